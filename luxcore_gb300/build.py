"""Builds liblrx.so (the C-ABI engine) in-tree for sm_103a.

Each translation unit compiles in parallel with nvcc (one -gencode, no
cmake); the host-only unit goes through g++ with the CUDA include path.
Host FP32 code is compiled with -ffp-contract=off so the restated
Matrix4x4::Inverse rounds exactly like the reference's.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OBJ_DIR = os.path.join(HERE, "_build")
LIB_DIR = os.path.join(HERE, "lib")
LIB_PATH = os.path.join(LIB_DIR, "liblrx.so")
ROOT = os.path.dirname(HERE)

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
              "-Xcompiler", "-fPIC,-ffp-contract=off", "-Xptxas", "-v"]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-Wall"]


def _cuda_home() -> str:
    for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if c and os.path.exists(os.path.join(c, "bin", "nvcc")):
            return c
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(nvcc))
    raise RuntimeError("nvcc not found")


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))


def headers():
    h = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    h.append(os.path.join(ROOT, "include", "lrx.h"))
    return h


def _compile(src: str, cuda: str, log_dir: str) -> str:
    obj = os.path.join(OBJ_DIR, os.path.basename(src) + ".o")
    if src.endswith(".cu"):
        cmd = [os.path.join(cuda, "bin", "nvcc"), *ARCH, *NVCC_FLAGS, "-c", src, "-o", obj]
    else:
        cmd = [os.environ.get("CXX", "g++"), *CXX_FLAGS, "-I", os.path.join(cuda, "include"), "-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    with open(os.path.join(log_dir, os.path.basename(src) + ".log"), "w") as f:
        f.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {src}\n{r.stdout}\n{r.stderr}")
    return obj


def up_to_date() -> bool:
    if not os.path.exists(LIB_PATH):
        return False
    t = os.path.getmtime(LIB_PATH)
    return all(os.path.getmtime(p) <= t for p in sources() + headers() + [__file__])


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and up_to_date():
        return LIB_PATH
    cuda = _cuda_home()
    os.makedirs(OBJ_DIR, exist_ok=True)
    os.makedirs(LIB_DIR, exist_ok=True)
    srcs = sources()
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(srcs), os.cpu_count() or 4))) as ex:
        objs = list(ex.map(lambda s: _compile(s, cuda, OBJ_DIR), srcs))
    tmp = LIB_PATH + f".tmp{os.getpid()}"
    cmd = [os.path.join(cuda, "bin", "nvcc"), *ARCH, "-shared", "-o", tmp, *objs,
           "-Xcompiler", "-fPIC", "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB_PATH)
    if verbose:
        for s in srcs:
            with open(os.path.join(OBJ_DIR, os.path.basename(s) + ".log")) as f:
                sys.stdout.write(f.read())
    return LIB_PATH


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
