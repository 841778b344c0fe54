"""The LuxRays-style C++ layer (include/lrx_luxrays.hpp): it compiles with
g++ alone (CPU test), and a C++ program driving it -- DataSet::Add of plain
and instanced meshes, GetAccelerator, NewHardwareIntersectionKernel,
EnqueueTraceRayBuffer, Update -- returns the oracle's hits (GPU test)."""
import os
import shutil
import subprocess
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.dirname(__file__))

from luxcore_gb300 import build as lbuild  # noqa: E402
from luxcore_gb300 import workloads as W  # noqa: E402
from parity import compare  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "luxrays_api_demo.cpp")
CUDA = "/usr/local/cuda"


def compile_demo(out_dir, syntax_only=False):
    cmd = ["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"), "-I", os.path.join(CUDA, "include"), SRC]
    if syntax_only:
        cmd += ["-fsyntax-only"]
    else:
        lib_dir = os.path.dirname(lbuild.LIB_PATH)
        cmd += ["-o", os.path.join(out_dir, "luxrays_api_demo"), "-L", lib_dir, "-llrx",
                f"-Wl,-rpath,{lib_dir}", "-L", os.path.join(CUDA, "lib64"), "-lcudart",
                f"-Wl,-rpath,{os.path.join(CUDA, 'lib64')}"]
    subprocess.check_call(cmd)
    return None if syntax_only else os.path.join(out_dir, "luxrays_api_demo")


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_header_compiles_with_gxx():
    compile_demo(None, syntax_only=True)


def scene_and_rays():
    base = W.displaced_icosphere(10, 601)
    objs = [(0, None), (1, None)]
    rng = np.random.default_rng(602)
    for k in range(30):
        m = np.eye(4, dtype=np.float32)
        m[:3, :3] *= rng.uniform(0.05, 0.15)
        m[:3, 3] = rng.uniform(0, 1, 3)
        objs.append((2, m))
    scene = W.SceneDesc([W.random_triangles(3000, 603), W.heightfield_mesh(30, 604), base], objs)
    moved = []
    for mi, m in objs:
        if m is None:
            moved.append((mi, None))
        else:
            m2 = m.copy()
            m2[:3, 3] += rng.uniform(-0.1, 0.1, 3).astype(np.float32)
            moved.append((mi, m2))
    return scene, W.SceneDesc(scene.meshes, moved), W.random_rays(30000, 605)


def write_input(path, scene, moved, rays):
    with open(path, "wb") as f:
        np.array([len(scene.meshes)], np.uint32).tofile(f)
        for m in scene.meshes:
            np.array([m.vertices.shape[0], m.triangles.shape[0]], np.uint32).tofile(f)
            np.ascontiguousarray(m.vertices, np.float32).tofile(f)
            np.ascontiguousarray(m.triangles, np.uint32).tofile(f)
        np.array([len(scene.objects)], np.uint32).tofile(f)
        for mi, m in scene.objects:
            np.array([mi, 0 if m is None else 1], np.uint32).tofile(f)
            (np.zeros(16, np.float32) if m is None else np.asarray(m, np.float32).reshape(16)).tofile(f)
        np.array([rays.shape[0]], np.uint32).tofile(f)
        np.ascontiguousarray(rays).tofile(f)
        for mi, m in moved.objects:
            (np.zeros(16, np.float32) if m is None else np.asarray(m, np.float32).reshape(16)).tofile(f)


@pytest.mark.gpu
def test_cpp_layer_matches_the_oracle(tmp_path, cuda_ready):
    from oracle import pyoracle as po
    exe = compile_demo(str(tmp_path))
    scene, moved, rays = scene_and_rays()
    inp = tmp_path / "scene.bin"
    write_input(str(inp), scene, moved, rays)
    out0, out1 = tmp_path / "hits0.bin", tmp_path / "hits1.bin"
    r = subprocess.run([exe, str(inp), str(out0), str(out1)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    for desc, out in ((scene, out0), (moved, out1)):
        gpu = np.fromfile(str(out), W.HIT_DTYPE)
        o = po.OracleScene(desc)
        ref, _ = o.intersect(rays)
        st = compare(gpu, ref, o, rays)
        assert st["ok"] and st["hit_rate"] > 0.05, st
