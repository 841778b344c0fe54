"""ctypes wrapper of the CPU oracle -- TEST INFRASTRUCTURE.

Only tests/, the smoke check and bench.py's CPU-baseline / reference legs
import this module.  The oracle restates LuxRays' BVHAccel / MBVHAccel
(src/luxrays/accelerators/bvhaccel.cpp:72-260, mbvhaccel.cpp:58-357); see
lrx_oracle.h for the full list of restated functions.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liblrx_oracle.so")
REF_LIB_PATH = os.path.join(HERE, "_ref", "liblrx_refcl.so")
REF_MBVH_LIB_PATH = os.path.join(HERE, "_ref", "liblrx_refcl_mbvh.so")
# the reference's CUDA kernel text (stitched by build_ref.sh from the LuxCore
# tree) and the host harness that compiles and launches it on the GPU
REFCU_SRC_PATH = os.path.join(HERE, "_ref", "refcu_bvh_kernel.cu")
REFCU_LIB_PATH = os.path.join(HERE, "_build", "liblrx_refcu.so")

ACCEL_BVH, ACCEL_MBVH = 0, 1

_lib = None
_lock = threading.Lock()


class OrcObject(ctypes.Structure):
    _fields_ = [("mesh", ctypes.c_uint32), ("has_transform", ctypes.c_uint32),
                ("m", ctypes.c_float * 16)]


class OrcInterval(ctypes.Structure):
    _fields_ = [("startTime", ctypes.c_float), ("endTime", ctypes.c_float), ("start", ctypes.c_float * 16),
                ("end", ctypes.c_float * 16), ("R", ctypes.c_float * 32), ("ST", ctypes.c_float * 12),
                ("Q", ctypes.c_float * 8), ("has", ctypes.c_int32 * 10)]


class OrcMotionDesc(ctypes.Structure):
    _fields_ = [("object", ctypes.c_uint32), ("count", ctypes.c_uint32), ("times", ctypes.c_void_p),
                ("transforms", ctypes.c_void_p)]


def build(force: bool = False) -> str:
    """Compile the oracle with g++ (-O2 -ffp-contract=off, no fast math)."""
    src = os.path.join(HERE, "lrx_oracle.cpp")
    deps = [src] + [os.path.join(HERE, h) for h in ("lrx_oracle.h", "lrx_oracle_motion.h")]
    if not force and os.path.exists(LIB_PATH) and os.path.getmtime(LIB_PATH) >= max(
            os.path.getmtime(d) for d in deps):
        return LIB_PATH
    os.makedirs(os.path.dirname(LIB_PATH), exist_ok=True)
    tmp = LIB_PATH + f".tmp{os.getpid()}"
    subprocess.check_call(["g++", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
                           "-std=c++17", "-pthread", src, "-o", tmp])
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


def _cuda_home() -> str | None:
    for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if c and os.path.exists(os.path.join(c, "include", "nvrtc.h")):
            return c
    return None


def build_refcu(force: bool = False) -> str | None:
    """Compile the host harness of the reference's CUDA kernel (NVRTC +
    driver API; it holds no kernel code of its own).  None when the CUDA
    toolkit's NVRTC is absent."""
    cuda = _cuda_home()
    if cuda is None:
        return None
    src = os.path.join(HERE, "refcu_harness.cpp")
    if not force and os.path.exists(REFCU_LIB_PATH) and os.path.getmtime(REFCU_LIB_PATH) >= os.path.getmtime(src):
        return REFCU_LIB_PATH
    os.makedirs(os.path.dirname(REFCU_LIB_PATH), exist_ok=True)
    lib64 = os.path.join(cuda, "lib64")
    tmp = REFCU_LIB_PATH + f".tmp{os.getpid()}"
    subprocess.check_call(["g++", "-O2", "-fPIC", "-shared", "-std=c++17", src, "-o", tmp,
                           "-I", os.path.join(cuda, "include"), "-L", lib64, "-L", os.path.join(lib64, "stubs"),
                           f"-Wl,-rpath,{lib64}", "-lnvrtc", "-lcuda"])
    os.replace(tmp, REFCU_LIB_PATH)
    return REFCU_LIB_PATH


class RefCudaKernel:
    """The reference's own CUDA intersection kernel (bvh.cl's
    Accelerator_Intersect_RayBuffer, compiled by NVRTC as the reference's
    CUDA device compiles it -- with its PATHOCL engine's --use_fast_math, or
    without it) on the current GPU, over the oracle's
    BVHArrayNode[] (OracleScene.bvh_nodes) and the concatenated mesh
    vertices.  `available` is False, with `reason`, when the kernel text (a
    build product of the reference tree) or the harness is missing."""

    def __init__(self, fast_math: bool = True):
        self.available, self.reason, self.info = False, "", ""
        self.fast_math = 1 if fast_math else 0
        if not os.path.exists(REFCU_SRC_PATH):
            self.reason = "reference kernel text not built (oracle/build_ref.sh needs the LuxCore source tree)"
            return
        path = build_refcu()
        if path is None:
            self.reason = "NVRTC not found"
            return
        try:
            self.L = ctypes.CDLL(path)
        except OSError as e:  # no CUDA driver on this machine
            self.reason = f"harness not loadable: {e}"
            return
        self.L.refcu_load.restype = ctypes.c_int
        self.L.refcu_load.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.c_char_p, ctypes.c_size_t]
        self.L.refcu_trace.restype = ctypes.c_int
        self.L.refcu_trace.argtypes = [ctypes.c_int, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint32,
                                       ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint32, ctypes.c_void_p]
        buf = ctypes.create_string_buffer(4096)
        rc = self.L.refcu_load(REFCU_SRC_PATH.encode(), self.fast_math, buf, len(buf))
        self.info = buf.value.decode(errors="replace")
        if rc != 0:
            self.reason = f"refcu_load failed ({rc}): {self.info}"
            return
        self.available = True

    def trace(self, d_rays: int, d_hits: int, count: int, d_verts: int, d_nodes: int, block: int = 32,
              stream: int = 0):
        rc = self.L.refcu_trace(self.fast_math, d_rays, d_hits, count, d_verts, d_nodes, block, ctypes.c_void_p(stream))
        if rc != 0:
            raise RuntimeError(f"refcu_trace: CUresult {rc}")


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            L = ctypes.CDLL(LIB_PATH)
            vp, u32, u64 = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint64
            L.orc_scene_create.restype = vp
            L.orc_scene_create.argtypes = [vp, vp, vp, vp, u32, vp, u32, ctypes.c_int, ctypes.c_int,
                                           ctypes.c_char_p, u64]
            L.orc_scene_create_motion.restype = vp
            L.orc_scene_create_motion.argtypes = [vp, vp, vp, vp, u32, vp, u32, vp, u32, ctypes.c_int,
                                                  ctypes.c_int, ctypes.c_char_p, u64]
            L.orc_scene_destroy.argtypes = [vp]
            L.orc_intersect.restype = ctypes.c_double
            L.orc_intersect.argtypes = [vp, vp, vp, u64, ctypes.c_int]
            L.orc_brute_force.argtypes = [vp, vp, vp, u64, ctypes.c_int]
            L.orc_triangle_hit.restype = ctypes.c_int
            L.orc_triangle_hit.argtypes = [vp, vp, u32, u32, vp, vp, vp]
            L.orc_bvh_node_count.restype = u64
            L.orc_bvh_node_count.argtypes = [vp]
            L.orc_bvh_nodes.argtypes = [vp, vp]
            L.orc_visit_stats.argtypes = [vp, vp, u64, vp, vp]
            L.orc_mbvh_export.restype = ctypes.c_int
            L.orc_mbvh_export.argtypes = [vp, vp, vp, vp, vp, vp, vp]
            L.orc_matrix_inverse.restype = ctypes.c_int
            L.orc_matrix_inverse.argtypes = [vp, vp]
            L.orc_machine_epsilon.restype = ctypes.c_float
            L.orc_machine_epsilon.argtypes = [ctypes.c_float]
            _lib = L
    return _lib


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


class OracleScene:
    """LuxRays DataSet + BVHAccel (accel=ACCEL_BVH) or MBVHAccel (ACCEL_MBVH),
    built with the classic builder (tree type 4 by default)."""

    def __init__(self, scene, accel: int | None = None, tree_type: int = 4):
        L = lib()
        if accel is None:
            accel = ACCEL_MBVH if scene.has_instances else ACCEL_BVH
        verts = [np.ascontiguousarray(m.vertices, np.float32).reshape(-1, 3) for m in scene.meshes]
        tris = [np.ascontiguousarray(m.triangles, np.uint32).reshape(-1, 3) for m in scene.meshes]
        self._verts = np.concatenate(verts) if verts else np.zeros((0, 3), np.float32)
        self._tris = np.concatenate(tris) if tris else np.zeros((0, 3), np.uint32)
        self._vo = np.zeros(len(verts) + 1, np.uint64)
        self._to = np.zeros(len(tris) + 1, np.uint64)
        self._vo[1:] = np.cumsum([v.shape[0] for v in verts])
        self._to[1:] = np.cumsum([t.shape[0] for t in tris])
        objs = (OrcObject * max(1, len(scene.objects)))()
        motions = []
        for i, (mi, m) in enumerate(scene.objects):
            objs[i].mesh = mi
            if m is not None and hasattr(m, "times"):
                motions.append((i, m))
            elif m is not None:
                objs[i].has_transform = 1
                flat = np.asarray(m, np.float32).reshape(16)
                for k in range(16):
                    objs[i].m[k] = float(flat[k])
        mds = (OrcMotionDesc * max(1, len(motions)))()
        self._motion_keep = []
        for k, (i, m) in enumerate(motions):
            t = np.ascontiguousarray(m.times, np.float32).reshape(-1)
            x = np.ascontiguousarray(m.transforms, np.float32).reshape(-1)
            self._motion_keep += [t, x]
            mds[k].object, mds[k].count = i, t.shape[0]
            mds[k].times, mds[k].transforms = t.ctypes.data, x.ctypes.data
        err = ctypes.create_string_buffer(512)
        self.handle = L.orc_scene_create_motion(_ptr(self._verts), _ptr(self._vo), _ptr(self._tris), _ptr(self._to),
                                                len(scene.meshes), objs, len(scene.objects), mds, len(motions),
                                                accel, tree_type, err, 512)
        if not self.handle:
            raise RuntimeError("oracle scene build failed: " + err.value.decode())
        self.accel = accel

    def __del__(self):
        if getattr(self, "handle", None) and _lib is not None:
            _lib.orc_scene_destroy(self.handle)
            self.handle = None

    def intersect(self, rays: np.ndarray, n_threads: int = 0):
        """Accelerator::Intersect per ray; returns (hits, seconds)."""
        from luxcore_gb300.workloads import HIT_DTYPE
        rays = np.ascontiguousarray(rays)
        hits = np.zeros(rays.shape[0], HIT_DTYPE)
        secs = lib().orc_intersect(self.handle, _ptr(rays), _ptr(hits), rays.shape[0], n_threads)
        return hits, secs

    def brute_force(self, rays: np.ndarray, n_threads: int = 0) -> np.ndarray:
        from luxcore_gb300.workloads import HIT_DTYPE
        rays = np.ascontiguousarray(rays)
        hits = np.zeros(rays.shape[0], HIT_DTYPE)
        lib().orc_brute_force(self.handle, _ptr(rays), _ptr(hits), rays.shape[0], n_threads)
        return hits

    def triangle_hit(self, ray: np.ndarray, mesh_index: int, tri_index: int):
        """(hit, t, b1, b2) of Triangle::Intersect against one triangle."""
        t, b1, b2 = ctypes.c_float(), ctypes.c_float(), ctypes.c_float()
        r = np.ascontiguousarray(ray.reshape(1))
        ok = lib().orc_triangle_hit(self.handle, _ptr(r), mesh_index, tri_index,
                                    ctypes.byref(t), ctypes.byref(b1), ctypes.byref(b2))
        return bool(ok), t.value, b1.value, b2.value

    def bvh_nodes(self) -> np.ndarray:
        n = lib().orc_bvh_node_count(self.handle)
        out = np.zeros((n, 8), np.uint32)
        if n:
            lib().orc_bvh_nodes(self.handle, _ptr(out))
        return out

    def mbvh_export(self):
        """The MBVH in MBVHKernel's upload layout: dict of nodes (n, 8) uint32,
        verts (n, 3) float32, mats (n, 16) float32, motion ranges (n, 2)
        uint32 and an OrcInterval array."""
        L = lib()
        counts = (ctypes.c_uint64 * 4)()
        if not L.orc_mbvh_export(self.handle, counts, None, None, None, None, None):
            raise ValueError("not an MBVH scene")
        nn, nv, nm, packed = (int(c) for c in counts)
        nms, nits = packed & 0xFFFFFFFF, packed >> 32
        out = {"nodes": np.zeros((nn, 8), np.uint32), "verts": np.zeros((max(nv, 1), 3), np.float32),
               "mats": np.zeros((max(nm, 1), 16), np.float32), "motion_ranges": np.zeros((max(nms, 1), 2), np.uint32),
               "intervals": (OrcInterval * max(nits, 1))(), "n_mats": nm, "n_motions": nms, "n_intervals": nits}
        L.orc_mbvh_export(self.handle, counts, _ptr(out["nodes"]), _ptr(out["verts"]), _ptr(out["mats"]),
                          _ptr(out["motion_ranges"]), out["intervals"])
        return out

    def visit_stats(self, rays: np.ndarray):
        rays = np.ascontiguousarray(rays)
        a, b = ctypes.c_double(), ctypes.c_double()
        lib().orc_visit_stats(self.handle, _ptr(rays), rays.shape[0], ctypes.byref(a), ctypes.byref(b))
        return a.value, b.value


def matrix_inverse(m: np.ndarray):
    m = np.ascontiguousarray(m, np.float32).reshape(16)
    out = np.zeros(16, np.float32)
    ok = lib().orc_matrix_inverse(_ptr(m), _ptr(out))
    return out.reshape(4, 4) if ok else None


def machine_epsilon(v: float) -> float:
    return lib().orc_machine_epsilon(v)
