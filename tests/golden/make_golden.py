"""Generates the golden fixtures tests/golden/*.npz from the REFERENCE'S OWN
kernel code, compiled for the CPU by oracle/build_ref.sh into oracle/_ref/:
include/luxrays/accelerators/bvh.cl with the geometry .cl files it is
stitched with (src/luxrays/accelerators/bvhaccelhw.cpp:189-202) for flat
scenes, and mbvh.cl with the matrix, quaternion, transform and motion-system
.cl files (mbvhaccelhw.cpp:225-247) for instanced and motion-blurred scenes.
The kernels walk the oracle's restated classic builds (BVHArrayNode[], and
for MBVH the layout MBVHKernel uploads).

Run in a checkout next to the LuxCore source tree:
    oracle/build_ref.sh /path/to/LuxCore && python tests/golden/make_golden.py
Each fixture holds the scene, the rays and the reference kernel's hits.
Hits of masked rays keep the sentinel the buffer was filled with; b1/b2 of
misses are undefined in the reference kernel (bvh.cl:219-223) and are not
compared.
"""
import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

from luxcore_gb300 import workloads as W  # noqa: E402
from oracle import pyoracle as po  # noqa: E402
from adversarial import adversarial_rays  # noqa: E402

SENTINEL = 0xDEADBEEF


def ref_trace(scene: W.SceneDesc, rays: np.ndarray) -> np.ndarray:
    lib = ctypes.CDLL(po.REF_LIB_PATH)
    lib.refcl_bvh_trace.argtypes = [ctypes.c_void_p] * 2 + [ctypes.c_uint, ctypes.c_void_p, ctypes.c_void_p,
                                                             ctypes.c_int]
    o = po.OracleScene(scene, po.ACCEL_BVH)
    nodes = o.bvh_nodes()
    verts = np.ascontiguousarray(np.concatenate([m.vertices for m in scene.meshes]), np.float32)
    hits = np.zeros(rays.shape[0], W.HIT_DTYPE)
    hits.view(np.uint32).reshape(-1)[:] = SENTINEL
    rays = np.ascontiguousarray(rays)
    lib.refcl_bvh_trace(rays.ctypes.data, hits.ctypes.data, rays.shape[0], verts.ctypes.data, nodes.ctypes.data, 0)
    return hits


def ref_mbvh_trace(scene: W.SceneDesc, rays: np.ndarray) -> np.ndarray:
    """The reference's mbvh.cl (oracle/_ref/liblrx_refcl_mbvh.so) over the
    oracle's MBVH in MBVHKernel's upload layout."""
    lib = ctypes.CDLL(po.REF_MBVH_LIB_PATH)
    vp, u64 = ctypes.c_void_p, ctypes.c_ulonglong
    lib.refcl_mbvh_trace.argtypes = [vp, vp, ctypes.c_uint, vp, vp, u64, vp, u64, vp, u64, vp, u64, ctypes.c_int]
    o = po.OracleScene(scene, po.ACCEL_MBVH)
    e = o.mbvh_export()
    hits = np.zeros(rays.shape[0], W.HIT_DTYPE)
    hits.view(np.uint32).reshape(-1)[:] = SENTINEL
    rays = np.ascontiguousarray(rays)
    lib.refcl_mbvh_trace(rays.ctypes.data, hits.ctypes.data, rays.shape[0], e["verts"].ctypes.data,
                         e["nodes"].ctypes.data, e["nodes"].shape[0], e["mats"].ctypes.data, e["n_mats"],
                         e["motion_ranges"].ctypes.data, e["n_motions"], ctypes.addressof(e["intervals"]),
                         e["n_intervals"], 0)
    return hits


def save(name: str, scene: W.SceneDesc, rays: np.ndarray):
    """Flat scenes go through bvh.cl, scenes with instances or motion
    through mbvh.cl; the objects are stored with the meshes."""
    hits = ref_mbvh_trace(scene, rays) if scene.has_instances else ref_trace(scene, rays)
    d = {"rays": rays.view(np.uint8), "hits": hits.view(np.uint8), "n_meshes": np.array(len(scene.meshes))}
    for i, m in enumerate(scene.meshes):
        d[f"v{i}"] = m.vertices
        d[f"t{i}"] = m.triangles
    if scene.has_instances:
        # objects: mesh, kind (0 plain, 1 matrix, 2 motion), matrix, keyframe range
        n = len(scene.objects)
        mesh, kind = np.zeros(n, np.uint32), np.zeros(n, np.uint32)
        mats, krange = np.zeros((n, 16), np.float32), np.zeros((n, 2), np.int64)
        times, keys = [], []
        for k, (mi, m) in enumerate(scene.objects):
            mesh[k] = mi
            if isinstance(m, W.Motion):
                kind[k] = 2
                krange[k] = (len(times), len(times) + len(m.times))
                times += list(np.asarray(m.times, np.float32))
                keys += list(np.asarray(m.transforms, np.float32).reshape(-1, 16))
            elif m is not None:
                kind[k] = 1
                mats[k] = np.asarray(m, np.float32).reshape(16)
        d.update(obj_mesh=mesh, obj_kind=kind, obj_mat=mats, obj_keys=krange,
                 key_times=np.asarray(times, np.float32), key_mats=np.asarray(keys, np.float32).reshape(-1, 16))
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **d)
    hr = (hits["meshIndex"] != W.NULL_INDEX) & (hits["meshIndex"] != SENTINEL)
    print(name, rays.shape[0], "rays, hit rate", hr.mean())


def load(name: str):
    z = np.load(os.path.join(HERE, name + ".npz"))
    n = int(z["n_meshes"])
    meshes = [W.Mesh(z[f"v{i}"], z[f"t{i}"]) for i in range(n)]
    objects = []
    if "obj_mesh" in z:
        for k in range(z["obj_mesh"].shape[0]):
            mi, kind = int(z["obj_mesh"][k]), int(z["obj_kind"][k])
            if kind == 2:
                a, b = z["obj_keys"][k]
                objects.append((mi, W.Motion(z["key_times"][a:b].copy(), z["key_mats"][a:b].reshape(-1, 4, 4).copy())))
            else:
                objects.append((mi, z["obj_mat"][k].reshape(4, 4).copy() if kind == 1 else None))
    scene = W.SceneDesc(meshes, objects)
    return scene, z["rays"].view(W.RAY_DTYPE).copy(), z["hits"].view(W.HIT_DTYPE).copy()


def main():
    if not (os.path.exists(po.REF_LIB_PATH) and os.path.exists(po.REF_MBVH_LIB_PATH)):
        sys.exit("oracle/_ref/liblrx_refcl*.so missing: run oracle/build_ref.sh first")
    # random small triangles (config-1 generator, scaled down) + adversarial rays
    sc = W.SceneDesc([W.random_triangles(2048, 11)])
    rays = np.concatenate([W.random_rays(4096, 12), adversarial_rays(sc.meshes[0], 13, 32)])
    save("golden_random", sc, rays)
    # heightfield with shared edges and vertices: ties
    hf = W.heightfield_mesh(33, 14)
    sc = W.SceneDesc([hf])
    rays = np.concatenate([W.pinhole_rays(48, 48), adversarial_rays(hf, 15, 32)])
    save("golden_heightfield", sc, rays)
    # several meshes: meshIndex = DataSet order
    sc = W.SceneDesc([W.random_triangles(700, 16), W.random_triangles(500, 17), W.heightfield_mesh(9, 18)])
    rays = W.random_rays(4096, 19)
    save("golden_multimesh", sc, rays)
    # two-level: plain meshes and affine instances (mbvh.cl with transforms)
    sc, closest, _ = W.config3(n_rays=4096, seed=20, n_meshes=3, freq=8, n_inst=60, extent=2.0, scale=(0.1, 0.3))
    sc = W.SceneDesc(sc.meshes + [W.random_triangles(300, 21)], sc.objects + [(3, None)])
    rays = np.concatenate([closest, adversarial_rays(sc.meshes[0], 22, 16)])
    save("golden_instanced", sc, rays)
    # motion systems: translating and static instances, ray times before, in and after the keyframes
    sc, closest, _ = W.config_motion(n_rays=4096, seed=23, n_meshes=3, freq=8, n_inst=60, extent=2.0,
                                     scale=(0.1, 0.3), kinds=("translate", "static"), time_range=(-0.25, 1.25),
                                     speed=0.02)
    save("golden_motion_translate", sc, closest)
    # turning, scaling and moving instances (Slerp): compared with a tolerance
    sc, closest, _ = W.config_motion(n_rays=4096, seed=24, n_meshes=3, freq=8, n_inst=60, extent=2.0,
                                     scale=(0.1, 0.3), kinds=("rigid", "translate", "static"),
                                     time_range=(-0.1, 1.1), speed=0.02)
    save("golden_motion_rigid", sc, closest)


if __name__ == "__main__":
    main()
