"""Generates the golden fixtures tests/golden/*.npz from the REFERENCE'S OWN
kernel code: include/luxrays/accelerators/bvh.cl with the geometry .cl files
it is stitched with (src/luxrays/accelerators/bvhaccelhw.cpp:189-202),
compiled for the CPU by oracle/build_ref.sh into oracle/_ref/.  The kernel
walks the BVHArrayNode[] of the oracle's restated classic builder.

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


def save(name: str, scene: W.SceneDesc, rays: np.ndarray):
    hits = ref_trace(scene, rays)
    d = {"rays": rays.view(np.uint8), "hits": hits.view(np.uint8), "n_meshes": np.array(len(scene.meshes))}
    for i, m in enumerate(scene.meshes):
        d[f"v{i}"] = m.vertices
        d[f"t{i}"] = m.triangles
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **d)
    hr = (hits["meshIndex"] != W.NULL_INDEX) & (hits["meshIndex"] != SENTINEL)
    print(name, rays.shape[0], "rays, hit rate", hr.mean())


def load(name: str):
    z = np.load(os.path.join(HERE, name + ".npz"))
    n = int(z["n_meshes"])
    scene = W.SceneDesc([W.Mesh(z[f"v{i}"], z[f"t{i}"]) for i in range(n)])
    return scene, z["rays"].view(W.RAY_DTYPE).copy(), z["hits"].view(W.HIT_DTYPE).copy()


def main():
    if not os.path.exists(po.REF_LIB_PATH):
        sys.exit("oracle/_ref/liblrx_refcl.so missing: run oracle/build_ref.sh first")
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


if __name__ == "__main__":
    main()
