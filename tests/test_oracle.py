"""CPU tests of the oracle: pinned against golden hits produced by the
reference's own kernel code, against brute force, and unit checks of the
restated helpers."""
import math
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.join(os.path.dirname(__file__), "golden"))

from luxcore_gb300 import workloads as W  # noqa: E402
from oracle import pyoracle as po  # noqa: E402
from make_golden import SENTINEL, load  # noqa: E402

# bvh.cl fixtures (flat scenes) and mbvh.cl fixtures (instances; translating
# motion systems): bit-exact pins
GOLDEN = ["golden_random", "golden_heightfield", "golden_multimesh", "golden_instanced", "golden_motion_translate"]


@pytest.mark.parametrize("name", GOLDEN)
def test_oracle_matches_reference_kernel(name):
    scene, rays, ref = load(name)
    o = po.OracleScene(scene)  # BVHAccel for flat scenes, MBVHAccel with instances
    hits, _ = o.intersect(rays, n_threads=2)
    written = ref["meshIndex"] != SENTINEL          # masked rays are not written by the reference
    masked = (rays["flags"] & W.RAY_FLAGS_MASKED) != 0
    assert np.array_equal(~written, masked)
    # NaN in o, d or maxt: BVHAccel::Intersect (CPU) reports a miss because
    # `t < rayHit->t` is false for NaN (bvhaccel.cpp:233), while the GPU
    # kernel's `t > *maxt` test accepts a NaN t (triangle_funcs.cl:136-137)
    # and reports a NaN-t hit.  The oracle and the engine follow the CPU.
    nan_ray = (np.isnan(rays["o"]).any(1) | np.isnan(rays["d"]).any(1) | np.isnan(rays["maxt"]))
    assert (hits["meshIndex"][nan_ray] == W.NULL_INDEX).all()
    written &= ~nan_ray
    h, r = hits[written], ref[written]
    # t is bit-exact for every written ray (hit or miss: t = maxt on a miss)
    tt = (h["t"] == r["t"]) | (np.isnan(h["t"]) & np.isnan(r["t"]))
    assert tt.all(), np.nonzero(~tt)[0][:5]
    hit = r["meshIndex"] != W.NULL_INDEX
    assert np.array_equal(h["meshIndex"] != W.NULL_INDEX, hit)
    same = (h["meshIndex"] == r["meshIndex"]) & (h["triangleIndex"] == r["triangleIndex"])
    # differences only where two triangles give the same t (the reference
    # kernel keeps the last such hit, BVHAccel::Intersect the first); the
    # adversarial rays aim at shared vertices and edges to provoke them
    assert same.mean() >= 0.98
    wr = rays[written]
    for i in np.nonzero(~same)[0]:
        ok, t, _, _ = o.triangle_hit(wr[i], int(r["meshIndex"][i]), int(r["triangleIndex"][i]))
        assert ok and t == h["t"][i]
    bb = same & hit
    assert np.array_equal(h["b1"][bb], r["b1"][bb]) and np.array_equal(h["b2"][bb], r["b2"][bb])


def test_oracle_motion_matches_reference_kernel_within_tolerance():
    """Turning and scaling motion systems: the reference's own CPU code
    (motionsystem.cpp, quaternion.cpp; restated by the oracle) and its
    OpenCL kernel (motionsystem_funcs.cl, quaternion_funcs.cl; the fixture)
    sum Slerp's dot product in different orders, so their sampled matrices
    differ in the last bits: same triangles, t within 1e-4 relative (1e-5
    absolute below t = 0.1), barycentrics within 1e-3."""
    scene, rays, ref = load("golden_motion_rigid")
    o = po.OracleScene(scene)
    hits, _ = o.intersect(rays, n_threads=2)
    same = (hits["meshIndex"] == ref["meshIndex"]) & (hits["triangleIndex"] == ref["triangleIndex"])
    assert same.mean() >= 0.999
    hit = same & (ref["meshIndex"] != W.NULL_INDEX)
    assert hit.mean() > 0.3
    dt = np.abs(hits["t"][hit].astype(np.float64) - ref["t"][hit]) / np.maximum(np.abs(ref["t"][hit]), 0.1)
    assert dt.max() <= 1e-4
    assert np.abs(hits["b1"][hit].astype(np.float64) - ref["b1"][hit]).max() <= 1e-3
    assert np.abs(hits["b2"][hit].astype(np.float64) - ref["b2"][hit]).max() <= 1e-3
    # translating instances of the same scene (every third object) agree to the bit
    trans = hit & (ref["meshIndex"] % 3 == 1)
    assert trans.any() and np.array_equal(hits["t"][trans], ref["t"][trans])


@pytest.mark.skipif(not os.path.exists(po.REF_MBVH_LIB_PATH), reason="reference MBVH kernel not built here")
def test_oracle_mbvh_matches_reference_kernel_live():
    """Larger instanced and translating-motion scenes, traced by the
    reference's mbvh.cl compiled for the CPU: bit-exact agreement."""
    from make_golden import ref_mbvh_trace
    for scene, rays in (W.config3(n_rays=20000, seed=31, n_meshes=4, freq=12, n_inst=400, extent=4.0,
                                  scale=(0.1, 0.4))[:2],
                        W.config_motion(n_rays=20000, seed=32, n_meshes=4, freq=12, n_inst=400, extent=4.0,
                                        scale=(0.1, 0.4), kinds=("translate", "static"), speed=0.02,
                                        time_range=(-0.2, 1.2))[:2]):
        ref = ref_mbvh_trace(scene, rays)
        hits, _ = po.OracleScene(scene).intersect(rays)
        hit = ref["meshIndex"] != W.NULL_INDEX
        assert hit.mean() > 0.3
        assert np.array_equal(hits["meshIndex"], ref["meshIndex"])
        assert np.array_equal(hits["triangleIndex"], ref["triangleIndex"])
        assert np.array_equal(hits["t"], ref["t"])
        assert np.array_equal(hits["b1"][hit], ref["b1"][hit]) and np.array_equal(hits["b2"][hit], ref["b2"][hit])


def test_oracle_bvh_equals_brute_force():
    scene, rays = W.config1(n_tris=3000, n_rays=6000, seed=5)
    o = po.OracleScene(scene)
    hits, _ = o.intersect(rays)
    bf = o.brute_force(rays)
    assert np.array_equal(hits["t"], bf["t"])
    assert np.array_equal(hits["meshIndex"], bf["meshIndex"])
    assert np.array_equal(hits["triangleIndex"], bf["triangleIndex"])


@pytest.mark.parametrize("tree_type", [2, 4, 8])
def test_tree_types_agree(tree_type):
    scene, rays = W.config1(n_tris=1500, n_rays=3000, seed=6)
    h4, _ = po.OracleScene(scene, tree_type=4).intersect(rays)
    hx, _ = po.OracleScene(scene, tree_type=tree_type).intersect(rays)
    assert np.array_equal(h4["t"], hx["t"])


def test_mbvh_equals_brute_force_and_bvh():
    scene, rays, _ = W.config3(n_rays=4000, n_meshes=3, freq=6, n_inst=40, extent=2.0, scale=(0.2, 0.5))
    o = po.OracleScene(scene)
    assert o.accel == po.ACCEL_MBVH
    hits, _ = o.intersect(rays)
    bf = o.brute_force(rays)
    assert (hits["meshIndex"] != W.NULL_INDEX).mean() > 0.05
    assert np.array_equal(hits["t"], bf["t"])
    same = (hits["meshIndex"] == bf["meshIndex"]) & (hits["triangleIndex"] == bf["triangleIndex"])
    assert same.mean() > 0.999
    # plain meshes through MBVH give the same answer as BVH
    flat = W.SceneDesc([W.random_triangles(800, 3), W.random_triangles(600, 4)])
    r = W.random_rays(3000, 5)
    a, _ = po.OracleScene(flat, po.ACCEL_BVH).intersect(r)
    b, _ = po.OracleScene(flat, po.ACCEL_MBVH).intersect(r)
    assert np.array_equal(a["t"], b["t"]) and np.array_equal(a["meshIndex"], b["meshIndex"])


def test_matrix_inverse_and_epsilon():
    m = np.eye(4, dtype=np.float32)
    m[:3, :3] = np.array([[0.0, -0.03, 0.0], [0.03, 0.0, 0.0], [0.0, 0.0, 0.03]], np.float32)
    m[:3, 3] = [4.0, 5.0, 6.0]
    inv = po.matrix_inverse(m)
    assert np.allclose(inv.astype(np.float64) @ m.astype(np.float64), np.eye(4), atol=2e-4)
    assert po.matrix_inverse(np.zeros((4, 4), np.float32)) is None
    assert po.machine_epsilon(0.0) == pytest.approx(1e-5)
    assert po.machine_epsilon(1e9) == pytest.approx(0.1)
    e1 = po.machine_epsilon(1.0)
    assert e1 == pytest.approx(128 * 2.0 ** -23, rel=1e-6) or e1 == pytest.approx(1e-5)


def test_empty_scene_misses():
    scene = W.SceneDesc([W.Mesh(np.zeros((0, 3), np.float32), np.zeros((0, 3), np.uint32))])
    rays = W.random_rays(100, 1)
    hits, _ = po.OracleScene(scene).intersect(rays)
    assert (hits["meshIndex"] == W.NULL_INDEX).all()
    assert np.array_equal(hits["t"], rays["maxt"])


def test_morton_expand_matches_bit_loop():
    # the builder's 21->63 bit spread (lrx_build.cu expand21), checked in Python
    def expand(v):
        x = v & 0x1FFFFF
        x = (x | x << 32) & 0x1F00000000FFFF
        x = (x | x << 16) & 0x1F0000FF0000FF
        x = (x | x << 8) & 0x100F00F00F00F00F
        x = (x | x << 4) & 0x10C30C30C30C30C3
        x = (x | x << 2) & 0x1249249249249249
        return x
    rng = np.random.default_rng(0)
    for v in list(rng.integers(0, 1 << 21, 200)) + [0, 1, (1 << 21) - 1]:
        v = int(v)
        slow = sum(((v >> b) & 1) << (3 * b) for b in range(21))
        assert expand(v) == slow


def test_reference_layout_bytes_per_ray():
    """bench.py's B_ref: the reference layout's bytes per ray from the
    oracle's BVHAccel walk counts (32 B per node visit, 48 B per leaf visit,
    68 B of ray and hit)."""
    import bench
    desc = W.SceneDesc([W.heightfield_mesh(65, 7)])
    o = po.OracleScene(desc, po.ACCEL_BVH)
    rays = W.pinhole_rays(32, 32)
    got = bench.reference_layout_bytes(o, [("primary", rays)], stride=1)["primary"]
    nodes, leaves = o.visit_stats(rays)
    assert leaves > 0 and nodes >= leaves
    assert got["bytes_per_ray"] == round(48 + 20 + 32 * nodes + 48 * leaves, 1)
    assert got["nodes_per_ray"] == round(nodes, 2) and got["leaves_per_ray"] == round(leaves, 2)
