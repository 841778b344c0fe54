"""GPU parity tests: the CUDA engine through the C ABI against the oracle
(BVHAccel / MBVHAccel restated) and against golden hits of the reference's
own kernel code.  Bar: parity.compare (>= 99.99 % index agreement, every
disagreement an exact-t tie re-tested on the oracle, t/b1/b2 within 1e-5
relative -- in practice bit-exact)."""
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.dirname(__file__))
sys.path.insert(0, os.path.join(os.path.dirname(__file__), "golden"))

from luxcore_gb300 import lrx  # noqa: E402
from luxcore_gb300 import workloads as W  # noqa: E402
from oracle import pyoracle as po  # noqa: E402
from adversarial import adversarial_rays  # noqa: E402
from parity import check_anyhit, compare  # noqa: E402

pytestmark = pytest.mark.gpu

SENT = 0xDEADBEEF
# launch configurations every parity test runs under:
# (block size, postpone, variant bits[, refill])
KERNEL_CONFIGS = [(128, 0, 0), (64, 8, 0), (256, 24, 0), (64, 8, 0xF), (128, 8, 0x7),
                  (64, 8, 0x10), (32, 8, 0x1F), (64, 8, 0x30),
                  (64, 8, 0x40), (128, 0, 0x41, 1), (32, 8, 0x46, 32),
                  (64, 8, 0x50, 8), (64, 8, 0xC0, 8), (256, 8, 0x80), (64, 8, 0x90),
                  (64, 8, 0x140, 8), (64, 8, 0x440, 8), (128, 8, 0x840, 8), (64, 8, 0x410), (128, 0, 0x800),
                  (64, 0, 0x2040, 8), (128, 8, 0x2046, 1)]
KERNELS = pytest.mark.parametrize("kernel", KERNEL_CONFIGS,
                                  ids=["b128", "b64-p8", "b256-p24", "b64-p8-allvariants", "b128-p8-mm3-hints",
                                       "b64-p8-sorted", "b32-p8-sorted-all", "b64-p8-octsort",
                                       "b64-p8-persistent", "b128-persistent-refill1",
                                       "b32-p8-persistent-refill32-hints", "b64-p8-sorted-persistent-refill8",
                                       "b64-p8-persistent-smemstack", "b256-p8-smemstack", "b64-p8-sorted-smemstack",
                                       "b64-p8-persistent-compact", "b64-p8-persistent-smemstack16",
                                       "b128-p8-persistent-smemstack32", "b64-p8-sorted-smemstack16",
                                       "b128-smemstack32", "b64-persistent-drainsplit",
                                       "b128-p8-persistent-drainsplit-hints-refill1"])


def make_scene(desc, kernel=(64, 8, 0), **kw):
    s = lrx.Scene(desc, **kw)
    refill = kernel[3] if len(kernel) > 3 else 0
    s.set_trace_config(*kernel[:3], refill=refill)
    assert s.trace_config() == {"block_size": kernel[0], "postpone": kernel[1], "variant": kernel[2],
                                "refill": refill}
    return s


@pytest.fixture(scope="module")
def torch_cuda(cuda_ready):
    import torch
    return torch


def gpu_trace(torch, scene, rays, mode=lrx.LRX_TRACE_CLOSEST, prefill=SENT, chunks=1):
    n = rays.shape[0]
    d_r = torch.from_numpy(np.ascontiguousarray(rays).view(np.uint8).reshape(-1).copy()).cuda()
    d_h = torch.empty(n * 20, dtype=torch.uint8, device="cuda")
    d_h.view(torch.int32).fill_(np.int32(np.uint32(prefill).view(np.int32)).item())
    st = torch.cuda.current_stream().cuda_stream
    bounds = np.linspace(0, n, chunks + 1).astype(np.int64)
    for a, b in zip(bounds[:-1], bounds[1:]):
        if b > a:
            scene.trace(d_r.data_ptr() + 48 * int(a), d_h.data_ptr() + 20 * int(a), int(b - a), mode, st)
    torch.cuda.synchronize()
    assert scene.device_status(st) == 0
    return d_h.cpu().numpy().view(W.HIT_DTYPE).copy()


def assert_parity(gpu, ref, oracle, rays, min_hit_rate=0.0):
    st = compare(gpu, ref, oracle, rays)
    assert st["ok"], st
    assert st["hit_rate"] >= min_hit_rate, st
    return st


# ---------------------------------------------------------------------------


@pytest.mark.parametrize("name", ["golden_random", "golden_heightfield", "golden_multimesh", "golden_instanced",
                                  "golden_motion_translate"])
@KERNELS
def test_golden_fixtures(torch_cuda, kernel, name):
    """Hits of the reference's own kernel text (bvh.cl, or mbvh.cl for the
    instanced and motion fixtures) compiled for the CPU."""
    from make_golden import load
    scene, rays, ref = load(name)
    s = make_scene(scene, kernel)
    gpu = gpu_trace(torch_cuda, s, rays)
    masked = (rays["flags"] & W.RAY_FLAGS_MASKED) != 0
    # masked rays: hit left untouched (bvh.cl:243-244)
    assert (gpu.view(np.uint32).reshape(-1, 5)[masked] == SENT).all()
    nan_ray = np.isnan(rays["o"]).any(1) | np.isnan(rays["d"]).any(1) | np.isnan(rays["maxt"])
    # NaN rays: misses, as BVHAccel::Intersect returns them
    assert (gpu["meshIndex"][nan_ray] == W.NULL_INDEX).all()
    keep = ~masked & ~nan_ray
    oracle = po.OracleScene(scene)
    g, r, rr = gpu[keep], ref[keep], rays[keep]
    st = compare(g, r, oracle, rr)
    assert st["bad_disagreements"] == 0 and st["values_ok"] and st["ties_valid"], st
    # and against the oracle itself: these fixtures aim rays at shared
    # vertices and edges, so the rate bar does not apply -- every
    # disagreement must be an exact-t tie that re-tests as a hit
    oh, _ = oracle.intersect(rays)
    st = compare(gpu[keep], oh[keep], oracle, rr)
    assert st["bad_disagreements"] == 0 and st["values_ok"] and st["ties_valid"], st
    assert st["agree"] >= 0.99, st


@KERNELS
def test_config1_full_scene(torch_cuda, kernel):
    """65,536 random triangles (config 1's scene), 262,144 of its rays."""
    scene, rays = W.config1(n_rays=1 << 18)
    s = make_scene(scene, kernel)
    oracle = po.OracleScene(scene)
    ref, _ = oracle.intersect(rays)
    gpu = gpu_trace(torch_cuda, s, rays)
    st = assert_parity(gpu, ref, oracle, rays, min_hit_rate=0.3)
    assert st["bitexact_t"] == 1.0
    anyh = gpu_trace(torch_cuda, s, rays, lrx.LRX_TRACE_ANY)
    a = check_anyhit(anyh, ref, oracle, rays)
    assert a["ok"], a


@KERNELS
def test_heightfield_primary_bounce_shadow(torch_cuda, kernel):
    """Config 2's three ray sets on a 256x256 heightfield."""
    mesh = W.heightfield_mesh(256, 21)
    scene = W.SceneDesc([mesh])
    s = make_scene(scene, kernel)
    oracle = po.OracleScene(scene)
    prim = W.pinhole_rays(256, 256)
    ref_p, _ = oracle.intersect(prim)
    gpu_p = gpu_trace(torch_cuda, s, prim)
    assert_parity(gpu_p, ref_p, oracle, prim, min_hit_rate=0.2)
    bounce = W.bounce_rays(scene, prim, gpu_p, 1 << 16, 22)
    ref_b, _ = oracle.intersect(bounce)
    gpu_b = gpu_trace(torch_cuda, s, bounce)
    assert_parity(gpu_b, ref_b, oracle, bounce, min_hit_rate=0.05)
    shadow = W.shadow_rays(bounce, 4, 23)
    ref_s, _ = oracle.intersect(shadow)
    any_s = gpu_trace(torch_cuda, s, shadow, lrx.LRX_TRACE_ANY)
    a = check_anyhit(any_s, ref_s, oracle, shadow)
    assert a["ok"], a


@KERNELS
def test_instanced_two_level(torch_cuda, kernel):
    """Config 3 in small: displaced icospheres under random affine instances."""
    scene, closest, anyr = W.config3(n_rays=1 << 15, n_meshes=4, freq=12, n_inst=300, extent=3.0,
                                     scale=(0.1, 0.4))
    s = make_scene(scene, kernel)
    info = s.info()
    assert info["two_level"] == 1 and info["instance_count"] == 300 and info["blas_count"] == 4
    oracle = po.OracleScene(scene)
    ref, _ = oracle.intersect(closest)
    gpu = gpu_trace(torch_cuda, s, closest)
    st = assert_parity(gpu, ref, oracle, closest, min_hit_rate=0.1)
    assert st["bitexact_t"] == 1.0
    ref_a, _ = oracle.intersect(anyr)
    gpu_a = gpu_trace(torch_cuda, s, anyr, lrx.LRX_TRACE_ANY)
    a = check_anyhit(gpu_a, ref_a, oracle, anyr)
    assert a["ok"], a


@KERNELS
def test_plain_and_instanced_objects_mixed(torch_cuda, kernel):
    base = W.displaced_icosphere(8, 31)
    objs = [(1, None), (0, None)]
    rng = np.random.default_rng(4)
    for k in range(20):
        m = np.eye(4, dtype=np.float32)
        m[:3, :3] *= rng.uniform(0.05, 0.2)
        m[:3, 3] = rng.uniform(0, 1, 3)
        objs.append((2, m))
    scene = W.SceneDesc([W.random_triangles(500, 32), W.random_triangles(300, 33), base], objs)
    s = make_scene(scene, kernel)
    rays = W.random_rays(20000, 34)
    oracle = po.OracleScene(scene)
    ref, _ = oracle.intersect(rays)
    gpu = gpu_trace(torch_cuda, s, rays)
    assert_parity(gpu, ref, oracle, rays, min_hit_rate=0.05)
    meshes_hit = set(np.unique(gpu["meshIndex"]).tolist())
    assert {0, 1} <= meshes_hit and any(m >= 2 and m != W.NULL_INDEX for m in meshes_hit)


@KERNELS
def test_adversarial_rays(torch_cuda, kernel):
    mesh = W.heightfield_mesh(64, 41)
    scene = W.SceneDesc([mesh])
    rays = adversarial_rays(mesh, 42, 64)
    s = make_scene(scene, kernel)
    gpu = gpu_trace(torch_cuda, s, rays)
    oracle = po.OracleScene(scene)
    ref, _ = oracle.intersect(rays)
    masked = (rays["flags"] & W.RAY_FLAGS_MASKED) != 0
    assert (gpu.view(np.uint32).reshape(-1, 5)[masked] == SENT).all()
    st = compare(gpu[~masked], ref[~masked], oracle, rays[~masked])
    assert st["bad_disagreements"] == 0 and st["values_ok"] and st["ties_valid"], st
    anyh = gpu_trace(torch_cuda, s, rays, lrx.LRX_TRACE_ANY)
    a = check_anyhit(anyh[~masked], ref[~masked], oracle, rays[~masked])
    assert a["ok"], a


def test_maxt_equal_to_the_hit_distance_is_a_miss(torch_cuda):
    """A ray whose maxt is exactly its closest hit's t misses that triangle
    (the reference keeps a hit only when t < the current t, which starts at
    maxt), in both modes; maxt one ulp above finds it again."""
    scene, rays = W.config1(n_tris=20000, n_rays=1 << 14, seed=77)
    oracle = po.OracleScene(scene)
    ref, _ = oracle.intersect(rays)
    hit = ref["meshIndex"] != W.NULL_INDEX
    assert hit.mean() > 0.1
    at = rays.copy()
    at["maxt"][hit] = ref["t"][hit]
    above = rays.copy()
    above["maxt"][hit] = np.nextafter(ref["t"][hit], np.float32(np.inf))
    s = lrx.Scene(scene)
    for r in (at, above):
        want, _ = oracle.intersect(r)
        assert_parity(gpu_trace(torch_cuda, s, r), want, oracle, r)
        a = check_anyhit(gpu_trace(torch_cuda, s, r, lrx.LRX_TRACE_ANY), want, oracle, r)
        assert a["ok"], a
    want_at, _ = oracle.intersect(at)
    assert (want_at["meshIndex"][hit] != ref["meshIndex"][hit]).mean() > 0.99


@pytest.mark.parametrize("n_tris", [0, 1, 2, 3, 4, 9, 25])
@KERNELS
def test_tiny_and_empty_scenes(torch_cuda, kernel, n_tris):
    mesh = W.random_triangles(n_tris, 50 + n_tris, size=0.3) if n_tris else W.Mesh(
        np.zeros((0, 3), np.float32), np.zeros((0, 3), np.uint32))
    scene = W.SceneDesc([mesh])
    s = make_scene(scene, kernel)
    rays = W.random_rays(4096, 51)
    gpu = gpu_trace(torch_cuda, s, rays)
    oracle = po.OracleScene(scene)
    ref, _ = oracle.intersect(rays)
    assert_parity(gpu, ref, oracle, rays)
    if n_tris == 0:
        assert np.array_equal(gpu["t"], rays["maxt"])


def test_degenerate_coincident_triangles(torch_cuda):
    """Many identical triangles: equal Morton codes, equal t -> lowest index."""
    v = np.array([[0.2, 0.2, 0.5], [0.8, 0.2, 0.5], [0.5, 0.8, 0.5]], np.float32)
    n = 3000
    mesh = W.Mesh(np.tile(v, (n, 1)), np.arange(3 * n, dtype=np.uint32).reshape(n, 3))
    scene = W.SceneDesc([mesh])
    s = lrx.Scene(scene)
    rng = np.random.default_rng(3)
    o = np.concatenate([rng.uniform(0.3, 0.6, (512, 2)), np.zeros((512, 1))], 1).astype(np.float32)
    rays = W.make_rays(o, np.tile(np.array([[0, 0, 1]], np.float32), (512, 1)), 1e-4, 1e30)
    gpu = gpu_trace(torch_cuda, s, rays)
    hit = gpu["meshIndex"] != W.NULL_INDEX
    assert hit.mean() > 0.5
    assert (gpu["triangleIndex"][hit] == 0).all()
    assert s.info()["max_depth"] <= 30


def test_host_entry_point_matches_device(torch_cuda):
    scene, rays = W.config1(n_tris=20000, n_rays=50000, seed=61)
    rays["flags"][::7] = W.RAY_FLAGS_MASKED
    s = lrx.Scene(scene)
    d = gpu_trace(torch_cuda, s, rays)
    hits = np.zeros(rays.shape[0], W.HIT_DTYPE)
    hits.view(np.uint32)[:] = SENT
    h = s.trace_host(rays, hits)
    assert np.array_equal(h.view(np.uint8), d.view(np.uint8))


def test_host_batches_overlap_and_match_device_traces(torch_cuda):
    """lrx_trace_host_batches over pinned and pageable host buffers, both
    modes and two scenes, a batch of more than one chunk: the same hits as
    device traces, masked slots untouched (pinned hit buffers are not copied
    in; their masked slots are read back), empty batches skipped."""
    torch = torch_cuda
    flat, frays = W.config1(n_tris=20000, n_rays=70000, seed=63)
    inst, irays, _ = W.config3(n_rays=50000, n_meshes=2, freq=8, n_inst=60, extent=2.0, scale=(0.1, 0.3))
    frays["flags"][::9] = W.RAY_FLAGS_MASKED
    sf, si = lrx.Scene(flat), lrx.Scene(inst)
    jobs = [(sf, frays, lrx.LRX_TRACE_CLOSEST, True), (si, irays, lrx.LRX_TRACE_ANY, False),
            (sf, frays[:0], lrx.LRX_TRACE_CLOSEST, False), (si, irays[:20000], lrx.LRX_TRACE_CLOSEST, True),
            (sf, frays[:33333], lrx.LRX_TRACE_ANY, False),
            (sf, np.tile(frays, 17)[:1_100_000], lrx.LRX_TRACE_CLOSEST, True),  # more than one chunk
            # any hit over more than one chunk: the scene's sorted configuration
            # runs persistent warps on the pipeline's chunks, same hits
            (sf, np.tile(frays, 17)[:1_200_000], lrx.LRX_TRACE_ANY, True)]
    keep, items, want = [], [], []
    for sc, r, mode, pinned in jobs:
        want.append(gpu_trace(torch, sc, r, mode) if r.shape[0] else None)
        hr = torch.from_numpy(np.ascontiguousarray(r).view(np.uint8).reshape(-1).copy())
        hh = torch.empty(max(1, r.shape[0]) * 20, dtype=torch.uint8)
        if pinned:
            hr, hh = hr.pin_memory(), hh.pin_memory()
        hh.view(torch.int32).fill_(np.int32(np.uint32(SENT).view(np.int32)).item())
        keep += [hr, hh]
        items.append((sc, hr.data_ptr(), hh.data_ptr(), r.shape[0], mode))
    lrx.trace_host_batches(items)
    for (sc, _r, h, n, _m), w, (_, _, _, _), hh in zip(items, want, jobs, keep[1::2]):
        if n == 0:
            continue
        got = hh.numpy()[:n * 20].view(W.HIT_DTYPE)
        assert np.array_equal(got.view(np.uint8), w.view(np.uint8))


CHUNK = 524288  # the host pipeline's chunk (rays)


@pytest.mark.parametrize("n", [CHUNK - 1, CHUNK, CHUNK + 1, 2 * CHUNK, 2 * CHUNK + 7])
def test_host_batches_at_chunk_boundaries(torch_cuda, n):
    """Batches just below, at and just above one and two host-pipeline
    chunks, closest and any hit, pinned and pageable, through
    lrx_trace_host_batches and lrx_trace_host: the device trace's hits, and
    masked slots untouched."""
    torch = torch_cuda
    flat, frays = W.config1(n_tris=20000, n_rays=70000, seed=64)
    rays = np.tile(frays, n // frays.shape[0] + 1)[:n].copy()
    rays["flags"][::13] = W.RAY_FLAGS_MASKED
    sc = lrx.Scene(flat)
    for mode in (lrx.LRX_TRACE_CLOSEST, lrx.LRX_TRACE_ANY):
        want = gpu_trace(torch, sc, rays, mode)
        for pinned in (True, False):
            hr = torch.from_numpy(rays.view(np.uint8).reshape(-1).copy())
            hh = torch.empty(n * 20, dtype=torch.uint8)
            if pinned:
                hr, hh = hr.pin_memory(), hh.pin_memory()
            hh.view(torch.int32).fill_(np.int32(np.uint32(SENT).view(np.int32)).item())
            lrx.trace_host_batches([(sc, hr.data_ptr(), hh.data_ptr(), n, mode)])
            got = hh.numpy().view(W.HIT_DTYPE)
            assert np.array_equal(got.view(np.uint8), want.view(np.uint8)), (mode, pinned)
        got = sc.trace_host(rays, hits=np.full(n * 5, SENT, dtype=np.uint32).view(W.HIT_DTYPE), mode=mode)
        assert np.array_equal(got.view(np.uint8), want.view(np.uint8)), mode
    sc.close()


@pytest.mark.parametrize("mode", [lrx.LRX_TRACE_CLOSEST, lrx.LRX_TRACE_ANY])
def test_host_entry_point_on_pinned_buffers(torch_cuda, mode):
    """lrx_trace_host on pinned host buffers: the same hits as device
    buffers, masked rays' slots untouched, and a buffer offset into a pinned
    allocation works too."""
    torch = torch_cuda
    scene, rays = W.config1(n_tris=20000, n_rays=60000, seed=62)
    rays["flags"][::5] = W.RAY_FLAGS_MASKED
    s = lrx.Scene(scene)
    d = gpu_trace(torch, s, rays, mode)
    h_rays = torch.from_numpy(rays.view(np.uint8).reshape(-1).copy()).pin_memory()
    h_hits = torch.empty(rays.shape[0] * 20 + 64, dtype=torch.uint8).pin_memory()
    h_hits.view(torch.int32).fill_(np.int32(np.uint32(SENT).view(np.int32)).item())
    off = 32  # hits start 32 bytes into the pinned allocation
    s.trace_host_ptr(h_rays.data_ptr(), h_hits.data_ptr() + off, rays.shape[0], mode)
    got = h_hits.numpy()[off:off + rays.shape[0] * 20].view(W.HIT_DTYPE)
    assert np.array_equal(got.view(np.uint8), d.view(np.uint8))
    assert (h_hits.numpy()[:off].view(np.uint32) == SENT).all()
    assert (h_hits.numpy()[off + rays.shape[0] * 20:].view(np.uint32) == SENT).all()


@KERNELS
def test_deterministic_and_batch_independent(torch_cuda, kernel):
    scene, rays = W.config1(n_tris=30000, n_rays=100000, seed=71)
    s = make_scene(scene, kernel)
    # whole batches (sorted when the variant asks) vs 7 small unsorted chunks,
    # for both modes: results must not depend on how rays are grouped
    for mode in (lrx.LRX_TRACE_CLOSEST, lrx.LRX_TRACE_ANY):
        a = gpu_trace(torch_cuda, s, rays, mode)
        b = gpu_trace(torch_cuda, s, rays, mode, chunks=7)
        assert np.array_equal(a.view(np.uint8), b.view(np.uint8)), mode


@pytest.mark.parametrize("layout", ["wide8", "compact4"])
def test_drain_split_hits_identical_to_the_plain_persistent_launch(torch_cuda, layout):
    """The drain split moves parts of a ray's walk to other lanes and merges
    their best hits; the merge order is the acceptance order itself, so every
    hit is bit-identical to the walk on one lane.  524,288 rays on the 512x512
    heightfield: about 3 rays per resident lane, so most of the launch is
    drain and most rays get helpers."""
    desc = W.SceneDesc([W.heightfield_mesh(512, W.BASE_SEED + 1)])
    kw = {} if layout == "wide8" else {"node_width": 4, "node_layout": lrx.LRX_NODES_COMPACT4, "leaf_max": 2}
    s = lrx.Scene(desc, **kw)
    prim = W.pinhole_rays(512, 512)
    s.set_trace_config(64, 0, lrx.LRX_VARIANT_PERSISTENT, modes=1, refill=8)
    ph = gpu_trace(torch_cuda, s, prim)
    sets = [prim, W.bounce_rays(desc, prim, ph, 1 << 19, 91), W.random_rays(1 << 19, 92)]
    for rays in sets:
        s.set_trace_config(64, 0, lrx.LRX_VARIANT_PERSISTENT, modes=1, refill=8)
        plain = gpu_trace(torch_cuda, s, rays)
        for pp, rf in ((0, 8), (8, 1), (24, 32)):
            s.set_trace_config(64, pp, lrx.LRX_VARIANT_PERSISTENT | lrx.LRX_VARIANT_DRAIN_SPLIT, modes=1, refill=rf)
            split = gpu_trace(torch_cuda, s, rays)
            assert np.array_equal(split.view(np.uint8), plain.view(np.uint8)), (pp, rf)
    # against the oracle on a stride sample of the bounce set
    oracle = po.OracleScene(desc)
    sample = sets[1][::8]
    ref, _ = oracle.intersect(sample)
    s.set_trace_config(64, 0, lrx.LRX_VARIANT_PERSISTENT | lrx.LRX_VARIANT_DRAIN_SPLIT, modes=1, refill=8)
    st = assert_parity(gpu_trace(torch_cuda, s, sets[1])[::8], ref, oracle, sample, min_hit_rate=0.05)
    assert st["bitexact_t"] == 1.0
    s.close()


@pytest.mark.parametrize("kind", ["instanced", "motion"])
def test_drain_split_on_two_level_scenes(torch_cuda, kind):
    """Two-level scenes: helpers take BLAS entries (instance-space ray and
    object) or TLAS entries (world ray); hits stay bit-identical to the plain
    persistent launch.  Motion scenes ignore the bit (the plain loop runs).
    262,144 rays, about two per resident lane."""
    torch = torch_cuda
    if kind == "instanced":
        desc, closest, _ = W.config3(n_rays=1 << 18, n_meshes=4, freq=12, n_inst=300, extent=3.0, scale=(0.1, 0.4))
    else:
        desc, closest, _ = W.config_motion(n_rays=1 << 18, n_meshes=4, freq=12, n_inst=300, extent=3.0,
                                           scale=(0.1, 0.4))
    s = lrx.Scene(desc)
    s.set_trace_config(64, 0, lrx.LRX_VARIANT_PERSISTENT, modes=1, refill=8)
    plain = gpu_trace(torch, s, closest)
    for pp, rf in ((0, 8), (8, 1)):
        s.set_trace_config(64, pp, lrx.LRX_VARIANT_PERSISTENT | lrx.LRX_VARIANT_DRAIN_SPLIT, modes=1, refill=rf)
        split = gpu_trace(torch, s, closest)
        assert np.array_equal(split.view(np.uint8), plain.view(np.uint8)), (pp, rf)
    if kind == "instanced":  # (motion against the oracle, within its tolerance: test_motion_gpu.py)
        oracle = po.OracleScene(desc)
        sample = closest[::16]
        ref, _ = oracle.intersect(sample)
        st = assert_parity(split[::16], ref, oracle, sample, min_hit_rate=0.05)
        assert st["bitexact_t"] == 1.0
    s.close()


def test_default_closest_config_is_the_drain_split(torch_cuda):
    s = lrx.Scene(W.SceneDesc([W.heightfield_mesh(16, 3)]))
    cfg = s.trace_config(lrx.LRX_TRACE_CLOSEST)
    assert cfg["variant"] == lrx.LRX_VARIANT_PERSISTENT | lrx.LRX_VARIANT_DRAIN_SPLIT, cfg
    s.close()


def test_instance_update_matches_rebuilt_oracle(torch_cuda):
    scene, closest, _ = W.config3(n_rays=20000, n_meshes=2, freq=8, n_inst=64, extent=2.0, scale=(0.1, 0.3))
    s = lrx.Scene(scene)
    rng = np.random.default_rng(9)
    moved = []
    for mi, m in scene.objects:
        m2 = np.array(m, np.float32).copy()
        m2[:3, 3] += rng.uniform(-0.3, 0.3, 3).astype(np.float32)
        moved.append((mi, m2))
    scene2 = W.SceneDesc(scene.meshes, moved)
    s.update_instances(scene2)
    oracle = po.OracleScene(scene2)
    ref, _ = oracle.intersect(closest)
    gpu = gpu_trace(torch_cuda, s, closest)
    assert_parity(gpu, ref, oracle, closest, min_hit_rate=0.02)


@KERNELS
def test_counted_trace(torch_cuda, kernel):
    scene, rays = W.config1(n_tris=20000, n_rays=40000, seed=81)
    s = make_scene(scene, kernel)
    torch = torch_cuda
    d_r = torch.from_numpy(rays.view(np.uint8).copy()).cuda()
    d_h = torch.empty(rays.shape[0] * 20, dtype=torch.uint8, device="cuda")
    c = torch.zeros(4, dtype=torch.int64, device="cuda")
    s.trace_counted(d_r.data_ptr(), d_h.data_ptr(), rays.shape[0], 0, c.data_ptr(),
                    torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    nodes, tris, insts, n = c.cpu().tolist()
    assert n == rays.shape[0] and insts == 0
    assert nodes >= n and tris > 0
    plain = gpu_trace(torch, s, rays)
    assert np.array_equal(d_h.cpu().numpy().view(W.HIT_DTYPE).view(np.uint8), plain.view(np.uint8))


def test_rejects_bad_arguments(torch_cuda):
    scene, rays = W.config1(n_tris=100, n_rays=64, seed=91)
    s = lrx.Scene(scene)
    torch = torch_cuda
    buf = torch.empty(64 * 48 + 16, dtype=torch.uint8, device="cuda")
    with pytest.raises(lrx.LrxError):
        s.trace(buf.data_ptr() + 4, buf.data_ptr(), 8, 0)      # misaligned rays
    with pytest.raises(lrx.LrxError):
        s.trace(buf.data_ptr(), buf.data_ptr(), 8, 7)          # unknown mode
    bad = W.SceneDesc([W.Mesh(np.zeros((3, 3), np.float32), np.array([[0, 1, 5]], np.uint32))])
    with pytest.raises(lrx.LrxError):
        lrx.Scene(bad)                                         # vertex index out of range
    sing = W.SceneDesc([W.random_triangles(10, 1)], [(0, np.zeros((4, 4), np.float32))])
    with pytest.raises(lrx.LrxError):
        lrx.Scene(sing)                                        # singular instance transform


def test_trace_config_struct_versions(torch_cuda):
    """The ABI-1 struct (no refill field) is still accepted on set and get;
    out-of-range values and unknown variant bits are rejected."""
    import ctypes
    scene, _ = W.config1(n_tris=100, n_rays=64, seed=92)
    s = lrx.Scene(scene)
    L = lrx.load()
    old = lrx.TraceConfig(20, 64, 4, lrx.LRX_VARIANT_PERSISTENT, 0, 99)  # refill beyond the 20 bytes: ignored
    assert L.lrx_scene_set_trace_config(s.handle, ctypes.byref(old)) == 0
    assert s.trace_config() == {"block_size": 64, "postpone": 4, "variant": lrx.LRX_VARIANT_PERSISTENT, "refill": 0}
    got = lrx.TraceConfig(20, 0, 0, 0, 0, 77)
    assert L.lrx_scene_get_trace_config(s.handle, ctypes.byref(got)) == 0
    assert (got.struct_size, got.block_size, got.refill) == (20, 64, 77)  # nothing past 20 bytes written
    for bad in [lrx.TraceConfig(16, 64, 8, 0, 0, 0), lrx.TraceConfig(24, 64, 8, 0x80000000, 0, 0),
                lrx.TraceConfig(24, 64, 8, 0x40, 0, 33), lrx.TraceConfig(24, 48, 8, 0, 0, 0),
                # a 32-entry shared-memory stack takes 256 B a thread: at most 128 threads a block
                lrx.TraceConfig(24, 256, 8, lrx.LRX_VARIANT_SMEM_STACK32, 0, 0),
                lrx.TraceConfig(24, 512, 8, lrx.LRX_VARIANT_SMEM_STACK16, 0, 0),
                # the library's internal build bits (motion, 64-byte records) are not variants
                lrx.TraceConfig(24, 64, 8, 0x200, 0, 0), lrx.TraceConfig(24, 64, 8, 0x1000, 0, 0)]:
        assert L.lrx_scene_set_trace_config(s.handle, ctypes.byref(bad)) == lrx.LRX_ERR_INVALID_ARGUMENT


@pytest.mark.parametrize("queue", ["fetch", "fetch-refill1", "tiles", "fetch-sorted", "tiles-sorted",
                                   "fetch-many-large"])
def test_trace_batches_equals_per_batch_traces(torch_cuda, queue):
    """lrx_trace_batches over a ragged mix of scenes, modes and sizes
    (including empty, single-ray and tile-boundary batches, and more batches
    than one queue launch holds) returns exactly what lrx_trace returns --
    with warp-level ray fetch (a scene config with the persistent variant,
    the closest-hit default) and with 64-ray tiles (no such config)."""
    torch = torch_cuda
    flat_desc, _ = W.config1(n_tris=20000, n_rays=1, seed=301)
    inst_desc, _, _ = W.config3(n_rays=1, n_meshes=2, freq=8, n_inst=50, extent=1.0, scale=(0.05, 0.2))
    scenes = [lrx.Scene(flat_desc), lrx.Scene(inst_desc)]
    for s in scenes:
        if queue == "tiles":
            s.set_trace_config(64, 8, 0)
        elif queue == "fetch-refill1":
            s.set_trace_config(64, 8, lrx.LRX_VARIANT_PERSISTENT, refill=1)
        elif queue == "fetch-sorted":  # batches >= 32,768 rays are reordered inside the queue launch
            s.set_trace_config(64, 8, lrx.LRX_VARIANT_PERSISTENT | lrx.LRX_VARIANT_SORT_RAYS, refill=8)
        elif queue == "tiles-sorted":
            s.set_trace_config(64, 8, lrx.LRX_VARIANT_SORT_RAYS)
    rng = np.random.default_rng(302)
    # 131,072 rays and more: launches of their own on side streams
    sizes = [0, 1, 63, 64, 65, 1000, 100_000, 40_000, 32_768, 131_071, 131_072, 300_000] + \
        rng.integers(1, 3000, 400).tolist()
    if queue == "fetch-many-large":  # more than 4 large batches: all of them stay in the queue launch
        sizes += [140_000, 150_000, 160_000]
    st = torch.cuda.current_stream().cuda_stream
    items, refs = [], []
    for k, n in enumerate(sizes):
        s = scenes[k % 2]
        mode = lrx.LRX_TRACE_ANY if k % 3 == 0 else lrx.LRX_TRACE_CLOSEST
        rays = W.random_rays(max(n, 1), 400 + k)[:n]
        rays["flags"][::17] = W.RAY_FLAGS_MASKED
        d_r = torch.from_numpy(rays.view(np.uint8).reshape(-1).copy()).cuda() if n else \
            torch.empty(48, dtype=torch.uint8, device="cuda")
        d_h = torch.empty(max(n, 1) * 20, dtype=torch.uint8, device="cuda")
        d_h.view(torch.int32).fill_(np.int32(np.uint32(SENT).view(np.int32)).item())
        items.append((s, d_r, d_h, n, mode))
        refs.append(gpu_trace(torch, s, rays, mode) if n else None)
    lrx.trace_batches([(s, r.data_ptr(), h.data_ptr(), n, m) for s, r, h, n, m in items], st)
    torch.cuda.synchronize()
    for s in scenes:
        assert s.device_status(st) == 0
    for (s, r, h, n, m), ref in zip(items, refs):
        if n == 0:
            continue
        got = h.cpu().numpy().view(W.HIT_DTYPE)[:n]
        bad = np.nonzero(got.view(np.uint32).reshape(-1, 5) != ref.view(np.uint32).reshape(-1, 5))[0]
        assert bad.size == 0, (n, m, bad[:5], got[bad[:3]], ref[bad[:3]])


def test_trace_batches_completion_flags_with_large_batches(torch_cuda):
    """lrx_trace_batches_ex: large batches (own launches on side streams) and
    queued ones all raise their completion flags and equal plain traces."""
    torch = torch_cuda
    flat_desc, _ = W.config1(n_tris=20000, n_rays=1, seed=321)
    s = lrx.Scene(flat_desc)
    sizes = [250_000, 3_000, 140_000, 0, 60_000]
    items, want = [], []
    for k, n in enumerate(sizes):
        mode = lrx.LRX_TRACE_ANY if k % 2 else lrx.LRX_TRACE_CLOSEST
        rays = W.random_rays(max(n, 1), 330 + k)[:n]
        d_r = torch.from_numpy(rays.view(np.uint8).reshape(-1).copy()).cuda() if n else \
            torch.empty(48, dtype=torch.uint8, device="cuda")
        d_h = torch.empty(max(n, 1) * 20, dtype=torch.uint8, device="cuda")
        items.append((s, d_r, d_h, n, mode))
        want.append(gpu_trace(torch, s, rays, mode) if n else None)
    tiles = torch.zeros(len(sizes), dtype=torch.int32, device="cuda")
    flags = torch.zeros(len(sizes), dtype=torch.int32, device="cuda")
    lrx.trace_batches([(sc, r.data_ptr(), h.data_ptr(), n, m) for sc, r, h, n, m in items],
                      torch.cuda.current_stream().cuda_stream, tiles.data_ptr(), flags.data_ptr())
    torch.cuda.synchronize()
    assert flags.cpu().tolist() == [1 if n else 0 for n in sizes]
    for (sc, r, h, n, m), w in zip(items, want):
        if n:
            assert np.array_equal(h.cpu().numpy()[:n * 20].view(np.uint32), w.view(np.uint32))


def test_trace_batches_in_a_cuda_graph(torch_cuda):
    """lrx_trace_batches captured in a CUDA graph -- large batches on forked
    side streams, small ones in the queue launch -- replays to the plain
    per-batch results, and again after new rays are written in place."""
    torch = torch_cuda
    flat_desc, _ = W.config1(n_tris=20000, n_rays=1, seed=311)
    inst_desc, _, _ = W.config3(n_rays=1, n_meshes=2, freq=8, n_inst=50, extent=1.0, scale=(0.05, 0.2))
    scenes = [lrx.Scene(flat_desc), lrx.Scene(inst_desc)]
    sizes = [200_000, 5_000, 140_000, 777, 1, 65_536]
    stream = torch.cuda.Stream()
    st = stream.cuda_stream
    items = []
    for k, n in enumerate(sizes):
        mode = lrx.LRX_TRACE_ANY if k % 2 else lrx.LRX_TRACE_CLOSEST
        d_r = torch.empty(n * 48, dtype=torch.uint8, device="cuda")
        d_h = torch.empty(n * 20, dtype=torch.uint8, device="cuda")
        items.append((scenes[k % 2], d_r, d_h, n, mode))
    arr = lrx.batch_array([(s, r.data_ptr(), h.data_ptr(), n, m) for s, r, h, n, m in items])

    def fill(seed):
        refs = []
        for k, (s, d_r, d_h, n, mode) in enumerate(items):
            rays = W.random_rays(n, seed + k)
            d_r.copy_(torch.from_numpy(rays.view(np.uint8).reshape(-1).copy()))
            refs.append(gpu_trace(torch, s, rays, mode))
        torch.cuda.synchronize()
        return refs

    fill(900)
    with torch.cuda.stream(stream):
        lrx.trace_batches([None] * len(items), st, arr=arr)  # first call on this thread: side streams created
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=stream):
        lrx.trace_batches([None] * len(items), st, arr=arr)
    for seed in (910, 920):
        refs = fill(seed)
        g.replay()
        torch.cuda.synchronize()
        for (s, d_r, d_h, n, mode), ref in zip(items, refs):
            got = d_h.cpu().numpy().view(W.HIT_DTYPE)
            assert np.array_equal(got.view(np.uint32), ref.view(np.uint32)), (n, mode)


def test_autotune_picks_a_valid_config_and_keeps_results(torch_cuda):
    """lrx_scene_autotune returns one of its candidates, installs it for that
    mode only, and traces under it match the oracle."""
    torch = torch_cuda
    scene, rays = W.config1(n_tris=30000, n_rays=50000, seed=501)
    s = lrx.Scene(scene)
    d_r = torch.from_numpy(rays.view(np.uint8).reshape(-1).copy()).cuda()
    before_any = s.trace_config(lrx.LRX_TRACE_ANY)
    st = torch.cuda.current_stream().cuda_stream
    chosen = s.autotune(d_r.data_ptr(), rays.shape[0], lrx.LRX_TRACE_CLOSEST, st)
    assert chosen["block_size"] in (32, 64, 128) and chosen["postpone"] in (0, 8, 16)
    assert chosen["variant"] in (0, lrx.LRX_VARIANT_STREAM_RAYS, lrx.LRX_VARIANT_SORT_RAYS,
                                 lrx.LRX_VARIANT_PERSISTENT, lrx.LRX_VARIANT_PERSISTENT | lrx.LRX_VARIANT_STREAM_RAYS)
    assert chosen["refill"] == (8 if chosen["variant"] & lrx.LRX_VARIANT_PERSISTENT else 0)
    assert s.trace_config(lrx.LRX_TRACE_CLOSEST) == chosen
    assert s.trace_config(lrx.LRX_TRACE_ANY) == before_any
    o = po.OracleScene(scene)
    ref, _ = o.intersect(rays)
    assert_parity(gpu_trace(torch, s, rays), ref, o, rays, min_hit_rate=0.05)


@pytest.mark.parametrize("passes", [1, 2, 3])
def test_treelet_restructured_builds_keep_parity(torch_cuda, passes):
    """Treelet SAH passes rewrite the binary tree before the collapse: the
    builder's structural validation must pass and traces must still match the
    oracle -- flat, heightfield, instanced and tiny scenes."""
    torch = torch_cuda
    scene, rays = W.config1(n_tris=30000, n_rays=40000, seed=700 + passes)
    s = lrx.Scene(scene, treelet_passes=passes)
    o = po.OracleScene(scene)
    ref, _ = o.intersect(rays)
    assert_parity(gpu_trace(torch, s, rays), ref, o, rays, min_hit_rate=0.2)
    a = check_anyhit(gpu_trace(torch, s, rays, lrx.LRX_TRACE_ANY), ref, o, rays)
    assert a["ok"], a
    hf = W.SceneDesc([W.heightfield_mesh(128, 710 + passes)])
    s = lrx.Scene(hf, treelet_passes=passes)
    prim = W.pinhole_rays(128, 128)
    o = po.OracleScene(hf)
    ref, _ = o.intersect(prim)
    assert_parity(gpu_trace(torch, s, prim), ref, o, prim, min_hit_rate=0.2)
    inst, closest, _ = W.config3(n_rays=1 << 13, n_meshes=3, freq=10, n_inst=100, extent=3.0, scale=(0.1, 0.4))
    s = lrx.Scene(inst, treelet_passes=passes)
    o = po.OracleScene(inst)
    ref, _ = o.intersect(closest)
    assert_parity(gpu_trace(torch, s, closest), ref, o, closest, min_hit_rate=0.05)
    for n in (1, 2, 3, 4, 7, 8, 9, 30):
        tiny, r = W.config1(n_tris=n, n_rays=2000, seed=720 + n)
        s = lrx.Scene(tiny, treelet_passes=passes)
        o = po.OracleScene(tiny)
        ref, _ = o.intersect(r)
        assert_parity(gpu_trace(torch, s, r), ref, o, r)


@pytest.mark.parametrize("width", [4, 5, 6, 7])
def test_narrower_nodes_keep_parity(torch_cuda, width):
    """Trees of 4- to 7-wide nodes (the same node format, deeper trees) give
    the oracle's hits, and closest hits equal the 8-wide tree's."""
    scene, rays = W.config1(n_tris=30000, n_rays=1 << 15, seed=91)
    oracle = po.OracleScene(scene)
    ref, _ = oracle.intersect(rays)
    s = lrx.Scene(scene, node_width=width)
    s8 = lrx.Scene(scene)
    if width == 4:  # (node counts need not fall monotonically with the width)
        assert s.info()["node_count"] > s8.info()["node_count"]
    for mode in (lrx.LRX_TRACE_CLOSEST, lrx.LRX_TRACE_ANY):
        gpu = gpu_trace(torch_cuda, s, rays, mode)
        if mode == lrx.LRX_TRACE_CLOSEST:
            assert_parity(gpu, ref, oracle, rays, min_hit_rate=0.05)
            assert np.array_equal(gpu.view(np.uint32), gpu_trace(torch_cuda, s8, rays, mode).view(np.uint32))
        else:
            a = check_anyhit(gpu, ref, oracle, rays)
            assert a["ok"], a
    with pytest.raises(lrx.LrxError):
        lrx.Scene(scene, node_width=3)


def test_autotuned_build_picks_a_candidate_and_keeps_results(torch_cuda):
    """lrx_scene_create_autotuned keeps one of the candidate builds with its
    tuned launch configuration; its closest hits equal the default build's."""
    torch = torch_cuda
    scene, rays = W.config1(n_tris=30000, n_rays=1 << 16, seed=92)
    d_r = torch.from_numpy(rays.view(np.uint8).reshape(-1).copy()).cuda()
    sc, opts, cfg = lrx.Scene.autotuned(scene, d_r.data_ptr(), rays.shape[0], lrx.LRX_TRACE_CLOSEST,
                                        torch.cuda.current_stream().cuda_stream, treelet_passes=1)
    assert opts["node_width"] in (4, 8) and opts["leaf_max"] in (2, 3) and opts["treelet_passes"] == 1
    assert sc.trace_config(lrx.LRX_TRACE_CLOSEST) == cfg
    want = gpu_trace(torch, lrx.Scene(scene), rays)
    assert np.array_equal(gpu_trace(torch, sc, rays).view(np.uint32), want.view(np.uint32))


@pytest.mark.parametrize("masked_frac", [0.0, 0.5, 0.97, 1.0])
def test_compaction_skips_masked_rays(torch_cuda, masked_frac):
    """The compacting launch traces only unmasked rays: their hits equal the
    plain launch's, masked rays' hit records stay untouched (all masked:
    nothing is written)."""
    torch = torch_cuda
    scene, rays = W.config1(n_tris=20000, n_rays=60000, seed=801)
    rng = np.random.default_rng(802)
    rays["flags"][rng.random(rays.shape[0]) < masked_frac] = W.RAY_FLAGS_MASKED
    plain = make_scene(scene, (64, 8, lrx.LRX_VARIANT_PERSISTENT, 8))
    comp = make_scene(scene, (64, 8, lrx.LRX_VARIANT_PERSISTENT | lrx.LRX_VARIANT_COMPACT, 8))
    # the drain split on the compacted list (device-side count, index indirection)
    comp_split = make_scene(scene, (64, 0, lrx.LRX_VARIANT_PERSISTENT | lrx.LRX_VARIANT_COMPACT
                                    | lrx.LRX_VARIANT_DRAIN_SPLIT, 8))
    for mode in (lrx.LRX_TRACE_CLOSEST, lrx.LRX_TRACE_ANY):
        a = gpu_trace(torch, plain, rays, mode)
        masked = (rays["flags"] & W.RAY_FLAGS_MASKED) != 0
        for c in (comp, comp_split):
            b = gpu_trace(torch, c, rays, mode)
            assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
            assert (b.view(np.uint32).reshape(-1, 5)[masked] == SENT).all()


def test_scene_blob_round_trip(torch_cuda):
    """lrx_scene_save / lrx_scene_load: a loaded scene traces bit-for-bit like
    the saved one (flat and two-level, both modes), keeps its trace configs
    and takes instance updates; corrupt or truncated blobs are rejected."""
    torch = torch_cuda
    flat, rays = W.config1(n_tris=20000, n_rays=30000, seed=901)
    inst, closest, anyr = W.config3(n_rays=1 << 14, n_meshes=3, freq=10, n_inst=120, extent=3.0, scale=(0.1, 0.4))
    for desc, r in ((flat, rays), (inst, closest)):
        a = lrx.Scene(desc)
        a.set_trace_config(128, 0, lrx.LRX_VARIANT_PERSISTENT, modes=1, refill=4)
        blob = a.save()
        b = lrx.Scene.from_blob(blob, desc=desc)
        assert b.trace_config(lrx.LRX_TRACE_CLOSEST) == a.trace_config(lrx.LRX_TRACE_CLOSEST)
        ia, ib = a.info(), b.info()
        assert {k: ia[k] for k in ia if k != "build_ms"} == {k: ib[k] for k in ib if k != "build_ms"}
        for mode in (lrx.LRX_TRACE_CLOSEST, lrx.LRX_TRACE_ANY):
            ha, hb = gpu_trace(torch, a, r, mode), gpu_trace(torch, b, r, mode)
            assert np.array_equal(ha.view(np.uint32), hb.view(np.uint32))
        for bad in (blob[:-1], blob[:30], blob[:100] + bytes([blob[100] ^ 1]) + blob[101:], b"x" * 64):
            with pytest.raises(lrx.LrxError):
                lrx.Scene.from_blob(bad)
    # instance update on the loaded scene equals the update on the original
    rng = np.random.default_rng(902)
    moved = []
    for mi, m in inst.objects:
        m2 = m.copy()
        m2[:3, 3] += rng.uniform(-0.2, 0.2, 3).astype(np.float32)
        moved.append((mi, m2))
    moved = W.SceneDesc(inst.meshes, moved)
    a = lrx.Scene(inst)
    b = lrx.Scene.from_blob(a.save(), desc=inst)
    a.update_instances(moved)
    b.update_instances(moved)
    for mode in (lrx.LRX_TRACE_CLOSEST, lrx.LRX_TRACE_ANY):
        ha, hb = gpu_trace(torch, a, anyr, mode), gpu_trace(torch, b, anyr, mode)
        assert np.array_equal(ha.view(np.uint32), hb.view(np.uint32))


def test_replicas_tracing_slices_equal_one_replica(torch_cuda):
    """Two scene replicas (as two GPUs would hold), each tracing its
    lrx.rank_slice of one RayBuffer, one after the other on this GPU with no
    exchange between them: the slices' hits concatenated in rank order equal
    one replica tracing the whole buffer, byte for byte, and the oracle's."""
    scene_desc, rays = W.config1(n_tris=30000, n_rays=200003, seed=93)
    whole = gpu_trace(torch_cuda, lrx.Scene(scene_desc), rays)
    parts = []
    for rank in range(2):
        b, e = lrx.rank_slice(rays.shape[0], rank, 2)
        replica = lrx.Scene(scene_desc)
        parts.append(gpu_trace(torch_cuda, replica, rays[b:e]))
        replica.close()
    got = np.concatenate(parts)
    assert np.array_equal(got.view(np.uint8), whole.view(np.uint8))
    oracle = po.OracleScene(scene_desc)
    ref, _ = oracle.intersect(rays)
    assert_parity(got, ref, oracle, rays)
