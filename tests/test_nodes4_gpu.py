"""The 64-byte node record (LRX_NODES_COMPACT4): 4-wide trees over flat
scenes stored with four child positions instead of eight slots.

It holds the same tree as the 80-byte record of a node_width-4 build -- the
same children, planes and meta bytes, repacked -- so every launch form must
give the same hits bit for bit in both modes, after the same node visits,
and the oracle's and the reference kernel's answers (the golden fixtures).
Also: the option's errors, scene info, blobs, batches (which trace compact
scenes through launches of their own) and the autotuner's candidates.
"""
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.dirname(__file__))
sys.path.insert(0, os.path.join(os.path.dirname(__file__), "golden"))

from luxcore_gb300 import lrx  # noqa: E402
from luxcore_gb300 import workloads as W  # noqa: E402
from oracle import pyoracle as po  # noqa: E402
from parity import check_anyhit, compare  # noqa: E402
from test_trace_gpu import KERNEL_CONFIGS, KERNELS, SENT, gpu_trace, make_scene  # noqa: E402

pytestmark = pytest.mark.gpu

C4 = {"node_width": 4, "node_layout": lrx.LRX_NODES_COMPACT4}
W4 = {"node_width": 4}


@pytest.fixture(scope="module")
def torch_cuda(cuda_ready):
    import torch
    return torch


@pytest.fixture(scope="module")
def flat():
    scene, rays = W.config1(n_tris=30000, n_rays=1 << 16, seed=941)
    return scene, rays


@pytest.mark.parametrize("name", ["golden_random", "golden_heightfield", "golden_multimesh"])
@KERNELS
def test_golden_fixtures_in_64_byte_records(torch_cuda, kernel, name):
    """Hits of the reference's own kernel text (bvh.cl) compiled for the CPU,
    under every launch configuration of the 80-byte parity tests."""
    from make_golden import load
    scene, rays, ref = load(name)
    s = make_scene(scene, kernel, **C4)
    assert s.info()["node_bytes"] == 64
    gpu = gpu_trace(torch_cuda, s, rays)
    masked = (rays["flags"] & W.RAY_FLAGS_MASKED) != 0
    assert (gpu.view(np.uint32).reshape(-1, 5)[masked] == SENT).all()
    nan_ray = np.isnan(rays["o"]).any(1) | np.isnan(rays["d"]).any(1) | np.isnan(rays["maxt"])
    assert (gpu["meshIndex"][nan_ray] == W.NULL_INDEX).all()
    keep = ~masked & ~nan_ray
    oracle = po.OracleScene(scene)
    st = compare(gpu[keep], ref[keep], oracle, rays[keep])
    assert st["bad_disagreements"] == 0 and st["values_ok"] and st["ties_valid"], st


@KERNELS
def test_same_hits_and_visits_as_the_80_byte_record(torch_cuda, flat, kernel):
    """Closest and any hit: bit-equal to the 80-byte record of the same
    4-wide tree (the traversal takes the same decisions), and the oracle's."""
    scene, rays = flat
    s4 = make_scene(scene, kernel, **C4)
    s8 = make_scene(scene, kernel, **W4)
    oracle = po.OracleScene(scene)
    ref, _ = oracle.intersect(rays)
    for mode in (lrx.LRX_TRACE_CLOSEST, lrx.LRX_TRACE_ANY):
        a, b = gpu_trace(torch_cuda, s4, rays, mode), gpu_trace(torch_cuda, s8, rays, mode)
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), mode
        if mode == lrx.LRX_TRACE_CLOSEST:
            st = compare(a, ref, oracle, rays)
            assert st["ok"] and st["bitexact_t"] == 1.0 and st["hit_rate"] > 0.3, st
        else:
            r = check_anyhit(a, ref, oracle, rays)
            assert r["ok"], r


def test_counted_visits_equal_and_info(torch_cuda, flat):
    """The counting trace sees the same node visits and triangle tests in
    both records; the 64-byte scene holds the same node count in 64 bytes
    each."""
    torch = torch_cuda
    scene, rays = flat
    s4, s8 = lrx.Scene(scene, **C4), lrx.Scene(scene, **W4)
    i4, i8 = s4.info(), s8.info()
    assert i4["node_bytes"] == 64 and i8["node_bytes"] == 80 and lrx.Scene(scene).info()["node_bytes"] == 80
    assert i4["node_count"] == i8["node_count"] and i4["max_depth"] == i8["max_depth"]
    assert i8["device_bytes"] - i4["device_bytes"] >= 16 * i4["node_count"]
    d_r = torch.from_numpy(rays.view(np.uint8).reshape(-1).copy()).cuda()
    st = torch.cuda.current_stream().cuda_stream
    for mode in (lrx.LRX_TRACE_CLOSEST, lrx.LRX_TRACE_ANY):
        counts = []
        for s in (s4, s8):
            d_h = torch.empty(rays.shape[0] * 20, dtype=torch.uint8, device="cuda")
            c = torch.zeros(4, dtype=torch.int64, device="cuda")
            s.trace_counted(d_r.data_ptr(), d_h.data_ptr(), rays.shape[0], mode, c.data_ptr(), st)
            torch.cuda.synchronize()
            counts.append(c.cpu().numpy().tolist())
        assert counts[0] == counts[1], (mode, counts)
        assert counts[0][0] > rays.shape[0]  # node visits


def test_option_errors(torch_cuda):
    scene, _ = W.config1(n_tris=2000, n_rays=16, seed=942)
    with pytest.raises(lrx.LrxError):  # 64-byte records hold 4 children
        lrx.Scene(scene, node_width=8, node_layout=lrx.LRX_NODES_COMPACT4)
    with pytest.raises(lrx.LrxError):
        lrx.Scene(scene, node_width=4, node_layout=7)
    inst, _c, _a = W.config3(n_rays=16, n_meshes=2, freq=6, n_inst=10)
    with pytest.raises(lrx.LrxError) as e:  # two-level scenes keep the 80-byte record
        lrx.Scene(inst, **C4)
    assert e.value.status == lrx.LRX_ERR_NOT_SUPPORTED


def test_blob_round_trip_of_a_64_byte_scene(torch_cuda, flat):
    scene, rays = flat
    a = lrx.Scene(scene, **C4)
    blob = a.save()
    b = lrx.Scene.from_blob(blob, desc=scene)
    ia, ib = a.info(), b.info()
    assert {k: ia[k] for k in ia if k != "build_ms"} == {k: ib[k] for k in ib if k != "build_ms"}
    for mode in (lrx.LRX_TRACE_CLOSEST, lrx.LRX_TRACE_ANY):
        ha, hb = gpu_trace(torch_cuda, a, rays, mode), gpu_trace(torch_cuda, b, rays, mode)
        assert np.array_equal(ha.view(np.uint32), hb.view(np.uint32))
    # the key tells the records apart
    assert lrx.scene_key(scene, node_width=4) != lrx.scene_key(scene, node_width=4,
                                                               node_layout=lrx.LRX_NODES_COMPACT4)


def test_batches_mixing_both_records(torch_cuda, flat):
    """A lrx_trace_batches call over 80- and 64-byte scenes (the latter in
    launches of their own) equals one lrx_trace per batch."""
    torch = torch_cuda
    scene, rays = flat
    other, orays = W.config1(n_tris=8000, n_rays=1 << 14, seed=943)
    s4, s8 = lrx.Scene(scene, **C4), lrx.Scene(other)
    d_r = torch.from_numpy(rays.view(np.uint8).reshape(-1).copy()).cuda()
    d_o = torch.from_numpy(orays.view(np.uint8).reshape(-1).copy()).cuda()
    n, no = rays.shape[0], orays.shape[0]
    d_h = torch.empty(n * 20, dtype=torch.uint8, device="cuda")
    d_ho = torch.empty(no * 20, dtype=torch.uint8, device="cuda")
    cut = [0, 1000, 5000, 20000, n]
    batches = [(s4, d_r.data_ptr() + 48 * a, d_h.data_ptr() + 20 * a, b - a, (k % 2))
               for k, (a, b) in enumerate(zip(cut[:-1], cut[1:]))]
    batches.append((s8, d_o.data_ptr(), d_ho.data_ptr(), no, lrx.LRX_TRACE_CLOSEST))
    st = torch.cuda.current_stream().cuda_stream
    lrx.trace_batches(batches, st)
    torch.cuda.synchronize()
    got = d_h.cpu().numpy().view(W.HIT_DTYPE).copy()
    for k, (a, b) in enumerate(zip(cut[:-1], cut[1:])):
        want = gpu_trace(torch, s4, rays[a:b], k % 2)
        assert np.array_equal(got[a:b].view(np.uint32), want.view(np.uint32)), k
    assert np.array_equal(d_ho.cpu().numpy().view(W.HIT_DTYPE).view(np.uint32),
                          gpu_trace(torch, s8, orays).view(np.uint32))


def test_autotuner_times_the_64_byte_candidates(torch_cuda, flat):
    """lrx_scene_create_autotuned reports which record it kept; its closest
    hits equal the default build's either way."""
    torch = torch_cuda
    scene, rays = flat
    d_r = torch.from_numpy(rays.view(np.uint8).reshape(-1).copy()).cuda()
    sc, opts, cfg = lrx.Scene.autotuned(scene, d_r.data_ptr(), rays.shape[0], lrx.LRX_TRACE_CLOSEST,
                                        torch.cuda.current_stream().cuda_stream, treelet_passes=1)
    assert opts["node_layout"] in (lrx.LRX_NODES_WIDE8, lrx.LRX_NODES_COMPACT4)
    assert opts["node_layout"] == lrx.LRX_NODES_WIDE8 or opts["node_width"] == 4
    assert sc.info()["node_bytes"] == (64 if opts["node_layout"] == lrx.LRX_NODES_COMPACT4 else 80)
    want = gpu_trace(torch, lrx.Scene(scene), rays)
    assert np.array_equal(gpu_trace(torch, sc, rays).view(np.uint32), want.view(np.uint32))


def test_kernel_configs_cover_the_64_byte_builds():
    """Every compile-time form the 64-byte records have (plain, MINMAX3,
    shared-memory stacks 8/16/32, persistent) is among the launch
    configurations above."""
    v = [k[2] for k in KERNEL_CONFIGS]
    assert any(x & lrx.LRX_VARIANT_MINMAX3 for x in v)
    for bit in (lrx.LRX_VARIANT_SMEM_STACK, lrx.LRX_VARIANT_SMEM_STACK16, lrx.LRX_VARIANT_SMEM_STACK32,
                lrx.LRX_VARIANT_PERSISTENT):
        assert any(x & bit for x in v), bit
