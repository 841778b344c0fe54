"""Failure detection on the GPU without a GPU fault.

A trace stops a ray when it exhausts its node-visit budget, and stops
starting rays once the launch's deadline has passed.  Either way the ray's
hit slot is left unwritten, the scene's status word records why, and
lrx_scene_device_status returns LRX_ERR_DEVICE -- nothing traps, and the
context stays usable.  These tests set tiny bounds through the public launch
configuration (lrx_trace_config.max_visits / deadline_us) on valid scenes
and check, for every launch form (persistent warps, one thread per ray,
sorted any-hit, queue launches with completion flags):
- the status bit is set and reported;
- every ray whose slot was written carries the oracle's answer, and the
  abandoned rays' slots still hold what the caller put there;
- with the default bounds the same scene traces cleanly afterwards (status
  0, full parity), so the default bounds never fire on a valid tree.
"""
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.dirname(__file__))

from luxcore_gb300 import lrx  # noqa: E402
from luxcore_gb300 import workloads as W  # noqa: E402
from oracle import pyoracle as po  # noqa: E402
from parity import check_anyhit, compare  # noqa: E402

pytestmark = pytest.mark.gpu

SENT = 0xDEADBEEF
STATUS_STACK, STATUS_VISITS, STATUS_DEADLINE = 1, 2, 4
LRX_ERR_DEVICE = 5

# (block size, postpone, variant, refill): persistent warps, one thread per
# ray, sorted before tracing
FORMS = {"persistent": (64, 8, lrx.LRX_VARIANT_PERSISTENT, 8), "thread-per-ray": (64, 8, 0, 0),
         "sorted": (64, 8, lrx.LRX_VARIANT_SORT_RAYS, 0),
         "drain-split": (64, 0, lrx.LRX_VARIANT_PERSISTENT | lrx.LRX_VARIANT_DRAIN_SPLIT, 8)}


@pytest.fixture(scope="module")
def torch_cuda(cuda_ready):
    import torch
    return torch


@pytest.fixture(scope="module")
def flat():
    desc = W.SceneDesc([W.heightfield_mesh(256, W.BASE_SEED + 1)])
    rays = W.random_rays(1 << 18, 301)
    oracle = po.OracleScene(desc)
    ref, _ = oracle.intersect(rays)
    return desc, rays, oracle, ref


def _status(scene, st):
    import ctypes
    v = ctypes.c_uint32()
    rc = lrx.load().lrx_scene_device_status(scene.handle, ctypes.byref(v), ctypes.c_void_p(st))
    return rc, v.value


def _trace(torch, scene, rays, mode):
    n = rays.shape[0]
    d_r = torch.from_numpy(np.ascontiguousarray(rays).view(np.uint8).reshape(-1).copy()).cuda()
    d_h = torch.empty(n * 20, dtype=torch.uint8, device="cuda")
    d_h.view(torch.int32).fill_(np.int32(np.uint32(SENT).view(np.int32)).item())
    st = torch.cuda.current_stream().cuda_stream
    scene.trace(d_r.data_ptr(), d_h.data_ptr(), n, mode, st)
    torch.cuda.synchronize()
    rc, status = _status(scene, st)
    return d_h.cpu().numpy().view(W.HIT_DTYPE).copy(), rc, status


def _written(hits):
    return ~(hits.view(np.uint32).reshape(-1, 5) == SENT).all(axis=1)


def _check_partial(hits, ref, oracle, rays, mode):
    """Written slots carry the oracle's answer; unwritten ones are untouched."""
    w = _written(hits)
    if not w.any():
        return w
    if mode == lrx.LRX_TRACE_CLOSEST:
        st = compare(hits[w], ref[w], oracle, rays[w])
        assert st["ok"] and st["bitexact_t"] == 1.0, st
    else:
        a = check_anyhit(hits[w], ref[w], oracle, rays[w])
        assert a["ok"], a
    return w


@pytest.mark.parametrize("form", list(FORMS))
@pytest.mark.parametrize("mode", [lrx.LRX_TRACE_CLOSEST, lrx.LRX_TRACE_ANY])
def test_visit_budget_abandons_rays_and_reports(torch_cuda, flat, form, mode):
    desc, rays, oracle, ref = flat
    scene = lrx.Scene(desc)
    bs, pp, var, rf = FORMS[form]
    scene.set_trace_config(bs, pp, var, refill=rf, max_visits=6)
    assert scene.trace_config(mode, bounds=True)["max_visits"] == 6
    hits, rc, status = _trace(torch_cuda, scene, rays, mode)
    assert rc == LRX_ERR_DEVICE and status == STATUS_VISITS, (rc, status)
    w = _check_partial(hits, ref, oracle, rays, mode)
    assert 0.05 < w.mean() < 0.999, w.mean()      # some rays finished within 6 visits, others did not
    # the default bounds: clean and complete
    scene.set_trace_config(bs, pp, var, refill=rf)
    hits, rc, status = _trace(torch_cuda, scene, rays, mode)
    assert rc == 0 and status == 0
    assert _written(hits).all()
    _check_partial(hits, ref, oracle, rays, mode)
    scene.close()


@pytest.mark.parametrize("form", ["persistent", "thread-per-ray", "drain-split"])
def test_deadline_stops_starting_rays_and_reports(torch_cuda, form):
    desc = W.SceneDesc([W.heightfield_mesh(512, W.BASE_SEED + 1)])
    rays = W.random_rays(1 << 21, 302)
    oracle = po.OracleScene(desc)
    ref, _ = oracle.intersect(rays)
    scene = lrx.Scene(desc)
    bs, pp, var, rf = FORMS[form]
    scene.set_trace_config(bs, pp, var, refill=rf, deadline_us=1, modes=1)
    hits, rc, status = _trace(torch_cuda, scene, rays, lrx.LRX_TRACE_CLOSEST)
    assert rc == LRX_ERR_DEVICE and status == STATUS_DEADLINE, (rc, status)
    # most rays were never started (with a 1 us deadline a persistent launch
    # may start none: its warps' first claims contend on one counter for
    # longer than that)
    w = _check_partial(hits, ref, oracle, rays, lrx.LRX_TRACE_CLOSEST)
    assert w.mean() < 0.9, w.mean()
    # the context is still usable: default bounds, full parity
    scene.set_trace_config(bs, pp, var, refill=rf, modes=1)
    hits, rc, status = _trace(torch_cuda, scene, rays, lrx.LRX_TRACE_CLOSEST)
    assert rc == 0 and status == 0 and _written(hits).all()
    _check_partial(hits, ref, oracle, rays, lrx.LRX_TRACE_CLOSEST)
    scene.close()


def test_queue_launch_with_flags_under_tiny_bounds(torch_cuda, flat):
    """Many small batches in one queue launch (persistent fetch) with
    completion flags: every batch's flag is still raised, the status word
    reports the visit budget, written slots are right."""
    torch = torch_cuda
    desc, rays, oracle, ref = flat
    scene = lrx.Scene(desc)
    scene.set_trace_config(64, 8, lrx.LRX_VARIANT_PERSISTENT, refill=8, max_visits=6)
    n = rays.shape[0]
    d_r = torch.from_numpy(np.ascontiguousarray(rays).view(np.uint8).reshape(-1).copy()).cuda()
    d_h = torch.empty(n * 20, dtype=torch.uint8, device="cuda")
    d_h.view(torch.int32).fill_(np.int32(np.uint32(SENT).view(np.int32)).item())
    cuts = np.linspace(0, n, 41).astype(np.int64)
    batches = [(scene, d_r.data_ptr() + 48 * int(a), d_h.data_ptr() + 20 * int(a), int(b - a), lrx.LRX_TRACE_CLOSEST)
               for a, b in zip(cuts[:-1], cuts[1:])]
    counters = torch.zeros(len(batches), dtype=torch.int32, device="cuda")
    flags = torch.zeros(len(batches), dtype=torch.int32, device="cuda")
    st = torch.cuda.current_stream().cuda_stream
    lrx.trace_batches(batches, st, d_tile_counters=counters.data_ptr(), d_done_flags=flags.data_ptr())
    torch.cuda.synchronize()
    assert (flags.cpu().numpy() == 1).all()
    rc, status = _status(scene, st)
    assert rc == LRX_ERR_DEVICE and status == STATUS_VISITS
    hits = d_h.cpu().numpy().view(W.HIT_DTYPE)
    w = _check_partial(hits, ref, oracle, rays, lrx.LRX_TRACE_CLOSEST)
    assert 0.05 < w.mean() < 0.999
    scene.close()


def test_instanced_budget_credits_each_instance_entry(torch_cuda):
    """Two-level scene: with the default bounds no ray runs out (each
    instance entry adds the largest BLAS's node count to the ray's budget);
    with a tiny cap the status word reports it."""
    desc, closest, _any = W.config3(n_meshes=4, freq=12, n_inst=300, n_rays=1 << 17)
    oracle = po.OracleScene(desc, po.ACCEL_MBVH)
    ref, _ = oracle.intersect(closest)
    scene = lrx.Scene(desc)
    hits, rc, status = _trace(torch_cuda, scene, closest, lrx.LRX_TRACE_CLOSEST)
    assert rc == 0 and status == 0 and _written(hits).all()
    _check_partial(hits, ref, oracle, closest, lrx.LRX_TRACE_CLOSEST)
    scene.set_trace_config(64, 8, lrx.LRX_VARIANT_PERSISTENT, refill=8, max_visits=4)
    hits, rc, status = _trace(torch_cuda, scene, closest, lrx.LRX_TRACE_CLOSEST)
    assert rc == LRX_ERR_DEVICE and status == STATUS_VISITS
    _check_partial(hits, ref, oracle, closest, lrx.LRX_TRACE_CLOSEST)
    scene.close()
