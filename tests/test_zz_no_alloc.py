"""lrx_trace_host_noalloc, the entry point for callers that cannot allocate
device memory -- a host loop sharing the GPU with other work in flight
(cudaFree can synchronise the whole device), or an application whose device
memory all belongs to its own fixed pool.  It stages rays and hits through a
static array reserved when the library loads instead of cudaMalloc'd buffers.

Checked here through the C ABI: on consecutive calls with different batches
(so a call could see the previous call's leftovers) it returns exactly what
lrx_trace_host returns, and it rejects a batch larger than its staging area.
This file is collected last so that a stopping run has run every other test
before it; it also passes on its own in a fresh process.
"""
import ctypes

import numpy as np
import pytest

from luxcore_gb300 import lrx
from luxcore_gb300 import workloads as W

pytestmark = pytest.mark.gpu

SENTINEL = 0xDEADBEEF


def _prefilled(n):
    h = np.zeros(n, W.HIT_DTYPE)
    h.view(np.uint32).reshape(-1)[:] = SENTINEL
    return h


def test_noalloc_matches_trace_host_on_consecutive_calls(cuda_ready):
    L = lrx.load()
    scene_desc, _ = W.config1(n_tris=40000, n_rays=1, seed=201)
    scene = lrx.Scene(scene_desc)
    # two calls in a row: a full-size batch, then a smaller one in the other mode
    batches = [(lrx.LRX_NOALLOC_MAX_RAYS, lrx.LRX_TRACE_CLOSEST, 202),
               (30011, lrx.LRX_TRACE_ANY, 203)]
    for n, mode, seed in batches:
        rays = W.random_rays(n, seed)
        rays["flags"][::13] = W.RAY_FLAGS_MASKED       # their hits must stay untouched
        expected = scene.trace_host(rays, _prefilled(n), mode)
        got = _prefilled(n)
        rc = L.lrx_trace_host_noalloc(scene.handle, rays.ctypes.data, got.ctypes.data, n, mode, None)
        assert rc == 0, L.lrx_last_error()
        # the parity tests' bar is bit-exact t/b1/b2 here; demand identical bytes
        assert np.array_equal(got.view(np.uint8), expected.view(np.uint8))
        hit = (got["meshIndex"] != W.NULL_INDEX) & (got["meshIndex"] != SENTINEL)
        assert hit.mean() > 0.2
    scene.close()


def test_noalloc_rejects_batches_beyond_the_staging_area(cuda_ready):
    L = lrx.load()
    scene = lrx.Scene(W.SceneDesc([W.random_triangles(100, 204)]))
    n = lrx.LRX_NOALLOC_MAX_RAYS + 1
    rays = W.random_rays(n, 205)
    hits = _prefilled(n)
    rc = L.lrx_trace_host_noalloc(scene.handle, rays.ctypes.data, hits.ctypes.data, n, 0, None)
    assert rc == 1
    assert b"limit" in L.lrx_last_error()
    assert (hits.view(np.uint32) == SENTINEL).all()     # nothing was written
    scene.close()
