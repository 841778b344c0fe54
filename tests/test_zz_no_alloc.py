"""lrx_trace_host_noalloc, the entry point for callers that cannot allocate
device memory -- a host loop sharing the GPU with other work in flight
(cudaFree can synchronise the whole device), or an application whose device
memory all belongs to its own fixed pool.  It stages rays and hits, and the
scratch of sorted and compacted launches, through a static array reserved
when the library loads instead of cudaMalloc'd or pooled buffers.

Checked here through the C ABI:
- on consecutive calls with different batches (so a call could see the
  previous call's leftovers) it returns exactly what lrx_trace_host returns,
  under the default launch configurations (closest hit on persistent warps,
  any hit through the ray sort at this size) and under ray compaction;
- in a fresh process, the device's free memory is the same before and after
  sorted and compacted calls of the largest size: nothing was allocated;
- it rejects a batch larger than its staging area.
This file is collected last so that a stopping run has run every other test
before it; it also passes on its own in a fresh process.
"""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

from luxcore_gb300 import lrx
from luxcore_gb300 import workloads as W

pytestmark = pytest.mark.gpu

SENTINEL = 0xDEADBEEF
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _prefilled(n):
    h = np.zeros(n, W.HIT_DTYPE)
    h.view(np.uint32).reshape(-1)[:] = SENTINEL
    return h


def _noalloc(L, scene, rays, mode):
    got = _prefilled(rays.shape[0])
    rc = L.lrx_trace_host_noalloc(scene.handle, rays.ctypes.data, got.ctypes.data, rays.shape[0], mode, None)
    assert rc == 0, L.lrx_last_error()
    return got


def _check_against_trace_host(L, scene, batches):
    for n, mode, seed in batches:
        rays = W.random_rays(n, seed)
        rays["flags"][::13] = W.RAY_FLAGS_MASKED       # their hits must stay untouched
        expected = scene.trace_host(rays, _prefilled(n), mode)
        got = _noalloc(L, scene, rays, mode)
        # the parity tests' bar is bit-exact t/b1/b2 here; demand identical bytes
        assert np.array_equal(got.view(np.uint8), expected.view(np.uint8)), (n, mode)
        hit = (got["meshIndex"] != W.NULL_INDEX) & (got["meshIndex"] != SENTINEL)
        assert hit.mean() > 0.2
        assert (got.view(np.uint32).reshape(n, 5)[::13] == SENTINEL).all()


def test_noalloc_matches_trace_host_on_consecutive_calls(cuda_ready):
    L = lrx.load()
    scene_desc, _ = W.config1(n_tris=40000, n_rays=1, seed=201)
    scene = lrx.Scene(scene_desc)
    # calls in a row: a full-size closest-hit batch (persistent warps), a
    # full-size any-hit batch (sorted before tracing), then a smaller any-hit
    # batch (below the sort threshold, traced in caller order)
    _check_against_trace_host(L, scene, [(lrx.LRX_NOALLOC_MAX_RAYS, lrx.LRX_TRACE_CLOSEST, 202),
                                         (lrx.LRX_NOALLOC_MAX_RAYS, lrx.LRX_TRACE_ANY, 203),
                                         (30011, lrx.LRX_TRACE_ANY, 206)])
    scene.close()


def test_noalloc_matches_trace_host_with_compaction(cuda_ready):
    L = lrx.load()
    scene_desc, _ = W.config1(n_tris=40000, n_rays=1, seed=207)
    scene = lrx.Scene(scene_desc)
    scene.set_trace_config(64, 8, lrx.LRX_VARIANT_PERSISTENT | lrx.LRX_VARIANT_COMPACT, modes=1, refill=8)
    scene.set_trace_config(64, 8, lrx.LRX_VARIANT_SORT_OCTANT | lrx.LRX_VARIANT_SORT_RAYS, modes=2)
    _check_against_trace_host(L, scene, [(lrx.LRX_NOALLOC_MAX_RAYS, lrx.LRX_TRACE_CLOSEST, 208),
                                         (lrx.LRX_NOALLOC_MAX_RAYS - 7, lrx.LRX_TRACE_CLOSEST, 209),
                                         (lrx.LRX_NOALLOC_MAX_RAYS, lrx.LRX_TRACE_ANY, 210)])
    scene.close()


# Run in a fresh process with every kernel loaded at start-up, so the only
# thing that could change the device's free memory between the two readings
# is an allocation (a memory pool reserving memory, a cudaMalloc).  The
# warm-up calls launch the same traversal kernels first, through paths that
# use no scratch, so the driver's local-memory reservation for them is
# already made.
_PROBE = r"""
import ctypes, json, sys
sys.path.insert(0, sys.argv[1])
import numpy as np
from luxcore_gb300 import lrx
from luxcore_gb300 import workloads as W

L = lrx.load()
cu = ctypes.CDLL("libcuda.so.1")

def free_bytes():
    ctx = ctypes.c_void_p()
    assert cu.cuCtxGetCurrent(ctypes.byref(ctx)) == 0 and ctx.value, "no current context"
    f, t = ctypes.c_size_t(), ctypes.c_size_t()
    assert cu.cuMemGetInfo_v2(ctypes.byref(f), ctypes.byref(t)) == 0
    return f.value

scene = lrx.Scene(W.config1(n_tris=40000, n_rays=1, seed=211)[0])
n = lrx.LRX_NOALLOC_MAX_RAYS

def call(rays, mode):
    hits = np.zeros(rays.shape[0], W.HIT_DTYPE)
    rc = L.lrx_trace_host_noalloc(scene.handle, rays.ctypes.data, hits.ctypes.data, rays.shape[0], mode, None)
    assert rc == 0, L.lrx_last_error()
    return hits

small = W.random_rays(1000, 212)
call(small, lrx.LRX_TRACE_CLOSEST)      # persistent warps, no scratch
call(small, lrx.LRX_TRACE_ANY)          # below the sort threshold, no scratch
before = free_bytes()
big = W.random_rays(n, 213)
for _ in range(2):
    call(big, lrx.LRX_TRACE_ANY)        # the ray sort's keys, indices and temp storage
scene.set_trace_config(64, 8, lrx.LRX_VARIANT_PERSISTENT | lrx.LRX_VARIANT_COMPACT, modes=1, refill=8)
for _ in range(2):
    call(big, lrx.LRX_TRACE_CLOSEST)    # the compaction's index list and temp storage
after = free_bytes()
print(json.dumps({"before": before, "after": after}))
"""


def test_noalloc_allocates_nothing_in_a_fresh_process(cuda_ready):
    env = dict(os.environ, CUDA_MODULE_LOADING="EAGER")
    r = subprocess.run([sys.executable, "-c", _PROBE, ROOT], env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    mem = json.loads(r.stdout.strip().splitlines()[-1])
    assert mem["after"] == mem["before"], mem


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
