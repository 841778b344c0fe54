"""Parity at the sizes the benchmark measures, on every ray.

- The heightfield (1024 x 1024 grid, 2,093,058 triangles, the default build
  with its treelet passes): 1,048,576 primary and 1,048,576 bounce rays
  (closest hit) and 4,194,304 shadow rays (any hit), traced as the benchmark
  traces one step -- one lrx_trace_batches call whose three batches run as
  launches of their own on side streams.
- Config 1 at full size: 65,536 random triangles, 1,048,576 rays.
- The instanced two-level scene: 16 displaced icospheres of 200,000
  triangles under 4,096 random affine instances, 8,388,608 closest-hit and
  8,388,608 any-hit rays, through the same batched call.

The oracle (BVHAccel::Intersect, bvhaccel.cpp:170-260, and
MBVHAccel::Intersect, mbvhaccel.cpp:252-357, restated) traces every ray
too; the bar is parity.compare / parity.check_anyhit.
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
THREADS = os.cpu_count() or 1


@pytest.fixture(scope="module")
def torch_cuda(cuda_ready):
    import torch
    return torch


def _device_sets(torch, sets):
    out = []
    for rays, mode in sets:
        d_r = torch.from_numpy(np.ascontiguousarray(rays).view(np.uint8).reshape(-1).copy()).cuda()
        d_h = torch.empty(rays.shape[0] * 20, dtype=torch.uint8, device="cuda")
        d_h.view(torch.int32).fill_(np.int32(np.uint32(SENT).view(np.int32)).item())
        out.append((d_r, d_h, rays.shape[0], mode))
    return out


def _trace_step(torch, scene, sets):
    """The sets as one lrx_trace_batches call on a side stream of torch's."""
    dev = _device_sets(torch, sets)
    stream = torch.cuda.Stream()
    st = stream.cuda_stream
    torch.cuda.synchronize()
    lrx.trace_batches([(scene, r.data_ptr(), h.data_ptr(), n, m) for r, h, n, m in dev], st)
    stream.synchronize()
    assert scene.device_status(st) == 0
    return [h.cpu().numpy().view(W.HIT_DTYPE).copy() for _r, h, _n, _m in dev]


def test_heightfield_step_every_ray(torch_cuda):
    desc = W.SceneDesc([W.heightfield_mesh(1024, W.BASE_SEED + 1)])
    scene = lrx.Scene(desc)
    assert scene.info()["triangle_count"] == 2_093_058
    oracle = po.OracleScene(desc, po.ACCEL_BVH)
    primary = W.pinhole_rays(1024, 1024)
    ref_p, _ = oracle.intersect(primary, n_threads=THREADS)
    bounce = W.bounce_rays(desc, primary, ref_p, 1 << 20, W.BASE_SEED + 100)
    shadow = W.shadow_rays(bounce, 4, W.BASE_SEED + 101)
    assert shadow.shape[0] == 4 << 20
    gp, gb, gs = _trace_step(torch_cuda, scene, [(primary, lrx.LRX_TRACE_CLOSEST), (bounce, lrx.LRX_TRACE_CLOSEST),
                                                 (shadow, lrx.LRX_TRACE_ANY)])
    st = compare(gp, ref_p, oracle, primary)
    assert st["ok"] and st["hit_rate"] > 0.3, st
    ref_b, _ = oracle.intersect(bounce, n_threads=THREADS)
    st = compare(gb, ref_b, oracle, bounce)
    assert st["ok"] and st["hit_rate"] > 0.01, st
    ref_s, _ = oracle.intersect(shadow, n_threads=THREADS)
    a = check_anyhit(gs, ref_s, oracle, shadow)
    assert a["ok"], a
    scene.close()


def test_config1_every_ray(torch_cuda):
    desc, rays = W.config1()
    assert rays.shape[0] == 1 << 20
    scene = lrx.Scene(desc)
    oracle = po.OracleScene(desc, po.ACCEL_BVH)
    ref, _ = oracle.intersect(rays, n_threads=THREADS)
    gc, ga = _trace_step(torch_cuda, scene, [(rays, lrx.LRX_TRACE_CLOSEST), (rays, lrx.LRX_TRACE_ANY)])
    st = compare(gc, ref, oracle, rays)
    assert st["ok"] and st["hit_rate"] > 0.3 and st["bitexact_t"] == 1.0, st
    a = check_anyhit(ga, ref, oracle, rays)
    assert a["ok"], a
    scene.close()


def test_instanced_4096_instances_every_ray(torch_cuda):
    desc, closest, anyr = W.config3()
    assert len(desc.objects) == 4096 and closest.shape[0] == anyr.shape[0] == 1 << 23
    scene = lrx.Scene(desc)
    oracle = po.OracleScene(desc, po.ACCEL_MBVH)
    gc, ga = _trace_step(torch_cuda, scene, [(closest, lrx.LRX_TRACE_CLOSEST), (anyr, lrx.LRX_TRACE_ANY)])
    ref_c, _ = oracle.intersect(closest, n_threads=THREADS)
    st = compare(gc, ref_c, oracle, closest)
    assert st["ok"] and st["hit_rate"] > 0.03, st
    ref_a, _ = oracle.intersect(anyr, n_threads=THREADS)
    a = check_anyhit(ga, ref_a, oracle, anyr)
    assert a["ok"], a
    scene.close()
