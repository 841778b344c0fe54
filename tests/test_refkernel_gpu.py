"""The reference's own CUDA intersection kernel on this GPU -- the comparison
arm bench.py times beside the engine.

The kernel text is the reference's bvh.cl with the OpenCL emulation prefix
its CUDA device adds, stitched by oracle/build_ref.sh from the LuxCore tree
and compiled here with NVRTC under the reference's options;
oracle/refcu_harness.cpp launches it with 32-thread blocks over the oracle's
BVHArrayNode[].  Checked:
- built exactly (--fmad=false in place of --use_fast_math), against the
  golden fixtures, which are the same kernel text run on the CPU
  (tests/golden/make_golden.py): the same triangles on every ray except
  exact-t ties, t/b1/b2 within the parity tolerance, masked rays untouched;
  and against the oracle on a config-1 scene: the parity bar;
- built as the reference's PATHOCL engine deploys it (--use_fast_math, the
  form bench.py times): the same triangles on nearly every ray, t within
  1e-4.
Skipped where the kernel text was not built (a checkout without the LuxCore
source tree).
"""
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.dirname(__file__))
sys.path.insert(0, os.path.join(os.path.dirname(__file__), "golden"))

from luxcore_gb300 import workloads as W  # noqa: E402
from oracle import pyoracle as po  # noqa: E402
from parity import compare  # noqa: E402

pytestmark = pytest.mark.gpu

SENT = 0xDEADBEEF


@pytest.fixture(scope="module")
def refk(cuda_ready):
    """The kernel built with --fmad=false instead of --use_fast_math: the
    same text and the same FP32 operations as its CPU run (compiled with
    -ffp-contract=off)."""
    import torch
    torch.cuda.init()
    k = po.RefCudaKernel(fast_math=False)
    if not k.available:
        pytest.skip(k.reason)
    return torch, k


def _ref_gpu_trace(torch, k, scene, rays):
    o = po.OracleScene(scene, po.ACCEL_BVH)
    nodes = torch.from_numpy(o.bvh_nodes().copy()).cuda()
    verts = torch.from_numpy(np.ascontiguousarray(np.concatenate([m.vertices for m in scene.meshes]),
                                                  np.float32).copy()).cuda()
    d_r = torch.from_numpy(np.ascontiguousarray(rays).view(np.uint8).reshape(-1).copy()).cuda()
    d_h = torch.empty(rays.shape[0] * 20, dtype=torch.uint8, device="cuda")
    d_h.view(torch.int32).fill_(np.int32(np.uint32(SENT).view(np.int32)).item())
    torch.cuda.synchronize()
    k.trace(d_r.data_ptr(), d_h.data_ptr(), rays.shape[0], verts.data_ptr(), nodes.data_ptr(), 32,
            torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    return d_h.cpu().numpy().view(W.HIT_DTYPE).copy(), o


@pytest.mark.parametrize("name", ["golden_random", "golden_heightfield", "golden_multimesh"])
def test_reference_kernel_on_gpu_matches_its_cpu_run(refk, name):
    from make_golden import load
    torch, k = refk
    scene, rays, golden = load(name)
    gpu, o = _ref_gpu_trace(torch, k, scene, rays)
    masked = (rays["flags"] & W.RAY_FLAGS_MASKED) != 0
    assert (gpu.view(np.uint32).reshape(-1, 5)[masked] == SENT).all()
    finite = ~masked & np.isfinite(rays["o"]).all(1) & np.isfinite(rays["d"]).all(1) & ~np.isnan(rays["maxt"])
    st = compare(gpu[finite], golden[finite], o, rays[finite])
    assert st["bad_disagreements"] == 0 and st["values_ok"] and st["agree"] >= 0.99, st


def test_reference_kernel_on_gpu_against_the_oracle(refk):
    torch, k = refk
    scene, rays = W.config1(n_tris=20000, n_rays=1 << 16, seed=61)
    gpu, o = _ref_gpu_trace(torch, k, scene, rays)
    ref, _ = o.intersect(rays)
    st = compare(gpu, ref, o, rays)
    assert st["bad_disagreements"] == 0 and st["values_ok"] and st["agree"] >= 0.999, st


def test_reference_kernel_with_fast_math_as_pathocl_builds_it(refk):
    """--use_fast_math (the reference's PATHOCL engine adds it): the same
    triangles on nearly every ray, t within 1e-4 relative -- the reference
    kernel as deployed, which bench.py times."""
    torch, _ = refk
    k = po.RefCudaKernel(fast_math=True)
    assert k.available, k.reason
    scene, rays = W.config1(n_tris=20000, n_rays=1 << 16, seed=62)
    gpu, o = _ref_gpu_trace(torch, k, scene, rays)
    ref, _ = o.intersect(rays)
    same = (gpu["meshIndex"] == ref["meshIndex"]) & (gpu["triangleIndex"] == ref["triangleIndex"])
    assert same.mean() >= 0.999
    hit = same & (ref["meshIndex"] != W.NULL_INDEX)
    rel = np.abs(gpu["t"][hit].astype(np.float64) - ref["t"][hit]) / np.abs(ref["t"][hit])
    assert rel.max() <= 1e-4, rel.max()
