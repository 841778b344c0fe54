"""The PATHOCL-style wavefront caller (luxcore_gb300/pathocl.py): one ray
buffer of path and shadow rays traced in place each iteration, masked tasks
included, with the buffer advanced on the device between traces.  Every
iteration's hits are checked against the oracle on the same rays, and the
masked rays' hit slots must stay untouched."""
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))

from luxcore_gb300 import lrx  # noqa: E402
from luxcore_gb300 import pathocl  # noqa: E402
from luxcore_gb300 import workloads as W  # noqa: E402
from oracle import pyoracle as po  # noqa: E402
from parity import compare  # noqa: E402

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda(cuda_ready):
    import torch
    return torch


@pytest.mark.parametrize("variant", [lrx.LRX_VARIANT_PERSISTENT, lrx.LRX_VARIANT_PERSISTENT | lrx.LRX_VARIANT_COMPACT,
                                     0],
                         ids=["persistent", "persistent-compact", "plain"])
def test_wavefront_iterations_match_the_oracle(torch_cuda, variant):
    torch = torch_cuda
    desc = W.SceneDesc([W.heightfield_mesh(65, 701), W.random_triangles(300, 702, size=0.05)])
    scene = lrx.Scene(desc)
    scene.set_trace_config(64, 8, variant, modes=1, refill=8 if variant else 0)
    oracle = po.OracleScene(desc)
    stream = torch.cuda.Stream()
    with torch.cuda.stream(stream):
        wf = pathocl.WavefrontPaths(scene, desc, 96, 96, max_depth=3, stream=stream)
        seen_masked = seen_shadow = 0
        for it in range(10):
            rays = wf.rays.cpu().numpy().copy().view(np.uint8).view(W.RAY_DTYPE).reshape(-1)
            before = wf.hits.cpu().numpy().copy()
            state = wf.state.cpu().numpy()
            wf.trace()
            stream.synchronize()
            hits = wf.hits.cpu().numpy().view(np.uint8).view(W.HIT_DTYPE).reshape(-1)
            masked = (rays["flags"] & W.RAY_FLAGS_MASKED) != 0
            seen_masked += int(masked.sum())
            seen_shadow += int(((state == pathocl.DIRECT_LIGHT) & ~masked).sum())
            # masked rays: hit slots untouched
            assert np.array_equal(hits.view(np.float32).reshape(-1, 5)[masked].view(np.uint32),
                                  before[masked].view(np.uint32))
            ref, _ = oracle.intersect(rays[~masked])
            st = compare(hits[~masked], ref, oracle, rays[~masked])
            assert st["ok"], (it, st)
            wf.advance()
        stream.synchronize()
    assert seen_masked > 0 and seen_shadow > 0
    assert wf.traced > 0
    img = wf.image()
    assert np.isfinite(img).all() and img.max() > 0
    assert float(wf.samples.sum()) > 0


def test_wavefront_on_an_instanced_scene_and_its_ray_harvest(torch_cuda):
    """Instances are shaded too (normals under the inverse transpose of the
    instance transform); the harvested bounce and shadow rays are rays of the
    scene that the oracle traces like the engine."""
    torch = torch_cuda
    desc, _c, _a = W.config3(n_rays=1, n_meshes=3, freq=10, n_inst=60, extent=2.0, scale=(0.2, 0.5))
    scene = lrx.Scene(desc)
    oracle = po.OracleScene(desc, po.ACCEL_MBVH)
    stream = torch.cuda.Stream()
    with torch.cuda.stream(stream):
        wf = pathocl.WavefrontPaths(scene, desc, 128, 128, max_depth=3, eye=(1.0, -1.2, 1.6), look=(1.0, 1.0, 0.8),
                                    light=(0.9, 1.1, 1.9), stream=stream)
        for it in range(4):
            rays = wf.rays.cpu().numpy().copy().view(np.uint8).view(W.RAY_DTYPE).reshape(-1)
            wf.trace()
            stream.synchronize()
            hits = wf.hits.cpu().numpy().view(np.uint8).view(W.HIT_DTYPE).reshape(-1)
            live = (rays["flags"] & W.RAY_FLAGS_MASKED) == 0
            ref, _ = oracle.intersect(rays[live])
            st = compare(hits[live], ref, oracle, rays[live])
            assert st["ok"], (it, st)
            wf.advance()
        bounce, shadow = wf.harvest(20000, 20000)
        stream.synchronize()
    assert bounce.shape == (20000, 12) and shadow.shape == (20000, 12)
    b = bounce.cpu().numpy().view(np.uint8).view(W.RAY_DTYPE).reshape(-1)
    s = shadow.cpu().numpy().view(np.uint8).view(W.RAY_DTYPE).reshape(-1)
    assert ((b["flags"] & W.RAY_FLAGS_MASKED) == 0).all() and ((s["flags"] & W.RAY_FLAGS_MASKED) == 0).all()
    assert (s["maxt"] < 1e29).all() and (b["maxt"] > 1e29).all()   # shadow rays stop short of the light
    # a bounce ray starts on a surface and leaves it: its origin is a hit point
    ref_b, _ = oracle.intersect(b)
    assert (ref_b["meshIndex"] != W.NULL_INDEX).mean() > 0.05
