"""GPU tests of the serving loop (lrx_server): every request's hits are the
same when it runs alone and when it runs mixed with others (continuous
batching through the queue kernel), scenes are evicted and rebuilt under a
tight HBM budget without changing results, and admission errors surface on
the request."""
import os
import sys
import threading

import numpy as np
import pytest

sys.path.insert(0, os.path.dirname(__file__))

from luxcore_gb300 import lrx  # noqa: E402
from luxcore_gb300 import workloads as W  # noqa: E402

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda(cuda_ready):
    import torch
    return torch


def scene_set():
    flat = W.SceneDesc([W.random_triangles(30000, 501)])
    multi = W.SceneDesc([W.random_triangles(8000, 502), W.heightfield_mesh(40, 503)])
    inst, _, _ = W.config3(n_rays=1, n_meshes=2, freq=8, n_inst=40, extent=1.0, scale=(0.05, 0.2))
    return [flat, multi, inst]


def make_requests(torch, n_scenes, n_req, seed):
    rng = np.random.default_rng(seed)
    reqs = []
    for k in range(n_req):
        n = int(rng.integers(1, 40000))
        sid = int(rng.integers(0, n_scenes))
        mode = lrx.LRX_TRACE_ANY if rng.random() < 0.3 else lrx.LRX_TRACE_CLOSEST
        rays = W.random_rays(n, seed * 1000 + k)
        rays["flags"][::23] = W.RAY_FLAGS_MASKED
        d_r = torch.from_numpy(rays.view(np.uint8).reshape(-1).copy()).cuda()
        d_h = torch.zeros(n * 20, dtype=torch.uint8, device="cuda")
        reqs.append((sid, d_r, d_h, n, mode))
    return reqs


def alone_results(torch, descs, reqs):
    # the server builds the plain LBVH (no treelet passes); any-hit results
    # depend on the tree, so the reference uses the same build
    scenes = [lrx.Scene(d, treelet_passes=0) for d in descs]
    out = []
    st = torch.cuda.current_stream().cuda_stream
    for sid, d_r, _, n, mode in reqs:
        h = torch.zeros(n * 20, dtype=torch.uint8, device="cuda")
        scenes[sid].trace(d_r.data_ptr(), h.data_ptr(), n, mode, st)
        out.append(h)
    torch.cuda.synchronize()
    res = [h.cpu().numpy() for h in out]
    for s in scenes:
        s.close()
    return res


def serve_all(server, ids, reqs):
    tickets = [server.submit(ids[sid], d_r.data_ptr(), d_h.data_ptr(), n, mode) for sid, d_r, d_h, n, mode in reqs]
    for t in tickets:
        server.wait(t)
    return [d_h.cpu().numpy() for _, _, d_h, _, _ in reqs]


@pytest.mark.parametrize("policy", [lrx.LRX_SERVE_BATCHED, lrx.LRX_SERVE_PLAIN], ids=["batched", "plain"])
def test_results_same_alone_and_in_the_mix(torch_cuda, policy):
    torch = torch_cuda
    descs = scene_set()
    reqs = make_requests(torch, len(descs), 60, 11)
    ref = alone_results(torch, descs, reqs)
    server = lrx.Server(policy=policy)
    ids = [server.add_scene(d) for d in descs]
    torch.cuda.synchronize()
    mixed = serve_all(server, ids, reqs)                    # all in flight together
    for k, (a, b) in enumerate(zip(ref, mixed)):
        assert np.array_equal(a, b), k
    for _, _, d_h, _, _ in reqs:
        d_h.zero_()
    torch.cuda.synchronize()
    one_by_one = []
    for r in reqs:                                           # each request alone in the server
        one_by_one += serve_all(server, ids, [r])
    for k, (a, b) in enumerate(zip(ref, one_by_one)):
        assert np.array_equal(a, b), k
    st = server.stats()
    assert st["requests_done"] == 2 * len(reqs) and st["requests_failed"] == 0
    assert st["scene_builds"] == len(descs) and st["scene_evictions"] == 0
    if policy == lrx.LRX_SERVE_BATCHED:
        assert st["launches"] < 2 * len(reqs)               # requests shared launches
    assert st["latency_p99_us"] >= st["latency_p50_us"] > 0
    server.close()


@pytest.mark.parametrize("cache", [True, False], ids=["blob-cache", "rebuild"])
def test_lru_eviction_under_a_tight_budget(torch_cuda, cache):
    """Scenes are evicted (LRU) and brought back -- from the host blob cache,
    or rebuilt without it -- with unchanged results."""
    torch = torch_cuda
    descs = scene_set()
    probe = [lrx.Scene(d, treelet_passes=0) for d in descs]  # the server's build
    sizes = [p.info()["device_bytes"] for p in probe]
    for p in probe:
        p.close()
    budget = max(sizes) + min(sizes) // 2                    # one scene at a time, roughly
    reqs = make_requests(torch, len(descs), 40, 12)
    ref = alone_results(torch, descs, reqs)
    server = lrx.Server(budget_bytes=budget, streams=2, host_cache_bytes=0 if cache else 2**64 - 1)
    ids = [server.add_scene(d) for d in descs]
    got = []
    for r in reqs:                                           # scene changes force evictions
        got += serve_all(server, ids, [r])
    for k, (a, b) in enumerate(zip(ref, got)):
        assert np.array_equal(a, b), k
    st = server.stats()
    assert st["scene_evictions"] > 0
    if cache:   # each scene built once, then reloaded from its blob
        assert st["scene_builds"] == len(set(r[0] for r in reqs)) and st["scene_reloads"] > 0
        assert st["host_cache_bytes"] > 0
    else:
        assert st["scene_builds"] > len(descs) and st["scene_reloads"] == 0
    assert st["peak_resident_bytes"] <= budget + max(sizes)
    server.close()


def test_budget_smaller_than_a_scene_fails_the_request(torch_cuda):
    torch = torch_cuda
    server = lrx.Server(budget_bytes=1024)
    sid = server.add_scene(W.SceneDesc([W.random_triangles(5000, 504)]))
    rays = W.random_rays(100, 505)
    d_r = torch.from_numpy(rays.view(np.uint8).reshape(-1).copy()).cuda()
    d_h = torch.zeros(100 * 20, dtype=torch.uint8, device="cuda")
    t = server.submit(sid, d_r.data_ptr(), d_h.data_ptr(), 100, lrx.LRX_TRACE_CLOSEST)
    with pytest.raises(lrx.LrxError) as e:
        server.wait(t)
    assert e.value.status == 7  # LRX_ERR_BUDGET
    assert server.stats()["requests_failed"] == 1
    server.close()


def test_launch_ray_cap_gives_each_larger_request_a_launch(torch_cuda):
    """max_rays_per_launch: a batched launch stops admitting requests once
    their rays reach the cap, so requests of more rays than the cap get one
    launch each, however they queue; their hits are those of lone traces."""
    torch = torch_cuda
    descs = scene_set()[:1]
    reqs = []
    for k in range(12):
        rays = W.random_rays(4096, 7700 + k)
        reqs.append((0, torch.from_numpy(rays.view(np.uint8).reshape(-1).copy()).cuda(),
                     torch.zeros(4096 * 20, dtype=torch.uint8, device="cuda"), 4096,
                     lrx.LRX_TRACE_CLOSEST if k % 2 == 0 else lrx.LRX_TRACE_ANY))
    ref = alone_results(torch, descs, reqs)
    server = lrx.Server(max_rays_per_launch=1000)
    ids = [server.add_scene(d) for d in descs]
    server.reset_stats()
    got = serve_all(server, ids, reqs)
    st = server.stats()
    server.close()
    assert st["launches"] == len(reqs) and st["requests_done"] == len(reqs), st
    for a, b in zip(got, ref):
        assert np.array_equal(a, b)


def test_concurrent_sessions(torch_cuda):
    torch = torch_cuda
    descs = scene_set()
    reqs = make_requests(torch, len(descs), 64, 13)
    ref = alone_results(torch, descs, reqs)
    server = lrx.Server(streams=4)
    ids = [server.add_scene(d) for d in descs]
    errors = []

    def session(chunk):
        try:
            for r in chunk:                                   # submit, wait, next bounce
                serve_all(server, ids, [r])
        except Exception as ex:  # noqa: BLE001
            errors.append(ex)

    threads = [threading.Thread(target=session, args=(reqs[i::8],)) for i in range(8)]
    for th in threads:
        th.start()
    for th in threads:
        th.join(timeout=120)
    assert not errors
    for k, (r, a) in enumerate(zip(reqs, ref)):
        assert np.array_equal(r[2].cpu().numpy(), a), k
    server.close()
