"""CPU tests of bench.py's multi-rank path with the gloo backend (world size
2 on 127.0.0.1): the barrier / max-over-ranks helper, and the reference arm
under torchrun, where rank 0 alone measures and prints and the other rank
exits 0 without work."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank_main(rank, world, port, out):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    sys.path.insert(0, ROOT)
    import bench
    d = bench.Dist(use_gpu=False)
    d.barrier()
    m = d.max(float(rank + 1) * 10.0)
    d.close()
    out.put((rank, m))


def test_dist_max_over_two_gloo_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res == {0: 20.0, 1: 20.0}


@pytest.mark.timeout(600)
def test_reference_arm_under_torchrun_two_ranks():
    port = free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), os.path.join(ROOT, "bench.py"),
           "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "3", "--ref-fraction", "256"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=580, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout          # rank 0 alone prints
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["cpu_baseline"]["kind"] == "port"


def _slice_rank_main(rank, world, port, out):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    sys.path.insert(0, ROOT)
    import numpy as np
    import torch.distributed as dist

    from luxcore_gb300 import lrx
    from luxcore_gb300 import workloads as W
    from oracle import pyoracle as po
    dist.init_process_group("gloo")
    desc, rays = W.config1(n_tris=3000, n_rays=10007, seed=91)
    b, e = lrx.rank_slice(rays.shape[0], rank, world)
    hits, _ = po.OracleScene(desc).intersect(rays[b:e])   # this rank's replica, its slice only
    parts = [None] * world
    dist.all_gather_object(parts, (rank, b, e, hits.tobytes()))
    dist.destroy_process_group()
    if rank == 0:
        full, _ = po.OracleScene(desc).intersect(rays)
        got = np.frombuffer(b"".join(p[3] for p in sorted(parts)), W.HIT_DTYPE)
        out.put((sorted((p[1], p[2]) for p in parts), bool(np.array_equal(got.view(np.uint8), full.view(np.uint8)))))


def test_ray_slices_of_two_gloo_ranks_concatenate_to_the_whole_buffer():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=_slice_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    ranges, equal = q.get(timeout=300)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert ranges == [(0, 5004), (5004, 10007)]
    assert equal


def test_rank_slice_covers_the_buffer():
    from luxcore_gb300 import lrx
    for n in (0, 1, 7, 1000, 1 << 20):
        for w in (1, 2, 3, 8):
            s = [lrx.rank_slice(n, r, w) for r in range(w)]
            assert s[0][0] == 0 and s[-1][1] == n
            assert all(a[1] == b[0] for a, b in zip(s, s[1:]))
            assert max(e - b for b, e in s) - min(e - b for b, e in s) <= 1
    with pytest.raises(ValueError):
        lrx.rank_slice(10, 2, 2)
