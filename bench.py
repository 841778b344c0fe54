#!/usr/bin/env python
"""Benchmark of the LuxRays intersection path on GB300.

Workload (one "step"): the fBm heightfield scene -- a 1024x1024 vertex grid
over [0,1]^2, 2,093,058 FP32 triangles, heights from seeded 6-octave value
noise scaled to [0, 0.2] -- traced with three ray sets:
  1,048,576 pinhole primary rays (eye (0.5,-0.5,0.6), look-at (0.5,0.5,0),
            vertical fov 60 deg), closest hit;
  1,048,576 cosine-hemisphere bounce rays from the primary hit points,
            closest hit;
  4,194,304 shadow rays from the bounce origins to 4 point lights in
            [0,1]^2 x [0.5,1], any hit.
All inputs are seeded synthetic data (no public scene is named for this
path).  Rays (302 MB) and hits (126 MB) exceed the 129 MB L2, so no flush is
needed between steps.

--impl lrx (default): the CUDA engine through liblrx.so.
--impl reference: the reference's CPU accelerator on the host cores (the
  oracle's restatement of BVHAccel::Intersect, all host threads).
Multi-GPU (torchrun): ray batches are independent, so each rank traces its
own copy of the workload on its own scene replica (weak scaling, no
collective on the data path); rank 0 prints the aggregate.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

from luxcore_gb300 import workloads as W  # noqa: E402

METRIC = "Mrays/s closest/any-hit (1 GB300, % HBM roofline); served p50/p99 vs plain launch"
UNIT = "Mrays/s"
WORKLOAD = "heightfield-2093058tri: 1048576 primary + 1048576 bounce (closest) + 4194304 shadow (any-hit)"
HEIGHTFIELD_RES = 1024
SHADOW_LIGHTS = 4
NODE_BYTES, TRI_BYTES, INST_BYTES, RAY_BYTES, HIT_BYTES = 80, 48, 80, 48, 20


def log(*a):
    print(*a, file=sys.stderr, flush=True)


# ---------------------------------------------------------------------------
# distributed helpers (torchrun)
# ---------------------------------------------------------------------------

def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class Dist:
    def __init__(self, use_gpu: bool):
        self.ws, self.rank, self.local = dist_env()
        self.pg = None
        if self.ws > 1:
            import torch
            import torch.distributed as dist
            if use_gpu:
                torch.cuda.set_device(self.local)
            dist.init_process_group("nccl" if use_gpu else "gloo")
            self.pg = dist

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def max(self, v: float) -> float:
        if not self.pg:
            return v
        import torch
        t = torch.tensor([v], dtype=torch.float64, device="cuda" if self.pg.get_backend() == "nccl" else "cpu")
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.pg:
            self.pg.destroy_process_group()


# ---------------------------------------------------------------------------
# clocks
# ---------------------------------------------------------------------------

class ClockSampler:
    """nvidia-smi sampled every 200 ms during the timed region."""
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------------
# workload
# ---------------------------------------------------------------------------

def make_scene():
    return W.SceneDesc([W.heightfield_mesh(HEIGHTFIELD_RES, W.BASE_SEED + 1)])


def derived_rays(scene, primary, primary_hits, seed):
    bounce = W.bounce_rays(scene, primary, primary_hits, 1 << 20, seed)
    shadow = W.shadow_rays(bounce, SHADOW_LIGHTS, seed + 1)
    return bounce, shadow


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


# DRAM bytes per ray of each ray set's traversal launch, from one ncu
# capture of this workload (dram__bytes_read.sum + dram__bytes_write.sum over
# the rays of the launch; the capture's command and table are in
# profiles/trace_heightfield_ncu.md).  A constant of that capture, not a
# figure of this run: the line says so in roofline.traffic_source.
TRAFFIC_PER_RAY = {"primary": 146.6, "bounce": 271.5, "shadow": 194.5}
TRAFFIC_SOURCE = ("ncu capture of the traversal launches of one step (profiles/trace_heightfield_ncu.md), "
                  "not this run; DRAM bytes per launch averaged over the three sets")


def count_kernel_launches(stream_handle, fn):
    """Kernels that fn() enqueues on the stream: the calls are captured into a
    CUDA graph (driver API, relaxed mode; nothing runs) and its kernel nodes
    counted -- this includes the ray-sort kernels of sorted launches.  None if
    the capture is not possible."""
    import ctypes
    try:
        cu = ctypes.CDLL("libcuda.so.1")
        s = ctypes.c_void_p(stream_handle)
        if cu.cuStreamBeginCapture_v2(s, ctypes.c_int(2)) != 0:  # CU_STREAM_CAPTURE_MODE_RELAXED
            return None
        ok = True
        try:
            fn()
        except Exception:  # a call that cannot be captured: no count
            ok = False
        g = ctypes.c_void_p()
        rc = cu.cuStreamEndCapture(s, ctypes.byref(g))
        if rc != 0 or not g.value:
            return None
        if not ok:
            cu.cuGraphDestroy(g)
            return None
        n = ctypes.c_size_t(0)
        cu.cuGraphGetNodes(g, None, ctypes.byref(n))
        nodes = (ctypes.c_void_p * n.value)()
        cu.cuGraphGetNodes(g, nodes, ctypes.byref(n))
        kernels = 0
        for k in range(n.value):
            t = ctypes.c_int(-1)
            cu.cuGraphNodeGetType(ctypes.c_void_p(nodes[k]), ctypes.byref(t))
            kernels += t.value == 0  # CU_GRAPH_NODE_TYPE_KERNEL
        cu.cuGraphDestroy(g)
        return kernels
    except (OSError, AttributeError):
        return None


# ---------------------------------------------------------------------------
# CPU arm (the reference's CPU accelerator, restated)
# ---------------------------------------------------------------------------

def cpu_measure(scene, sets, threads: int, accel: str = "bvh", keep_hits: bool = False):
    """Times the oracle's BVHAccel::Intersect (or MBVHAccel::Intersect for
    instanced scenes) over the given ray sets; with keep_hits, also returns
    the oracle's hits per set (for the parity check of the GPU's)."""
    from oracle import pyoracle as po
    o = po.OracleScene(scene, po.ACCEL_MBVH if accel == "mbvh" else po.ACCEL_BVH)
    total, secs, hits = 0, 0.0, []
    for rays in sets:
        h, s = o.intersect(rays, n_threads=threads)
        secs += s
        total += rays.shape[0]
        if keep_hits:
            hits.append(h)
    if keep_hits:
        return total, secs, o, hits
    return total, secs, o


def parity_block(oracle_scene, sets, gpu_hits, ref_hits, stride: int):
    """The GPU hits of the timed step against the oracle's on the CPU
    sample (every `stride`-th ray of each set): closest-hit sets by
    oracle.parity.compare, any-hit sets by oracle.parity.check_anyhit."""
    from oracle.parity import check_anyhit, compare
    out, ok = {}, True
    for (name, rays, mode), g, r in zip(sets, gpu_hits, ref_hits):
        g = np.ascontiguousarray(g[::stride])
        rs = np.ascontiguousarray(rays[::stride])
        if mode == 0:
            c = compare(g, r, oracle_scene, rs)
            out[name] = {k: c[k] for k in ("n", "agree", "ties", "bad_disagreements", "bitexact_t", "values_ok",
                                           "ties_valid", "ok")}
        else:
            c = check_anyhit(g, r, oracle_scene, rs)
            out[name] = {"n": c["n"], "hitmiss_agree": c["hitmiss_agree"], "valid": c["valid"], "ok": c["ok"]}
        ok = ok and out[name]["ok"]
    out["ok"] = bool(ok)
    out["sample"] = f"every {stride}th ray of each set, GPU hits of the last timed step"
    return out


def reference_layout_bytes(o, sets, stride: int = 16):
    """B_ref: the bytes per ray that the reference's own layout fetches for the
    same rays -- one 32-B BVHArrayNode per node visit and, per leaf visit,
    three 12-B vertices plus the 12-B index triple -- with the ray read and
    the 20-B RayHit write, counted by the oracle's BVHAccel walk
    (bvhaccel.cpp:170-260; `o` an OracleScene) over every `stride`-th ray of
    each set."""
    out = {}
    for name, rays in sets:
        nodes, leaves = o.visit_stats(np.ascontiguousarray(rays[::stride]))
        out[name] = {"nodes_per_ray": round(nodes, 2), "leaves_per_ray": round(leaves, 2),
                     "bytes_per_ray": round(RAY_BYTES + HIT_BYTES + 32 * nodes + 48 * leaves, 1)}
    return out


def reference_gpu_arm(torch, oracle_scene, scene_desc, sets, ref_hits, stride, stream, device, reps=3):
    """The reference's own CUDA kernel (bvh.cl as its CUDA device compiles it,
    oracle.pyoracle.RefCudaKernel) on this GPU over the oracle's
    BVHArrayNode[] with 32-thread blocks: Mrays/s per set (CUDA events on
    `stream`, `reps` launches after one warm-up) and its hits' parity with
    the oracle on the CPU sample.  The reference kernel has no any-hit mode,
    so every set, shadow rays included, is a closest-hit trace."""
    from oracle import pyoracle as po
    from oracle.parity import compare
    k = po.RefCudaKernel(fast_math=True)
    if not k.available:
        return {"unavailable": k.reason}
    nodes = torch.from_numpy(oracle_scene.bvh_nodes().copy()).to(device)
    verts = torch.from_numpy(np.ascontiguousarray(np.concatenate([m.vertices for m in scene_desc.meshes]),
                                                  np.float32).copy()).to(device)
    st = stream.cuda_stream
    per_ms, per_mrays, parity = {}, {}, {}
    total_rays, total_ms = 0, 0.0
    for (name, rays, _mode), rh in zip(sets, ref_hits):
        n = rays.shape[0]
        d_r = torch.from_numpy(np.ascontiguousarray(rays).view(np.uint8).reshape(-1).copy()).to(device)
        d_h = torch.empty(n * HIT_BYTES, dtype=torch.uint8, device=device)
        torch.cuda.synchronize()
        k.trace(d_r.data_ptr(), d_h.data_ptr(), n, verts.data_ptr(), nodes.data_ptr(), 32, st)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            k.trace(d_r.data_ptr(), d_h.data_ptr(), n, verts.data_ptr(), nodes.data_ptr(), 32, st)
        e1.record(stream)
        e1.synchronize()
        ms = e0.elapsed_time(e1) / reps
        per_ms[name] = round(ms, 4)
        per_mrays[name] = round(n / (ms / 1e3) / 1e6, 1)
        total_rays += n
        total_ms += ms
        hits = d_h.cpu().numpy().view(W.HIT_DTYPE)
        c = compare(np.ascontiguousarray(hits[::stride]), rh, oracle_scene, np.ascontiguousarray(rays[::stride]))
        parity[name] = {kk: c[kk] for kk in ("n", "agree", "ties", "bad_disagreements", "bitexact_t")}
        del d_r, d_h
    return {"Mrays": round(total_rays / (total_ms / 1e3) / 1e6, 1), "ms_per_step": round(total_ms, 4),
            "per_set_ms": per_ms, "per_set_Mrays": per_mrays, "parity_vs_oracle": parity,
            "compiled": k.info, "block": 32,
            "layout": "the oracle's BVHArrayNode[] (classic builder, 4-ary), one vertex page, one node page; "
                      "every set traced closest-hit (no any-hit mode in the reference kernel)",
            "sample": f"parity on every {stride}th ray of each set, against the oracle's BVHAccel (fast math "
                      "moves t, b1, b2 in the last bits and flips a few near-ties)"}


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    threads = os.cpu_count() or 1
    from oracle import pyoracle as po
    scene = make_scene()
    primary = W.pinhole_rays(1024, 1024)
    o = po.OracleScene(scene, po.ACCEL_BVH)
    ph, _ = o.intersect(primary, n_threads=threads)
    bounce, shadow = derived_rays(scene, primary, ph, W.BASE_SEED + 100)
    frac = args.ref_fraction
    sample = [primary[::frac], bounce[::frac], shadow[::frac]]
    n_sample = sum(s.shape[0] for s in sample)
    for _ in range(args.warmup):
        for s in sample:
            o.intersect(s, n_threads=threads)
    secs = []
    for _ in range(args.steps):
        t = 0.0
        for s in sample:
            _, dt = o.intersect(s, n_threads=threads)
            t += dt
        secs.append(t)
    total = sum(secs)
    value = n_sample * args.steps / total / 1e6
    desc = f"every {frac}th ray of each set ({n_sample} rays per step), classic-builder BVH, {threads} threads"
    line = {
        "impl": "reference", "metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(1e3 * total / args.steps, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded)",
        "config": {"workload": WORKLOAD, "sample": desc},
        "cpu_baseline": {"value": round(value, 3), "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": desc},
        "e2e": {"value": round(value, 3), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------

def run_lrx(args):
    import torch

    from luxcore_gb300 import lrx

    d = Dist(use_gpu=True)
    ws, rank, local = d.ws, d.rank, d.local
    torch.cuda.set_device(local)
    stream = torch.cuda.Stream()
    st = stream.cuda_stream

    scene_desc = make_scene()
    t0 = time.perf_counter()
    build_kw = {} if args.treelet_passes is None else {"treelet_passes": args.treelet_passes}
    with torch.cuda.stream(stream):
        scene = lrx.Scene(scene_desc, stream=st, **build_kw)
    build_s = time.perf_counter() - t0
    if args.block_size is not None or args.postpone is not None or args.variant is not None:
        scene.set_trace_config(args.block_size or 64, 0 if args.postpone is None else args.postpone,
                               args.variant or 0, refill=args.refill or 0)
    saved_cfg = {m: scene.trace_config(m) for m in (lrx.LRX_TRACE_CLOSEST, lrx.LRX_TRACE_ANY)}
    info = scene.info()

    primary = W.pinhole_rays(1024, 1024)

    def up(a):
        return torch.from_numpy(np.ascontiguousarray(a).view(np.uint8).reshape(-1).copy()).cuda(local)

    log(f"[bench] {time.strftime('%H:%M:%S')} scene built {info}")
    d_prim = up(primary)
    d_ph = torch.empty(primary.shape[0] * HIT_BYTES, dtype=torch.uint8, device=f"cuda:{local}")
    torch.cuda.synchronize()
    scene.trace(d_prim.data_ptr(), d_ph.data_ptr(), primary.shape[0], lrx.LRX_TRACE_CLOSEST, st)
    stream.synchronize()
    log(f"[bench] {time.strftime('%H:%M:%S')} primary hits traced")
    ph = d_ph.cpu().numpy().view(W.HIT_DTYPE)
    bounce, shadow = derived_rays(scene_desc, primary, ph, W.BASE_SEED + 100)
    sets = [("primary", primary, lrx.LRX_TRACE_CLOSEST), ("bounce", bounce, lrx.LRX_TRACE_CLOSEST),
            ("shadow", shadow, lrx.LRX_TRACE_ANY)]
    dev = []
    for name, r, mode in sets:
        dr = up(r)
        dh = torch.empty(r.shape[0] * HIT_BYTES, dtype=torch.uint8, device=f"cuda:{local}")
        dev.append((name, dr, dh, r.shape[0], mode))
    rays_per_step = sum(x[3] for x in dev)

    # traversal counters (untimed): nodes / triangles fetched per ray
    counts = {}
    cbuf = torch.zeros(4, dtype=torch.int64, device=f"cuda:{local}")
    log(f"[bench] {time.strftime('%H:%M:%S')} rays ready, counting pass")
    for name, dr, dh, n, mode in dev:
        cbuf.zero_()
        torch.cuda.synchronize()  # the zeroing ran on torch's stream, the trace runs on `st`
        scene.trace_counted(dr.data_ptr(), dh.data_ptr(), n, mode, cbuf.data_ptr(), st)
        stream.synchronize()
        nodes, tris, insts, rays = cbuf.cpu().tolist()
        counts[name] = (nodes / n, tris / n, insts / n)
    if scene.device_status(st) != 0:
        raise RuntimeError("device status word set during the counting pass")
    log(f"[bench] {time.strftime('%H:%M:%S')} counting done {counts}")
    alg_bytes = {}
    for name, dr, dh, n, mode in dev:
        nn, nt, ni = counts[name]
        alg_bytes[name] = n * (RAY_BYTES + HIT_BYTES + nn * NODE_BYTES + nt * TRI_BYTES + ni * INST_BYTES)

    def seq_step(evs=None):
        # one lrx_trace per set, back to back on one stream
        for k, (name, dr, dh, n, mode) in enumerate(dev):
            if evs is not None:
                evs[k][0].record(stream)
            scene.trace(dr.data_ptr(), dh.data_ptr(), n, mode, st)
            if evs is not None:
                evs[k][1].record(stream)

    batch_arr = lrx.batch_array([(scene, dr.data_ptr(), dh.data_ptr(), n, mode) for _nm, dr, dh, n, mode in dev])

    def batched_step(evs=None):
        # the three sets as one lrx_trace_batches call: each (>= 131,072 rays)
        # is a launch of its own on a side stream, all three side by side
        lrx.trace_batches([None] * len(dev), st, arr=batch_arr)

    step = batched_step if args.step_form == "batched" else seq_step
    for _ in range(args.warmup):
        step()
        seq_step()
    stream.synchronize()
    if scene.device_status(st) != 0:
        raise RuntimeError("device status word set during warm-up")
    launches_per_step = count_kernel_launches(st, step)
    log(f"[bench] {time.strftime('%H:%M:%S')} warm-up done, timing {args.steps} steps")

    ev = [[(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in dev]
          for _ in range(args.steps)]
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    clocks = ClockSampler(local)
    d.barrier()
    torch.cuda.synchronize()
    clocks.start()
    start.record(stream)
    for k in range(args.steps):
        step(ev[k])
    end.record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    log(f"[bench] {time.strftime('%H:%M:%S')} timed region done")
    if scene.device_status(st) != 0:
        raise RuntimeError("device status word set during the timed steps")
    # the last timed step's hits, for the parity check on the CPU sample
    step_hits = [dh.cpu().numpy().view(W.HIT_DTYPE).copy() for _nm, _dr, dh, _n, _m in dev] if rank == 0 else None
    d.barrier()
    elapsed_ms = start.elapsed_time(end)
    elapsed_ms = d.max(elapsed_ms)
    if args.step_form == "batched":
        # per-launch times: the same sets as sequential launches, each between
        # events on its stream (outside the timed region)
        seq_t0, seq_t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        seq_t0.record(stream)
        for k in range(args.steps):
            seq_step(ev[k])
        seq_t1.record(stream)
        torch.cuda.synchronize()
        seq_step_ms = seq_t0.elapsed_time(seq_t1) / args.steps
    else:
        seq_step_ms = elapsed_ms / args.steps
    kern_ms = {name: statistics.mean(ev[k][j][0].elapsed_time(ev[k][j][1]) for k in range(args.steps))
               for j, (name, *_rest) in enumerate(dev)}
    value = rays_per_step * args.steps * ws / (elapsed_ms / 1e3) / 1e6

    # the same sets under other launch configurations (block size, postpone),
    # for comparison; outside the timed region
    alt = {}
    if args.sweep:
        for bs, pp, var, rf in [(64, 8, 64, 8), (64, 8, 72, 8), (128, 8, 72, 8), (64, 0, 72, 8), (64, 8, 65, 8),
                                (64, 8, 16, 0), (64, 8, 80, 8), (64, 8, 0xC0, 8), (64, 8, 0x440, 8),
                                (64, 8, 0x840, 8), (64, 8, 0x410, 0), (64, 8, 0x810, 0)]:
            scene.set_trace_config(bs, pp, var, refill=rf)
            key = f"b{bs}-p{pp}-v{var}-r{rf}"
            alt[key] = {}
            for name, dr, dh, n, mode in dev:
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                scene.trace(dr.data_ptr(), dh.data_ptr(), n, mode, st)
                e0.record(stream)
                for _ in range(5):
                    scene.trace(dr.data_ptr(), dh.data_ptr(), n, mode, st)
                e1.record(stream)
                e1.synchronize()
                alt[key][name] = round(n * 5 / (e0.elapsed_time(e1) / 1e3) / 1e6, 1)
        for m, c in saved_cfg.items():
            scene.set_trace_config(c["block_size"], c["postpone"], c["variant"], modes=2 if m == lrx.LRX_TRACE_ANY else 1,
                                   refill=c["refill"])
    builds = {}
    if args.build_sweep:
        # the same sets on trees built with 0-3 treelet passes, leaf size 2, and
        # 4- and 6-wide nodes, the 4-wide ones also in 64-byte node records
        # (default launch configs)
        C4 = lrx.LRX_NODES_COMPACT4
        for passes, leaf, width, layout in ((0, 3, 8, 0), (1, 3, 8, 0), (2, 3, 8, 0), (3, 3, 8, 0), (2, 2, 8, 0),
                                            (2, 3, 4, 0), (2, 3, 4, C4), (2, 2, 4, C4), (2, 3, 6, 0)):
            with torch.cuda.stream(stream):
                sc = lrx.Scene(scene_desc, stream=st, treelet_passes=passes, leaf_max=leaf, node_width=width,
                               node_layout=layout)
            inf = sc.info()
            row = {"build_ms": round(inf["build_ms"], 2), "wide_nodes": inf["node_count"], "depth": inf["max_depth"],
                   "node_bytes": inf["node_bytes"]}
            for name, dr, dh, n, mode in dev:
                cb = torch.zeros(4, dtype=torch.int64, device=f"cuda:{local}")
                torch.cuda.synchronize()
                sc.trace_counted(dr.data_ptr(), dh.data_ptr(), n, mode, cb.data_ptr(), st)
                stream.synchronize()
                nn, nt, _ni, _nr = cb.cpu().tolist()
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                sc.trace(dr.data_ptr(), dh.data_ptr(), n, mode, st)
                e0.record(stream)
                for _ in range(5):
                    sc.trace(dr.data_ptr(), dh.data_ptr(), n, mode, st)
                e1.record(stream)
                e1.synchronize()
                row[name] = {"Mrays": round(n * 5 / (e0.elapsed_time(e1) / 1e3) / 1e6, 1),
                             "nodes_per_ray": round(nn / n, 2), "tris_per_ray": round(nt / n, 2)}
            sc.close()
            builds[f"treelet{passes}-leaf{leaf}-width{width}" + ("-nodes64" if layout else "")] = row
        # the build lrx_scene_create_autotuned keeps for each set (its
        # candidates: width 8 / 4 in 80-byte records, width 4 in 64-byte
        # records, leaf 3 / 2; each at its tuned launch config), on the
        # set's first 262,144 rays
        for name, dr, dh, n, mode in dev:
            with torch.cuda.stream(stream):
                sc, opts, cfg = lrx.Scene.autotuned(scene_desc, dr.data_ptr(), min(n, 1 << 18), mode, st)
            builds[f"autotuned-{name}"] = {**opts, **cfg}
            sc.close()
        log(f"[bench] {time.strftime('%H:%M:%S')} build sweep done")

    if args.sweep:
        # compaction: the bounce set with half of its rays masked (finished paths)
        name, dr, dh, n, mode = dev[1]
        half = dr.clone()
        words = half.view(torch.int32).view(-1, 12)
        g = torch.Generator(device=f"cuda:{local}")
        g.manual_seed(5)
        words[:, 9] = torch.where(torch.rand(n, generator=g, device=f"cuda:{local}") < 0.5,
                                  torch.ones_like(words[:, 9]), words[:, 9])
        alt["bounce-half-masked"] = {}
        for key, var in (("persistent", 64), ("persistent+compact", 64 | 256)):
            scene.set_trace_config(64, 8, var, modes=1, refill=8)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            scene.trace(half.data_ptr(), dh.data_ptr(), n, mode, st)
            e0.record(stream)
            for _ in range(5):
                scene.trace(half.data_ptr(), dh.data_ptr(), n, mode, st)
            e1.record(stream)
            e1.synchronize()
            alt["bounce-half-masked"][key + "_ms"] = round(e0.elapsed_time(e1) / 5, 4)
        c = saved_cfg[lrx.LRX_TRACE_CLOSEST]
        scene.set_trace_config(c["block_size"], c["postpone"], c["variant"], modes=1, refill=c["refill"])
        del half

        # each set as a one-batch lrx_trace_batches call (the queue kernel)
        alt["queue-1batch"] = {}
        for name, dr, dh, n, mode in dev:
            one = [(scene, dr.data_ptr(), dh.data_ptr(), n, mode)]
            arr1 = lrx.batch_array(one)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            lrx.trace_batches(one, st, arr=arr1)
            e0.record(stream)
            for _ in range(5):
                lrx.trace_batches(one, st, arr=arr1)
            e1.record(stream)
            e1.synchronize()
            alt["queue-1batch"][name] = round(n * 5 / (e0.elapsed_time(e1) / 1e3) / 1e6, 1)

    # roofline of the traversal kernels: algorithmic bytes / time -- over the
    # timed step (the batched step's three launches run side by side), and
    # per launch from the sequential per-set times
    peak, peak_kind = load_peaks()
    tot_alg = sum(alg_bytes.values())
    achieved = tot_alg / (elapsed_ms / args.steps / 1e3) / 1e9
    per_launch_frac = {name: round(alg_bytes[name] / (kern_ms[name] / 1e3) / 1e9 / peak, 4) for name, *_r in dev}
    # the bounce kernel on a launch large enough to amortise its drain: 8 M
    # distinct cosine-hemisphere rays from the same primary hit points (the
    # step's own bounce set is 1 M rays per launch); outside the timed region
    big_bounce = None
    if not args.no_big_bounce:
        nb = 8 << 20
        b8 = W.bounce_rays(scene_desc, primary, ph, nb, W.BASE_SEED + 200)
        d_b8 = up(b8)
        d_h8 = torch.empty(nb * HIT_BYTES, dtype=torch.uint8, device=f"cuda:{local}")
        cbuf.zero_()
        torch.cuda.synchronize()
        scene.trace_counted(d_b8.data_ptr(), d_h8.data_ptr(), nb, lrx.LRX_TRACE_CLOSEST, cbuf.data_ptr(), st)
        stream.synchronize()
        bn, bt, _bi, _br = cbuf.cpu().tolist()
        for _ in range(2):
            scene.trace(d_b8.data_ptr(), d_h8.data_ptr(), nb, lrx.LRX_TRACE_CLOSEST, st)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(5):
            scene.trace(d_b8.data_ptr(), d_h8.data_ptr(), nb, lrx.LRX_TRACE_CLOSEST, st)
        e1.record(stream)
        e1.synchronize()
        ms8 = e0.elapsed_time(e1) / 5
        bpr = RAY_BYTES + HIT_BYTES + bn / nb * NODE_BYTES + bt / nb * TRI_BYTES
        big_bounce = {"rays": nb, "Mrays": round(nb / (ms8 / 1e3) / 1e6, 1), "ms_per_launch": round(ms8, 4),
                      "nodes_tris_per_ray": [round(bn / nb, 2), round(bt / nb, 2)],
                      "frac": round(nb * bpr / (ms8 / 1e3) / 1e9 / peak, 4)}
        del d_b8, d_h8
    # DRAM bytes per trace launch, averaged over the sets
    traffic = round(sum(TRAFFIC_PER_RAY[name] * n for name, _dr, _dh, n, _m in dev) / len(dev))

    # end to end: host rays in pinned memory -> lrx_trace_host -> host hits
    e2e_value = None
    pinned = []
    for name, r, mode in (sets if not args.no_e2e else []):
        hr = torch.from_numpy(np.ascontiguousarray(r).view(np.uint8).reshape(-1).copy()).pin_memory()
        hh = torch.empty(r.shape[0] * HIT_BYTES, dtype=torch.uint8).pin_memory()
        pinned.append((hr, hh, r.shape[0], mode))

    def e2e_seq_step():
        for hr, hh, n, mode in pinned:
            scene.trace_host_ptr(hr.data_ptr(), hh.data_ptr(), n, mode, st)

    host_arr = lrx.host_batch_array([(scene, hr.data_ptr(), hh.data_ptr(), n, mode) for hr, hh, n, mode in pinned])

    def e2e_batched_step():
        # one lrx_trace_host_batches call: each set's copies overlap the others' traces
        lrx.trace_host_batches([None] * len(pinned), st, arr=host_arr)

    e2e_step = e2e_batched_step if args.step_form == "batched" else e2e_seq_step
    e2e_seq_value = None
    if not args.no_e2e:
        for _ in range(max(1, args.warmup)):
            e2e_step()
            e2e_seq_step()
        # the steps in five timed windows, the median window's rate: host
        # time moves with bursts of other work on the host, and one window
        # caught by one would misstate the rest
        d.barrier()
        n_win = 5 if args.steps >= 5 else 1
        per_win = [args.steps // n_win + (1 if k < args.steps % n_win else 0) for k in range(n_win)]
        e2e_windows = []
        for nw in per_win:
            t1 = time.perf_counter()
            for _ in range(nw):
                e2e_step()
            e2e_s = d.max(time.perf_counter() - t1)
            e2e_windows.append(rays_per_step * nw * ws / e2e_s / 1e6)
        e2e_value = round(float(np.median(e2e_windows)), 3)
        # the sequential form likewise: the median of three windows
        seq_windows = []
        n_seq = max(1, args.steps // 30)
        for _ in range(3):
            t1 = time.perf_counter()
            for _ in range(n_seq):
                e2e_seq_step()
            seq_windows.append(rays_per_step * n_seq / (time.perf_counter() - t1) / 1e6)
        e2e_seq_value = round(float(np.median(seq_windows)), 3)
    # lrx_trace_host copies rays and hits in (masked rays keep the caller's
    # hits); lrx_trace_host_batches copies only the rays of pinned buffers
    # (the hit buffer's masked slots -- none here -- are read back directly)
    h2d = rays_per_step * (RAY_BYTES + (0 if args.step_form == "batched" else HIT_BYTES))
    d2h = rays_per_step * HIT_BYTES

    line = None
    if rank == 0:
        cpu = None
        parity = None
        ref_gpu = None
        if not args.no_cpu_baseline:
            threads = os.cpu_count() or 1
            frac = args.ref_fraction
            sample = [primary[::frac], bounce[::frac], shadow[::frac]]
            n_s, secs, oracle_scene, ref_hits = cpu_measure(scene_desc, sample, threads, keep_hits=True)
            cpu = {"value": round(n_s / secs / 1e6, 3), "unit": UNIT, "cores": threads, "kind": "port",
                   "sample": f"every {frac}th ray of each of the 3 sets ({n_s} rays), oracle BVHAccel::Intersect "
                             f"restatement, classic-builder BVH, {threads} threads"}
            parity = parity_block(oracle_scene, sets, step_hits, ref_hits, frac)
            if not args.no_ref_gpu:
                ref_gpu = reference_gpu_arm(torch, oracle_scene, scene_desc, sets, ref_hits, frac, stream,
                                            f"cuda:{local}")
            # the reference layout's bytes per ray on the same rays, beside this
            # build's (roofline.bytes_per_ray): a worse tree cannot raise the
            # roofline fraction unnoticed
            bref = reference_layout_bytes(oracle_scene, [(nm, r) for nm, r, _m in sets])
            step_bref = sum(bref[nm]["bytes_per_ray"] * r.shape[0] for nm, r, _m in sets) / rays_per_step
            cpu["b_ref"] = {"per_set": bref, "step_bytes_per_ray": round(step_bref, 1),
                            "sample": "every 16th ray of each set, oracle BVHAccel walk (classic builder, 4-ary)",
                            "formula": "48 + 20 + 32 x node visits + (3 x 12 + 12) x leaf visits"}
        line = {
            "metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(elapsed_ms / args.steps, 4), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
            "config": {
                "workload": WORKLOAD, "rays_per_step": rays_per_step, "triangles": info["triangle_count"],
                "l2": "inputs larger than L2 (rays 302 MB + hits 126 MB + scene per step)",
                "parallelism": f"replicas x{ws}", "build_ms": round(info["build_ms"], 1),
                "scene_build_wall_s": round(build_s, 3), "wide_nodes": info["node_count"],
                "bvh_depth": info["max_depth"],
                "step_form": ("one lrx_trace_batches call (3 launches on side streams)" if args.step_form == "batched"
                              else "3 sequential lrx_trace launches"),
                "sequential_step_Mrays": round(rays_per_step / (seq_step_ms / 1e3) / 1e6, 1),
                "per_set_ms": {k: round(v, 4) for k, v in kern_ms.items()},
                "per_set_Mrays": {name: round(n / (kern_ms[name] / 1e3) / 1e6, 1) for name, _, _, n, _ in dev},
                "nodes_tris_per_ray": {k: [round(v[0], 2), round(v[1], 2)] for k, v in counts.items()},
                "trace_config": {"closest": scene.trace_config(lrx.LRX_TRACE_CLOSEST),
                                 "any": scene.trace_config(lrx.LRX_TRACE_ANY)},
                "config_sweep_Mrays": alt,
                "build_sweep": builds,
                "treelet_passes": args.treelet_passes,
            },
            "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                         "frac": round(achieved / peak, 4), "traffic": traffic, "traffic_source": TRAFFIC_SOURCE,
                         "peak_kind": peak_kind, "scope": "the timed step (algorithmic bytes / step time)",
                         "per_launch_frac": per_launch_frac,
                         "bounce_8M_launch": big_bounce,
                         "bytes_per_ray": round(tot_alg / rays_per_step, 1)},
            "cpu_baseline": cpu,
            "parity": parity,
            "reference_gpu": ref_gpu,
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h,
                    "api": ("lrx_trace_host_batches over the 3 sets (pinned host buffers)" if args.step_form == "batched"
                            else "lrx_trace_host per set (pinned host buffers)"),
                    "sequential_lrx_trace_host_value": e2e_seq_value,
                    "estimator": "median of the Mrays/s of 5 timed windows of steps/5 steps each",
                    "windows_Mrays": [round(v, 1) for v in e2e_windows] if not args.no_e2e else None},
            "gpu_launches": (launches_per_step if launches_per_step is not None else len(dev)) * args.steps,
            "gpu_launches_per_step": launches_per_step,
            "clocks": clk,
        }
        if ws == 1 and not args.no_extras:
            # the metric's second half, bounded: uneven batches (batched over
            # plain with the same autotuned configs) and the serving loop
            # (p50 / p99, batched over plain); outside the timed region
            dev.clear()
            for key, fn in (("batching", lambda: batching_line(args, 3)),
                            ("serving", lambda: serving_line(args, [2000.0, 800.0], 2.0, budget_runs=False))):
                t_x = time.perf_counter()
                try:
                    x = fn()
                    cfg = {k: v for k, v in x["config"].items() if k != "autotuned"}
                    line[key] = {"metric": x["metric"], "value": x["value"], "unit": x["unit"], **cfg,
                                 "wall_s": round(time.perf_counter() - t_x, 1)}
                except Exception as e:  # reported in the line; the headline stands
                    line[key] = {"error": repr(e)[:500]}
                log(f"[bench] {time.strftime('%H:%M:%S')} {key} done in {time.perf_counter() - t_x:.1f}s")
        print(json.dumps(line), flush=True)
    scene.close()
    d.close()
    return 0


# ---------------------------------------------------------------------------
# Instanced two-level scene: 16 x 200,000-triangle icospheres, 4,096 instances
# ---------------------------------------------------------------------------

def run_instanced(args, motion: bool = False):
    """16 displaced icospheres of 200,000 triangles under 4,096 random affine
    instances (819,200,000 effective triangles) in [0,10]^3; per step
    8,388,608 closest-hit and 8,388,608 any-hit rays (maxt U[0.5, 5]).
    motion: the same meshes under W.motion_scene's instances -- a third each
    translating (two keyframes), turning/scaling/moving (three keyframes)
    and static -- with ray times uniform over the shutter [0, 1]."""
    import torch

    from luxcore_gb300 import lrx

    torch.cuda.set_device(0)
    t0 = time.perf_counter()
    if motion:
        scene_desc, closest, anyr = W.config_motion(n_rays=args.inst_rays)
    else:
        scene_desc, closest, anyr = W.config3(n_rays=args.inst_rays)
    tag = "motion" if motion else "instanced"
    log(f"[{tag}] {time.strftime('%H:%M:%S')} scene and rays generated in {time.perf_counter() - t0:.1f}s")
    stream = torch.cuda.Stream()
    st = stream.cuda_stream
    t0 = time.perf_counter()
    with torch.cuda.stream(stream):
        scene = lrx.Scene(scene_desc, stream=st)
    build_s = time.perf_counter() - t0
    info = scene.info()
    log(f"[{tag}] scene built {info}")
    dev = []
    for name, r, mode in (("closest", closest, lrx.LRX_TRACE_CLOSEST), ("any", anyr, lrx.LRX_TRACE_ANY)):
        dr = torch.from_numpy(np.ascontiguousarray(r).view(np.uint8).reshape(-1).copy()).cuda()
        dh = torch.empty(r.shape[0] * HIT_BYTES, dtype=torch.uint8, device="cuda")
        dev.append((name, dr, dh, r.shape[0], mode))
    rays_per_step = sum(x[3] for x in dev)
    counts, alg = {}, {}
    cbuf = torch.zeros(4, dtype=torch.int64, device="cuda")
    for name, dr, dh, n, mode in dev:
        cbuf.zero_()
        torch.cuda.synchronize()
        scene.trace_counted(dr.data_ptr(), dh.data_ptr(), n, mode, cbuf.data_ptr(), st)
        stream.synchronize()
        nn, nt, ni, _ = cbuf.cpu().tolist()
        counts[name] = (nn / n, nt / n, ni / n)
        alg[name] = n * (RAY_BYTES + HIT_BYTES + nn / n * NODE_BYTES + nt / n * TRI_BYTES + ni / n * INST_BYTES)
    # size-independent check at full size: any-hit hit/miss equals closest-hit hit/miss
    name, dr, dh, n, _ = dev[1]
    dh_c = torch.empty_like(dh)
    scene.trace(dr.data_ptr(), dh_c.data_ptr(), n, lrx.LRX_TRACE_CLOSEST, st)
    scene.trace(dr.data_ptr(), dh.data_ptr(), n, lrx.LRX_TRACE_ANY, st)
    stream.synchronize()
    mi_any = dh.view(torch.int32).view(-1, 5)[:, 3].cpu().numpy().view(np.uint32)
    mi_cl = dh_c.view(torch.int32).view(-1, 5)[:, 3].cpu().numpy().view(np.uint32)
    hit_any, hit_cl = mi_any != W.NULL_INDEX, mi_cl != W.NULL_INDEX
    anyhit_consistent = bool(np.array_equal(hit_any, hit_cl))
    del dh_c

    def step(evs=None):
        for k, (name, dr, dh, n, mode) in enumerate(dev):
            if evs is not None:
                evs[k][0].record(stream)
            scene.trace(dr.data_ptr(), dh.data_ptr(), n, mode, st)
            if evs is not None:
                evs[k][1].record(stream)

    for _ in range(args.warmup):
        step()
    stream.synchronize()
    if scene.device_status(st) != 0:
        raise RuntimeError("device status word set during warm-up")
    launches_per_step = count_kernel_launches(st, step)
    ev = [[(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in dev]
          for _ in range(args.steps)]
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    clocks = ClockSampler(0)
    torch.cuda.synchronize()
    clocks.start()
    start.record(stream)
    for k in range(args.steps):
        step(ev[k])
    end.record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    if scene.device_status(st) != 0:
        raise RuntimeError("device status word set during the timed steps")
    elapsed_ms = start.elapsed_time(end)
    kern_ms = {name: statistics.mean(ev[k][j][0].elapsed_time(ev[k][j][1]) for k in range(args.steps))
               for j, (name, *_rest) in enumerate(dev)}
    value = rays_per_step * args.steps / (elapsed_ms / 1e3) / 1e6
    peak, peak_kind = load_peaks()
    achieved = sum(alg.values()) / (sum(kern_ms.values()) / 1e3) / 1e9
    cpu = None
    if not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        frac = args.ref_fraction * 64
        sample = [closest[::frac], anyr[::frac]]
        n_s, secs, _o = cpu_measure(scene_desc, sample, threads, accel="mbvh")
        cpu = {"value": round(n_s / secs / 1e6, 3), "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"every {frac}th ray of both sets ({n_s} rays), oracle MBVHAccel::Intersect restatement "
                         f"(closest hit for both), {threads} threads"}
    line = {
        "metric": ("Mrays/s closest/any-hit on motion-blurred instances (1 GB300, % HBM roofline)" if motion else
                   "Mrays/s closest/any-hit on the instanced two-level scene (1 GB300, % HBM roofline)"),
        "value": round(value, 3), "unit": UNIT, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(elapsed_ms / args.steps, 4), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
        "config": {
            "workload": f"{tag}: {info['blas_count']} meshes x 200000 tris, {info['instance_count']} instances "
                        f"({info['triangle_count']} effective tris"
                        + ("; 1/3 translating, 1/3 turning+scaling+moving, 1/3 static, ray time U[0,1)" if motion else "")
                        + f"); {dev[0][3]} closest + {dev[1][3]} any-hit rays",
            "rays_per_step": rays_per_step, "build_ms": round(info["build_ms"], 1),
            "scene_build_wall_s": round(build_s, 3), "wide_nodes": info["node_count"],
            "device_MB": round(info["device_bytes"] / 1e6, 1),
            "per_set_ms": {k: round(v, 4) for k, v in kern_ms.items()},
            "per_set_Mrays": {name: round(n / (kern_ms[name] / 1e3) / 1e6, 1) for name, _, _, n, _ in dev},
            "nodes_tris_insts_per_ray": {k: [round(x, 2) for x in v] for k, v in counts.items()},
            "hit_rate": {"closest": round(float((dh_hits(dev[0]) != W.NULL_INDEX).mean()), 4),
                         "any": round(float(hit_any.mean()), 4)},
            "anyhit_hitmiss_equals_closest": anyhit_consistent,
            "l2": "inputs larger than L2 (rays 805 MB + hits 336 MB per step)",
        },
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "traffic": None, "peak_kind": peak_kind,
                     "bytes_per_ray": round(sum(alg.values()) / rays_per_step, 1),
                     **({"note": "motion intervals read at instance entry are not counted"} if motion else {})},
        "cpu_baseline": cpu,
        "gpu_launches": (launches_per_step if launches_per_step is not None else len(dev)) * args.steps,
        "gpu_launches_per_step": launches_per_step,
        "clocks": clk,
    }
    print(json.dumps(line), flush=True)
    scene.close()
    return 0


def run_pathocl(args):
    """PATHOCL-style wavefront loop on the heightfield (luxcore_gb300/pathocl.py):
    1,048,576 tasks (one per pixel of a 1024 x 1024 image), one ray buffer of
    path and shadow rays traced in place per iteration, masked tasks
    included, advanced on the device between traces; depth limit 4.  A step
    is 8 iterations.  Reported: unmasked rays traced per second over the
    whole loop (trace + AdvancePaths stand-in) and over the trace launches
    alone, for the default closest-hit config and with ray compaction."""
    import torch

    from luxcore_gb300 import lrx
    from luxcore_gb300 import pathocl

    torch.cuda.set_device(0)
    stream = torch.cuda.Stream()
    st = stream.cuda_stream
    desc = make_scene()
    with torch.cuda.stream(stream):
        scene = lrx.Scene(desc, stream=st)
    iters = 8
    forms = {}
    default = scene.trace_config(lrx.LRX_TRACE_CLOSEST)  # the library's closest-hit default
    for form, (pp, variant) in (("default", (default["postpone"], default["variant"])),
                                ("default+compact", (default["postpone"], default["variant"] | lrx.LRX_VARIANT_COMPACT)),
                                ("persistent, no drain split", (8, lrx.LRX_VARIANT_PERSISTENT))):
        scene.set_trace_config(default["block_size"], pp, variant, modes=1, refill=default["refill"] or 8)
        with torch.cuda.stream(stream):
            wf = pathocl.WavefrontPaths(scene, desc, 1024, 1024, max_depth=4, stream=stream)
            wf.iterate(args.warmup * iters)
            torch.cuda.synchronize()
            t0 = int(wf.traced_dev)
            ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
                  for _ in range(args.steps * iters)]
            start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            clocks = ClockSampler(0)
            clocks.start()
            start.record(stream)
            for k in range(args.steps * iters):
                ev[k][0].record(stream)
                wf.trace()
                ev[k][1].record(stream)
                wf.advance()
            end.record(stream)
            torch.cuda.synchronize()
            clk = clocks.stop()
        if scene.device_status(st) != 0:
            raise RuntimeError("device status word set during the wavefront loop")
        rays = int(wf.traced_dev) - t0
        loop_ms = start.elapsed_time(end)
        trace_ms = sum(a.elapsed_time(b) for a, b in ev)
        forms[form] = {"loop_Mrays": round(rays / (loop_ms / 1e3) / 1e6, 1),
                       "trace_Mrays": round(rays / (trace_ms / 1e3) / 1e6, 1),
                       "unmasked_rays_per_iteration": round(rays / (args.steps * iters)),
                       "ms_per_iteration": round(loop_ms / (args.steps * iters), 4),
                       "trace_ms_per_iteration": round(trace_ms / (args.steps * iters), 4), "clocks": clk}
        del wf
    best = forms["default"]
    line = {
        "metric": "Mrays/s traced in a PATHOCL-style wavefront loop (trace + AdvancePaths stand-in on the device)",
        "value": best["loop_Mrays"], "unit": UNIT, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(best["ms_per_iteration"] * iters, 4), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
        "config": {"workload": "heightfield-2093058tri, 1048576 tasks (1024x1024), depth 4, one in-place buffer of "
                               "path + shadow rays per iteration, 8 iterations per step",
                   "forms": forms},
        "clocks": best["clocks"],
    }
    print(json.dumps(line), flush=True)
    scene.close()
    return 0


def dh_hits(entry):
    """meshIndex column of a device hit buffer (host copy)."""
    import torch
    _name, _dr, dh, _n, _mode = entry
    return dh.view(torch.int32).view(-1, 5)[:, 3].cpu().numpy().view(np.uint32)


# ---------------------------------------------------------------------------
# Uneven batches over several resident scenes: plain vs queue kernel
# ---------------------------------------------------------------------------

def device_random_rays(torch, n, extent, seed, device):
    """Rays on the device: origins ~ U[0,extent]^3, directions uniform on the
    sphere, mint 1e-4, maxt 1e30 (48-byte luxrays::Ray records)."""
    g = torch.Generator(device=device)
    g.manual_seed(seed)
    rec = torch.zeros((n, 12), dtype=torch.float32, device=device)
    rec[:, 0:3] = torch.rand((n, 3), generator=g, device=device) * extent
    d = torch.randn((n, 3), generator=g, device=device)
    rec[:, 3:6] = d / d.norm(dim=1, keepdim=True).clamp_min(1e-20)
    rec[:, 6] = 1e-4
    rec[:, 7] = 1e30
    return rec


def run_batching(args):
    print(json.dumps(batching_line(args, args.steps)), flush=True)
    return 0


def batching_line(args, steps: int) -> dict:
    """The uneven-batch workload (512 batches of log-uniform size over 8
    random-triangle scenes): one lrx_trace per RayBuffer against one
    lrx_trace_batches call, eager and as replayed CUDA
    graphs, each timed over `steps` repetitions with the same autotuned
    per-scene configs (plus the plain form under the library defaults)."""
    import torch

    from luxcore_gb300 import lrx

    dev = "cuda:0"
    torch.cuda.set_device(0)
    tri_counts, extents, batches = W.uneven_batches(n_batches=args.batches)
    log(f"[batching] scenes {tri_counts.tolist()}")
    scenes = []
    for k, (n, ext) in enumerate(zip(tri_counts.tolist(), extents.tolist())):
        scenes.append(lrx.Scene(W.SceneDesc([W.random_triangles(int(n), W.BASE_SEED + 40 + k, extent=ext)])))
    stream = torch.cuda.Stream()
    st = stream.cuda_stream
    items = []
    for k, (si, n, anyhit) in enumerate(batches):
        rec = device_random_rays(torch, int(n), float(extents[si]), W.BASE_SEED + 1000 + k, dev)
        hits = torch.empty(int(n) * HIT_BYTES, dtype=torch.uint8, device=dev)
        items.append((scenes[si], rec, hits, int(n), lrx.LRX_TRACE_ANY if anyhit else lrx.LRX_TRACE_CLOSEST))
    total_rays = sum(x[3] for x in items)
    torch.cuda.synchronize()
    log(f"[batching] {len(items)} batches, {total_rays} rays resident")

    def plain():
        for s, rec, hits, n, mode in items:
            s.trace(rec.data_ptr(), hits.data_ptr(), n, mode, st)

    # the plain form under the library's default launch configuration,
    # before any autotuning
    def timed_plain_default():
        with torch.cuda.stream(stream):
            plain()
            stream.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(steps):
                plain()
            e1.record(stream)
        e1.synchronize()
        return e0.elapsed_time(e1) / steps

    default_ms = timed_plain_default()

    # per-scene autotune on a 262,144-ray sample of each mode
    tuned = {}
    if not args.no_autotune:
        for k, s in enumerate(scenes):
            sample = device_random_rays(torch, 1 << 18, float(extents[k]), W.BASE_SEED + 7 + k, dev)
            tuned[k] = {m: s.autotune(sample.data_ptr(), 1 << 18, m, st)
                        for m in (lrx.LRX_TRACE_CLOSEST, lrx.LRX_TRACE_ANY)}
        torch.cuda.synchronize()

    arr = lrx.batch_array([(s, rec.data_ptr(), hits.data_ptr(), n, mode) for s, rec, hits, n, mode in items])

    def batched():
        lrx.trace_batches(items, st, arr=arr)

    def timed(fn, reps):
        with torch.cuda.stream(stream):
            fn()
        stream.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0 = time.perf_counter()
        with torch.cuda.stream(stream):  # graph replays launch on the current stream
            e0.record(stream)
            for _ in range(reps):
                fn()
            e1.record(stream)
        e1.synchronize()
        return e0.elapsed_time(e1) / reps, (time.perf_counter() - t0) * 1e3 / reps

    def graphed(fn):
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=stream):
            fn_st = torch.cuda.current_stream().cuda_stream
            assert fn_st == st
            fn()
        return lambda: g.replay()

    res = {}
    res["plain"] = timed(plain, steps)
    plain_hits = [h.clone() for _, _, h, _, _ in items[:8]]
    res["batched"] = timed(batched, steps)
    same = all(torch.equal(a, b[2]) for a, b in zip(plain_hits, items[:8]))
    res["plain_graph"] = timed(graphed(plain), steps)
    for _, _, h, _, _ in items[:8]:
        h.zero_()
    torch.cuda.synchronize()
    res["batched_graph"] = timed(graphed(batched), steps)
    same = same and all(torch.equal(a, b[2]) for a, b in zip(plain_hits, items[:8]))
    for s in scenes:
        if s.device_status(st) != 0:
            raise RuntimeError("device status word set")
    mrays = {k: round(total_rays / (v[0] / 1e3) / 1e6, 1) for k, v in res.items()}
    mrays["plain_default_config"] = round(total_rays / (default_ms / 1e3) / 1e6, 1)
    line = {
        "metric": "Mrays/s on uneven batches (batched queue kernel + CUDA graph vs one launch per RayBuffer)",
        "value": mrays["batched_graph"], "unit": UNIT, "n_gpus": 1, "steps": steps, "warmup": 1,
        "ms_per_step": round(res["batched_graph"][0], 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
        "config": {"workload": f"{len(items)} batches log-uniform [1024, 2097152] rays over 8 scenes "
                               f"({int(min(tri_counts))}-{int(max(tri_counts))} triangles), 70/30 closest/any",
                   "rays_per_step": total_rays, "Mrays_by_form": mrays,
                   "device_ms_by_form": {k: round(v[0], 3) for k, v in res.items()},
                   "host_ms_by_form": {k: round(v[1], 3) for k, v in res.items()},
                   "batched_over_plain": round(mrays["batched_graph"] / mrays["plain"], 3),
                   "batched_over_plain_default_config": round(mrays["batched_graph"] / mrays["plain_default_config"], 3),
                   "plain": "one lrx_trace per RayBuffer with the autotuned per-scene configs (the same configs "
                            "the batched form uses); plain_default_config: the library defaults, no autotune",
                   "results_equal_plain": bool(same), "autotuned": tuned},
    }
    for s in scenes:
        s.close()
    del items
    if args.build_sweep:
        line["config"]["build_sweep"] = batching_build_sweep(torch, lrx, tri_counts, extents, stream)
    return line


def batching_build_sweep(torch, lrx, tri_counts, extents, stream) -> dict:
    """Per scene of the uneven-batch workload: closest- and any-hit Mrays/s
    of a 262,144-ray random sample under each candidate build of the
    autotuner -- node width 8 or 4, 80- or 64-byte node records, 3 or 2
    triangles per leaf -- at the library's default launch configs, and the
    build lrx_scene_create_autotuned keeps for each mode (tuned launch
    config included)."""
    st = stream.cuda_stream
    n = 1 << 18
    C4 = lrx.LRX_NODES_COMPACT4
    out = {}
    for k, (tris, ext) in enumerate(zip(tri_counts.tolist(), extents.tolist())):
        desc = W.SceneDesc([W.random_triangles(int(tris), W.BASE_SEED + 40 + k, extent=ext)])
        rec = device_random_rays(torch, n, float(ext), W.BASE_SEED + 5000 + k, "cuda:0")
        hits = torch.empty(n * HIT_BYTES, dtype=torch.uint8, device="cuda:0")
        row = {}
        for width, layout, leaf in ((8, 0, 3), (8, 0, 2), (4, 0, 3), (4, 0, 2), (4, C4, 3), (4, C4, 2)):
            with torch.cuda.stream(stream):
                sc = lrx.Scene(desc, stream=st, leaf_max=leaf, node_width=width, node_layout=layout)
            r = {}
            for mode in (lrx.LRX_TRACE_CLOSEST, lrx.LRX_TRACE_ANY):
                sc.trace(rec.data_ptr(), hits.data_ptr(), n, mode, st)
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                for _ in range(5):
                    sc.trace(rec.data_ptr(), hits.data_ptr(), n, mode, st)
                e1.record(stream)
                e1.synchronize()
                r["closest" if mode == lrx.LRX_TRACE_CLOSEST else "any"] = round(
                    n * 5 / (e0.elapsed_time(e1) / 1e3) / 1e6, 1)
            sc.close()
            row[f"width{width}-leaf{leaf}" + ("-nodes64" if layout else "")] = r
        for mode in (lrx.LRX_TRACE_CLOSEST, lrx.LRX_TRACE_ANY):
            sc, opts, cfg = lrx.Scene.autotuned(desc, rec.data_ptr(), n, mode, st)
            row["autotuned_" + ("closest" if mode == lrx.LRX_TRACE_CLOSEST else "any")] = {**opts, **cfg}
            sc.close()
        out[f"scene{k}-{int(tris)}tri"] = row
        log(f"[batching] build sweep scene {k}: {row}")
    return out


# ---------------------------------------------------------------------------
# Serving: 64 sessions over 12 scenes, Poisson arrivals, LRU under a budget
# ---------------------------------------------------------------------------

SERVE_SIZE_RANGE = (4096, 4_194_304)


def collect(server, ticket, timeout_ms=600_000):
    """Waits for a ticket; True once it is finished (a failed request counts
    as finished -- the server's statistics record it), False on timeout."""
    from luxcore_gb300 import lrx
    try:
        server.wait(ticket, timeout_ms)
    except lrx.LrxError as e:
        if e.status == 9:  # LRX_ERR_TIMEOUT: still running
            return False
    return True


def serving_scenes(max_tris):
    """12 scenes with log-uniform triangle counts in [100k, max_tris]; every
    third is instanced (displaced icospheres under random transforms)."""
    rng = W.Rng(W.BASE_SEED + 5, 21)
    counts = W.log_uniform_int(rng, 12, 100_000, max_tris).tolist()
    descs, extents = [], []
    for k, n in enumerate(counts):
        if k % 3 == 2:
            n_inst = max(1, n // 14_580)  # 8 unique icospheres of 20 * 27^2 = 14,580 triangles
            ext = max(1.0, (n_inst / 64.0) ** (1.0 / 3.0))
            descs.append(W.instanced_scene(n_meshes=8, freq=27, n_inst=n_inst, seed=W.BASE_SEED + 60 + k,
                                           scale=(0.1, 0.4), extent=ext))
        else:
            ext = (n / 65536.0) ** (1.0 / 3.0)
            descs.append(W.SceneDesc([W.random_triangles_fast(n, W.BASE_SEED + 60 + k, extent=ext)]))
        extents.append(ext)
    return counts, descs, extents


def run_serving(args):
    line = serving_line(args, args.serve_rates, args.serve_seconds, budget_runs=True)
    print(json.dumps(line), flush=True)
    return 0


def wavefront_pools(torch, descs, extents, pool_n, device, seed):
    """Per scene, the bounce (closest-hit) and shadow (any-hit) rays of a
    PATHOCL-style wavefront path tracer over it (luxcore_gb300.pathocl,
    1,048,576 tasks, camera outside the scene's cube looking in, one light
    near its top), pool_n of each, cycled if the scene yields fewer."""
    from luxcore_gb300 import lrx
    from luxcore_gb300.pathocl import WavefrontPaths
    pools = []
    for k, (d, ext) in enumerate(zip(descs, extents)):
        sc = lrx.Scene(d, treelet_passes=0)
        wp = WavefrontPaths(sc, d, 1024, 1024, max_depth=4, eye=(0.5 * ext, -0.6 * ext, 0.8 * ext),
                            look=(0.5 * ext, 0.5 * ext, 0.4 * ext), light=(0.45 * ext, 0.55 * ext, 0.95 * ext),
                            seed=seed + k, device=device)
        b, sh = wp.harvest(pool_n, pool_n)
        torch.cuda.synchronize()
        sc.close()
        out = []
        for r in (b, sh):
            if r.shape[0] == 0:
                raise RuntimeError(f"serving scene {k}: the wavefront produced no rays")
            reps = (pool_n + r.shape[0] - 1) // r.shape[0]
            out.append(r.repeat(reps, 1)[:pool_n].contiguous())
        pools.append((out[0], out[1]))
        del wp, b, sh
    return pools


def serving_line(args, rates, seconds: float, budget_runs: bool) -> dict:
    """The serving workload: 64 sessions over 12 scenes with Poisson arrivals at
    each rate in `rates`, `seconds` each, batched (continuous batching) and
    plain servers; with budget_runs also a scaled HBM budget that forces
    evictions (with and without the blob cache).  Rays: the bounce and shadow
    rays of a wavefront path tracer over each scene (--serve-rays wavefront)
    or uniformly random rays (random)."""
    import torch

    from luxcore_gb300 import lrx

    dev = "cuda:0"
    torch.cuda.set_device(0)
    t0 = time.perf_counter()
    counts, descs, extents = serving_scenes(args.serve_max_tris)
    log(f"[serving] scenes {counts} generated in {time.perf_counter() - t0:.1f}s")
    pool_n = SERVE_SIZE_RANGE[1]
    t0 = time.perf_counter()
    if args.serve_rays == "wavefront":
        pools = wavefront_pools(torch, descs, extents, pool_n, dev, W.BASE_SEED + 2000)
    else:
        pools = []
        for k, ext in enumerate(extents):
            closest = device_random_rays(torch, pool_n, ext, W.BASE_SEED + 2000 + k, dev)
            anyr = device_random_rays(torch, pool_n, ext, W.BASE_SEED + 3000 + k, dev)
            anyr[:, 7] = torch.rand(pool_n, device=dev) * (0.5 * ext) + 0.05 * ext  # shadow-ray lengths
            pools.append((closest, anyr))
    log(f"[serving] {args.serve_rays} ray pools ready in {time.perf_counter() - t0:.1f}s")
    n_sess, k_buf = args.sessions, 4
    hits = [[torch.empty(pool_n * HIT_BYTES, dtype=torch.uint8, device=dev) for _ in range(k_buf)]
            for _ in range(n_sess)]
    torch.cuda.synchronize()

    def schedule(rate, duration, seed):
        g = np.random.default_rng(seed)
        n = int(rate * duration * 1.5) + 16
        t = np.cumsum(g.exponential(1.0 / rate, n))
        t = t[t < duration]
        lo, hi = SERVE_SIZE_RANGE
        sizes = np.floor(np.exp(g.uniform(np.log(lo), np.log(hi), t.size))).astype(np.int64)
        sess = g.integers(0, n_sess, t.size)
        return list(zip(t.tolist(), sess.tolist(), sizes.tolist()))

    def one_run(policy, budget, rate, cache=True, seed=W.BASE_SEED + 77):
        server = lrx.Server(policy=policy, budget_bytes=budget, streams=args.serve_streams,
                            host_cache_bytes=0 if cache else 2 ** 64 - 1)
        ids = [server.add_scene(d) for d in descs]
        if not budget or budget >= (150 << 30):
            for k in range(len(descs)):  # make every scene resident before the clock starts
                c, _ = pools[k]
                server.wait(server.submit(ids[k], c.data_ptr(), hits[0][0].data_ptr(), 1024, lrx.LRX_TRACE_CLOSEST))
        server.reset_stats()
        sched = schedule(rate, seconds, seed)
        step = [0] * n_sess
        inflight = [[None] * k_buf for _ in range(n_sess)]
        deferred = 0
        start = time.perf_counter()
        for t_arr, s, n in sched:
            while time.perf_counter() - start < t_arr:
                pass
            free = [b for b in range(k_buf) if inflight[s][b] is None]
            if not free:  # the session still has k_buf batches in flight: wait for its oldest
                deferred += 1
                b = 0
                collect(server, inflight[s][0])
                inflight[s][0] = None
                free = [0]
            b = free[0]
            sid = s % len(descs)
            mode = lrx.LRX_TRACE_CLOSEST if step[s] % 2 == 0 else lrx.LRX_TRACE_ANY  # bounce, then shadow
            step[s] += 1
            rays = pools[sid][0 if mode == lrx.LRX_TRACE_CLOSEST else 1]
            inflight[s][b] = server.submit(ids[sid], rays.data_ptr(), hits[s][b].data_ptr(), int(n), mode)
            # collect what has finished so buffers come back
            for ss in (s,):
                for bb in range(k_buf):
                    tk = inflight[ss][bb]
                    if tk is not None and bb != b and collect(server, tk, 0):
                        inflight[ss][bb] = None
        for s in range(n_sess):
            for b in range(k_buf):
                if inflight[s][b] is not None:
                    collect(server, inflight[s][b])
        wall = time.perf_counter() - start
        st = server.stats()
        server.close()
        return {"offered_batches_per_s": rate, "batches": len(sched), "deferred_by_session": deferred,
                "p50_us": round(st["latency_p50_us"], 1), "p99_us": round(st["latency_p99_us"], 1),
                "mean_us": round(st["latency_mean_us"], 1), "max_us": round(st["latency_max_us"], 1),
                "Mrays_per_s": round(st["rays_done"] / max(wall, 1e-9) / 1e6, 1),
                "wall_s": round(wall, 3), "launches": st["launches"], "failed": st["requests_failed"],
                "builds": st["scene_builds"], "evictions": st["scene_evictions"],
                "reloads_from_blob_cache": st["scene_reloads"],
                "peak_resident_GB": round(st["peak_resident_bytes"] / 2 ** 30, 3)}

    full = 150 << 30
    res = {}
    for rate in rates:
        res[f"batched@{rate}"] = one_run(lrx.LRX_SERVE_BATCHED, full, rate)
        res[f"plain@{rate}"] = one_run(lrx.LRX_SERVE_PLAIN, full, rate)
    # the first rate is above what the GPU serves: its backlog, and so p50 and
    # p99, move from run to run (the same schedule gave p99/p50 from 2.3 to
    # 4.7), so the batched server is run there twice more, on other Poisson
    # schedules, and the line also gives the median ratio of the three runs
    head_rate = rates[0]
    repeats = [res[f"batched@{head_rate}"]]
    for k in (1, 2):
        r = one_run(lrx.LRX_SERVE_BATCHED, full, head_rate, seed=W.BASE_SEED + 77 + k)
        res[f"batched@{head_rate}-schedule{k + 1}"] = r
        repeats.append(r)
    ratios = [round(v["p99_us"] / max(v["p50_us"], 1e-9), 2) for v in repeats]
    # scaled budget: ~40 % of the scene bytes, so scenes are evicted and rebuilt
    probe_total, probe_max = 0, 0
    for d in descs:
        s = lrx.Scene(d, treelet_passes=0)  # as the server builds
        probe_total += s.info()["device_bytes"]
        probe_max = max(probe_max, s.info()["device_bytes"])
        s.close()
    small = int(max(probe_total * 0.4, probe_max * 1.25))  # the largest scene must still fit
    if budget_runs:
        low_rate = min(rates)
        res[f"batched@{low_rate}-budget40pct"] = one_run(lrx.LRX_SERVE_BATCHED, small, low_rate)
        res[f"batched@{low_rate}-budget40pct-no-blob-cache"] = one_run(lrx.LRX_SERVE_BATCHED, small, low_rate,
                                                                       cache=False)
    head = res[f"batched@{rates[0]}"]
    plain = res[f"plain@{rates[0]}"]
    line = {
        "metric": "served p50/p99 batch latency and Mrays/s (continuous batching vs plain launch)",
        "value": head["Mrays_per_s"], "unit": UNIT, "n_gpus": 1, "steps": 1, "warmup": 1,
        "ms_per_step": round(head["wall_s"] * 1e3, 1), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
        "config": {"workload": f"{n_sess} sessions over 12 scenes ({min(counts)}-{max(counts)} triangles, 4 "
                               f"instanced), Poisson arrivals, sizes log-uniform {list(SERVE_SIZE_RANGE)}, "
                               f"bounce (closest) / shadow (any) alternating per session",
                   "rays": ("bounce and shadow rays of a wavefront path tracer over each scene (1,048,576 tasks, "
                            "depth 4)" if args.serve_rays == "wavefront" else "uniformly random rays"),
                   "seconds_per_run": seconds,
                   "scene_bytes_total_GB": round(probe_total / 2 ** 30, 3), "budgets_GB": [150, round(small / 2 ** 30, 3)],
                   "runs": res,
                   "p99_over_p50": {k: round(v["p99_us"] / max(v["p50_us"], 1e-9), 2) for k, v in res.items()},
                   f"batched@{head_rate}_p99_over_p50_median_of_3_schedules": float(np.median(ratios)),
                   "batched_over_plain_Mrays": {f"@{r}": round(res[f"batched@{r}"]["Mrays_per_s"] /
                                                               max(res[f"plain@{r}"]["Mrays_per_s"], 1e-9), 3)
                                                for r in rates}},
    }
    del pools, hits
    return line


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=300)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="lrx", choices=["lrx", "reference"])
    ap.add_argument("--sessions", type=int, default=64)
    ap.add_argument("--serve-max-tris", type=int, default=20_000_000)
    ap.add_argument("--serve-seconds", type=float, default=2.0)
    ap.add_argument("--serve-rates", type=float, nargs="+", default=[2000.0, 800.0])
    ap.add_argument("--serve-streams", type=int, default=4)
    ap.add_argument("--serve-rays", default="wavefront", choices=["wavefront", "random"],
                    help="serving ray pools: a wavefront path tracer's bounce and shadow rays, or random rays")
    ap.add_argument("--no-extras", action="store_true",
                    help="default workload: skip the bounded batching and serving runs after the main line's timing")
    ap.add_argument("--workload", default="heightfield", choices=["heightfield", "batching", "serving", "instanced",
                                                                      "motion", "pathocl"],
                    help="heightfield = the headline line; batching = uneven batches, plain vs queue kernel")
    ap.add_argument("--batches", type=int, default=512)
    ap.add_argument("--step-form", default="batched", choices=["batched", "sequential"],
                    help="heightfield step: one lrx_trace_batches call over the 3 sets, or 3 lrx_trace calls")
    ap.add_argument("--inst-rays", type=int, default=1 << 23, help="instanced workload: rays per set")
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--ref-fraction", type=int, default=4,
                    help="CPU legs trace every Nth ray of each set")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-ref-gpu", action="store_true",
                    help="skip the reference's own CUDA kernel on this GPU (needs the CPU baseline's oracle)")
    ap.add_argument("--no-e2e", action="store_true", help="skip the host-buffer (lrx_trace_host) leg")
    ap.add_argument("--no-big-bounce", action="store_true", help="skip the 8 M-ray bounce launch")
    ap.add_argument("--sweep", action="store_true", help="also time other launch configurations")
    ap.add_argument("--treelet-passes", type=int, default=None, help="BVH treelet passes (default: the library's)")
    ap.add_argument("--build-sweep", action="store_true",
                    help="also build with 0-3 treelet passes and time each tree (outside the timed region)")
    ap.add_argument("--block-size", type=int, default=None, help="override the per-mode defaults")
    ap.add_argument("--postpone", type=int, default=None)
    ap.add_argument("--variant", type=int, default=None, help="LRX_VARIANT_* bits")
    ap.add_argument("--refill", type=int, default=None, help="with LRX_VARIANT_PERSISTENT: idle lanes per claim")
    args = ap.parse_args()
    if args.warmup < 3:
        log("warmup raised to 3 (timing rule)")
        args.warmup = 3
    if args.workload == "serving" and args.impl == "lrx":
        return run_serving(args)
    if args.workload == "batching" and args.impl == "lrx":
        return run_batching(args)
    if args.workload == "instanced" and args.impl == "lrx":
        return run_instanced(args)
    if args.workload == "motion" and args.impl == "lrx":
        return run_instanced(args, motion=True)
    if args.workload == "pathocl" and args.impl == "lrx":
        return run_pathocl(args)
    if args.impl == "reference":
        return run_reference(args)
    return run_lrx(args)


if __name__ == "__main__":
    sys.exit(main())
