#!/usr/bin/env python
"""Throughput of the policy + value evaluation path on GB300.

Workload (one "step"): 8192 positions through BOTH benchmark nets -- policy
(5x5 24->128, 11x 3x3 128->128, 1x1 head, ReLU, softmax over 361) and value
(same trunk, FC 361->256 ReLU, FC 256->1, tanh) -- in batches of 256, on the
BF16 tensor-core path.  Positions: the 1024 seeded positions of
tests/golden/positions_s0.npz (empty board, komi 7.5, k~U[0,250] uniform legal
moves, planes from the reference's own feature gather) under the 8 board
symmetries = 8192 distinct inputs.  Weights: He-normal, zero biases, seeds 1
(policy) and 2 (value).

Reported (one JSON line on rank 0):
  value       positions/s with inputs resident in HBM (lg_*_device)
  e2e         positions/s through the host C ABI from boards
              (lg_policy_boards / lg_value_boards: 362 bytes a position in,
              input planes gathered on the GPU, results out; the copies and
              the gather timed) -- the counterpart of get_scored_moves /
              get_value, whose gather runs on the host.  e2e_planes: the same
              through lg_policy / lg_value with host-gathered planes.
  roofline    the dominant kernel (tensor-core 3x3 conv), CUDA-event timed
              inside the timed region, against the measured BF16 peak
  cpu_baseline  the reference algorithm (im2col + OpenBLAS sgemm, one
              position per thread) on this host's cores, bounded sample
  fp32_plain_batch1  the plain FP32 drop-in path at batch 1 (the ratio
              target's denominator), and top-1 agreement of BF16 vs FP64

--impl reference: the reference's CPU path (the C restatement of
Network.cpp's im2col + sgemm + bias + activation over scipy's OpenBLAS; the
reference engine itself cannot be built where its sources are absent) on all
host threads, same metric and config.
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

METRIC = "positions/sec policy+value net, BF16 vs FP32 plain on GB300 at ≥99% top-1 agree"
BATCH = 256
POSITIONS = 8192
# Algorithmic FLOPs of one 3x3 128->128 conv per position: 2 * 361 * 128 * 1152.
FLOP_3X3_PER_POS = 2 * 361 * 128 * 1152
# ... of the 5x5 24->128 first layer: 2 * 361 * 128 * 600.
FLOP_5X5_PER_POS = 2 * 361 * 128 * 600
# Policy (1,226,637,568) + value (1,226,822,912) FLOP per position.
FLOP_PAIR_PER_POS = 2_453_460_480


def load_positions():
    d = np.load(os.path.join(ROOT, "tests", "golden", "positions_s0.npz"))
    pp = np.unpackbits(d["planes_p"], axis=-1)[:, :24, :361]
    pv = np.unpackbits(d["planes_v"], axis=-1)[:, :24, :361]
    import leela_gb300 as lg
    P = np.concatenate([pp[..., lg.ROTATE[s]] for s in range(8)])
    V = np.concatenate([pv[..., lg.ROTATE[s]] for s in range(8)])
    return np.ascontiguousarray(P), np.ascontiguousarray(V)


def load_boards(with_moves: bool = False):
    """The 1024 fixture boards under the 8 symmetries, in the order of
    load_positions(): squares [8192][361] int8 and to_move [8192] int8 (and
    moves [8192][4]: last move, the move before, ko point -- rotated with the
    board -- and the komi flag)."""
    d = np.load(os.path.join(ROOT, "tests", "golden", "positions_s0.npz"))
    import leela_gb300 as lg
    sq = np.concatenate([d["squares"][:, lg.ROTATE[s]] for s in range(8)])
    tm = np.tile(d["meta"][:, 0].astype(np.int8), 8)
    if not with_moves:
        return np.ascontiguousarray(sq, dtype=np.int8), tm
    mv = []
    for s in range(8):
        inv = np.argsort(lg.ROTATE[s])  # old point -> its index on the rotated board
        m = d["moves"].copy()
        for k in range(3):
            m[:, k] = np.where(m[:, k] >= 0, inv[np.maximum(m[:, k], 0)], -1)
        mv.append(m)
    return np.ascontiguousarray(sq, dtype=np.int8), tm, np.ascontiguousarray(np.concatenate(mv), np.int32)


def make_weights():
    from oracle import oracle as O
    P, V = O.make_net(O.CFG_POLICY), O.make_net(O.CFG_VALUE)
    return P, V, O.he_weights(P, O.POLICY_SEED), O.he_weights(V, O.VALUE_SEED)


def read_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return p.get("bf16_tflops_sustained", 1700.0), p.get("hbm_gbs", 6800.0), "measured"
    except (OSError, ValueError):
        return 1700.0, 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi samples during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
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
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.t.join(timeout=2)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for n, v in zip(names, parts[3:7]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x: float, world: int) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ------------------------------------------------------------- CPU baseline

def cpu_baseline(planes_p, planes_v, seconds: float = 12.0, nthreads: int = 0):
    """The reference algorithm on the host: im2col + OpenBLAS sgemm + bias +
    activation per layer (Network.cpp:345-423), one position per thread
    (Network.cpp:239), every host core."""
    from oracle import oracle as O
    P, V, wp, wv = make_weights()
    blas = O.enable_blas()
    n = nthreads or os.cpu_count()
    sample = planes_p[:512], planes_v[:512]
    t = O.time_pair_f32(P, wp, V, wv, sample[0], sample[1], n, n)
    iters = max(n, int(seconds / max(t, 1e-3) * n))
    el = O.time_pair_f32(P, wp, V, wv, sample[0], sample[1], iters, n)
    O.disable_blas()
    return {"value": iters / el, "unit": "positions/s", "cores": n, "kind": "port",
            "sample": f"{iters} policy+value evaluations over 512 positions, "
                      f"{'OpenBLAS sgemm' if blas else 'plain-loop GEMM'}, {el:.1f} s"}


def run_reference(args, world, rank):
    if rank != 0:
        return
    from oracle import oracle as O
    planes_p, planes_v = load_positions()
    P, V, wp, wv = make_weights()
    blas = O.enable_blas()
    n = os.cpu_count()
    per_step = 4 * n
    for _ in range(args.warmup):
        O.time_pair_f32(P, wp, V, wv, planes_p[:512], planes_v[:512], per_step, n)
    total = 0.0
    for _ in range(args.steps):
        total += O.time_pair_f32(P, wp, V, wv, planes_p[:512], planes_v[:512], per_step, n)
    value = per_step * args.steps / total
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "positions/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * total / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "config-1 policy+value nets (5x5 24->128, 11x 3x3 128->128, "
                               "1x1 head, ReLU, FC 361->256->1 tanh), CPU", "batch": 1,
                   "positions_per_step": per_step},
        "cpu_baseline": {"value": value, "unit": "positions/s", "cores": n, "kind": "port",
                         "sample": f"{per_step} policy+value evaluations per step over 512 "
                                   f"positions, one per thread, "
                                   f"{'OpenBLAS sgemm' if blas else 'plain-loop GEMM'}"},
        "e2e": {"value": value, "unit": "positions/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    O.disable_blas()
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------- GPU arm

def run_ours(args, world, rank, local):
    import torch

    import leela_gb300 as lg
    from leela_gb300 import build as B
    B.build()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    planes_p, planes_v = load_positions()
    P, V, wp, wv = make_weights()
    ctx = lg.Context(policy=lg.NetDesc.config1_policy(wp, "bf16"),
                     value=lg.NetDesc.config1_value(wv, "bf16"), device=local, max_batch=BATCH)
    import tempfile
    if args.profile_run:
        # fixed kernel choice (the autotuner's pick at batch 256 on GB300), so
        # that a profiler's launch list holds only the measured step's kernels
        ctx.set_tuning(BATCH, 3, 0)
    else:
        ctx.autotune(os.path.join(tempfile.gettempdir(), f"leela_gb300_tune_{BATCH}.json"))
    d_p = torch.from_numpy(planes_p).to(dev)
    d_v = torch.from_numpy(planes_v).to(dev)
    d_probs = torch.empty((POSITIONS, 361), dtype=torch.float32, device=dev)
    d_val = torch.empty(POSITIONS, dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream(dev)
    sp = stream.cuda_stream

    def step():
        ctx.policy_device(d_p.data_ptr(), POSITIONS, d_probs.data_ptr(), 1.0, None, sp)
        ctx.value_device(d_v.data_ptr(), POSITIONS, d_val.data_ptr(), sp)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    # ---------------- timed region: inputs resident in HBM (142 MB > L2)
    launches0 = ctx.stats()["kernel_launches"]
    ctx.profile(True)
    clocks = ClockSampler(local)
    clocks.start()
    barrier(world)
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(args.steps):
        step()
    ev1.record(stream)
    torch.cuda.synchronize()
    barrier(world)
    clk = clocks.stop()
    ms = ev0.elapsed_time(ev1)
    gpu_launches = ctx.stats()["kernel_launches"] - launches0
    n3, ms3 = ctx.profile_read(lg.PROF_TC_3X3)
    nh, msh = ctx.profile_read(lg.PROF_TC_HEAD)
    nf, msf = ctx.profile_read(lg.PROF_TC_FIRST)
    no, mso = ctx.profile_read(lg.PROF_OTHER)
    ntr, mstr = ctx.profile_read(lg.PROF_TC_TRUNK)
    npk, mspk = ctx.profile_read(lg.PROF_PACK)
    ntl, mstl = ctx.profile_read(lg.PROF_TAIL)
    tuning = ctx.tuning(BATCH)
    ctx.profile(False)
    ms_max = max_over_ranks(ms, world)
    value = world * POSITIONS * args.steps / (ms_max / 1e3)
    if args.profile_run:
        ctx.close()
        if rank == 0:
            print(json.dumps({"profile_run": True, "value": value}), flush=True)
        return

    # ---------------- e2e: host boards through lg_policy_boards / lg_value_boards
    squares, to_move = load_boards()
    ctx.policy_boards(squares[:BATCH], to_move[:BATCH])
    ctx.value_boards(squares[:BATCH], to_move[:BATCH])
    e2e_steps = max(3, min(args.steps, 10))
    barrier(world)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        probs = ctx.policy_boards(squares, to_move)
        vals = ctx.value_boards(squares, to_move)
    t_e2e = max_over_ranks(time.perf_counter() - t0, world)
    e2e = {"value": world * POSITIONS * e2e_steps / t_e2e, "unit": "positions/s",
           "h2d_bytes_per_step": int(2 * (squares.nbytes + to_move.nbytes)),
           "d2h_bytes_per_step": int(probs.nbytes + vals.nbytes),
           "call": "lg_policy_boards + lg_value_boards (gather on the GPU)"}
    # the same with planes gathered on the host (lg_policy / lg_value)
    host_p = np.ascontiguousarray(planes_p)
    host_v = np.ascontiguousarray(planes_v)
    ctx.policy(host_p[:BATCH])
    ctx.value(host_v[:BATCH])
    barrier(world)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        probs = ctx.policy(host_p)
        vals = ctx.value(host_v)
    t_e2p = max_over_ranks(time.perf_counter() - t0, world)
    e2e_planes = {"value": world * POSITIONS * e2e_steps / t_e2p, "unit": "positions/s",
                  "h2d_bytes_per_step": int(host_p.nbytes + host_v.nbytes),
                  "d2h_bytes_per_step": int(probs.nbytes + vals.nbytes),
                  "call": "lg_policy + lg_value (planes gathered on the host)"}

    extras = {}
    if rank == 0:
        extras = secondary_measurements(lg, ctx, wp, wv, planes_p, planes_v, d_p, d_v, dev, sp)
        extras["e2e_planes"] = e2e_planes
        extras["gather"] = gather_throughput(lg, squares, to_move, dev, sp)

    if rank != 0:
        ctx.close()
        return
    peak, hbm, peak_kind = read_peaks()
    if ntr and tuning.get("conv3x3") == 3:
        # persistent kernel: the 5x5 first layer and all 11 3x3 layers of one net
        kernel_name = "tc_trunk_kernel (5x5 24->128 + 11 x 3x3 128->128 in one launch, batch 256)"
        n_dom, ms_dom = ntr, mstr
        flop_launch = (11 * FLOP_3X3_PER_POS + FLOP_5X5_PER_POS) * BATCH
    elif ntr:
        # persistent kernel: all 11 3x3 layers of one net per launch
        kernel_name = "tc_trunk_kernel (11 x 3x3 128->128 in one launch, batch 256)"
        n_dom, ms_dom = ntr, mstr
        flop_launch = 11 * FLOP_3X3_PER_POS * BATCH
    else:
        kernel_name = "tc_convT_kernel<2,0,0> (3x3 128->128, batch 256)"
        n_dom, ms_dom = n3, ms3
        flop_launch = FLOP_3X3_PER_POS * BATCH
    avg3 = ms_dom / max(n_dom, 1) / 1e3
    achieved = flop_launch / avg3 / 1e12 if n_dom else None
    traffic = None
    tpath = os.path.join(ROOT, "profiles", "roofline_traffic.json")
    if os.path.exists(tpath):
        with open(tpath) as f:
            traffic = json.load(f).get("tc_trunk_kernel" if ntr else "tc_convT_kernel<2,0,0>")
    line = {
        "metric": METRIC, "value": value, "unit": "positions/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_max / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "bf16",
        "data": "synthetic: 1024 seeded positions (reference feature gather) x 8 symmetries, "
                "He-normal weights",
        "config": {"workload": "config-1 policy+value nets (5x5 24->128, 11x 3x3 128->128, 1x1 "
                               "head, ReLU, FC 361->256->1 tanh), BF16, batch 256",
                   "batch": BATCH, "positions_per_step": POSITIONS, "precision": "bf16",
                   "parallelism": f"replicas x{world}",
                   "l2": "inputs 142 MB per step > L2 129 MB; no flush"},
        "e2e": e2e,
        "roofline": {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                     "frac": (achieved / peak) if achieved else None, "traffic": traffic,
                     "kernel": kernel_name,
                     "peak_source": f"bf16_tflops_sustained ({peak_kind})",
                     "launches": n_dom, "avg_launch_us": avg3 * 1e6,
                     "flop_per_launch": flop_launch},
        "kernel_time_share": {
            "tc_3x3": ms3, "tc_3x3_fused_head": msh, "tc_trunk": mstr, "tc_5x5_first": msf,
            "pack_planes": mspk, "softmax_value_fc": mstl, "other": mso,
            "launches": {"tc_3x3": n3, "tc_head": nh, "tc_trunk": ntr, "tc_first": nf,
                         "pack_planes": npk, "softmax_value_fc": ntl, "other": no}},
        "kernel_choice_batch256": tuning,
        "clocks": clk,
        "gpu_launches": gpu_launches,
        "pair_flop_rate_tflops": FLOP_PAIR_PER_POS * value / world / 1e12,
    }
    line.update(extras)
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(planes_p, planes_v, seconds=args.cpu_seconds)
    ctx.close()
    print(json.dumps(line), flush=True)


def serving_config3(lg, wp, wv, planes_p, planes_v, device, n_req=100_000, rate=200_000.0,
                    mean_batch=48, max_batch=512):
    """Uneven batching as the search produces it: n_req single-position
    requests with Poisson arrivals (rate per second, seed 2), grouped into
    batches of Geometric(mean 48) sizes clipped to [1, 512] (seed 3).  Each
    batch is submitted to both nets (lg_submit) at its last arrival; the
    server merges what is queued, pads to a power-of-two bucket and replays
    that bucket's CUDA graph.  Latency = completion of both nets - arrival."""
    import tempfile
    import threading as th
    arrivals = np.cumsum(np.random.default_rng(2).exponential(1.0 / rate, n_req))
    rng = np.random.default_rng(3)
    sizes, total = [], 0
    while total < n_req:
        b = int(min(max(rng.geometric(1.0 / mean_batch), 1), max_batch, n_req - total))
        sizes.append(b)
        total += b
    n_pos = planes_p.shape[0]
    with lg.Context(policy=lg.NetDesc.config1_policy(wp, "bf16"),
                    value=lg.NetDesc.config1_value(wv, "bf16"), device=device,
                    max_batch=max_batch) as ctx:
        ctx.autotune(os.path.join(tempfile.gettempdir(), f"leela_gb300_tune_{max_batch}.json"))
        # Capture every bucket's graphs (both server slots) before the clock starts.
        b, tag = 1, 10_000_000
        while b <= max_batch:
            for _ in range(2):
                for net, src in ((lg.LG_NET_POLICY, planes_p), (lg.LG_NET_VALUE, planes_v)):
                    x = np.ascontiguousarray(src[:b])
                    o = np.empty((b, 361) if net == lg.LG_NET_POLICY else b, np.float32)
                    tag += 1
                    ctx.submit(net, x, o, tag=tag)
                    for _ in range(5000):
                        if ctx.poll(4, timeout_us=1000):
                            break
            b *= 2
        batches, start = [], 0
        for k, sz in enumerate(sizes):
            idx = np.arange(start, start + sz) % n_pos
            batches.append((np.ascontiguousarray(planes_p[idx]), np.ascontiguousarray(planes_v[idx]),
                            np.empty((sz, 361), np.float32), np.empty(sz, np.float32), start, sz))
            start += sz
        done = {}
        stop = th.Event()

        def poller():
            while not stop.is_set() or len(done) < 2 * len(batches):
                for t in ctx.poll(512, timeout_us=2000):
                    done[t] = time.perf_counter()
                if stop.is_set() and len(done) >= 2 * len(batches):
                    break

        pt = th.Thread(target=poller, daemon=True)
        pt.start()
        t0 = time.perf_counter() + 0.01
        for k, (bp, bv, op, ov, st, sz) in enumerate(batches):
            due = t0 + arrivals[st + sz - 1]
            while time.perf_counter() < due:
                pass
            ctx.submit(lg.LG_NET_POLICY, bp, op, tag=2 * k + 1)
            ctx.submit(lg.LG_NET_VALUE, bv, ov, tag=2 * k + 2)
        stop.set()
        pt.join(timeout=60)
        served = ctx.stats()["batches"]
    if len(done) < 2 * len(batches):
        return {"error": f"only {len(done)} of {2 * len(batches)} submissions completed"}
    lat = np.empty(n_req)
    last = 0.0
    for k, (_, _, _, _, st, sz) in enumerate(batches):
        comp = max(done[2 * k + 1], done[2 * k + 2])
        last = max(last, comp)
        lat[st:st + sz] = comp - (t0 + arrivals[st:st + sz])
    return {"requests": n_req, "arrival_rate_per_s": rate, "client_batches": len(sizes),
            "server_batches": int(served), "mean_client_batch": float(np.mean(sizes)),
            "throughput_positions_per_s": n_req / (last - (t0 + arrivals[0])),
            "latency_p50_ms": float(np.percentile(lat, 50) * 1e3),
            "latency_p99_ms": float(np.percentile(lat, 99) * 1e3),
            "note": "policy + value per request; BF16; CUDA graph per power-of-two bucket "
                    "(host copies inside the graph); autotuned kernel choice per bucket"}


def secondary_measurements(lg, ctx, wp, wv, planes_p, planes_v, d_p, d_v, dev, sp):
    """FP32 batch-1 throughput, BF16 at the other batch sizes, and top-1
    agreement with the FP64 oracle."""
    import torch
    out = {}
    # FP32 plain path at batch 1 (policy + value per position).
    with lg.Context(policy=lg.NetDesc.config1_policy(wp, "fp32"),
                    value=lg.NetDesc.config1_value(wv, "fp32"), device=dev.index,
                    max_batch=1) as c32:
        n = 200
        for i in range(5):
            c32.policy(planes_p[i:i + 1])
            c32.value(planes_v[i:i + 1])
        t0 = time.perf_counter()
        for i in range(n):
            c32.policy(planes_p[i:i + 1])
            c32.value(planes_v[i:i + 1])
        host_rate = n / (time.perf_counter() - t0)
        probs = torch.empty((1, 361), device=dev)
        val = torch.empty(1, device=dev)
        for i in range(5):
            c32.policy_device(d_p[i].data_ptr(), 1, probs.data_ptr(), 1.0, None, sp)
            c32.value_device(d_v[i].data_ptr(), 1, val.data_ptr(), sp)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for i in range(n):
            c32.policy_device(d_p[i].data_ptr(), 1, probs.data_ptr(), 1.0, None, sp)
            c32.value_device(d_v[i].data_ptr(), 1, val.data_ptr(), sp)
        e1.record()
        torch.cuda.synchronize()
        dev_rate = n / (e0.elapsed_time(e1) / 1e3)
    out["fp32_plain_batch1"] = {"host_api_positions_per_s": host_rate,
                                "device_positions_per_s": dev_rate}
    # BF16 at the other configured batch sizes (device-resident inputs),
    # autotuned as a user's context would be.
    import tempfile
    by_batch = {}
    for b in (1, 8, 64, 256):
        with lg.Context(policy=lg.NetDesc.config1_policy(wp, "bf16"),
                        value=lg.NetDesc.config1_value(wv, "bf16"), device=dev.index,
                        max_batch=b) as cb:
            cb.autotune(os.path.join(tempfile.gettempdir(), f"leela_gb300_tune_{b}.json"))
            probs = torch.empty((b, 361), device=dev)
            val = torch.empty(b, device=dev)
            reps = max(4, min(200, 4096 // b))
            for i in range(3):
                cb.policy_device(d_p.data_ptr(), b, probs.data_ptr(), 1.0, None, sp)
                cb.value_device(d_v.data_ptr(), b, val.data_ptr(), sp)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            for i in range(reps):
                off = (i * b) % (8192 - b + 1)
                cb.policy_device(d_p[off].data_ptr(), b, probs.data_ptr(), 1.0, None, sp)
                cb.value_device(d_v[off].data_ptr(), b, val.data_ptr(), sp)
            e1.record()
            torch.cuda.synchronize()
            by_batch[str(b)] = b * reps / (e0.elapsed_time(e1) / 1e3)
    out["bf16_by_batch_positions_per_s"] = by_batch
    out["ratio_bf16_batched_vs_fp32_batch1"] = by_batch["256"] / dev_rate
    # Top-1 agreement with the FP64 oracle (BF16 and FP8 weights), 256 positions.
    from oracle import oracle as O
    P, V = O.make_net(O.CFG_POLICY), O.make_net(O.CFG_VALUE)
    idx = np.arange(0, 8192, 32)
    O.enable_blas()
    l64 = O.forward_f64(P, wp, planes_p[idx])
    v64 = O.forward_f64(V, wv, planes_v[idx])
    O.disable_blas()
    p64 = O.softmax_f64(l64, 1.0)
    agree = {}
    for prec in ("bf16", "fp8w"):
        with lg.Context(policy=lg.NetDesc.config1_policy(wp, prec),
                        value=lg.NetDesc.config1_value(wv, prec), device=dev.index,
                        max_batch=256) as cq:
            pr, lo = cq.policy(planes_p[idx], 1.0, return_logits=True)
            vq = cq.value(planes_v[idx])
        agree[prec] = {"top1": float((lo.argmax(1) == l64.argmax(1)).mean()),
                       "prob_max_abs_err": float(np.abs(pr - p64).max()),
                       "prob_mean_abs_err": float(np.abs(pr - p64).mean()),
                       "value_max_abs_err": float(np.abs(vq - v64).max()),
                       "value_mean_abs_err": float(np.abs(vq - v64).mean()),
                       "positions": int(idx.size)}
    out["vs_fp64_oracle"] = agree
    out["serving_config3"] = serving_config3(lg, wp, wv, planes_p, planes_v, dev.index)
    out["distill_config4"] = distill_config4(wp, wv, planes_p, planes_v, dev.index)
    return out


def gather_throughput(lg, squares, to_move, dev, sp, reps=20):
    """lg_gather_device alone, boards resident in HBM: 8192 boards -> 24
    policy planes and 24 value planes (the benchmark nets' inputs;
    algorithmic bytes per board and set 362 in + 24 * 361 out), and -> all 32
    planes of both sets (ladder reader, ko, last moves, komi)."""
    import torch
    B = squares.shape[0]
    _, _, moves = load_boards(with_moves=True)
    d_sq = torch.from_numpy(squares).to(dev)
    d_tm = torch.from_numpy(to_move).to(dev)
    d_mv = torch.from_numpy(moves).to(dev)
    out_p = torch.empty((B, 32, 361), dtype=torch.uint8, device=dev)
    out_v = torch.empty((B, 32, 361), dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream(dev)

    def timed(nplanes):
        def run():
            for which, out in ((0, out_p), (1, out_v)):
                lg.gather_device(d_sq.data_ptr(), d_tm.data_ptr(), B, which, nplanes, out.data_ptr(), sp,
                                 d_mv.data_ptr())
        for _ in range(3):
            run()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            run()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps

    ms = timed(24)
    ms32 = timed(32)
    per_launch = B * (362 + 24 * 361)
    _, hbm, _ = read_peaks()
    gbs = 2 * per_launch / (ms / 1e3) / 1e9
    return {"boards_per_s_both_sets": B / (ms / 1e3), "us_per_launch": ms * 1e3 / 2,
            "boards_per_launch": B, "algorithmic_bytes_per_launch": per_launch,
            "achieved_gbs": gbs, "hbm_peak_gbs": hbm, "frac_of_hbm": gbs / hbm if hbm else None,
            "all_32_planes_boards_per_s_both_sets": B / (ms32 / 1e3),
            "all_32_planes_us_per_launch": ms32 * 1e3 / 2}


def gather_run(reps):
    """lg_gather_device alone on 8192 boards (gather_throughput), one JSON line."""
    import torch
    import leela_gb300 as lg
    dev = torch.device("cuda", 0)
    squares, to_move = load_boards()
    sp = torch.cuda.current_stream(dev).cuda_stream
    res = gather_throughput(lg, squares, to_move, dev, sp, reps=reps)
    print(json.dumps({"gather_run": True, **res}), flush=True)


def distill_config4(wp, wv, planes_p, planes_v, device):
    """The distilled student (64-wide net, entropy-gated fallback to the full
    net) on the fixture positions: the student is trained on
    positions 0..895 (x8 symmetries), evaluated on 896..1023; labels are the
    full FP32 policy net's softmax and 2*mc_owner(64)-1.  Run at the
    specified teacher temperature 1 and, as an ablation, at 0.05 (the
    He-normal teacher's policies are nearly flat at temperature 1)."""
    from leela_gb300 import distill
    mc = np.load(os.path.join(ROOT, "tests", "golden", "mcowner_s0.npz"))["mcowner"]
    pos_index = np.arange(planes_p.shape[0]) % 1024
    res = {}
    for name, temp in (("teacher_T1", 1.0), ("teacher_T0.05", 0.05)):
        res[name] = distill.run_config4(planes_p, planes_v, pos_index, mc, wp, wv, device,
                                        teacher_temperature=temp, time_budget_s=25.0)
    return res


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--profile-run", action="store_true",
                    help="only the device-resident warm-up and timed steps (for ncu)")
    ap.add_argument("--gather-run", action="store_true",
                    help="only the gather timing: 8192 boards, 24 and 32 planes, both sets (for ncu)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.gather_run:
        gather_run(reps=5)
        return
    world, rank, local = dist_setup()
    if args.impl == "reference":
        run_reference(args, world, rank)
    else:
        run_ours(args, world, rank, local)


if __name__ == "__main__":
    main()
