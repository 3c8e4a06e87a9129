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
  roofline    the dominant kernel (the persistent trunk), timed with CUDA
              events around every launch in a second pass over the same
              steps (the first pass, which gives `value`, has no events
              between launches: they would serialise the programmatic
              dependent launches), against the measured BF16 peak
  cpu_baseline  the reference algorithm (im2col + OpenBLAS sgemm, one
              position per thread) on this host's cores, bounded sample
  summary     the plain FP32 drop-in path at batch 1 (the ratio target's
              denominator), BF16 and FP16 at other batch sizes, the same step
              in FP16 (the variant at >= 99% top-1 vs FP64), top-1 agreement
              vs FP64 over 65,536 positions, the 8-symmetry ensemble (a
              search's root, and 32 positions a call), serving, the
              distilled path, and leaf evaluations/s under the engine's
              request pattern (search_pattern.cpp)

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
    """(BF16 burst TFLOP/s, BF16 sustained TFLOP/s, HBM GB/s, source)."""
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return (p.get("bf16_tflops", 1900.0), p.get("bf16_tflops_sustained", 1700.0), p.get("hbm_gbs", 6800.0),
                "measured")
    except (OSError, ValueError):
        return 1900.0, 1700.0, 6800.0, "fallback"


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
    # ---------------- the same steps again with CUDA events around every
    # launch (per-kernel times: the roofline's trunk launches and the
    # kernel-time shares); the events serialise the launches, so this
    # region's step time is reported beside `value`, not as it
    ctx.profile(True)
    torch.cuda.synchronize()
    ep0, ep1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ep0.record(stream)
    for _ in range(args.steps):
        step()
    ep1.record(stream)
    torch.cuda.synchronize()
    ms_prof = ep0.elapsed_time(ep1)
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
        extras = secondary_measurements(lg, ctx, wp, wv, planes_p, planes_v, d_p, d_v, dev, sp,
                                        quick=args.quick)
        extras["e2e_planes"] = e2e_planes
        extras["gather"] = gather_throughput(lg, squares, to_move, dev, sp)

    if rank != 0:
        ctx.close()
        return
    peak_burst, peak_sust, hbm, peak_kind = read_peaks()
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
    total_ms = sum(x for x in (ms3, msh, msf, mso, mstr, mspk, mstl))
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
        "roofline": {"bound": "tensor", "achieved": achieved, "peak": peak_burst, "unit": "TFLOP/s",
                     "frac": (achieved / peak_burst) if achieved else None, "traffic": traffic,
                     "kernel": kernel_name,
                     "peak_source": f"bf16_tflops, burst ({peak_kind}): the kernel runs in a sub-second "
                                    f"region at max clocks",
                     "frac_of_sustained": (achieved / peak_sust) if achieved else None,
                     "launches": n_dom, "avg_launch_us": avg3 * 1e6, "flop_per_launch": flop_launch},
        "kernel_time_share": {k: round(v / total_ms, 4) for k, v in (
            ("tc_trunk", mstr), ("tc_3x3", ms3 + msh), ("tc_5x5_first", msf), ("pack_planes", mspk),
            ("softmax_value_fc", mstl), ("other", mso)) if v},
        "kernel_choice_batch256": tuning,
        "ms_per_step_with_launch_events": ms_prof / args.steps,
        "clocks": clk,
        "gpu_launches": gpu_launches,
        "pair_flop_rate_tflops": FLOP_PAIR_PER_POS * value / world / 1e12,
    }
    # the key secondary numbers in the line (short, so that it survives
    # whole); everything in --detail
    line["summary"] = summarize(extras, value)
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(planes_p, planes_v, seconds=args.cpu_seconds)
    if args.detail:
        with open(args.detail, "w") as f:
            json.dump({"line": line, "extras": extras}, f, indent=1)
    ctx.close()
    print(json.dumps(line), flush=True)


def summarize(x, value):
    """A few figures of the secondary measurements for the JSON line."""
    r = lambda v, n=4: None if v is None else round(v, n)  # noqa: E731
    out = {}
    b1 = x.get("fp32_batch1", {})
    if b1:
        out["fp32_batch1_pairs_per_s"] = r(b1.get("small_batch_device_pairs_per_s"), 1)
        out["fp32_batch1_host_api_pairs_per_s"] = r(b1.get("small_batch_host_api_pairs_per_s"), 1)
        # the headline value (a step of 8192 through batches of 256) and the
        # autotuned batch-256 pair rates of BF16 and FP16 against FP32 at batch 1
        out["ratio_bf16_b256_vs_fp32_b1"] = r(value / b1["small_batch_device_pairs_per_s"], 1)
        if "bf16_by_batch_positions_per_s" in x:
            out["ratio_bf16_b256_pair_rate_vs_fp32_b1"] = r(
                x["bf16_by_batch_positions_per_s"]["256"] / b1["small_batch_device_pairs_per_s"], 1)
        if "fp16_b256_pairs_per_s" in x:
            out["ratio_fp16_b256_pair_rate_vs_fp32_b1"] = r(
                x["fp16_b256_pairs_per_s"] / b1["small_batch_device_pairs_per_s"], 1)
        if "fp16_step_positions_per_s" in x:
            out["ratio_fp16_step_vs_fp32_b1"] = r(
                x["fp16_step_positions_per_s"] / b1["small_batch_device_pairs_per_s"], 1)
    f32 = x.get("fp32_roofline", {})
    if f32:
        pk = f32["fp32_sgemm_tflops"]
        out["fp32_peak_tflops"] = r(pk, 1)
        out["fp32_b1_frac_of_fp32_peak"] = r(f32["b1_tflops"] / pk, 3)
        out["fp32_b256_pairs_per_s"] = round(f32["b256_pairs_per_s"])
        out["fp32_b256_frac_of_fp32_peak"] = r(f32["b256_tflops"] / pk, 3)
    if "bf16_by_batch_positions_per_s" in x:
        out["bf16_pairs_per_s_by_batch"] = {k: round(v) for k, v in x["bf16_by_batch_positions_per_s"].items()}
    if "fp16_b256_pairs_per_s" in x:
        out["fp16_b256_pairs_per_s"] = round(x["fp16_b256_pairs_per_s"])
    if "fp16_step_positions_per_s" in x:
        out["fp16_step_positions_per_s"] = round(x["fp16_step_positions_per_s"])
    sp_runs = x.get("search_pattern", {})
    if sp_runs and "unavailable" not in sp_runs:
        out["search_pattern_leaf_evals_per_s"] = {k: round(v["leaf_evals_per_s"]) for k, v in sp_runs.items()
                                                  if "leaf_evals_per_s" in v}
    ens = x.get("ensemble_avg8", {})
    if ens:
        out["avg8_root_us_per_pair"] = r(ens["1"]["us_per_call_pair"], 1)
        out["avg8_b32_positions_per_s"] = round(ens["32"]["positions_per_s"])
    c2 = x.get("config2_vs_fp64", {})
    for prec, d in c2.items():
        if isinstance(d, dict) and "top1" in d:
            out[f"top1_vs_fp64_{prec}"] = r(d["top1"])
    if "positions" in c2:
        out["top1_positions"] = c2["positions"]
    sv = x.get("serving_config3", {})
    if "by_rate" in sv:
        out["serving"] = {k: [round(v["throughput_positions_per_s"]), r(v["latency_p50_ms"], 2),
                              r(v["latency_p99_ms"], 2)] for k, v in sv["by_rate"].items() if "latency_p50_ms" in v}
    d4 = x.get("distill", {})
    if "student_only_evals_per_s" in d4:
        out["distill"] = {"student_only_evals_per_s": round(d4["student_only_evals_per_s"]),
                          "full_pair_evals_per_s": round(d4["full_pair_evals_per_s"]),
                          "student_only_speedup": r(d4["student_only_speedup"], 2),
                          "gated_speedup_at_fallback": {k[9:]: r(d4[k]["speedup"], 2)
                                                        for k in ("fallback_0", "fallback_10pct", "fallback_100")
                                                        if k in d4}}
    return out


def serving_config3(lg, wp, wv, planes_p, planes_v, device, rates=(100_000.0, 200_000.0, 400_000.0, 800_000.0),
                    n_req=100_000, mean_batch=48, max_batch=512):
    """Uneven batching as the search produces it: n_req single-position
    requests with Poisson arrivals (at each of `rates` per second, seed 2),
    grouped into batches of Geometric(mean 48) sizes clipped to [1, 512]
    (seed 3).  Each batch is submitted to both nets (lg_submit) at its last
    arrival; the server merges what is queued, pads to a power-of-two bucket
    and replays that bucket's CUDA graph.  Latency = completion of both nets
    - arrival; throughput = requests / (last completion - first arrival).
    The client sleeps until each due time (the interpreter's thread switch
    interval is set to 20 us), so that the thread timing completions is not
    held off by a busy-waiting submitter."""
    import sys as _sys
    import tempfile
    import threading as th
    old_switch = _sys.getswitchinterval()
    _sys.setswitchinterval(2e-5)
    rng = np.random.default_rng(3)
    sizes, total = [], 0
    while total < n_req:
        b = int(min(max(rng.geometric(1.0 / mean_batch), 1), max_batch, n_req - total))
        sizes.append(b)
        total += b
    n_pos = planes_p.shape[0]
    res = {}
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
        for rate in rates:
            arrivals = np.cumsum(np.random.default_rng(2).exponential(1.0 / rate, n_req))
            done = {}
            stop = th.Event()
            served0 = ctx.stats()["batches"]

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
                wait = due - time.perf_counter()
                if wait > 2e-4:
                    time.sleep(wait - 1e-4)
                while time.perf_counter() < due:
                    pass
                ctx.submit(lg.LG_NET_POLICY, bp, op, tag=2 * k + 1)
                ctx.submit(lg.LG_NET_VALUE, bv, ov, tag=2 * k + 2)
            stop.set()
            pt.join(timeout=60)
            served = ctx.stats()["batches"] - served0
            if len(done) < 2 * len(batches):
                res[f"{int(rate)}"] = {"error": f"only {len(done)} of {2 * len(batches)} submissions completed"}
                continue
            lat = np.empty(n_req)
            last = 0.0
            for k, (_, _, _, _, st, sz) in enumerate(batches):
                comp = max(done[2 * k + 1], done[2 * k + 2])
                last = max(last, comp)
                lat[st:st + sz] = comp - (t0 + arrivals[st:st + sz])
            res[f"{int(rate)}"] = {
                "throughput_positions_per_s": n_req / (last - (t0 + arrivals[0])),
                "latency_p50_ms": float(np.percentile(lat, 50) * 1e3),
                "latency_p99_ms": float(np.percentile(lat, 99) * 1e3),
                "server_batches": int(served), "client_batches": len(sizes)}
    _sys.setswitchinterval(old_switch)
    return {"requests_per_rate": n_req, "mean_client_batch": float(np.mean(sizes)), "by_rate": res,
            "note": "policy + value per request; BF16; CUDA graph per power-of-two bucket (host copies inside "
                    "the graph); autotuned kernel choice per bucket"}


def config2_vs_fp64(lg, wp, wv, device, sp, subset=512):
    """Precision variants against the FP64 oracle over the 65,536 positions of
    the precision configuration: top-1 agreement against the oracle's FP64
    answers (tests/golden/config2_f64.npz, make_config2.py), value errors
    against its FP64 values, probability errors on `subset` positions
    computed live by the oracle, and the share of top-1 flips whose FP64
    top-1/top-2 gap is below twice the largest logit error seen on the
    subset."""
    import hashlib

    import torch
    from oracle import oracle as O
    d = np.load(os.path.join(ROOT, "tests", "golden", "config2_f64.npz"))
    n = int(d["n"])
    sq, tm, _ = O.config_boards(n, int(d["seed"]))
    if hashlib.sha256(sq.tobytes()).hexdigest()[:16] != str(d["squares_sha256"]):
        return {"error": "position generator does not reproduce the fixture"}
    dev = torch.device("cuda", device)
    d_sq, d_tm = torch.from_numpy(sq).to(dev), torch.from_numpy(tm).to(dev)
    planes = {}
    for which, key in ((0, "p"), (1, "v")):
        t = torch.empty((n, 24, 361), dtype=torch.uint8, device=dev)
        lg.gather_device(d_sq.data_ptr(), d_tm.data_ptr(), n, which, 24, t.data_ptr(), sp)
        planes[key] = t
    torch.cuda.synchronize()
    sub = np.arange(0, n, n // subset)
    P, V = O.make_net(O.CFG_POLICY), O.make_net(O.CFG_VALUE)
    O.enable_blas()
    l64 = O.forward_f64(P, wp, planes["p"][sub].cpu().numpy())
    O.disable_blas()
    p64 = O.softmax_f64(l64, 1.0)
    out = {"positions": n, "prob_error_subset": int(sub.size)}
    for prec in ("bf16", "fp16", "fp8w"):
        logits = torch.empty((n, 361), device=dev)
        probs = torch.empty((n, 361), device=dev)
        val = torch.empty(n, device=dev)
        with lg.Context(policy=lg.NetDesc.config1_policy(wp, prec), value=lg.NetDesc.config1_value(wv, prec),
                        device=device, max_batch=256) as c:
            c.policy_device(planes["p"].data_ptr(), n, probs.data_ptr(), 1.0, logits.data_ptr(), sp)
            c.value_device(planes["v"].data_ptr(), n, val.data_ptr(), sp)
            torch.cuda.synchronize()
        agree = logits.argmax(1).cpu().numpy() == d["top1"]
        verr = np.abs(val.cpu().numpy() - d["value"])
        emax = float(np.abs(logits[sub].cpu().numpy() - l64).max())
        perr = np.abs(probs[sub].cpu().numpy() - p64)
        gaps = d["gap"][~agree]
        out[prec] = {"top1": float(agree.mean()), "flips": int((~agree).sum()),
                     "flips_within_2x_logit_error": float((gaps < 2 * emax).mean()) if gaps.size else 1.0,
                     "logit_max_abs_err_subset": emax,
                     "prob_max_abs_err": float(perr.max()), "prob_mean_abs_err": float(perr.mean()),
                     "value_max_abs_err": float(verr.max()), "value_mean_abs_err": float(verr.mean())}
    ncap = d["top1_w_bf16"].size
    out["weight_rounding_only_top1"] = {"bf16": float((d["top1_w_bf16"] == d["top1"][:ncap]).mean()),
                                        "fp16": float((d["top1_w_fp16"] == d["top1"][:ncap]).mean()),
                                        "positions": int(ncap)}
    return out


def pair_rate_device(lg, wp, wv, prec, B, d_p, d_v, dev, sp, choice=None, reps=None, autotune=True):
    """Policy + value pairs per second, device-resident inputs, batch B."""
    import tempfile

    import torch
    with lg.Context(policy=lg.NetDesc.config1_policy(wp, prec),
                    value=lg.NetDesc.config1_value(wv, prec), device=dev.index, max_batch=B) as cb:
        if choice is not None:
            cb.set_tuning(B, *choice)
        elif autotune:
            cb.autotune(os.path.join(tempfile.gettempdir(), f"leela_gb300_tune_{prec}_{B}.json"))
        probs = torch.empty((B, 361), device=dev)
        val = torch.empty(B, device=dev)
        reps = reps or max(4, min(200, 4096 // B))
        for i in range(3):
            cb.policy_device(d_p.data_ptr(), B, probs.data_ptr(), 1.0, None, sp)
            cb.value_device(d_v.data_ptr(), B, val.data_ptr(), sp)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for i in range(reps):
            off = (i * B) % (8192 - B + 1)
            cb.policy_device(d_p[off].data_ptr(), B, probs.data_ptr(), 1.0, None, sp)
            cb.value_device(d_v[off].data_ptr(), B, val.data_ptr(), sp)
        e1.record()
        torch.cuda.synchronize()
        return B * reps / (e0.elapsed_time(e1) / 1e3), cb.tuning(B)


def ensemble_rates(lg, wp, wv, d_p, d_v, dev, sp):
    """The 8-symmetry ensemble (AVERAGE_ALL: lg_policy_avg8_device +
    lg_value_avg8_device, BF16, inputs resident): the root evaluation of a
    search (1 position = 8 rotated evaluations per net, the small-batch
    kernel) as microseconds per policy + value call pair, and 32 positions a
    call (256 evaluations per net, the persistent trunk) as positions/s."""
    import torch
    out = {}
    with lg.Context(policy=lg.NetDesc.config1_policy(wp, "bf16"),
                    value=lg.NetDesc.config1_value(wv, "bf16"), device=dev.index, max_batch=256) as c:
        for B, reps in ((1, 200), (32, 100)):
            probs = torch.empty((B, 361), device=dev)
            val = torch.empty(B, device=dev)

            def call(i):
                off = (i * B) % (8192 - B + 1)
                c.policy_avg8_device(d_p[off].data_ptr(), B, probs.data_ptr(), 1.0, sp)
                c.value_avg8_device(d_v[off].data_ptr(), B, val.data_ptr(), sp)
            for i in range(3):
                call(i)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            for i in range(reps):
                call(i)
            e1.record()
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1) / reps
            out[str(B)] = {"us_per_call_pair": ms * 1e3, "positions_per_s": B / (ms / 1e3)}
    return out


def search_pattern_rates(dev, runs=(("bf16", 64, "server"), ("bf16", 64, "direct"), ("bf16", 16, "server"),
                                        ("fp32", 64, "server"), ("fp32", 64, "direct")), seconds=3.0):
    """Leaf evaluations per second under the engine's request pattern
    (leela_gb300/integration/search_pattern.cpp, a C++ program over the C
    ABI): N threads, each with up to 2 asynchronous policy requests
    outstanding and one value evaluation per leaf, either through the
    batching server (merged across threads, as the backend does) or as
    blocking one-position calls.  Synthetic: no tree, board or host gather."""
    src = os.path.join(ROOT, "leela_gb300", "integration", "search_pattern.cpp")
    exe = os.path.join(ROOT, "leela_gb300", "integration", "_build", "search_pattern")
    os.makedirs(os.path.dirname(exe), exist_ok=True)
    r = subprocess.run(["g++", "-O2", "-std=c++17", "-pthread", src, "-I" + os.path.join(ROOT, "include"),
                        "-L" + os.path.join(ROOT, "leela_gb300"), "-lleela_gb300",
                        "-Wl,-rpath," + os.path.join(ROOT, "leela_gb300"), "-o", exe], capture_output=True, text=True)
    if r.returncode != 0:
        return {"unavailable": r.stderr[-300:]}
    out = {}
    env = dict(os.environ, CUDA_VISIBLE_DEVICES=os.environ.get("CUDA_VISIBLE_DEVICES", str(dev.index)))
    for prec, threads, mode in runs:
        p = subprocess.run([exe, str(threads), str(seconds), mode, prec, "64"], capture_output=True, text=True,
                           timeout=120, env=env)
        key = f"{prec}_{mode}_{threads}t"
        try:
            out[key] = json.loads(p.stdout.strip().splitlines()[-1])
        except (IndexError, ValueError):
            out[key] = {"error": (p.stderr or p.stdout)[-300:]}
    return out


def step_rate_device(lg, wp, wv, prec, d_p, d_v, dev, sp, steps=10):
    """The headline step (8192 positions through both nets in chained calls
    of 256, inputs resident) at another precision: positions/s."""
    import tempfile

    import torch
    with lg.Context(policy=lg.NetDesc.config1_policy(wp, prec),
                    value=lg.NetDesc.config1_value(wv, prec), device=dev.index, max_batch=BATCH) as c:
        c.autotune(os.path.join(tempfile.gettempdir(), f"leela_gb300_tune_{prec}_{BATCH}.json"))
        probs = torch.empty((POSITIONS, 361), device=dev)
        val = torch.empty(POSITIONS, device=dev)

        def step():
            c.policy_device(d_p.data_ptr(), POSITIONS, probs.data_ptr(), 1.0, None, sp)
            c.value_device(d_v.data_ptr(), POSITIONS, val.data_ptr(), sp)

        for _ in range(3):
            step()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(steps):
            step()
        e1.record()
        torch.cuda.synchronize()
        return POSITIONS * steps / (e0.elapsed_time(e1) / 1e3)


def fp32_peak_tflops(dev, n=8192, reps=8):
    """FP32 throughput of the GPU's FFMA pipes, the roofline of the plain FP32
    path: an n^3 FP32 GEMM through cuBLAS (torch.matmul with TF32 off, so
    FP32 FFMA, no tensor cores), best of reps, CUDA events."""
    import torch
    prev = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = False
    try:
        a = torch.randn(n, n, device=dev)
        b = torch.randn(n, n, device=dev)
        for _ in range(2):
            a @ b
        torch.cuda.synchronize()
        best = None
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            a @ b
            e1.record()
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1)
            best = ms if best is None else min(best, ms)
        del a, b
        return 2.0 * n ** 3 / (best / 1e3) / 1e12
    finally:
        torch.backends.cuda.matmul.allow_tf32 = prev


def secondary_measurements(lg, ctx, wp, wv, planes_p, planes_v, d_p, d_v, dev, sp, quick=False):
    """FP32 batch 1 (the ratio's denominator), BF16 at the other batch sizes,
    FP16 at batch 256, the precision variants against FP64 over 65,536
    positions, serving and distillation."""
    out = {}
    # FP32 plain path at batch 1 (policy + value per position): the
    # small-batch kernel (the default at batch 1) and the per-layer kernels
    r_lat, _ = pair_rate_device(lg, wp, wv, "fp32", 1, d_p, d_v, dev, sp, choice=(4, 0), reps=400)
    r_gen, _ = pair_rate_device(lg, wp, wv, "fp32", 1, d_p, d_v, dev, sp, choice=(0, 0), reps=200)
    with lg.Context(policy=lg.NetDesc.config1_policy(wp, "fp32"),
                    value=lg.NetDesc.config1_value(wv, "fp32"), device=dev.index, max_batch=1) as c32:
        for i in range(5):
            c32.policy(planes_p[i:i + 1])
            c32.value(planes_v[i:i + 1])
        n = 300
        t0 = time.perf_counter()
        for i in range(n):
            c32.policy(planes_p[i:i + 1])
            c32.value(planes_v[i:i + 1])
        host_rate = n / (time.perf_counter() - t0)
    # the FP32 path batched, and the FP32 peak both are measured against
    r_b256, _ = pair_rate_device(lg, wp, wv, "fp32", 256, d_p, d_v, dev, sp, reps=8)
    peak32 = fp32_peak_tflops(dev)
    out["fp32_roofline"] = {"fp32_sgemm_tflops": peak32, "b1_tflops": r_lat * FLOP_PAIR_PER_POS / 1e12,
                            "b256_pairs_per_s": r_b256, "b256_tflops": r_b256 * FLOP_PAIR_PER_POS / 1e12,
                            "note": "peak: cuBLAS FP32 GEMM 8192^3 with TF32 off (FFMA), best of 8"}
    out["fp32_batch1"] = {"small_batch_device_pairs_per_s": r_lat, "per_layer_device_pairs_per_s": r_gen,
                          "small_batch_host_api_pairs_per_s": host_rate,
                          "note": "policy + value per position, batch 1; device = inputs resident, CUDA "
                                  "events; host API = lg_policy + lg_value blocking calls"}
    by_batch, choices = {}, {}
    for b in (1, 8, 64, 256):
        by_batch[str(b)], choices[str(b)] = pair_rate_device(lg, wp, wv, "bf16", b, d_p, d_v, dev, sp)
    out["bf16_by_batch_positions_per_s"] = by_batch
    out["bf16_kernel_choice_by_batch"] = choices
    out["fp16_b256_pairs_per_s"], _ = pair_rate_device(lg, wp, wv, "fp16", 256, d_p, d_v, dev, sp)
    # the headline step itself in FP16 (the variant at >= 99% top-1 vs FP64)
    out["fp16_step_positions_per_s"] = step_rate_device(lg, wp, wv, "fp16", d_p, d_v, dev, sp)
    out["ensemble_avg8"] = ensemble_rates(lg, wp, wv, d_p, d_v, dev, sp)
    out["ratio_bf16_batched_vs_fp32_batch1"] = by_batch["256"] / r_lat
    out["config2_vs_fp64"] = config2_vs_fp64(lg, wp, wv, dev.index, sp)
    if not quick:
        out["serving_config3"] = serving_config3(lg, wp, wv, planes_p, planes_v, dev.index)
        out["distill"] = distill_rates(wp, wv, planes_p, planes_v, dev.index)
        out["search_pattern"] = search_pattern_rates(dev)
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
    _, _, hbm, _ = read_peaks()
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


def latency_run(B, reps):
    """The small-batch kernel alone at batch B: `reps` policy + value calls
    of the FP32 and the BF16 benchmark nets, inputs resident, one JSON line
    of device microseconds per net call."""
    import torch

    import leela_gb300 as lg
    from leela_gb300 import build as Bld
    Bld.build()
    dev = torch.device("cuda", 0)
    planes_p, planes_v = load_positions()
    _, _, wp, wv = make_weights()
    d_p = torch.from_numpy(planes_p[:64]).to(dev)
    d_v = torch.from_numpy(planes_v[:64]).to(dev)
    sp = torch.cuda.current_stream(dev).cuda_stream
    out = {"latency_run": True, "batch": B}
    for prec in ("fp32", "bf16"):
        with lg.Context(policy=lg.NetDesc.config1_policy(wp, prec), value=lg.NetDesc.config1_value(wv, prec),
                        max_batch=max(B, 1)) as c:
            c.set_tuning(B, 4, 0)
            probs = torch.empty((B, 361), device=dev)
            val = torch.empty(B, device=dev)
            for _ in range(3):
                c.policy_device(d_p.data_ptr(), B, probs.data_ptr(), 1.0, None, sp)
                c.value_device(d_v.data_ptr(), B, val.data_ptr(), sp)
            torch.cuda.synchronize()
            c.profile(True)
            for i in range(reps):
                c.policy_device(d_p[i % 32].data_ptr(), B, probs.data_ptr(), 1.0, None, sp)
                c.value_device(d_v[i % 32].data_ptr(), B, val.data_ptr(), sp)
            torch.cuda.synchronize()
            n, ms = c.profile_read(lg.PROF_LAT)
            c.profile(False)
            out[prec] = {"launches": n, "us_per_launch": ms * 1e3 / max(n, 1)}
    print(json.dumps(out), flush=True)


def student_run(reps):
    """The fused student kernel (and its finish kernels) alone on the 8192
    benchmark inputs: `reps` calls, one JSON line of evaluations per second."""
    import torch

    from leela_gb300 import build as Bld
    from leela_gb300 import distill
    Bld.build()
    dev = torch.device("cuda", 0)
    planes_p, _ = load_positions()
    N = planes_p.shape[0]
    d_p = torch.from_numpy(planes_p).to(dev)
    st = distill.Student(max_batch=8)
    st.init_he(0)
    params = st.get_params()
    st.close()
    s = torch.cuda.current_stream(dev).cuda_stream
    with distill.FastNet(params, max_batch=N) as fast:
        probs = torch.empty((N, 361), device=dev)
        val = torch.empty(N, device=dev)
        for _ in range(3):
            fast.device(d_p.data_ptr(), N, probs.data_ptr(), val.data_ptr(), 1.0, None, None, s)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            fast.device(d_p.data_ptr(), N, probs.data_ptr(), val.data_ptr(), 1.0, None, None, s)
        e1.record()
        fast.status(s)
        ms = e0.elapsed_time(e1) / max(reps, 1)
    print(json.dumps({"student_run": True, "positions": N, "ms_per_call": ms, "evals_per_s": N / (ms / 1e3)}),
          flush=True)


def distill_rates(wp, wv, planes_p, planes_v, device, N=8192):
    """Leaf evaluations per second of the learned fast path's pieces on the
    8192 benchmark inputs (resident on the GPU): the full BF16 pair
    (autotuned, batches of up to 1024, its fastest serving size here), the
    student alone (fused kernel, one call of 8192), and the gated path at
    fallback rates of 0%, ~10% and 100% (thresholds at entropy percentiles
    of this student).  The speed does not depend on what the student
    learned -- the fallback rate does (the trained students: bench.py
    --distill-run)."""
    import tempfile

    import torch

    import leela_gb300 as lg
    from leela_gb300 import distill
    dev = torch.device("cuda", device)
    s = torch.cuda.current_stream(dev).cuda_stream
    d_p = torch.from_numpy(planes_p[:N]).to(dev)
    d_v = torch.from_numpy(planes_v[:N]).to(dev)
    st = distill.Student(max_batch=8, device=device)
    st.init_he(0)
    params = st.get_params()
    st.close()

    def timed(fn, reps=5):
        for _ in range(2):
            fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            fn()
        e1.record()
        torch.cuda.synchronize()
        return N / (e0.elapsed_time(e1) / reps / 1e3)

    out = {}
    with lg.Context(policy=lg.NetDesc.config1_policy(wp, "bf16"), value=lg.NetDesc.config1_value(wv, "bf16"),
                    device=device, max_batch=1024) as cf, distill.FastNet(params, max_batch=N, device=device) as fast:
        cf.autotune(os.path.join(tempfile.gettempdir(), "leela_gb300_tune_1024.json"))
        fp = torch.empty((N, 361), device=dev)
        fv = torch.empty(N, device=dev)
        se = torch.empty(N, device=dev)

        def full():
            cf.policy_device(d_p.data_ptr(), N, fp.data_ptr(), 1.0, None, s)
            cf.value_device(d_v.data_ptr(), N, fv.data_ptr(), s)

        def student():
            fast.device(d_p.data_ptr(), N, fp.data_ptr(), fv.data_ptr(), 1.0, None, se.data_ptr(), s)

        out["full_pair_evals_per_s"] = timed(full)
        out["student_only_evals_per_s"] = timed(student)
        fast.status(s)
        ent = se.cpu().numpy()
        out["student_only_speedup"] = out["student_only_evals_per_s"] / out["full_pair_evals_per_s"]
        for name, thr in (("fallback_0", 1e9), ("fallback_10pct", float(np.percentile(ent, 90))),
                          ("fallback_100", -1.0)):
            g = distill.GatedEvaluator(fast, cf, thr)
            buf = [None]

            def gated():
                buf[0] = g.evaluate(d_p, d_v, s, buf[0])

            rate = timed(gated)
            out[name] = {"fallback_rate": int(buf[0][3].item()) / N, "evals_per_s": rate,
                         "speedup": rate / out["full_pair_evals_per_s"]}
        fast.status(s)
    return out


def distill_run():
    """The learned fast path at its configuration's scale (one JSON line):
    1,048,576 positions from the seeded generator, value labels from the
    reference's own Playout::mc_owner(64) (tests/golden/config4_mcowner.npz,
    made by tests/golden/make_config4.py), policy labels from the full FP32
    net, the student trained by this library's kernels, judged on 65,536
    held-out positions by the full BF16 nets (leela_gb300.distill.run_config4)."""
    import hashlib

    import torch

    from leela_gb300 import build as B
    from leela_gb300 import distill
    from oracle import oracle as O
    B.build()
    d = np.load(os.path.join(ROOT, "tests", "golden", "config4_mcowner.npz"))
    n, seed = int(d["n"]), int(d["seed"])
    t0 = time.perf_counter()
    sq, tm, _ = O.config_boards(n, seed)
    gen_s = time.perf_counter() - t0
    if hashlib.sha256(sq.tobytes()).hexdigest()[:16] != str(d["squares_sha256"]):
        print(json.dumps({"distill_run": True, "error": "the position generator does not reproduce the labels' boards"}))
        return
    _, _, wp, wv = make_weights()
    res = distill.run_config4(sq, tm, d["winrate_x128"].astype(np.float32) / 128.0, wp, wv, 0)
    res["board_generation_seconds"] = gen_s
    print(json.dumps({"distill_run": True, **res}), flush=True)


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
    ap.add_argument("--quick", action="store_true",
                    help="skip the serving replay and the distillation experiment")
    ap.add_argument("--detail", default=None, help="write every secondary measurement to this JSON file")
    ap.add_argument("--gather-run", action="store_true",
                    help="only the gather timing: 8192 boards, 24 and 32 planes, both sets (for ncu)")
    ap.add_argument("--latency-run", type=int, default=0, metavar="B",
                    help="only the small-batch kernel at batch B, --steps calls per net and precision (for ncu)")
    ap.add_argument("--student-run", action="store_true",
                    help="only the fused student kernel on the 8192 benchmark inputs, --steps calls (for ncu)")
    ap.add_argument("--distill-run", action="store_true",
                    help="the learned fast path at its configuration's scale (1M positions; minutes)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.gather_run:
        gather_run(reps=5)
        return
    if args.latency_run:
        latency_run(args.latency_run, reps=args.steps)
        return
    if args.student_run:
        student_run(reps=args.steps)
        return
    if args.distill_run:
        distill_run()
        return
    world, rank, local = dist_setup()
    if args.impl == "reference":
        run_reference(args, world, rank)
    else:
        run_ours(args, world, rank, local)


if __name__ == "__main__":
    main()
