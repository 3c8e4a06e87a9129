"""Distilled fast path: a small student net trained on the GPU by this
library's own forward/backward kernels (lg_student_*), served in BF16, that
answers leaves first and hands a position to the full nets when the
student's policy entropy is above a threshold.

The reference has no learned fast path; its search evaluates every leaf
with the full net (UCTNode.cpp:74-121, 316-344).  Labels are the full
policy net's softmax and Monte-Carlo win rates (Playout::mc_owner,
Playout.cpp:174-217, mapped to [-1, 1]); the full net is also the judge of
the student's top-1 agreement.
"""
from __future__ import annotations

import ctypes
import math
import time

import numpy as np

from . import (LG_ACT_RELU, LG_NET_POLICY, Context, LeelaGPUError, NetDesc, _check,
               library)

STUDENT_SHAPE = dict(c_in=24, width=64, n3x3=5, fc_hidden=64)


def _bind():
    L = library()
    if getattr(L, "_student_bound", False):
        return L
    vp, i32, f32 = ctypes.c_void_p, ctypes.c_int, ctypes.c_float
    P = ctypes.POINTER
    L.lg_student_create.argtypes = [i32, i32, i32, i32, i32, i32, P(vp)]
    L.lg_student_destroy.argtypes = [vp]
    L.lg_student_destroy.restype = None
    L.lg_student_param_count.argtypes = [vp]
    L.lg_student_param_count.restype = ctypes.c_size_t
    L.lg_student_set_params.argtypes = [vp, vp, ctypes.c_size_t]
    L.lg_student_get_params.argtypes = [vp, vp, ctypes.c_size_t]
    L.lg_student_train_step.argtypes = [vp, vp, i32, vp, vp, f32, f32, vp, vp]
    L.lg_student_grads.argtypes = [vp, vp, i32, vp, vp, f32, vp, vp]
    L.lg_student_forward.argtypes = [vp, vp, i32, vp, vp, vp]
    L.lg_fast_param_count.argtypes = [i32, i32, i32]
    L.lg_fast_param_count.restype = ctypes.c_size_t
    L.lg_fast_create.argtypes = [i32, i32, i32, i32, i32, vp, P(vp)]
    L.lg_fast_set_weights.argtypes = [vp, vp]
    L.lg_fast_destroy.argtypes = [vp]
    L.lg_fast_destroy.restype = None
    L.lg_fast_device.argtypes = [vp, vp, i32, f32, vp, vp, vp, vp, vp]
    L.lg_fast_status.argtypes = [vp, vp]
    L.lg_gated_device.argtypes = [vp, vp, vp, vp, i32, f32, f32, vp, vp, vp, vp, vp]
    L._student_bound = True
    return L


class Student:
    """The student net on one GPU (FP32 parameters, Adam state)."""

    def __init__(self, c_in=24, width=64, n3x3=5, fc_hidden=64, max_batch=256, device=0):
        L = _bind()
        self.shape = dict(c_in=c_in, width=width, n3x3=n3x3, fc_hidden=fc_hidden)
        self._h = ctypes.c_void_p()
        _check(L.lg_student_create(device, c_in, width, n3x3, fc_hidden, max_batch,
                                   ctypes.byref(self._h)))
        self.n = int(L.lg_student_param_count(self._h))

    def close(self):
        if self._h:
            library().lg_student_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- parameters (flat host layout, see include/leela_gpu.h)
    def init_he(self, seed: int = 0):
        """He-normal weights N(0, 2/fan_in), zero biases."""
        rng = np.random.default_rng(seed)
        s = self.shape
        parts = []
        for l in range(s["n3x3"] + 1):
            k = 5 if l == 0 else 3
            cin = s["c_in"] if l == 0 else s["width"]
            fan = cin * k * k
            parts += [rng.normal(0, math.sqrt(2 / fan), s["width"] * fan), np.zeros(s["width"])]
        W = s["width"]
        H = s["fc_hidden"]
        parts += [rng.normal(0, math.sqrt(2 / W), W), np.zeros(1),
                  rng.normal(0, math.sqrt(2 / W), W), np.zeros(1),
                  rng.normal(0, math.sqrt(2 / 361), H * 361), np.zeros(H),
                  rng.normal(0, math.sqrt(2 / H), H), np.zeros(1)]
        self.set_params(np.concatenate(parts).astype(np.float32))

    def set_params(self, p: np.ndarray):
        p = np.ascontiguousarray(p, dtype=np.float32)
        _check(library().lg_student_set_params(self._h, p.ctypes.data, p.size))

    def get_params(self) -> np.ndarray:
        p = np.empty(self.n, dtype=np.float32)
        _check(library().lg_student_get_params(self._h, p.ctypes.data, p.size))
        return p

    def _split(self, p):
        s = self.shape
        W = s["width"]
        trunk = 0
        for l in range(s["n3x3"] + 1):
            k = 5 if l == 0 else 3
            cin = s["c_in"] if l == 0 else W
            trunk += W * cin * k * k + W
        pol = p[:trunk + W + 1]
        val = np.concatenate([p[:trunk], p[trunk + W + 1:]])
        return pol, val

    def policy_desc(self, precision="bf16", params=None) -> NetDesc:
        s = self.shape
        pol, _ = self._split(self.get_params() if params is None else params)
        return NetDesc(pol, s["c_in"], s["width"], s["width"], s["n3x3"], 1, LG_ACT_RELU, 0, 0,
                       precision=precision)

    def value_desc(self, precision="bf16", params=None) -> NetDesc:
        s = self.shape
        _, val = self._split(self.get_params() if params is None else params)
        return NetDesc(val, s["c_in"], s["width"], s["width"], s["n3x3"], 1, LG_ACT_RELU, 0, 1,
                       s["fc_hidden"], 0, precision=precision)

    # ---- device-pointer calls
    def train_step(self, planes_ptr, B, target_ptr, value_ptr, lr, value_weight=1.0,
                   stream=None, want_loss=False):
        loss = (ctypes.c_float * 2)() if want_loss else None
        _check(library().lg_student_train_step(self._h, planes_ptr, B, target_ptr, value_ptr, lr,
                                               value_weight, loss, stream))
        return (loss[0], loss[1]) if want_loss else None

    def grads(self, planes_ptr, B, target_ptr, value_ptr, value_weight=1.0):
        g = np.empty(self.n, dtype=np.float32)
        loss = (ctypes.c_float * 2)()
        _check(library().lg_student_grads(self._h, planes_ptr, B, target_ptr, value_ptr,
                                          value_weight, g.ctypes.data, loss))
        return (loss[0], loss[1]), g

    def forward(self, planes_ptr, B, probs_ptr, value_ptr, stream=None):
        _check(library().lg_student_forward(self._h, planes_ptr, B, probs_ptr, value_ptr, stream))


def train(student: Student, planes, target_probs, target_value, steps: int, batch: int = 256,
          lr: float = 1e-3, value_weight: float = 1.0, seed: int = 0, log_every: int = 100,
          time_budget_s: float | None = None):
    """Adam on random minibatches of device tensors planes [N][c_in][361]
    uint8, target_probs [N][361], target_value [N]; returns the loss log."""
    import torch
    g = torch.Generator(device="cpu").manual_seed(seed)
    N = planes.shape[0]
    log = []
    t0 = time.perf_counter()
    stream = torch.cuda.current_stream().cuda_stream
    for it in range(steps):
        idx = torch.randint(0, N, (batch,), generator=g).to(planes.device)
        p = planes.index_select(0, idx).contiguous()
        t = target_probs.index_select(0, idx).contiguous()
        v = target_value.index_select(0, idx).contiguous()
        want = (it % log_every == 0) or it == steps - 1
        loss = student.train_step(p.data_ptr(), batch, t.data_ptr(), v.data_ptr(), lr,
                                  value_weight, stream, want_loss=want)
        if want:
            log.append((it, float(loss[0]), float(loss[1])))
        if time_budget_s and time.perf_counter() - t0 > time_budget_s:
            log.append((it, float("nan"), float("nan")))
            break
    torch.cuda.synchronize()
    return log


def entropy(probs):
    """Shannon entropy in nats of each row of a [B][361] tensor."""
    import torch
    p = probs.clamp_min(1e-30)
    return -(probs * torch.log(p)).sum(dim=1)


class FastNet:
    """The student served by the fused BF16 kernel (lg_fast_*): trunk and
    both heads in one launch, then softmax (+ entropy) and the value FC.
    `params` in the Student flat layout (width 64)."""

    def __init__(self, params, c_in=24, n3x3=5, fc_hidden=64, max_batch=8192, device=0):
        L = _bind()
        self.shape = dict(c_in=c_in, n3x3=n3x3, fc_hidden=fc_hidden)
        self.max_batch = max_batch
        n = int(L.lg_fast_param_count(c_in, n3x3, fc_hidden))
        p = np.ascontiguousarray(params, dtype=np.float32)
        if p.size != n:
            raise ValueError(f"student weights have {p.size} floats, the shape needs {n}")
        self._h = ctypes.c_void_p()
        _check(L.lg_fast_create(device, c_in, n3x3, fc_hidden, max_batch, p.ctypes.data, ctypes.byref(self._h)))

    def set_weights(self, params):
        p = np.ascontiguousarray(params, dtype=np.float32)
        _check(library().lg_fast_set_weights(self._h, p.ctypes.data))

    def device(self, planes_ptr, B, probs_ptr, value_ptr, temperature=1.0, logits_ptr=None, entropy_ptr=None,
               stream=None):
        _check(library().lg_fast_device(self._h, planes_ptr, B, temperature, probs_ptr, logits_ptr, value_ptr,
                                        entropy_ptr, stream))

    def status(self, stream=None):
        _check(library().lg_fast_status(self._h, stream))

    def close(self):
        if self._h:
            library().lg_fast_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class GatedEvaluator:
    """The learned fast path (lg_gated_device): the student answers every
    position, positions whose student policy entropy exceeds `threshold`
    nats are handed to the full nets on the device -- compaction, the full
    nets' batch sizes and the write-back all stay on the GPU, with no host
    synchronisation."""

    def __init__(self, fast: FastNet, full_ctx: Context, threshold: float = 2.5):
        self.s = fast
        self.f = full_ctx
        self.threshold = threshold

    def evaluate(self, planes_p, planes_v, stream=None, out=None, temperature=1.0):
        """planes_p / planes_v: device uint8 [B][24][361] (policy / value
        planes of the same positions).  Returns device tensors (probs [B][361],
        values [B], fallback [B] uint8, count [1] int32); `out`, a tuple of
        those four, is reused when given."""
        import torch
        B = planes_p.shape[0]
        dev = planes_p.device
        if out is None:
            out = (torch.empty((B, 361), device=dev), torch.empty(B, device=dev),
                   torch.empty(B, dtype=torch.uint8, device=dev), torch.empty(1, dtype=torch.int32, device=dev))
        probs, values, fb, cnt = out
        s = stream if stream is not None else torch.cuda.current_stream().cuda_stream
        _check(_bind().lg_gated_device(self.s._h, self.f._h, planes_p.data_ptr(), planes_v.data_ptr(), B,
                                       temperature, self.threshold, probs.data_ptr(), values.data_ptr(),
                                       fb.data_ptr(), cnt.data_ptr(), s))
        return probs, values, fb, cnt


def calibrate_threshold(entropy_np, agree_np, target=0.97):
    """Largest entropy threshold such that answering every position with
    entropy <= threshold from the student, and the rest from the full net
    (which agrees with itself), keeps overall top-1 agreement >= target.
    Returns (threshold, student share, overall agreement)."""
    order = np.argsort(entropy_np)
    n = len(order)
    wrong = np.cumsum(~agree_np[order])
    ok = np.nonzero(1.0 - wrong / n >= target)[0]
    if len(ok) == 0:
        return float("-inf"), 0.0, 1.0
    k = int(ok[-1]) + 1
    thr = float(entropy_np[order[k - 1]])
    return thr, k / n, 1.0 - wrong[k - 1] / n


def run_config4(squares, to_move, mc_winrate, wp, wv, device=0, holdout=65536, train_steps=6000,
                batch=512, lr=1e-3, teacher_temperatures=(1.0, 0.05), time_budget_s=240.0,
                eval_batch=8192, seed=0):
    """The learned fast path at the scale of its configuration.

    Positions: squares [N][361] / to_move [N] (host), planes 0..23 of both
    sets gathered on the GPU.  Labels: the full FP32 policy net's softmax at
    each teacher temperature, and 2 * mc_winrate - 1 (Playout::mc_owner(64)
    win rates of the side to move).  The student (5x5 24->64, 5x 3x3
    64->64, two heads) is trained by this library's FP32 kernels on the
    first N - holdout positions and judged on the last `holdout` by the
    full BF16 nets, as served.  Reports, per teacher temperature: training
    cost, the student's top-1 agreement with the full net, the fallback rate
    and agreement of the gate at 2.5 nats and at the threshold calibrated
    for 97% agreement, and leaf evaluations per second of the full pair,
    the student alone and the gated path (inputs resident on the GPU,
    batches of `eval_batch`)."""
    import torch
    from . import gather_device
    dev = torch.device("cuda", device)
    N = squares.shape[0]
    stream = torch.cuda.current_stream(dev).cuda_stream
    d_sq = torch.from_numpy(np.ascontiguousarray(squares)).to(dev)
    d_tm = torch.from_numpy(np.ascontiguousarray(to_move)).to(dev)
    d_pp = torch.empty((N, 24, 361), dtype=torch.uint8, device=dev)
    d_pv = torch.empty((N, 24, 361), dtype=torch.uint8, device=dev)
    gather_device(d_sq.data_ptr(), d_tm.data_ptr(), N, 0, 24, d_pp.data_ptr(), stream)
    gather_device(d_sq.data_ptr(), d_tm.data_ptr(), N, 1, 24, d_pv.data_ptr(), stream)
    del d_sq, d_tm
    ntr = N - holdout
    vt = torch.from_numpy((2.0 * mc_winrate - 1.0).astype(np.float32)).to(dev)
    t0 = time.perf_counter()
    logits = torch.empty((N, 361), device=dev)
    with Context(policy=NetDesc.config1_policy(wp, "fp32"), device=device, max_batch=1024) as t32:
        probs = torch.empty((min(N, 65536), 361), device=dev)
        for b0 in range(0, N, 65536):
            nb = min(65536, N - b0)
            t32.policy_device(d_pp[b0].data_ptr(), nb, probs.data_ptr(), 1.0, logits[b0].data_ptr(), stream)
        del probs
    torch.cuda.synchronize()
    label_s = time.perf_counter() - t0
    te_p, te_v = d_pp[ntr:], d_pv[ntr:]
    T = (holdout // eval_batch) * eval_batch
    te_p, te_v = te_p[:T], te_v[:T]
    out = {"positions": int(N), "train_positions": int(ntr), "holdout_positions": int(T),
           "teacher_label_seconds": label_s, "value_labels": "2 * mc_owner(64) - 1 (reference Playout.cpp)"}
    with Context(policy=NetDesc.config1_policy(wp, "bf16"), value=NetDesc.config1_value(wv, "bf16"),
                 device=device, max_batch=1024) as cf:
        for b in (256, 1024):
            cf.set_tuning(b, 3, 0)
        fp = torch.empty((T, 361), device=dev)
        fv = torch.empty(T, device=dev)
        cf.policy_device(te_p.data_ptr(), T, fp.data_ptr(), 1.0, None, stream)
        cf.value_device(te_v.data_ptr(), T, fv.data_ptr(), stream)
        full_top1 = fp.argmax(1)

        def timed(fn, reps=3):
            fn()
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            for _ in range(reps):
                fn()
            e1.record()
            torch.cuda.synchronize()
            return reps * T / (e0.elapsed_time(e1) / 1e3)

        def full_pair():
            cf.policy_device(te_p.data_ptr(), T, fp.data_ptr(), 1.0, None, stream)
            cf.value_device(te_v.data_ptr(), T, fv.data_ptr(), stream)

        out["full_pair_evals_per_s"] = timed(full_pair)
        for tt in teacher_temperatures:
            target = torch.softmax(logits[:ntr] / tt, dim=1)
            st = Student(max_batch=batch, device=device)
            st.init_he(seed)
            t0 = time.perf_counter()
            log = train(st, d_pp[:ntr], target, vt[:ntr], train_steps, batch=batch, lr=lr, seed=seed,
                        log_every=500, time_budget_s=time_budget_s)
            train_s = time.perf_counter() - t0
            del target
            params = st.get_params()
            te_t = torch.softmax(logits[ntr:ntr + T] / tt, dim=1)
            kl, mse = heldout_loss(st, te_p, te_t, vt[ntr:ntr + T], batch=batch)
            st.close()
            del te_t
            res = {"train_steps": int(log[-1][0]) + 1, "batch": batch, "train_seconds": train_s,
                   "samples_per_s": (int(log[-1][0]) + 1) * batch / train_s,
                   "heldout_policy_kl": kl, "heldout_value_mse": mse,
                   "loss_first_last": [log[0], log[-1]]}
            with FastNet(params, max_batch=eval_batch, device=device) as fast:
                sp = torch.empty((T, 361), device=dev)
                sv = torch.empty(T, device=dev)
                se = torch.empty(T, device=dev)
                for b0 in range(0, T, eval_batch):
                    fast.device(te_p[b0].data_ptr(), eval_batch, sp[b0].data_ptr(), sv[b0:].data_ptr(), 1.0,
                                None, se[b0:].data_ptr(), stream)
                fast.status(stream)
                ent = se.cpu().numpy()
                agree = (sp.argmax(1) == full_top1).cpu().numpy()
                res["student_top1_agreement_with_full_net"] = float(agree.mean())
                res["student_value_mae_vs_full_net"] = float((sv - fv).abs().mean().item())
                res["student_entropy_nats"] = {"p10": float(np.percentile(ent, 10)),
                                               "median": float(np.median(ent)),
                                               "p90": float(np.percentile(ent, 90))}
                thr_cal, share_cal, agree_cal = calibrate_threshold(ent, agree)

                def student_only():
                    for b0 in range(0, T, eval_batch):
                        fast.device(te_p[b0].data_ptr(), eval_batch, sp[b0].data_ptr(), sv[b0:].data_ptr(), 1.0,
                                    None, se[b0:].data_ptr(), stream)

                res["student_only_evals_per_s"] = timed(student_only)
                for name, thr in (("gate_2.5", 2.5), ("gate_calibrated_97", thr_cal)):
                    if not np.isfinite(thr):
                        res[name] = {"threshold_nats": None, "note": "no threshold keeps 97% agreement"}
                        continue
                    g = GatedEvaluator(fast, cf, thr)
                    bufs = [None]
                    counts = torch.zeros(T // eval_batch, dtype=torch.int32, device=dev)

                    def gated():
                        for i, b0 in enumerate(range(0, T, eval_batch)):
                            bufs[0] = g.evaluate(te_p[b0:b0 + eval_batch], te_v[b0:b0 + eval_batch], stream,
                                                 bufs[0])
                            counts[i:i + 1].copy_(bufs[0][3])

                    rate = timed(gated)
                    fb = float(counts.sum().item()) / T
                    mask = ent > thr
                    res[name] = {"threshold_nats": float(thr), "fallback_rate": fb,
                                 "fallback_rate_host_check": float(mask.mean()),
                                 "top1_agreement": float(1.0 - (~agree & ~mask).mean()),
                                 "leaf_evals_per_s": rate,
                                 "speedup_vs_full_pair": rate / out["full_pair_evals_per_s"]}
                res["student_only_speedup_vs_full_pair"] = res["student_only_evals_per_s"] / out[
                    "full_pair_evals_per_s"]
            out[f"teacher_T{tt:g}"] = res
            torch.cuda.synchronize()
    return out


def _policy_len(shape):
    W = shape["width"]
    n = 0
    for l in range(shape["n3x3"] + 1):
        k = 5 if l == 0 else 3
        cin = shape["c_in"] if l == 0 else W
        n += W * cin * k * k + W
    return n + W + 1


def _value_part(params, shape):
    trunk = _policy_len(shape) - shape["width"] - 1
    return np.concatenate([params[:trunk], params[trunk + shape["width"] + 1:]])


def heldout_loss(student: Student, planes, target_probs, target_value, value_weight=1.0,
                 batch=256):
    """Mean policy KL and value MSE of `student` on device tensors (no update)."""
    N = planes.shape[0]
    kl = mse = 0.0
    n = 0
    for b0 in range(0, N, batch):
        nb = min(batch, N - b0)
        (a, b), _ = student.grads(planes[b0].data_ptr(), nb, target_probs[b0].data_ptr(),
                                  target_value[b0:].data_ptr(), value_weight)
        kl += a * nb
        mse += b * nb
        n += nb
    return kl / n, mse / n
