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


class GatedEvaluator:
    """Student first (BF16, both heads), full nets for the positions whose
    student policy entropy exceeds `threshold` nats."""

    def __init__(self, student_ctx: Context, full_ctx: Context, threshold: float = 2.5):
        self.s = student_ctx
        self.f = full_ctx
        self.threshold = threshold

    def evaluate(self, planes_p, planes_v, stream=None):
        """planes_p / planes_v: device uint8 [B][24][361] (policy / value
        planes of the same positions).  Returns (probs, values, fallback mask)."""
        import torch
        B = planes_p.shape[0]
        dev = planes_p.device
        sp = torch.empty((B, 361), device=dev)
        sv = torch.empty(B, device=dev)
        s = stream if stream is not None else torch.cuda.current_stream().cuda_stream
        self.s.policy_device(planes_p.data_ptr(), B, sp.data_ptr(), 1.0, None, s)
        self.s.value_device(planes_p.data_ptr(), B, sv.data_ptr(), s)
        mask = entropy(sp) > self.threshold
        idx = torch.nonzero(mask).flatten()
        k = int(idx.numel())
        if k:
            fp = planes_p.index_select(0, idx).contiguous()
            fv = planes_v.index_select(0, idx).contiguous()
            op = torch.empty((k, 361), device=dev)
            ov = torch.empty(k, device=dev)
            self.f.policy_device(fp.data_ptr(), k, op.data_ptr(), 1.0, None, s)
            self.f.value_device(fv.data_ptr(), k, ov.data_ptr(), s)
            sp.index_copy_(0, idx, op)
            sv.index_copy_(0, idx, ov)
        return sp, sv, mask


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


def run_config4(planes_p, planes_v, position_index, mc_winrate, wp, wv, device=0,
                train_positions=896, steps=3000, time_budget_s=30.0, teacher_temperature=1.0,
                threshold=2.5, batch=256, seed=0):
    """Distillation experiment (a distilled 64-wide student with an entropy
    gate, at the scale of the fixture positions): labels = the full FP32 policy net's softmax at
    teacher_temperature and 2*mc_owner-1 values; train on positions
    < train_positions (all symmetries), evaluate on the rest.  Reports the
    student's top-1 agreement with the full BF16 net, the fallback rate at
    `threshold` nats and at a threshold calibrated for >= 97% agreement, and
    leaf evaluations per second of the gated evaluator against the full net
    alone (inputs resident on the GPU, batches of `batch`)."""
    import torch
    dev = torch.device("cuda", device)
    N = planes_p.shape[0]
    d_pp = torch.from_numpy(np.ascontiguousarray(planes_p)).to(dev)
    d_pv = torch.from_numpy(np.ascontiguousarray(planes_v)).to(dev)
    stream = torch.cuda.current_stream(dev).cuda_stream
    with Context(policy=NetDesc.config1_policy(wp, "fp32"), device=device, max_batch=256) as t32:
        logits = torch.empty((N, 361), device=dev)
        probs = torch.empty((N, 361), device=dev)
        t32.policy_device(d_pp.data_ptr(), N, probs.data_ptr(), 1.0, logits.data_ptr(), stream)
    target = torch.softmax(logits / teacher_temperature, dim=1).contiguous()
    vt = torch.from_numpy((2.0 * mc_winrate[position_index] - 1.0).astype(np.float32)).to(dev)
    train_idx = torch.from_numpy(np.nonzero(position_index < train_positions)[0]).to(dev)
    test_idx = torch.from_numpy(np.nonzero(position_index >= train_positions)[0]).to(dev)
    st = Student(max_batch=batch, device=device)
    st.init_he(seed)
    t0 = time.perf_counter()
    log = train(st, d_pp.index_select(0, train_idx).contiguous(),
                target.index_select(0, train_idx).contiguous(),
                vt.index_select(0, train_idx).contiguous(), steps, batch=batch, lr=1e-3,
                seed=seed, log_every=250, time_budget_s=time_budget_s)
    train_s = time.perf_counter() - t0
    params = st.get_params()
    st.close()
    tp = d_pp.index_select(0, test_idx).contiguous()
    tv = d_pv.index_select(0, test_idx).contiguous()
    T = tp.shape[0]
    T = (T // batch) * batch
    tp, tv = tp[:T], tv[:T]
    shape = STUDENT_SHAPE
    sdesc = dict(policy=NetDesc(params[:_policy_len(shape)], shape["c_in"], shape["width"],
                                shape["width"], shape["n3x3"], 1, LG_ACT_RELU, 0, 0,
                                precision="bf16"),
                 value=NetDesc(_value_part(params, shape), shape["c_in"], shape["width"],
                               shape["width"], shape["n3x3"], 1, LG_ACT_RELU, 0, 1,
                               shape["fc_hidden"], 0, precision="bf16"))
    with Context(device=device, max_batch=batch, **sdesc) as cs, \
            Context(policy=NetDesc.config1_policy(wp, "bf16"),
                    value=NetDesc.config1_value(wv, "bf16"), device=device,
                    max_batch=batch) as cf:
        # both nets with their kernel choices tuned, as a serving context runs
        cs.autotune()
        cf.autotune()
        sp = torch.empty((T, 361), device=dev)
        fp = torch.empty((T, 361), device=dev)
        fv = torch.empty(T, device=dev)
        cs.policy_device(tp.data_ptr(), T, sp.data_ptr(), 1.0, None, stream)
        cf.policy_device(tp.data_ptr(), T, fp.data_ptr(), 1.0, None, stream)
        torch.cuda.synchronize()
        ent = entropy(sp).cpu().numpy()
        agree = (sp.argmax(1) == fp.argmax(1)).cpu().numpy()
        thr_cal, share_cal, agree_cal = calibrate_threshold(ent, agree)

        def timed(fn, reps=3):
            for _ in range(2):
                fn()
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            for _ in range(reps):
                fn()
            e1.record()
            torch.cuda.synchronize()
            return reps * T / (e0.elapsed_time(e1) / 1e3)

        def full_only():
            for b0 in range(0, T, batch):
                cf.policy_device(tp[b0].data_ptr(), batch, fp[b0].data_ptr(), 1.0, None, stream)
                cf.value_device(tv[b0].data_ptr(), batch, fv[b0:].data_ptr(), stream)

        def gated(thr):
            g = GatedEvaluator(cs, cf, thr)

            def run():
                fb = 0
                for b0 in range(0, T, batch):
                    _, _, m = g.evaluate(tp[b0:b0 + batch], tv[b0:b0 + batch], stream)
                    fb += int(m.sum())
                return fb
            return run

        full_rate = timed(full_only)
        student_rate = timed(gated(1e9))
        spec_rate = timed(gated(threshold))
        cal_rate = timed(gated(thr_cal)) if np.isfinite(thr_cal) else None
    mask_spec = ent > threshold
    return {
        "positions_train": int(train_idx.numel()), "positions_test": int(T),
        "teacher_temperature": teacher_temperature, "train_steps": int(log[-1][0]) + 1,
        "train_seconds": train_s, "loss_log": log[::max(1, len(log) // 6)] + [log[-1]],
        "student_top1_agreement_with_full_net": float(agree.mean()),
        "student_entropy_nats": {"p10": float(np.percentile(ent, 10)),
                                 "median": float(np.median(ent)),
                                 "p90": float(np.percentile(ent, 90))},
        "gate_spec": {"threshold_nats": threshold, "fallback_rate": float(mask_spec.mean()),
                      "top1_agreement": float(1.0 - (~agree & ~mask_spec).mean()),
                      "leaf_evals_per_s": spec_rate,
                      "speedup_vs_full_net": spec_rate / full_rate},
        "gate_calibrated_97": {"threshold_nats": thr_cal, "fallback_rate": 1.0 - share_cal,
                               "top1_agreement": agree_cal, "leaf_evals_per_s": cal_rate,
                               "speedup_vs_full_net": (cal_rate / full_rate) if cal_rate else None},
        "student_only_leaf_evals_per_s": student_rate,
        "full_net_leaf_evals_per_s": full_rate,
    }


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
