"""The distilled student: GPU training kernels against the FP64 oracle, a
training run that lowers the loss, export to the serving paths, and the
entropy-gated fallback."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def student_mod(gpu_lib):
    from leela_gb300 import distill
    return distill


def _targets(rng, B):
    logits = rng.normal(0, 2.0, (B, 361))
    t = np.exp(logits - logits.max(1, keepdims=True))
    return (t / t.sum(1, keepdims=True)).astype(np.float32), rng.uniform(-0.8, 0.8, B).astype(np.float32)


def test_student_gradients_match_fp64_oracle(student_mod, positions):
    import torch
    from oracle import distill_oracle as D
    st = student_mod.Student(max_batch=8)
    st.init_he(3)
    p = st.get_params()
    rng = np.random.default_rng(5)
    # small random biases so that no layer is exactly at a ReLU kink
    planes = np.ascontiguousarray(positions["planes_p"][10:13, :24])
    t, vt = _targets(rng, 3)
    d_planes = torch.from_numpy(planes).cuda()
    d_t = torch.from_numpy(t).cuda()
    d_v = torch.from_numpy(vt).cuda()
    (kl, mse), g = st.grads(d_planes.data_ptr(), 3, d_t.data_ptr(), d_v.data_ptr(), 0.5)
    (kl64, mse64), g64 = D.loss_and_grads(p, planes, t, vt, 0.5, 24, 64, 5, 64)
    assert abs(kl - kl64) <= 1e-4 * abs(kl64) + 1e-6
    assert abs(mse - mse64) <= 1e-4 * abs(mse64) + 1e-6
    # per parameter tensor, norm-wise relative error; the floor covers
    # tensors whose exact gradient is zero (the policy-head bias: the
    # softmax and the target both sum to 1)
    floor = 1e-4 * np.abs(g64).max()
    off = 0
    for s in D.shapes(24, 64, 5, 64):
        sizes = [s[3] * s[2] * s[1] * s[1], s[3]] if s[0] == "conv" else [s[1]]
        for n in sizes:
            a, b = g[off:off + n], g64[off:off + n]
            off += n
            denom = max(np.abs(b).max(), floor)
            assert np.abs(a - b).max() / denom <= 2e-3, (s, n, np.abs(a - b).max(), denom)
    st.close()


def test_training_lowers_the_loss(student_mod, positions):
    import torch
    st = student_mod.Student(max_batch=64)
    st.init_he(1)
    rng = np.random.default_rng(7)
    planes = torch.from_numpy(np.ascontiguousarray(positions["planes_p"][:64, :24])).cuda()
    t, vt = _targets(rng, 64)
    d_t, d_v = torch.from_numpy(t).cuda(), torch.from_numpy(vt).cuda()
    log = student_mod.train(st, planes, d_t, d_v, steps=300, batch=64, lr=2e-3, log_every=50)
    first, last = log[0], log[-1]
    assert last[1] + last[2] < 0.7 * (first[1] + first[2]), log
    st.close()


def test_exported_nets_match_the_student_forward(student_mod, gpu_lib, positions):
    import torch
    lg = gpu_lib
    st = student_mod.Student(max_batch=32)
    st.init_he(2)
    planes = torch.from_numpy(np.ascontiguousarray(positions["planes_p"][:20, :24])).cuda()
    probs = torch.empty((20, 361), device="cuda")
    val = torch.empty(20, device="cuda")
    st.forward(planes.data_ptr(), 20, probs.data_ptr(), val.data_ptr())
    torch.cuda.synchronize()
    with lg.Context(policy=st.policy_desc("fp32"), value=st.value_desc("fp32"), max_batch=32) as c:
        p2 = c.policy(planes.cpu().numpy())
        v2 = c.value(planes.cpu().numpy())
    assert np.abs(probs.cpu().numpy() - p2).max() < 1e-5
    assert np.abs(val.cpu().numpy() - v2).max() < 1e-5
    st.close()


@pytest.mark.parametrize("B", [40, 300])
def test_gate_routes_by_entropy(student_mod, gpu_lib, weights, positions, B):
    """lg_gated_device: with a threshold no entropy reaches, the student's
    answers (bit-identical to lg_fast_device); with one below every entropy,
    the full nets' answers for every position (bit-identical to the full
    context on the persistent trunk); at the median entropy, each position
    from the side its entropy picks, and the device-side count equal to the
    number of fallbacks.  B = 300 spans two chunks of the full context."""
    import torch
    lg = gpu_lib
    st = student_mod.Student(max_batch=8)
    st.init_he(4)
    params = st.get_params()
    st.close()
    idx = np.arange(B) % 1024
    pp = torch.from_numpy(np.ascontiguousarray(positions["planes_p"][idx, :24])).cuda()
    pv = torch.from_numpy(np.ascontiguousarray(positions["planes_v"][idx, :24])).cuda()
    with student_mod.FastNet(params, max_batch=512) as fast, \
            lg.Context(policy=lg.NetDesc.config1_policy(weights["cfg_p"][1], "bf16"),
                       value=lg.NetDesc.config1_value(weights["cfg_v"][1], "bf16"),
                       max_batch=256) as cf:
        sp = torch.empty((B, 361), device="cuda")
        sv = torch.empty(B, device="cuda")
        se = torch.empty(B, device="cuda")
        fast.device(pp.data_ptr(), B, sp.data_ptr(), sv.data_ptr(), 1.0, None, se.data_ptr())
        fast.status()
        sp, sv, se = sp.cpu().numpy(), sv.cpu().numpy(), se.cpu().numpy()
        # the full nets as the gated path runs them: persistent trunk with
        # the first layer inside, chunks of 256
        for b in (B % 256 or 256, 256):
            cf.set_tuning(b, 3, 0)
        fp = cf.policy(pp.cpu().numpy())
        fv = cf.value(pv.cpu().numpy())
        for thr, expect in ((1e9, "student"), (-1.0, "full"), (float(np.median(se)), "mixed")):
            g = student_mod.GatedEvaluator(fast, cf, threshold=thr)
            p, v, m, n = g.evaluate(pp, pv)
            torch.cuda.synchronize()
            fast.status()
            p, v, m, n = p.cpu().numpy(), v.cpu().numpy(), m.cpu().numpy().astype(bool), int(n.item())
            want = se > thr
            assert np.array_equal(m, want), thr
            assert n == int(want.sum())
            assert np.array_equal(p[~want], sp[~want]) and np.array_equal(v[~want], sv[~want]), thr
            assert np.array_equal(p[want], fp[want]) and np.array_equal(v[want], fv[want]), thr
            if expect == "student":
                assert n == 0
            elif expect == "full":
                assert n == B
            else:
                assert 0 < n < B


def test_gate_needs_tensor_core_full_nets(student_mod, gpu_lib, weights, positions):
    import torch
    lg = gpu_lib
    n = int(student_mod._bind().lg_fast_param_count(24, 5, 64))
    pp = torch.zeros((4, 24, 361), dtype=torch.uint8, device="cuda")
    with student_mod.FastNet(np.zeros(n, np.float32), max_batch=8) as fast, \
            lg.Context(policy=lg.NetDesc.config1_policy(weights["cfg_p"][1], "fp32"),
                       value=lg.NetDesc.config1_value(weights["cfg_v"][1], "fp32"), max_batch=8) as c32:
        with pytest.raises(lg.LeelaGPUError):
            student_mod.GatedEvaluator(fast, c32, 2.5).evaluate(pp, pp)


def test_training_gains_over_the_untrained_student(student_mod, gpu_lib, weights, positions):
    """What the trained network buys over having none: trained on the
    config-4 labels (the full FP32 policy net's softmax, 2*mc_owner-1 values)
    of positions 0..895, the student approximates the full net on the
    held-out positions 896..1023 far better than the untrained student:
    lower policy KL to the full net and lower value error."""
    import os

    import torch
    lg = gpu_lib
    from conftest import GOLDEN
    mc = np.load(os.path.join(GOLDEN, "mcowner_s0.npz"))["mcowner"]
    pp = np.ascontiguousarray(positions["planes_p"][:, :24])
    with lg.Context(policy=lg.NetDesc.config1_policy(weights["cfg_p"][1]), max_batch=256) as c:
        probs = c.policy(pp, 1.0)
    d_pp = torch.from_numpy(pp).cuda()
    d_t = torch.from_numpy(probs).cuda()
    d_v = torch.from_numpy((2 * mc - 1).astype(np.float32)).cuda()
    tr, te = slice(0, 896), slice(896, 1024)
    st = student_mod.Student(max_batch=256)
    st.init_he(0)
    before = student_mod.heldout_loss(st, d_pp[te].contiguous(), d_t[te].contiguous(),
                                      d_v[te].contiguous())
    student_mod.train(st, d_pp[tr].contiguous(), d_t[tr].contiguous(), d_v[tr].contiguous(),
                      steps=400, batch=128, lr=1e-3, log_every=100)
    after = student_mod.heldout_loss(st, d_pp[te].contiguous(), d_t[te].contiguous(),
                                     d_v[te].contiguous())
    st.close()
    print("held-out (KL, value MSE) untrained", before, "trained", after)
    assert after[0] < 0.5 * before[0]
    assert after[1] < before[1]
