"""The student served by the fused BF16 kernel (lg_fast_*), called through
the C ABI: against the same nets served layer by layer in BF16 by a
context (same weight and activation rounding, another summation order),
against the FP32 student forward, independence of the batch a position
sits in, and the argument checks."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def dmod(gpu_lib):
    from leela_gb300 import distill
    return distill


def _student(dmod, seed, max_batch=64, bias_scale=0.05):
    """A He-normal student with small random biases (no layer sits exactly
    at ReLU kinks); returns (Student, flat params)."""
    st = dmod.Student(max_batch=max_batch)
    st.init_he(seed)
    p = st.get_params()
    rng = np.random.default_rng(seed + 100)
    # biases: every conv's bias block and the heads' biases
    s = st.shape
    off = 0
    for l in range(s["n3x3"] + 1):
        k = 5 if l == 0 else 3
        cin = s["c_in"] if l == 0 else s["width"]
        off += s["width"] * cin * k * k
        p[off:off + s["width"]] = rng.normal(0, bias_scale, s["width"])
        off += s["width"]
    st.set_params(p)
    return st, p


def _run_fast(dmod, fast, planes, T=1.0):
    import torch
    B = planes.shape[0]
    probs = torch.empty((B, 361), device="cuda")
    logits = torch.empty((B, 361), device="cuda")
    val = torch.empty(B, device="cuda")
    ent = torch.empty(B, device="cuda")
    fast.device(planes.data_ptr(), B, probs.data_ptr(), val.data_ptr(), T, logits.data_ptr(), ent.data_ptr())
    fast.status()
    return probs.cpu().numpy(), logits.cpu().numpy(), val.cpu().numpy(), ent.cpu().numpy()


def test_fast_net_matches_the_bf16_layer_path(dmod, gpu_lib, positions):
    """Same BF16 rounding of weights and activations, FP32 accumulation in
    another order (an activation that lands near a rounding boundary can
    round the other way, one BF16 step = 2^-8 relative): probabilities
    within 2e-5, values within 3e-3, head outputs within 8e-3 norm-wise (two
    BF16 steps), top-1 equal up to near-ties, entropy equal to -sum p ln p
    of the output.  (Measured on GB300: 7.7e-6, 1.2e-3, 2.5e-3.)"""
    import torch
    lg = gpu_lib
    st, p = _student(dmod, 11)
    B = 64
    pp = torch.from_numpy(np.ascontiguousarray(positions["planes_p"][:B, :24])).cuda()
    with dmod.FastNet(p, max_batch=B) as fast, \
            lg.Context(policy=st.policy_desc("bf16"), value=st.value_desc("bf16"), max_batch=B) as c:
        c.set_tuning(B, 0, 0)
        fp, fl, fv, fe = _run_fast(dmod, fast, pp)
        ref_p, ref_l = c.policy(pp.cpu().numpy(), 1.0, return_logits=True)
        ref_v = c.value(pp.cpu().numpy())
    st.close()
    dp = np.abs(fp - ref_p).max()
    dv = np.abs(fv - ref_v).max()
    dl = np.abs(fl - ref_l).max() / np.abs(ref_l).max()
    print(f"fast vs layer path: prob {dp:.3g}, value {dv:.3g}, logit (norm-wise) {dl:.3g}")
    assert dp <= 2e-5 and dv <= 3e-3 and dl <= 8e-3
    from conftest import top1_same_up_to_ties
    assert top1_same_up_to_ties(fl, ref_l, 2 * dl).all()
    h = -(fp * np.log(np.maximum(fp, 1e-30))).sum(1)
    assert np.abs(fe - h).max() <= 1e-4


def test_fast_net_close_to_fp32_student(dmod, positions):
    """Against the FP32 student forward (the trained net itself): the BF16
    serving error."""
    import torch
    st, p = _student(dmod, 12)
    B = 48
    pp = torch.from_numpy(np.ascontiguousarray(positions["planes_p"][100:100 + B, :24])).cuda()
    probs = torch.empty((B, 361), device="cuda")
    val = torch.empty(B, device="cuda")
    st.forward(pp.data_ptr(), B, probs.data_ptr(), val.data_ptr())
    torch.cuda.synchronize()
    with dmod.FastNet(p, max_batch=B) as fast:
        fp, _, fv, _ = _run_fast(dmod, fast, pp)
    st.close()
    dp = np.abs(fp - probs.cpu().numpy()).max()
    dv = np.abs(fv - val.cpu().numpy()).max()
    print(f"fast (BF16) vs FP32 student: prob {dp:.3g}, value {dv:.3g}")
    assert dp <= 2e-4 and dv <= 3e-2


def test_fast_net_batch_independent(dmod, positions):
    """A position's answer does not depend on the batch or on its partner
    in the two-board group: bit-identical at B = 1, 3, 37 and 300."""
    import torch
    st, p = _student(dmod, 13, max_batch=8)
    st.close()
    pp = torch.from_numpy(np.ascontiguousarray(positions["planes_p"][:300, :24])).cuda()
    with dmod.FastNet(p, max_batch=300) as fast:
        full = _run_fast(dmod, fast, pp)
        for start, B in ((0, 1), (5, 3), (17, 37), (1, 299)):
            part = _run_fast(dmod, fast, pp[start:start + B].contiguous())
            for a, b in zip(part, full):
                assert np.array_equal(a, b[start:start + B]), (start, B)


def test_fast_net_arguments(dmod, gpu_lib):
    import torch
    L = dmod._bind()
    n = int(L.lg_fast_param_count(24, 5, 64))
    p = np.zeros(n, np.float32)
    h = ctypes.c_void_p()
    assert L.lg_fast_create(0, 22, 5, 64, 8, p.ctypes.data, ctypes.byref(h)) == -1  # c_in not a multiple of 4
    assert L.lg_fast_create(0, 24, 0, 64, 8, p.ctypes.data, ctypes.byref(h)) == -1
    with dmod.FastNet(p, max_batch=8) as fast:
        planes = torch.zeros((9 * 24 * 361 + 4,), dtype=torch.uint8, device="cuda")
        probs = torch.empty((9, 361), device="cuda")
        val = torch.empty(9, device="cuda")
        with pytest.raises(gpu_lib.LeelaGPUError):   # B above max_batch
            fast.device(planes.data_ptr(), 9, probs.data_ptr(), val.data_ptr())
        with pytest.raises(gpu_lib.LeelaGPUError):   # planes not 4-byte aligned
            fast.device(planes.data_ptr() + 1, 2, probs.data_ptr(), val.data_ptr())
        # zero weights: uniform policy, entropy ln 361, value tanh(0) = 0
        fp, _, fv, fe = _run_fast(dmod, fast, planes[:4 * 24 * 361].view(4, 24, 361))
        assert np.allclose(fp, 1.0 / 361, rtol=1e-6)
        assert np.allclose(fe, np.log(361.0), atol=1e-5)
        assert np.all(fv == 0.0)
