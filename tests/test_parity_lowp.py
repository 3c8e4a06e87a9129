"""BF16 and FP8-weight tensor-core paths against the FP64 host oracle.

Tolerances (stated per result, on the benchmark nets with He-normal weights):
  top-1 agreement with FP64              >= 95% of 64 positions (the >= 99%
                                            benchmark-scale figure is measured
                                            by bench.py over more positions)
  policy probabilities, max |p - p64|    <= 2e-3
  norm-wise logit error max|a-b|/max|b|  <= 5e-2
  value, max |v - v64|                   <= 3e-2
"""
import numpy as np
import pytest

from conftest import rel_logit_err

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def f64_refs(positions, weights, oracle_mod):
    """FP64 oracle outputs with exact weights ('exact') and with the weights
    each variant defines ('bf16': BF16-rounded, 'fp8w': E4M3 per output
    channel, BF16 FC)."""
    O = oracle_mod
    pp, pv = positions["planes_p"][:64, :24], positions["planes_v"][:64, :24]
    (P, wp), (V, wv) = weights["cfg_p"], weights["cfg_v"]
    out = {}
    O.enable_blas()
    try:
        for mode in ("exact", "bf16", "fp8w"):
            qp = wp if mode == "exact" else O.quantize_weights(P, wp, "fp8" if mode == "fp8w" else "bf16")
            qv = wv if mode == "exact" else O.quantize_weights(V, wv, "fp8" if mode == "fp8w" else "bf16")
            lp = O.forward_f64(P, qp, pp)
            out[mode] = (lp, O.softmax_f64(lp, 1.0), O.forward_f64(V, qv, pv))
    finally:
        O.disable_blas()
    return out


@pytest.mark.parametrize("prec", ["bf16", "fp8w"])
def test_lowp_vs_fp64(gpu_lib, weights, positions, f64_refs, prec):
    """Against the FP64 oracle run with the variant's own weights, the only
    error left is the BF16 activation rounding: top-1 >= 95%, probabilities
    within 2e-3, norm-wise logit error <= 5e-2, value within 3e-2.  Against
    the exact weights, BF16 meets the same bars; E4M3 weights carry their own
    quantisation error (top-1 ~60%, logit error ~0.4 on these nets, the same
    as FP64 arithmetic with E4M3 weights), bounded here at 0.6 / 0.1."""
    lg = gpu_lib
    with lg.Context(policy=lg.NetDesc.config1_policy(weights["cfg_p"][1], prec),
                    value=lg.NetDesc.config1_value(weights["cfg_v"][1], prec), max_batch=64) as c:
        probs, logits = c.policy(positions["planes_p"][:64, :24], 1.0, return_logits=True)
        v = c.value(positions["planes_v"][:64, :24])
    for ref_kind in (prec, "exact"):
        lp64, p64, v64 = f64_refs[ref_kind]
        agree = (logits.argmax(1) == lp64.argmax(1)).mean()
        perr = np.abs(probs - p64).max()
        lerr = rel_logit_err(logits, lp64).max()
        verr = np.abs(v - v64).max()
        print(f"{prec} vs fp64[{ref_kind}]: top1 {agree:.3f} prob_err {perr:.2e} "
              f"logit_err {lerr:.2e} value_err {verr:.2e}")
        if ref_kind == prec or prec == "bf16":
            assert agree >= 0.95
            assert perr <= 2e-3
            assert lerr <= 5e-2
            assert verr <= 3e-2
        else:
            assert lerr <= 0.6
            assert verr <= 0.1


def test_bf16_batch_independent(gpu_lib, weights, positions):
    """A position's result does not depend on its batch or its slot in it."""
    lg = gpu_lib
    with lg.Context(policy=lg.NetDesc.config1_policy(weights["cfg_p"][1], "bf16"),
                    max_batch=64) as c:
        planes = positions["planes_p"][:37, :24]
        full = c.policy(planes)
        one = np.concatenate([c.policy(planes[i:i + 1]) for i in (0, 17, 36)])
    assert np.array_equal(one, full[[0, 17, 36]])


def test_bf16_device_path(gpu_lib, weights, positions):
    import torch
    lg = gpu_lib
    with lg.Context(policy=lg.NetDesc.config1_policy(weights["cfg_p"][1], "bf16"),
                    max_batch=128) as c:
        planes = np.ascontiguousarray(positions["planes_p"][:100, :24])
        host = c.policy(planes)
        d = torch.from_numpy(planes).cuda()
        out = torch.empty((100, 361), device="cuda")
        s = torch.cuda.current_stream()
        c.policy_device(d.data_ptr(), 100, out.data_ptr(), 1.0, None, s.cuda_stream)
        s.synchronize()
        assert np.array_equal(out.cpu().numpy(), host)


def test_lowp_rejects_unsupported_shape(gpu_lib, weights):
    lg = gpu_lib
    with pytest.raises(lg.LeelaGPUError):
        lg.Context(policy=lg.NetDesc.reference_policy(weights["ref_p"][1], "bf16"), max_batch=4)
