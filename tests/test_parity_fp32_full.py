"""The FP32 drop-in path over the whole of the benchmark configurations.

Config 0: the policy net at batch 1 over all 1024 positions, against the
reference's own compiled CPU/BLAS outputs (tests/golden/config0_s0.npz,
written by make_golden.py --only config0).  Config 1: policy and value nets
at batch 8, 64 and 256 over the 8192 symmetry inputs (1024 positions x 8
rotations), against the oracle, which reproduces the reference bit for bit
with OpenBLAS (tests/test_oracle.py).

Bars: norm-wise relative logit error max|a-b| / max|b| <= 1e-4 per position;
the same top-1 move, except where the reference's two best logits are
within that tolerance of each other (a tie at FP32 precision; counted and
printed); values within 1e-5.  The element-wise metric
max|a-b| / max(|b|, 1e-3 max|b|) is reported beside it: on near-zero logits
it measures FP32 rounding itself, so its bar is relative -- against FP64
arithmetic (the oracle), the GPU's FP32 logits must be no further off than
the reference's own FP32 logits are (config 0), and GPU and oracle may
differ by at most 1e-2 (config 1; measured 6e-3).
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN, elem_rel_err, rel_logit_err, top1_same_up_to_ties

pytestmark = pytest.mark.gpu

LOGIT_TOL = 1e-4
ELEM_TOL = 1e-2


@pytest.fixture(scope="module")
def config0():
    return dict(np.load(os.path.join(GOLDEN, "config0_s0.npz")))


def test_config0_batch1_all_positions_vs_reference(gpu_lib, weights, positions, config0, oracle_mod):
    lg, O = gpu_lib, oracle_mod
    planes_p, planes_v = positions["planes_p"][:, :24], positions["planes_v"][:, :24]
    n = planes_p.shape[0]
    logits = np.empty((n, 361), np.float32)
    probs = np.empty((n, 361), np.float32)
    value = np.empty(n, np.float32)
    with lg.Context(policy=lg.NetDesc.config1_policy(weights["cfg_p"][1]),
                    value=lg.NetDesc.config1_value(weights["cfg_v"][1]), max_batch=1) as c:
        for i in range(n):
            probs[i:i + 1], logits[i:i + 1] = c.policy(planes_p[i:i + 1], 1.0, return_logits=True)
            value[i:i + 1] = c.value(planes_v[i:i + 1])
    ref = config0["logits_r0"]
    norm, elem = rel_logit_err(logits, ref), elem_rel_err(logits, ref)
    same = logits.argmax(1) == ref.argmax(1)
    print(f"config0 batch 1, {n} positions: norm-wise max {norm.max():.2e}, element-wise max "
          f"{elem.max():.2e}, top-1 equal {same.mean():.4f}, value err {np.abs(value - config0['value_r0']).max():.2e}")
    assert norm.max() <= LOGIT_TOL
    assert elem.max() <= ELEM_TOL
    assert top1_same_up_to_ties(logits, ref, LOGIT_TOL).all()
    assert np.abs(value - config0["value_r0"]).max() <= 1e-5
    # element-wise against exact arithmetic: no worse than the reference's own FP32
    O.enable_blas()
    try:
        l64 = O.forward_f64(weights["cfg_p"][0], weights["cfg_p"][1], planes_p)
    finally:
        O.disable_blas()
    e_gpu, e_ref = elem_rel_err(logits, l64).max(), elem_rel_err(ref, l64).max()
    print(f"element-wise vs FP64: GPU FP32 {e_gpu:.2e}, reference FP32 {e_ref:.2e}")
    assert e_gpu <= 1.5 * e_ref
    # probabilities: the reference softmax (restated, pinned) of the reference logits
    assert np.abs(probs - O.softmax_f32(ref, 1.0)).max() <= 1e-6


@pytest.fixture(scope="module")
def config1_oracle(weights, positions, oracle_mod, gpu_lib):
    O, lg = oracle_mod, gpu_lib
    pp = np.concatenate([positions["planes_p"][:, :24][..., lg.ROTATE[r]] for r in range(8)])
    pv = np.concatenate([positions["planes_v"][:, :24][..., lg.ROTATE[r]] for r in range(8)])
    O.enable_blas()
    try:
        lref = O.forward_f32(weights["cfg_p"][0], weights["cfg_p"][1], pp)
        vref = O.forward_f32(weights["cfg_v"][0], weights["cfg_v"][1], pv)
    finally:
        O.disable_blas()
    return np.ascontiguousarray(pp), np.ascontiguousarray(pv), lref, vref


@pytest.mark.parametrize("B", [8, 64, 256])
def test_config1_symmetry_inputs_vs_oracle(gpu_lib, weights, config1_oracle, B):
    lg = gpu_lib
    pp, pv, lref, vref = config1_oracle
    n = pp.shape[0]
    logits = np.empty((n, 361), np.float32)
    value = np.empty(n, np.float32)
    with lg.Context(policy=lg.NetDesc.config1_policy(weights["cfg_p"][1]),
                    value=lg.NetDesc.config1_value(weights["cfg_v"][1]), max_batch=B) as c:
        for i in range(0, n, B):
            _, logits[i:i + B] = c.policy(pp[i:i + B], 1.0, return_logits=True)
            value[i:i + B] = c.value(pv[i:i + B])
    norm, elem = rel_logit_err(logits, lref), elem_rel_err(logits, lref)
    same = logits.argmax(1) == lref.argmax(1)
    print(f"config1 batch {B}, {n} inputs: norm-wise max {norm.max():.2e}, element-wise max {elem.max():.2e}, "
          f"top-1 equal {same.mean():.5f} ({(~same).sum()} ties), value err {np.abs(value - vref).max():.2e}")
    assert norm.max() <= LOGIT_TOL
    assert elem.max() <= ELEM_TOL
    assert top1_same_up_to_ties(logits, lref, LOGIT_TOL).all()
    assert np.abs(value - vref).max() <= 1e-5
