"""Kernel variants for 128-wide tensor-core layers and the autotuner that
picks between them per batch bucket (lg_autotune / lg_tuning /
lg_set_tuning)."""
import json
import os

import numpy as np
import pytest

from conftest import rel_logit_err

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def f64(positions, weights, oracle_mod):
    O = oracle_mod
    O.enable_blas()
    try:
        lp = O.forward_f64(weights["cfg_p"][0], weights["cfg_p"][1], positions["planes_p"][:64, :24])
        v = O.forward_f64(weights["cfg_v"][0], weights["cfg_v"][1], positions["planes_v"][:64, :24])
    finally:
        O.disable_blas()
    return lp, v


@pytest.mark.parametrize("v3,v1", [(0, 0), (1, 0), (0, 1), (1, 1), (2, 0), (2, 1), (3, 0)])
@pytest.mark.parametrize("B", [1, 5, 64])
def test_every_variant_meets_the_bf16_bars(gpu_lib, weights, positions, f64, v3, v1, B):
    lg = gpu_lib
    lp64, v64 = f64
    with lg.Context(policy=lg.NetDesc.config1_policy(weights["cfg_p"][1], "bf16"),
                    value=lg.NetDesc.config1_value(weights["cfg_v"][1], "bf16"), max_batch=64) as c:
        c.set_tuning(B, v3, v1)
        _, logits = c.policy(positions["planes_p"][:B, :24], 1.0, return_logits=True)
        v = c.value(positions["planes_v"][:B, :24])
    assert rel_logit_err(logits, lp64[:B]).max() <= 5e-2
    assert np.abs(v - v64[:B]).max() <= 3e-2
    if B == 64:
        assert (logits.argmax(1) == lp64.argmax(1)).mean() >= 0.95


def test_autotune_writes_and_reloads_its_cache(gpu_lib, weights, positions, tmp_path):
    lg = gpu_lib
    path = str(tmp_path / "tune.json")
    kw = dict(policy=lg.NetDesc.config1_policy(weights["cfg_p"][1], "bf16"),
              value=lg.NetDesc.config1_value(weights["cfg_v"][1], "bf16"), max_batch=32)
    with lg.Context(**kw) as c:
        assert not c.tuning(4)["tuned"]
        ref = c.policy(positions["planes_p"][:20, :24])
        c.autotune(path)
        table = {b: c.tuning(b) for b in (1, 2, 4, 8, 16, 32)}
        assert all(t["tuned"] for t in table.values())
        after = c.policy(positions["planes_p"][:20, :24])
        assert np.abs(after - ref).max() < 1e-4
    with open(path) as f:
        saved = json.load(f)
    assert set(saved["table"]) == {"1", "2", "4", "8", "16", "32"}
    with lg.Context(**kw) as c2:
        c2.autotune(path)  # loads, no timing
        assert {b: c2.tuning(b) for b in table} == table


@pytest.mark.parametrize("B", [1, 3, 64])
@pytest.mark.parametrize("v3", [2, 3])
@pytest.mark.parametrize("prec", ["fp8w", "fp16"])
def test_trunk_matches_per_layer_kernels(gpu_lib, weights, positions, B, v3, prec):
    """The persistent trunk kernel (3x3 choice 2; choice 3 with the first
    layer in the same launch) computes the same layers as the per-layer
    launches, FP8 weights (per-channel scales) and FP16 operands included."""
    lg = gpu_lib
    with lg.Context(policy=lg.NetDesc.config1_policy(weights["cfg_p"][1], prec),
                    value=lg.NetDesc.config1_value(weights["cfg_v"][1], prec), max_batch=64) as c:
        c.set_tuning(B, 0, 0)
        p0, l0 = c.policy(positions["planes_p"][:B, :24], 1.0, return_logits=True)
        v0 = c.value(positions["planes_v"][:B, :24])
        c.set_tuning(B, v3, 0)
        p2, l2 = c.policy(positions["planes_p"][:B, :24], 1.0, return_logits=True)
        v2 = c.value(positions["planes_v"][:B, :24])
    assert rel_logit_err(l2, l0).max() < 1e-5
    assert np.abs(v2 - v0).max() < 1e-5


@pytest.mark.parametrize("B", [1, 7, 64, 256])
def test_fused_first_layer_trunk_equals_separate_first_layer(gpu_lib, weights, positions, B):
    """Choice 3 (first layer as work items of the trunk launch) and choice 2
    (first layer in its own launch, same 256-row tiles and K order) give the
    same BF16 results; B = 7 leaves a ragged last L5 chunk (2793 rows)."""
    lg = gpu_lib
    idx = np.arange(B) % 1024
    with lg.Context(policy=lg.NetDesc.config1_policy(weights["cfg_p"][1], "bf16"),
                    value=lg.NetDesc.config1_value(weights["cfg_v"][1], "bf16"), max_batch=256) as c:
        c.set_tuning(B, 2, 0)
        _, l2 = c.policy(positions["planes_p"][idx, :24], 1.0, return_logits=True)
        v2 = c.value(positions["planes_v"][idx, :24])
        c.set_tuning(B, 3, 0)
        _, l3 = c.policy(positions["planes_p"][idx, :24], 1.0, return_logits=True)
        v3 = c.value(positions["planes_v"][idx, :24])
    assert rel_logit_err(l3, l2).max() < 1e-5
    assert np.abs(v3 - v2).max() < 1e-5


def test_untuned_defaults(gpu_lib, weights):
    """Without tuning a context takes the measured defaults: with a 16-bit
    net the small-batch kernel (choice 4) up to 2 positions and the
    persistent trunk with the first layer inside (choice 3) above; FP32
    nets the small-batch kernel up to 8 positions and their per-layer
    kernels above."""
    lg = gpu_lib
    with lg.Context(policy=lg.NetDesc.config1_policy(weights["cfg_p"][1], "bf16"),
                    value=lg.NetDesc.config1_value(weights["cfg_v"][1], "bf16"), max_batch=256) as c:
        got = {b: c.tuning(b)["conv3x3"] for b in (1, 2, 3, 8, 9, 256)}
        assert got == {1: 4, 2: 4, 3: 3, 8: 3, 9: 3, 256: 3}
        assert not c.tuning(256)["tuned"]
    with lg.Context(policy=lg.NetDesc.config1_policy(weights["cfg_p"][1]),
                    value=lg.NetDesc.config1_value(weights["cfg_v"][1]), max_batch=64) as c:
        got = {b: c.tuning(b)["conv3x3"] for b in (1, 8, 9, 64)}
        assert got == {1: 4, 8: 4, 9: 0, 64: 0}
