"""The CPU oracle against the reference's own outputs (tests/golden, made by
tests/golden/make_golden.py from the reference's compiled CPU/BLAS code)."""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN, rel_logit_err


def test_weights_match_golden_checksums(weights, oracle_mod):
    with open(os.path.join(GOLDEN, "weights.json")) as f:
        sums = json.load(f)
    assert oracle_mod.checksum(weights["cfg_p"][1]) == sums["cfg_policy"]
    assert oracle_mod.checksum(weights["cfg_v"][1]) == sums["cfg_value"]
    assert oracle_mod.checksum(weights["ref_p"][1]) == sums["ref_policy"]
    assert oracle_mod.checksum(weights["ref_v"][1]) == sums["ref_value"]


def test_he_normal_statistics(weights, oracle_mod):
    n, w = weights["cfg_p"]
    shapes = oracle_mod.conv_shapes(n)
    k, ci, co, off = shapes[1]
    W = w[off:off + co * ci * k * k]
    assert abs(W.mean()) < 3e-3
    assert abs(W.std() - np.sqrt(2.0 / (ci * k * k))) / np.sqrt(2.0 / (ci * k * k)) < 0.01
    b = w[off + co * ci * k * k: off + co * ci * k * k + co]
    assert np.all(b == 0)


def test_det_log(oracle_mod):
    L = oracle_mod.lib()
    for x in [1e-300, 1e-9, 0.001, 0.37, 0.5, 0.999999, 1.0, 7.0]:
        assert abs(L.or_det_log(x) - np.log(x)) <= 4e-16 * max(1.0, abs(np.log(x)))


@pytest.mark.parametrize("rot", [0, 3])
def test_config1_policy_matches_reference(positions, golden_config1, weights, oracle_mod, rot):
    O = oracle_mod
    n, w = weights["cfg_p"]
    planes = np.stack([O.rotate_planes(p[:24], rot) for p in positions["planes_p"][:6]])
    ref = golden_config1[f"logits_r{rot}"][:6]
    O.enable_blas()
    try:
        blas = O.forward_f32(n, w, planes)
    finally:
        O.disable_blas()
    # With the same BLAS the restatement reproduces the reference bit for bit.
    if O.find_openblas():
        assert np.array_equal(blas, ref)
    loops = O.forward_f32(n, w, planes)
    assert rel_logit_err(loops, ref).max() < 1e-5
    assert np.array_equal(loops.argmax(1), ref.argmax(1))
    probs = O.softmax_f32(ref, 1.0)
    assert np.abs(probs - golden_config1[f"probs_r{rot}"][:6]).max() < 1e-7
    f64 = O.forward_f64(n, w, planes)
    assert rel_logit_err(f64, ref).max() < 1e-5


def test_config1_value_matches_reference(positions, golden_config1, weights, oracle_mod):
    O = oracle_mod
    n, w = weights["cfg_v"]
    v = O.forward_f32(n, w, positions["planes_v"][:6, :24])
    assert np.abs(v - golden_config1["value_r0"][:6]).max() < 1e-5
    v64 = O.forward_f64(n, w, positions["planes_v"][:6, :24])
    assert np.abs(v64 - golden_config1["value_r0"][:6]).max() < 1e-5


@pytest.mark.parametrize("rot", [0, 5])
def test_reference_shaped_nets_match_reference(positions, golden_refexact, weights, oracle_mod,
                                               rot):
    """ELU everywhere, 3x3 heads, 32->96->128 policy, 64-wide value with the
    (1+tanh)/2 map: the reference's own Network.cpp forward."""
    O = oracle_mod
    n, w = weights["ref_p"]
    planes = np.stack([O.rotate_planes(p, rot) for p in positions["planes_p"][:4]])
    lo = O.forward_f32(n, w, planes)
    ref = golden_refexact[f"logits_r{rot}"][:4]
    assert rel_logit_err(lo, ref).max() < 1e-5
    nv, wv = weights["ref_v"]
    pv = np.stack([O.rotate_planes(p, rot) for p in positions["planes_v"][:4]])
    v = O.forward_f32(nv, wv, pv)
    assert np.abs(v - golden_refexact[f"value_r{rot}"][:4]).max() < 1e-5


def test_scored_moves_unrotation_and_ladder(positions, golden_refexact, weights, oracle_mod):
    """Netresult assembly (Network.cpp:656-667, 820-829): softmax at the
    search temperature 0.75, un-rotate, EMPTY points only, losing ladders 0."""
    O = oracle_mod
    import leela_gb300 as lg
    n, w = weights["ref_p"]
    for rot in (0, 5):
        for i in range(3):
            planes = O.rotate_planes(positions["planes_p"][i], rot)[None]
            probs = O.softmax_f32(O.forward_f32(n, w, planes), 0.75)[0]
            sq = positions["squares"][i]
            ladder = positions["planes_p"][i][25]
            got = np.full(361, -1.0, dtype=np.float32)
            for idx in range(361):
                if sq[idx] == 2:
                    got[idx] = 0.0 if ladder[idx] else probs[lg.REV_ROTATE[rot][idx]]
            ref = golden_refexact[f"probs_r{rot}"][i]
            assert np.array_equal(got < 0, ref < 0)
            assert np.abs(got - ref).max() < 1e-6


def test_rotation_tables(oracle_mod):
    import leela_gb300 as lg
    for s in range(8):
        for v in range(361):
            assert oracle_mod.rotate_nn_idx(v, s) == lg.rotate_nn_idx(v, s)
            assert lg.rotate_nn_idx(lg.rev_rotate_nn_idx(v, s), s) == v


def test_softmax_edge_cases(oracle_mod):
    O = oracle_mod
    x = np.zeros(361, dtype=np.float32)
    p = O.softmax_f32(x, 1.0)
    assert np.allclose(p, 1.0 / 361)
    x = np.full(361, -1e4, dtype=np.float32)
    x[7] = 80.0
    p = O.softmax_f32(x, 0.75)
    assert p[7] == 1.0 and np.isfinite(p).all()
    x = np.random.default_rng(0).normal(size=361).astype(np.float32) * 40
    p32 = O.softmax_f32(x, 0.75)
    p64 = O.softmax_f64(x.astype(np.float64), 0.75)
    assert np.abs(p32 - p64).max() < 1e-6


def test_e4m3_rounding(oracle_mod):
    r = oracle_mod.e4m3_round
    assert r(448.0) == 448.0 and r(1000.0) == 448.0 and r(-1000.0) == -448.0
    assert r(1.0) == 1.0 and r(1.0625) == 1.0 and r(1.1875) == 1.25  # ties to even
    assert r(2.0 ** -9) == 2.0 ** -9 and r(2.0 ** -11) == 0.0
    assert r(0.3) == 0.3125 - 0.0 or abs(r(0.3) - 0.3) <= 2.0 ** -5


def test_mcowner_labels_in_range():
    d = np.load(os.path.join(GOLDEN, "mcowner_s0.npz"))["mcowner"]
    assert d.shape == (1024,) and np.all((d >= 0) & (d <= 1))


def test_config2_fixture_weight_rounding_caps():
    """The precision fixture's own finding (FP64 arithmetic, exact
    activations, 16-bit weights, first 8,192 of its positions): weights
    rounded to BF16 alone keep the FP64 top-1 below 99%, FP16 weights above."""
    d = np.load(os.path.join(os.path.dirname(__file__), "golden", "config2_f64.npz"))
    n = d["top1_w_bf16"].size
    cap_b = (d["top1_w_bf16"] == d["top1"][:n]).mean()
    cap_h = (d["top1_w_fp16"] == d["top1"][:n]).mean()
    assert cap_b < 0.99 < cap_h


def test_config2_generator_reproduces_the_fixture(oracle_mod):
    """oracle.config_boards regenerates the precision fixture's 65,536 boards
    bit for bit (the GPU test regenerates them on its own host)."""
    import hashlib
    d = np.load(os.path.join(os.path.dirname(__file__), "golden", "config2_f64.npz"))
    sq, tm, mv = oracle_mod.config_boards(int(d["n"]), int(d["seed"]))
    assert hashlib.sha256(sq.tobytes()).hexdigest()[:16] == str(d["squares_sha256"])
    assert hashlib.sha256(tm.tobytes()).hexdigest()[:16] == str(d["to_move_sha256"])
    # positions of the configurations' kind: stone density near the fixture's
    assert 0.2 < (sq != 2).mean() < 0.45 and (mv[:, 3] == 1).all()


def test_config4_labels_fixture(oracle_mod):
    """The learned fast path's value labels (tests/golden/make_config4.py):
    one Playout::mc_owner(64) win rate of the side to move per position of
    oracle.config_boards(n, seed 4), stored exactly as multiples of 1/128;
    the generator reproduces the boards they belong to."""
    import hashlib
    d = np.load(os.path.join(GOLDEN, "config4_mcowner.npz"))
    n = int(d["n"])
    w = d["winrate_x128"]
    assert n == 1 << 20 and w.shape == (n,) and int(d["playouts"]) == 64
    assert w.max() <= 128 and 0.45 < w.mean() / 128 < 0.55
    sq, tm, _ = oracle_mod.config_boards(n, int(d["seed"]))
    assert hashlib.sha256(sq.tobytes()).hexdigest()[:16] == str(d["squares_sha256"])
    assert hashlib.sha256(tm.tobytes()).hexdigest()[:16] == str(d["to_move_sha256"])


def test_config4_labels_agree_with_a_fresh_reference_labelling(oracle_mod):
    """Where the reference sources are at hand (LEELA_REF), the reference's
    own mc_owner(64) run again on the first 512 positions (other random
    playouts) agrees with the stored labels as two 64-playout estimates of
    one win rate do: mean absolute difference below 0.1, correlation above
    0.8."""
    import subprocess
    import tempfile
    ref = os.environ.get("LEELA_REF")
    if not ref or not os.path.isdir(ref):
        pytest.skip("LEELA_REF not set")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    subprocess.run(["make", "-s", "-j8", "-C", os.path.join(root, "oracle"), "ref", f"REF={ref}"], check=True)
    d = np.load(os.path.join(GOLDEN, "config4_mcowner.npz"))
    n = 512
    sq, tm, mv = oracle_mod.config_boards(n, int(d["seed"]))
    with tempfile.TemporaryDirectory() as td:
        pre = os.path.join(td, "c")
        sq.tofile(pre + ".sq")
        tm.tofile(pre + ".tm")
        mv.tofile(pre + ".mv")
        subprocess.run([os.path.join(root, "oracle", "_ref", "ref_harness"), "mcfile", pre + ".sq", pre + ".tm",
                        pre + ".mv", str(n), "64", str(min(8, os.cpu_count() or 1)), pre], check=True,
                       stderr=subprocess.DEVNULL)
        w = np.fromfile(pre + ".mcowner", np.float32)
    stored = d["winrate_x128"][:n] / 128.0
    assert np.abs(w - stored).mean() < 0.1
    assert np.corrcoef(w, stored)[0, 1] > 0.8
