"""FP32 drop-in path on the GPU against the reference's CPU/BLAS outputs
(tests/golden) and the CPU oracle.  Bar: same top-1 move and norm-wise
relative logit error max|a-b|/max|b| <= 1e-4 per position."""
import numpy as np
import pytest

from conftest import rel_logit_err

pytestmark = pytest.mark.gpu

LOGIT_TOL = 1e-4


@pytest.fixture(scope="module")
def ctx_cfg(gpu_lib, weights):
    lg = gpu_lib
    c = lg.Context(policy=lg.NetDesc.config1_policy(weights["cfg_p"][1]),
                   value=lg.NetDesc.config1_value(weights["cfg_v"][1]), max_batch=256)
    yield c
    c.close()


@pytest.fixture(scope="module")
def ctx_ref(gpu_lib, weights):
    lg = gpu_lib
    c = lg.Context(policy=lg.NetDesc.reference_policy(weights["ref_p"][1]),
                   value=lg.NetDesc.reference_value(weights["ref_v"][1]), max_batch=64)
    yield c
    c.close()


@pytest.mark.parametrize("rot", [0, 3])
def test_config1_policy_vs_reference(ctx_cfg, gpu_lib, positions, golden_config1, rot):
    planes = gpu_lib.rotate_planes(positions["planes_p"][:64, :24], rot)
    probs, logits = ctx_cfg.policy(planes, 1.0, return_logits=True)
    ref = golden_config1[f"logits_r{rot}"]
    err = rel_logit_err(logits, ref)
    assert err.max() <= LOGIT_TOL, err.max()
    assert np.array_equal(logits.argmax(1), ref.argmax(1))
    assert np.abs(probs - golden_config1[f"probs_r{rot}"]).max() < 1e-6


def test_config1_value_vs_reference(ctx_cfg, positions, golden_config1):
    v = ctx_cfg.value(positions["planes_v"][:64, :24])
    assert np.abs(v - golden_config1["value_r0"]).max() < 1e-5


@pytest.mark.parametrize("rot", [0, 5])
def test_reference_shaped_nets_vs_reference(ctx_ref, gpu_lib, positions, golden_refexact, rot):
    """The reference's own shapes (ELU, 3x3 heads, 32->96->128 / 64-wide)."""
    planes = gpu_lib.rotate_planes(positions["planes_p"][:64], rot)
    _, logits = ctx_ref.policy(planes, 0.75, return_logits=True)
    ref = golden_refexact[f"logits_r{rot}"]
    assert rel_logit_err(logits, ref).max() <= LOGIT_TOL
    assert np.array_equal(logits.argmax(1), ref.argmax(1))
    pv = gpu_lib.rotate_planes(positions["planes_v"][:64], rot)
    v = ctx_ref.value(pv)
    assert np.abs(v - golden_refexact[f"value_r{rot}"]).max() < 1e-5


def test_scored_moves_vs_reference_netresult(ctx_ref, gpu_lib, positions, golden_refexact):
    """get_scored_moves: rotation, EMPTY filter and ladder pruning exactly as
    Network::get_scored_moves(DIRECT, rot) returns them."""
    for rot in (0, 5):
        for i in range(8):
            res = gpu_lib.get_scored_moves(ctx_ref, positions["planes_p"][i],
                                           positions["squares"][i], positions["planes_p"][i][25],
                                           rotation=rot, temperature=0.75)
            ref = golden_refexact[f"probs_r{rot}"][i]
            assert [p for _, p in res] == [int(j) for j in np.nonzero(ref >= 0)[0]]
            got = np.array([v for v, _ in res])
            assert np.abs(got - ref[ref >= 0]).max() < 1e-6


@pytest.mark.parametrize("B", [1, 3, 8, 257])
def test_batch_sizes_vs_oracle(ctx_cfg, positions, weights, oracle_mod, B):
    """Ragged and oversize batches (257 > max_batch splits into two calls)."""
    O = oracle_mod
    idx = np.arange(B) % 1024
    planes = positions["planes_p"][idx, :24]
    O.enable_blas()
    try:
        ref = O.forward_f32(weights["cfg_p"][0], weights["cfg_p"][1], planes)
        vref = O.forward_f32(weights["cfg_v"][0], weights["cfg_v"][1],
                             positions["planes_v"][idx, :24])
    finally:
        O.disable_blas()
    _, logits = ctx_cfg.policy(planes, 1.0, return_logits=True)
    assert rel_logit_err(logits, ref).max() <= LOGIT_TOL
    assert np.array_equal(logits.argmax(1), ref.argmax(1))
    v = ctx_cfg.value(positions["planes_v"][idx, :24])
    assert np.abs(v - vref).max() < 1e-5


def test_empty_batch(ctx_cfg):
    out = ctx_cfg.policy(np.zeros((0, 24, 361), np.uint8))
    assert out.shape == (0, 361)


def test_empty_board_and_full_planes(ctx_cfg, weights, oracle_mod):
    """Extreme inputs: all-zero planes and all-one planes."""
    O = oracle_mod
    planes = np.stack([np.zeros((24, 361), np.uint8), np.ones((24, 361), np.uint8)])
    _, logits = ctx_cfg.policy(planes, 1.0, return_logits=True)
    ref = O.forward_f32(weights["cfg_p"][0], weights["cfg_p"][1], planes)
    assert rel_logit_err(logits, ref).max() <= LOGIT_TOL


def test_device_entry_points_match_host(ctx_cfg, positions):
    import torch
    planes = np.ascontiguousarray(positions["planes_p"][:16, :24])
    host_probs = ctx_cfg.policy(planes, 0.75)
    d_planes = torch.from_numpy(planes).cuda()
    d_probs = torch.empty((16, 361), dtype=torch.float32, device="cuda")
    s = torch.cuda.current_stream()
    ctx_cfg.policy_device(d_planes.data_ptr(), 16, d_probs.data_ptr(), 0.75, None, s.cuda_stream)
    s.synchronize()
    assert np.abs(d_probs.cpu().numpy() - host_probs).max() < 1e-6
    pv = torch.from_numpy(np.ascontiguousarray(positions["planes_v"][:16, :24])).cuda()
    d_v = torch.empty(16, dtype=torch.float32, device="cuda")
    ctx_cfg.value_device(pv.data_ptr(), 16, d_v.data_ptr(), s.cuda_stream)
    s.synchronize()
    assert np.abs(d_v.cpu().numpy() - ctx_cfg.value(positions["planes_v"][:16, :24])).max() < 1e-6


def test_avg8_ensemble_matches_oracle(gpu_lib, weights, positions, oracle_mod):
    """AVERAGE_ALL (Network.cpp:642-654, 606-615): the device ensemble equals
    the average of the 8 rotated oracle evaluations, un-rotated."""
    import torch
    lg, O = gpu_lib, oracle_mod
    B = 3
    pp = np.ascontiguousarray(positions["planes_p"][:B, :24])
    pv = np.ascontiguousarray(positions["planes_v"][:B, :24])
    with lg.Context(policy=lg.NetDesc.config1_policy(weights["cfg_p"][1]),
                    value=lg.NetDesc.config1_value(weights["cfg_v"][1]), max_batch=32) as c:
        out = torch.empty((B, 361), device="cuda")
        val = torch.empty(B, device="cuda")
        s = torch.cuda.current_stream()
        c.policy_avg8_device(torch.from_numpy(pp).cuda().data_ptr(), B, out.data_ptr(), 0.75,
                             s.cuda_stream)
        c.value_avg8_device(torch.from_numpy(pv).cuda().data_ptr(), B, val.data_ptr(), s.cuda_stream)
        s.synchronize()
    O.enable_blas()
    try:
        ref = np.zeros((B, 361))
        vref = np.zeros(B)
        for r in range(8):
            rp = np.stack([O.rotate_planes(x, r) for x in pp])
            pr = O.softmax_f32(O.forward_f32(weights["cfg_p"][0], weights["cfg_p"][1], rp), 0.75)
            ref += pr[:, lg.REV_ROTATE[r]]
            rv = np.stack([O.rotate_planes(x, r) for x in pv])
            vref += O.forward_f32(weights["cfg_v"][0], weights["cfg_v"][1], rv)
    finally:
        O.disable_blas()
    assert np.abs(out.cpu().numpy() - ref / 8).max() < 1e-6
    assert np.abs(val.cpu().numpy() - vref / 8).max() < 1e-5


@pytest.mark.parametrize("B", [1, 2, 5, 8])
@pytest.mark.parametrize("shapes", ["config1", "reference"])
def test_small_batch_kernel_matches_per_layer_path(gpu_lib, weights, positions, B, shapes):
    """The small-batch kernel (every layer in one launch, 8-way input-channel
    splits summed in a fixed order) against the per-layer FP32 kernels, for
    the benchmark nets and the reference's own shapes (ELU, 3x3 heads,
    32->96->128 and 64-wide value trunk, (1+tanh)/2): same top-1, logits
    within 1e-5 norm-wise, probabilities within 1e-6, values within 1e-5."""
    lg = gpu_lib
    if shapes == "config1":
        pol = lg.NetDesc.config1_policy(weights["cfg_p"][1])
        val = lg.NetDesc.config1_value(weights["cfg_v"][1])
        pp, pv = positions["planes_p"][:B, :24], positions["planes_v"][:B, :24]
    else:
        pol = lg.NetDesc.reference_policy(weights["ref_p"][1])
        val = lg.NetDesc.reference_value(weights["ref_v"][1])
        pp, pv = positions["planes_p"][:B], positions["planes_v"][:B]
    with lg.Context(policy=pol, value=val, max_batch=8) as c:
        assert c.tuning(B)["conv3x3"] == 4  # the default for small batches
        c.set_tuning(B, 0, 0)
        p0, l0 = c.policy(pp, 0.75, return_logits=True)
        v0 = c.value(pv)
        c.set_tuning(B, 4, 0)
        n0 = c.stats()["kernel_launches"]
        p4, l4 = c.policy(pp, 0.75, return_logits=True)
        v4 = c.value(pv)
        assert c.stats()["kernel_launches"] - n0 == 2  # one launch per net
    assert rel_logit_err(l4, l0).max() <= 1e-5
    assert np.array_equal(l4.argmax(1), l0.argmax(1))
    assert np.abs(p4 - p0).max() < 1e-6
    assert np.abs(v4 - v0).max() < 1e-5


def test_small_batch_kernel_repeated_calls(gpu_lib, weights, positions):
    """Counters reset between launches: many calls in a row on one stream
    (alternating batch sizes, so that rows unused by one call are used by
    the next) give the same answer every time."""
    lg = gpu_lib
    with lg.Context(policy=lg.NetDesc.config1_policy(weights["cfg_p"][1]),
                    value=lg.NetDesc.config1_value(weights["cfg_v"][1]), max_batch=8) as c:
        ref1 = c.policy(positions["planes_p"][:1, :24])
        ref8 = c.policy(positions["planes_p"][:8, :24])
        vref = c.value(positions["planes_v"][:8, :24])
        for i in range(20):
            assert np.array_equal(c.policy(positions["planes_p"][:1, :24]), ref1)
            assert np.array_equal(c.policy(positions["planes_p"][:8, :24]), ref8)
            assert np.array_equal(c.value(positions["planes_v"][:8, :24]), vref)


@pytest.mark.parametrize("fc_hidden", [64, 192, 256, 320])
def test_value_head_widths_vs_fp64(gpu_lib, oracle_mod, positions, fc_hidden):
    """The value head's FC chain at several widths against the FP64 oracle
    (FP32 nets, small trunk): up to 256 hidden units it runs on clusters of
    2 x ceil(H/64) CTAs (64 and 192 leave a partial or odd cluster), wider
    heads on the split-K kernel whose last CTAs finish the reduction.  Over
    more than one chunk (max_batch 32, 70 positions) and at batch 1."""
    lg, O = gpu_lib, oracle_mod
    shape = dict(c_in=24, width1=64, width=64, n3x3=2, head_k=1, act=O.RELU, act_head=1,
                 value_head=1, fc_hidden=fc_hidden, value_map=0)
    n = O.make_net(shape)
    w = O.he_weights(n, 11)
    src = positions["planes_v"][:70, :24]
    O.enable_blas()
    try:
        ref = O.forward_f64(n, w, src)
    finally:
        O.disable_blas()
    with lg.Context(value=lg.NetDesc(w, **shape, precision="fp32"), max_batch=32) as c:
        v = c.value(src)
        v1 = c.value(src[:1])
    assert np.abs(v - ref).max() < 1e-5
    assert np.abs(v1 - ref[:1]).max() < 1e-5
