"""BF16, FP16 and FP8-weight tensor-core paths against the FP64 host oracle.

Tolerances (stated per result, on the benchmark nets with He-normal weights,
64 positions; the top-1 agreement at scale is asserted over 65,536 positions
in test_config2_precision.py):
  top-1 agreement with FP64              >= 95%
  policy probabilities, max |p - p64|    <= 2e-3
  norm-wise logit error max|a-b|/max|b|  <= 5e-2 (FP16: 1e-2)
  value, max |v - v64|                   <= 3e-2 (FP16: 5e-3)
"""
import numpy as np
import pytest

from conftest import rel_logit_err

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def f64_refs(positions, weights, oracle_mod):
    """FP64 oracle outputs with exact weights ('exact') and with the weights
    each variant defines ('bf16': BF16-rounded, 'fp16': FP16-rounded, 'fp8w':
    E4M3 per output channel, BF16 FC)."""
    O = oracle_mod
    pp, pv = positions["planes_p"][:64, :24], positions["planes_v"][:64, :24]
    (P, wp), (V, wv) = weights["cfg_p"], weights["cfg_v"]
    out = {}
    O.enable_blas()
    try:
        for mode in ("exact", "bf16", "fp16", "fp8w"):
            qmode = {"fp8w": "fp8"}.get(mode, mode)
            qp = wp if mode == "exact" else O.quantize_weights(P, wp, qmode)
            qv = wv if mode == "exact" else O.quantize_weights(V, wv, qmode)
            lp = O.forward_f64(P, qp, pp)
            out[mode] = (lp, O.softmax_f64(lp, 1.0), O.forward_f64(V, qv, pv))
    finally:
        O.disable_blas()
    return out


@pytest.mark.parametrize("prec", ["bf16", "fp16", "fp8w"])
def test_lowp_vs_fp64(gpu_lib, weights, positions, f64_refs, prec):
    """Against the FP64 oracle run with the variant's own weights, the only
    error left is the activation rounding: top-1 >= 95%, probabilities
    within 2e-3, norm-wise logit error <= 5e-2, value within 3e-2 (FP16, with
    three more mantissa bits: 1e-2 and 5e-3).  Against the exact weights,
    BF16 and FP16 meet the same bars; E4M3 weights carry their own
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
        if ref_kind == prec or prec in ("bf16", "fp16"):
            assert agree >= 0.95
            assert perr <= 2e-3
            assert lerr <= (1e-2 if prec == "fp16" else 5e-2)
            assert verr <= (5e-3 if prec == "fp16" else 3e-2)
        else:
            assert lerr <= 0.6
            assert verr <= 0.1


def test_bf16_batch_independent(gpu_lib, weights, positions):
    """For one kernel choice, a position's result does not depend on its
    batch or its slot in it (bit for bit).  (Buckets of up to 8 positions
    default to the small-batch kernel, whose FP32 sums run in another
    order; here they are set to the per-layer kernels.)"""
    lg = gpu_lib
    with lg.Context(policy=lg.NetDesc.config1_policy(weights["cfg_p"][1], "bf16"),
                    max_batch=64) as c:
        c.set_tuning(1, 0, 0)
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


@pytest.mark.parametrize("prec", ["bf16", "fp16", "fp8w"])
def test_chunked_device_call_equals_one_call_per_chunk(gpu_lib, weights, positions, prec):
    """A device call over several chunks packs chunk k+1's planes in the CTAs
    of chunk k's finish launch (softmax, or the value head).  The results
    equal those of calling each chunk alone, bit for bit: when every chunk
    runs on the trunk, and when the last chunk runs on the small-batch
    kernel (which reads the planes, so nothing is packed for it)."""
    import torch
    lg = gpu_lib
    mb = 64
    with lg.Context(policy=lg.NetDesc.config1_policy(weights["cfg_p"][1], prec),
                    value=lg.NetDesc.config1_value(weights["cfg_v"][1], prec), max_batch=mb) as c:
        c.set_tuning(mb, 3, 0)  # buckets 33..64: the trunk with the first layer inside
        c.set_tuning(5, 4, 0)   # buckets 5..8: the small-batch kernel
        s = torch.cuda.current_stream()
        for B in (4 * mb + 5, 3 * mb + 40):
            pp = torch.from_numpy(np.ascontiguousarray(positions["planes_p"][:B, :24])).cuda()
            pv = torch.from_numpy(np.ascontiguousarray(positions["planes_v"][:B, :24])).cuda()
            probs = torch.empty((B, 361), device="cuda")
            logits = torch.empty((B, 361), device="cuda")
            vals = torch.empty(B, device="cuda")
            c.policy_device(pp.data_ptr(), B, probs.data_ptr(), 1.0, logits.data_ptr(), s.cuda_stream)
            c.value_device(pv.data_ptr(), B, vals.data_ptr(), s.cuda_stream)
            probs1 = torch.empty_like(probs)
            logits1 = torch.empty_like(logits)
            vals1 = torch.empty_like(vals)
            for b0 in range(0, B, mb):
                nb = min(mb, B - b0)
                c.policy_device(pp[b0].data_ptr(), nb, probs1[b0].data_ptr(), 1.0, logits1[b0].data_ptr(),
                                s.cuda_stream)
                c.value_device(pv[b0].data_ptr(), nb, vals1[b0].data_ptr(), s.cuda_stream)
            s.synchronize()
            assert torch.equal(probs, probs1), B
            assert torch.equal(logits, logits1), B
            assert torch.equal(vals, vals1), B


def test_lowp_rejects_unsupported_shape(gpu_lib, weights):
    lg = gpu_lib
    with pytest.raises(lg.LeelaGPUError):
        lg.Context(policy=lg.NetDesc.reference_policy(weights["ref_p"][1], "bf16"), max_batch=4)


@pytest.mark.parametrize("value_head", [0, 1])
def test_bf16_64_wide_net(gpu_lib, oracle_mod, positions, value_head):
    """64-wide nets (the distilled-net shape: 5x5 24->64, 5x 3x3 64->64, 1x1
    head) run on the M=128-rows tensor-core kernel; same bars as above
    against the FP64 oracle with BF16-rounded weights."""
    lg, O = gpu_lib, oracle_mod
    shape = dict(c_in=24, width1=64, width=64, n3x3=5, head_k=1, act=O.RELU, act_head=0,
                 value_head=value_head, fc_hidden=64 if value_head else 0, value_map=0)
    n = O.make_net(shape)
    w = O.he_weights(n, 7)
    src = positions["planes_v" if value_head else "planes_p"][:64, :24]
    O.enable_blas()
    try:
        ref = O.forward_f64(n, O.quantize_weights(n, w, "bf16"), src)
    finally:
        O.disable_blas()
    desc = lg.NetDesc(w, **shape, precision="bf16")
    with lg.Context(policy=None if value_head else desc, value=desc if value_head else None,
                    max_batch=64) as c:
        if value_head:
            v = c.value(src)
            assert np.abs(v - ref).max() <= 3e-2
        else:
            _, logits = c.policy(src, 1.0, return_logits=True)
            assert (logits.argmax(1) == ref.argmax(1)).mean() >= 0.95
            assert rel_logit_err(logits, ref).max() <= 5e-2


@pytest.mark.parametrize("c_in", [24, 18])
def test_bf16_planes_with_other_byte_values(gpu_lib, oracle_mod, positions, c_in):
    """Plane bytes other than 0/1 reach the first layer exactly: doubling
    plane 1's bytes gives, bit for bit, what doubling plane 1's first-layer
    weights gives (x2 is exact in FP32 and in BF16).  The two calls take the
    packing kernel's two paths (byte conversion; 0/1 bit masks)."""
    lg, O = gpu_lib, oracle_mod
    n = 24
    shape = dict(c_in=c_in, width1=128, width=128, n3x3=2, head_k=1, act=O.RELU, act_head=0,
                 value_head=0, fc_hidden=0, value_map=0)
    w = O.he_weights(O.make_net(shape), 11)
    w2 = w.copy()
    w2[:128 * c_in * 25].reshape(128, c_in, 25)[:, 1, :] *= 2
    planes = np.ascontiguousarray(positions["planes_p"][:n, :c_in])
    doubled = planes.copy()
    doubled[:, 1] *= 2
    assert doubled.max() == 2

    def desc(ww):
        return lg.NetDesc(ww, c_in, 128, 128, 2, 1, O.RELU, 0, 0, precision="bf16")

    with lg.Context(policy=desc(w), max_batch=32) as a, lg.Context(policy=desc(w2), max_batch=32) as b:
        _, la = a.policy(doubled, 1.0, return_logits=True)
        _, lb = b.policy(planes, 1.0, return_logits=True)
    assert np.array_equal(la, lb)


@pytest.mark.parametrize("prec", ["bf16", "fp16", "fp8w"])
@pytest.mark.parametrize("B", [1, 3, 8])
def test_small_batch_kernel_lowp(gpu_lib, weights, positions, f64_refs, prec, B):
    """Choice 4 -- the whole net in one launch, the 3x3 layers on the warp
    MMA, the first layer and the head in FP32 on the rounded weights -- rounds
    the activations where the tensor-core trunk does; only the order of the
    FP32 sums differs.  Same bars against the FP64 oracle (with the variant's
    own weights) as the batched kernels, one launch per net, and within the
    same distance of the per-layer kernels' results."""
    lg = gpu_lib
    pp, pv = positions["planes_p"][:B, :24], positions["planes_v"][:B, :24]
    with lg.Context(policy=lg.NetDesc.config1_policy(weights["cfg_p"][1], prec),
                    value=lg.NetDesc.config1_value(weights["cfg_v"][1], prec), max_batch=8) as c:
        c.set_tuning(B, 0, 0)
        _, l0 = c.policy(pp, 1.0, return_logits=True)
        v0 = c.value(pv)
        c.set_tuning(B, 4, 0)
        n0 = c.stats()["kernel_launches"]
        _, l4 = c.policy(pp, 1.0, return_logits=True)
        v4 = c.value(pv)
        assert c.stats()["kernel_launches"] - n0 == 2
    lp64, _, v64 = f64_refs[prec]
    lbar, vbar = (1e-2, 5e-3) if prec == "fp16" else (5e-2, 3e-2)
    assert rel_logit_err(l4, lp64[:B]).max() <= lbar
    assert np.abs(v4 - v64[:B]).max() <= vbar
    assert rel_logit_err(l4, l0).max() <= lbar
    assert np.abs(v4 - v0).max() <= vbar


def test_chained_and_pipelined_calls_random_sizes(gpu_lib, weights, positions):
    """Many call sizes (seeded: ragged last chunks, small-batch tails, one and
    many chunks) through the chained device calls and the pipelined board
    calls, each compared bit for bit with one call per chunk.  The launches
    of a chained call overlap (programmatic dependent launches, two
    first-layer buffers, a ring of board slots), so this guards the order
    of their reads and writes."""
    import torch
    lg = gpu_lib
    mb = 128
    rng = np.random.default_rng(7)
    sizes = [int(x) for x in rng.integers(1, 6 * mb, size=12)] + [mb + 1, 2 * mb, 3 * mb + 7]
    with lg.Context(policy=lg.NetDesc.config1_policy(weights["cfg_p"][1], "bf16"),
                    value=lg.NetDesc.config1_value(weights["cfg_v"][1], "bf16"), max_batch=mb) as c:
        c.set_tuning(mb, 3, 0)     # buckets 65..128: the trunk
        c.set_tuning(64, 3, 0)     # 33..64
        c.set_tuning(32, 2, 0)     # 17..32: trunk, first layer in its own launch
        c.set_tuning(16, 0, 0)     # 9..16: per-layer kernels
        c.set_tuning(8, 4, 0)      # 1..8: the small-batch kernel
        s = torch.cuda.current_stream()
        for B in sizes:
            idx = (np.arange(B) * 7 + B) % 1024
            pp_h = np.ascontiguousarray(positions["planes_p"][idx, :24])
            pv_h = np.ascontiguousarray(positions["planes_v"][idx, :24])
            pp, pv = torch.from_numpy(pp_h).cuda(), torch.from_numpy(pv_h).cuda()
            probs = torch.empty((B, 361), device="cuda")
            vals = torch.empty(B, device="cuda")
            c.policy_device(pp.data_ptr(), B, probs.data_ptr(), 1.0, None, s.cuda_stream)
            c.value_device(pv.data_ptr(), B, vals.data_ptr(), s.cuda_stream)
            p1 = torch.empty_like(probs)
            v1 = torch.empty_like(vals)
            for b0 in range(0, B, mb):
                nb = min(mb, B - b0)
                c.policy_device(pp[b0].data_ptr(), nb, p1[b0].data_ptr(), 1.0, None, s.cuda_stream)
                c.value_device(pv[b0].data_ptr(), nb, v1[b0].data_ptr(), s.cuda_stream)
            s.synchronize()
            assert torch.equal(probs, p1), B
            assert torch.equal(vals, v1), B
            # the same positions from boards (pipelined when B > max_batch)
            sq, tm = positions["squares"][idx], positions["meta"][idx, 0]
            pb = c.policy_boards(sq, tm)
            vb = c.value_boards(sq, tm)
            assert np.array_equal(pb, p1.cpu().numpy()), B
            assert np.array_equal(vb, v1.cpu().numpy()), B
        assert c.device_error() == 0


@pytest.mark.parametrize("B,choice", [(32, 3), (1, 4)])
def test_avg8_ensemble_on_tensor_cores(gpu_lib, weights, positions, oracle_mod, B, choice):
    """AVERAGE_ALL on the BF16 path (Network.cpp:642-654, 606-615): the 8
    rotated copies of each position run as one batch (8 x 32 = 256 through
    the persistent trunk; 8 x 1 through the small-batch kernel), then are
    un-rotated and averaged in symmetry order.  Bit for bit the same as the
    plane-input calls on the rotated planes (board-major, symmetry-minor),
    averaged in float32 in the same order."""
    import torch
    lg, O = gpu_lib, oracle_mod
    pp = np.ascontiguousarray(positions["planes_p"][:B, :24])
    pv = np.ascontiguousarray(positions["planes_v"][:B, :24])
    rp = np.stack([O.rotate_planes(x, r) for x in pp for r in range(8)])
    rv = np.stack([O.rotate_planes(x, r) for x in pv for r in range(8)])
    with lg.Context(policy=lg.NetDesc.config1_policy(weights["cfg_p"][1], "bf16"),
                    value=lg.NetDesc.config1_value(weights["cfg_v"][1], "bf16"), max_batch=256) as c:
        c.set_tuning(8 * B, choice, 0)
        out = torch.empty((B, 361), device="cuda")
        val = torch.empty(B, device="cuda")
        s = torch.cuda.current_stream()
        c.policy_avg8_device(torch.from_numpy(pp).cuda().data_ptr(), B, out.data_ptr(), 0.75, s.cuda_stream)
        c.value_avg8_device(torch.from_numpy(pv).cuda().data_ptr(), B, val.data_ptr(), s.cuda_stream)
        s.synchronize()
        p8 = c.policy(rp, 0.75)
        v8 = c.value(rv)
    ref = np.zeros((B, 361), np.float32)
    vref = np.zeros(B, np.float32)
    for r in range(8):
        ref = ref + p8[r::8][:, lg.REV_ROTATE[r]]
        vref = vref + v8[r::8]
    assert np.array_equal(out.cpu().numpy(), ref / np.float32(8))
    assert np.array_equal(val.cpu().numpy(), vref / np.float32(8))
