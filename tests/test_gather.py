"""GPU input-plane gather (lg_gather_device) and the board-input evaluation
calls (lg_policy_boards / lg_value_boards).

Bit-exact: the gathered planes equal the reference gather's planes 0..23 on
the 1024 fixture positions, and the oracle's on random boards (dense ones,
with captures) and hand-built edge cases.  The board-input calls return
exactly what the plane-input calls return on the gathered planes."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

POINTS = 361


def _gather(lg, squares, to_move, which, nplanes=24, moves=None):
    import torch
    sq = torch.from_numpy(np.array(squares, dtype=np.int8).reshape(-1, POINTS)).cuda()
    B = sq.shape[0]
    tm = torch.from_numpy(np.array(np.broadcast_to(np.asarray(to_move, dtype=np.int8), (B,)))).cuda()
    mv = None if moves is None else torch.from_numpy(np.array(moves, dtype=np.int32).reshape(B, 4)).cuda()
    out = torch.full((max(B, 1), nplanes, POINTS), 7, dtype=torch.uint8, device="cuda")
    s = torch.cuda.current_stream().cuda_stream
    lg.gather_device(sq.data_ptr(), tm.data_ptr(), B, which, nplanes, out.data_ptr(), s,
                     None if mv is None else mv.data_ptr())
    torch.cuda.synchronize()
    return out[:B].cpu().numpy()


def _synthetic_moves(squares, to_move, seed):
    """Last move = a stone of the side that just moved, the move before = a
    stone of the side to move (or -1), a ko point on some boards, komi on
    most -- the extra inputs planes 24..31 read."""
    rng = np.random.default_rng(seed)
    mv = np.full((len(squares), 4), -1, np.int32)
    for i, (sq, tm) in enumerate(zip(squares, to_move)):
        last = np.flatnonzero(sq == 1 - tm)
        prev = np.flatnonzero(sq == tm)
        empty = np.flatnonzero(sq == 2)
        if last.size and rng.random() < 0.9:
            mv[i, 0] = rng.choice(last)
            if prev.size and rng.random() < 0.9:
                mv[i, 1] = rng.choice(prev)
        if empty.size and rng.random() < 0.2:
            mv[i, 2] = rng.choice(empty)
        mv[i, 3] = int(rng.random() < 0.8)
    return mv


@pytest.mark.parametrize("which,key", [(0, "planes_p"), (1, "planes_v")])
def test_gather_matches_reference_planes(gpu_lib, positions, which, key):
    got = _gather(gpu_lib, positions["squares"], positions["meta"][:, 0], which)
    ref = positions[key][:, :24]
    bad = np.argwhere(got != ref)
    assert bad.size == 0, bad[:5]


@pytest.mark.parametrize("which,key", [(0, "planes_p"), (1, "planes_v")])
def test_gather_all_32_planes_match_reference(gpu_lib, positions, which, key):
    """Ladders, ko, the last two moves, komi and the third line too."""
    got = _gather(gpu_lib, positions["squares"], positions["meta"][:, 0], which, 32, positions["moves"])
    bad = np.argwhere(got != positions[key])
    assert bad.size == 0, bad[:5]


@pytest.mark.parametrize("seed,kmax", [(4, 250), (5, 350)])
def test_gather_32_planes_match_oracle_on_random_boards(gpu_lib, oracle_mod, seed, kmax):
    sq, tm = oracle_mod.random_boards(256, seed, kmax=kmax)
    mv = _synthetic_moves(sq, tm, seed)
    for which in (0, 1):
        got = _gather(gpu_lib, sq, tm, which, 32, mv)
        ref = oracle_mod.gather_planes(sq, tm, which, 32, mv)
        assert (got == ref).all(), np.argwhere(got != ref)[:5]


@pytest.mark.parametrize("seed,kmax", [(1, 250), (2, 400), (3, 600)])
def test_gather_matches_oracle_on_random_boards(gpu_lib, oracle_mod, seed, kmax):
    sq, tm = oracle_mod.random_boards(256, seed, kmax=kmax)
    for which in (0, 1):
        got = _gather(gpu_lib, sq, tm, which)
        ref = oracle_mod.gather_planes(sq, tm, which)
        assert (got == ref).all(), np.argwhere(got != ref)[:5]


def _edge_boards():
    boards = []
    boards.append(np.full(POINTS, 2, np.int8))                      # empty board
    b = np.full(POINTS, 2, np.int8); b[0] = 0; boards.append(b)     # one corner stone
    b = np.full(POINTS, 0, np.int8); b[[0, 200]] = 2; boards.append(b)  # one string, 2 liberties
    b = np.full(POINTS, 0, np.int8); b[180] = 2; boards.append(b)   # one string, 1 liberty
    # a white stone in atari inside black: capture and after-move planes
    b = np.full(POINTS, 2, np.int8)
    b[[20 - 1, 20 + 1, 20 - 19]] = 0; b[20] = 1; boards.append(b)
    # a large white string with 1 liberty next to a black eye
    b = np.full(POINTS, 1, np.int8); b[0:19] = 0; b[19:38] = 1; b[5] = 2; b[360] = 2
    boards.append(b)
    # alternate rows of black and white with one gap each (long strings)
    b = np.empty(POINTS, np.int8)
    for y in range(19):
        b[y * 19:(y + 1) * 19] = y % 2
        b[y * 19 + (y * 7) % 19] = 2
    boards.append(b)
    return np.stack(boards)


def test_gather_edge_cases(gpu_lib, oracle_mod):
    sq = _edge_boards()
    for tm in (0, 1):
        for which in (0, 1):
            got = _gather(gpu_lib, sq, tm, which)
            ref = oracle_mod.gather_planes(sq, np.full(len(sq), tm), which)
            assert (got == ref).all(), (tm, which, np.argwhere(got != ref)[:5])


def test_gather_prefix_and_arguments(gpu_lib, positions):
    lg = gpu_lib
    sq, tm = positions["squares"][:8], positions["meta"][:8, 0]
    got = _gather(lg, sq, tm, 0, nplanes=18)
    assert (got == positions["planes_p"][:8, :18]).all()
    _gather(lg, sq[:0], tm[:0], 0)   # B = 0 is a no-op
    import torch
    dsq = torch.from_numpy(np.ascontiguousarray(sq)).cuda()
    dtm = torch.from_numpy(np.ascontiguousarray(tm.astype(np.int8))).cuda()
    out = torch.zeros((8, 32, POINTS), dtype=torch.uint8, device="cuda")
    for which, nplanes in ((0, 33), (0, 0), (2, 24), (0, 25)):  # 25: planes 24.. need moves
        with pytest.raises(lg.LeelaGPUError):
            lg.gather_device(dsq.data_ptr(), dtm.data_ptr(), 8, which, nplanes, out.data_ptr(), None)
    with pytest.raises(lg.LeelaGPUError):
        lg.gather_device(0, 0, 4, 0, 24, 0, None)
    torch.cuda.synchronize()


@pytest.mark.parametrize("prec", ["fp32", "bf16", "fp16", "fp8w"])
def test_board_calls_equal_plane_calls(gpu_lib, positions, weights, prec):
    lg = gpu_lib
    n = 160  # more than max_batch: two chunks plus a ragged one
    sq, tm = positions["squares"][:n], positions["meta"][:n, 0]
    with lg.Context(policy=lg.NetDesc.config1_policy(weights["cfg_p"][1], prec),
                    value=lg.NetDesc.config1_value(weights["cfg_v"][1], prec), max_batch=64) as c:
        pb, lb = c.policy_boards(sq, tm, 1.0, return_logits=True)
        vb = c.value_boards(sq, tm)
        pp, lp = c.policy(positions["planes_p"][:n, :24], 1.0, return_logits=True)
        vp = c.value(positions["planes_v"][:n, :24])
    assert np.array_equal(pb, pp) and np.array_equal(lb, lp) and np.array_equal(vb, vp)


@pytest.mark.parametrize("prec", ["bf16", "fp16"])
def test_board_call_pipeline_on_the_trunk(gpu_lib, positions, weights, prec):
    """Board calls over several chunks run as a pipeline: super-chunks of
    2048 positions through a ring of four slots (copies on their own stream,
    one gather launch per super-chunk, then the chained device path), a
    first one of one chunk and a short last one, all starting on chunk
    boundaries.  Bit for bit the plane calls' results: with the persistent
    trunk for full chunks, the small-batch kernel for a ragged last chunk,
    and, at 10,317 positions, seven super-chunks that wrap the ring."""
    lg = gpu_lib
    mb = 64
    with lg.Context(policy=lg.NetDesc.config1_policy(weights["cfg_p"][1], prec),
                    value=lg.NetDesc.config1_value(weights["cfg_v"][1], prec), max_batch=mb) as c:
        c.set_tuning(mb, 3, 0)  # buckets 33..64: the trunk with the first layer inside
        c.set_tuning(5, 4, 0)   # buckets 5..8: the small-batch kernel
        for n in (4 * mb + 5, 3 * mb + 40, 8 * mb + 5, 1024, 2048 + mb + 3, 5 * 2048 + 77):
            idx = np.arange(n) % 1024
            sq, tm = positions["squares"][idx], positions["meta"][idx, 0]
            pb, lb = c.policy_boards(sq, tm, 1.0, return_logits=True)
            vb = c.value_boards(sq, tm)
            pp, lp = c.policy(positions["planes_p"][idx, :24], 1.0, return_logits=True)
            vp = c.value(positions["planes_v"][idx, :24])
            assert np.array_equal(pb, pp) and np.array_equal(lb, lp) and np.array_equal(vb, vp), n


def test_board_calls_feed_32_plane_nets(gpu_lib, weights, positions):
    """The reference-shaped nets read all 32 planes: from boards + moves they
    give exactly what they give from the reference gather's planes (FP32);
    without moves the call is refused."""
    lg = gpu_lib
    n = 40
    sq, tm, mv = positions["squares"][:n], positions["meta"][:n, 0], positions["moves"][:n]
    with lg.Context(policy=lg.NetDesc.reference_policy(weights["ref_p"][1]),
                    value=lg.NetDesc.reference_value(weights["ref_v"][1]), max_batch=16) as c:
        with pytest.raises(lg.LeelaGPUError):
            c.policy_boards(sq[:2], tm[:2])
        pb = c.policy_boards(sq, tm, moves=mv)
        vb = c.value_boards(sq, tm, moves=mv)
        pp = c.policy(positions["planes_p"][:n])
        vp = c.value(positions["planes_v"][:n])
    assert np.array_equal(pb, pp) and np.array_equal(vb, vp)


@pytest.mark.parametrize("c_in", [32, 18])
def test_bf16_board_calls_write_the_first_layer_input(gpu_lib, oracle_mod, positions, c_in):
    """Tensor-core nets fed from boards take the first layer's expanded input
    rows straight from the gather (no planes, no packing pass): the same
    outputs, bit for bit, as from the reference gather's planes.  32 planes:
    160 channels in three 64-channel halves; 18 planes: groups of 8 channels
    that span two x shifts."""
    lg, O = gpu_lib, oracle_mod
    n = 40
    sq, tm, mv = positions["squares"][:n], positions["meta"][:n, 0], positions["moves"][:n]
    nets = {}
    for vh in (0, 1):
        fc = 256 if vh else 0
        shape = dict(c_in=c_in, width1=128, width=128, n3x3=2, head_k=1, act=O.RELU, act_head=0,
                     value_head=vh, fc_hidden=fc, value_map=0)
        w = O.he_weights(O.make_net(shape), 7 + vh)
        nets[vh] = lg.NetDesc(w, c_in, 128, 128, 2, 1, O.RELU, 0, vh, fc, 0, precision="bf16")
    kw = dict(moves=mv) if c_in > 24 else {}
    with lg.Context(policy=nets[0], value=nets[1], max_batch=16) as c:
        pb, lb = c.policy_boards(sq, tm, 1.0, return_logits=True, **kw)
        vb = c.value_boards(sq, tm, **kw)
        pp, lp = c.policy(positions["planes_p"][:n, :c_in], 1.0, return_logits=True)
        vp = c.value(positions["planes_v"][:n, :c_in])
    assert np.array_equal(pb, pp) and np.array_equal(lb, lp) and np.array_equal(vb, vp)
