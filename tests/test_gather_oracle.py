"""The oracle's restatement of the input-plane gather (all 32 planes of the
policy and value sets, the ladder reader included) against the planes the
reference's own gather wrote for the 1024 fixture positions
(Network.cpp:883-1201), and the oracle's random-board generator.  CPU only."""
import numpy as np


def test_gather_matches_reference_planes(positions, oracle_mod):
    sq, tm = positions["squares"], positions["meta"][:, 0]
    for which, key in ((0, "planes_p"), (1, "planes_v")):
        got = oracle_mod.gather_planes(sq, tm, which)
        ref = positions[key][:, :24]
        bad = np.argwhere(got != ref)
        assert bad.size == 0, (key, bad[:5])


def test_gather_all_32_planes_match_reference(positions, oracle_mod):
    """Ladders (FastBoard.cpp:2530-2837), ko, the last two moves, komi and the
    third line as well: 269 ladder and 1482 ladder-win points in the fixture."""
    sq, tm, mv = positions["squares"], positions["meta"][:, 0], positions["moves"]
    for which, key in ((0, "planes_p"), (1, "planes_v")):
        got = oracle_mod.gather_planes(sq, tm, which, 32, mv)
        ref = positions[key]
        bad = np.argwhere(got != ref)
        assert bad.size == 0, (key, bad[:5])
    ladder = positions["planes_p"][:, 25].sum()
    win = positions["planes_p"][:, 26].sum()
    assert ladder > 200 and win > 1000


def test_fixture_covers_every_plane(positions):
    """Every plane 0..23 of both sets is set somewhere in the fixture, and
    some empty points are suicides for the side to move (no after-move plane
    set), so the parity cases exercise each branch."""
    pp, pv = positions["planes_p"][:, :24], positions["planes_v"][:, :24]
    assert (pp.sum(axis=(0, 2)) > 0).all()
    assert (pv.sum(axis=(0, 2)) > 0).all()
    suicide = (pp[:, 0] == 1) & (pp[:, 13:19].sum(axis=1) == 0)
    assert suicide.sum() > 100


def _strings_have_liberties(sq):
    """Every string of the board has a liberty (flood fill in numpy-free
    Python; small boards only)."""
    seen = np.zeros(361, bool)
    for p in range(361):
        if sq[p] == 2 or seen[p]:
            continue
        stack, libs, c = [p], set(), sq[p]
        seen[p] = True
        while stack:
            q = stack.pop()
            x, y = q % 19, q // 19
            for nx, ny in ((x - 1, y), (x + 1, y), (x, y - 1), (x, y + 1)):
                if 0 <= nx < 19 and 0 <= ny < 19:
                    r = ny * 19 + nx
                    if sq[r] == 2:
                        libs.add(r)
                    elif sq[r] == c and not seen[r]:
                        seen[r] = True
                        stack.append(r)
        if not libs:
            return False
    return True


def test_random_boards_are_legal_and_deterministic(oracle_mod):
    a, ta = oracle_mod.random_boards(16, 7, kmax=400)
    b, tb = oracle_mod.random_boards(16, 7, kmax=400)
    assert (a == b).all() and (ta == tb).all()
    assert set(np.unique(a)) <= {0, 1, 2}
    for sq in a:
        assert _strings_have_liberties(sq)
    # dense boards reach captures: fewer stones than moves played somewhere
    assert (a != 2).sum(axis=1).max() > 150
