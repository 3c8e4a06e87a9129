"""Shared fixtures.  Tests marked `gpu` need a CUDA device and the built
library; everything else runs on the CPU."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the built CUDA library")


def unpack_planes(packed):
    return np.unpackbits(packed, axis=-1)[..., :361].astype(np.uint8)


@pytest.fixture(scope="session")
def positions():
    d = np.load(os.path.join(GOLDEN, "positions_s0.npz"))
    return {"planes_p": unpack_planes(d["planes_p"]), "planes_v": unpack_planes(d["planes_v"]),
            "squares": d["squares"], "meta": d["meta"], "moves": d["moves"]}


@pytest.fixture(scope="session")
def golden_config1():
    return dict(np.load(os.path.join(GOLDEN, "config1_s0.npz")))


@pytest.fixture(scope="session")
def golden_refexact():
    return dict(np.load(os.path.join(GOLDEN, "refexact_s0.npz")))


@pytest.fixture(scope="session")
def oracle_mod():
    from oracle import oracle as O
    O.build()
    return O


@pytest.fixture(scope="session")
def weights(oracle_mod):
    O = oracle_mod
    nets = {"cfg_p": O.CFG_POLICY, "cfg_v": O.CFG_VALUE, "ref_p": O.REF_POLICY,
            "ref_v": O.REF_VALUE}
    out = {}
    for k, preset in nets.items():
        seed = O.VALUE_SEED if k.endswith("_v") else O.POLICY_SEED
        n = O.make_net(preset)
        out[k] = (n, O.he_weights(n, seed))
    return out


def rel_logit_err(a, b):
    """Per-position norm-wise relative error max|a-b| / max|b|, the parity
    metric for logits (the L-inf error relative to the logit vector's scale)."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return np.abs(a - b).max(axis=-1) / np.maximum(np.abs(b).max(axis=-1), 1e-30)


def elem_rel_err(a, b, floor=1e-3):
    """Per-position element-wise relative error with a floor,
    max_i |a_i - b_i| / max(|b_i|, floor * max_j |b_j|).  On near-zero logits
    it is dominated by FP32 rounding: the reference's own FP32 logits differ
    from FP64 arithmetic by 1.8e-3 on this metric."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    den = np.maximum(np.abs(b), floor * np.abs(b).max(axis=-1, keepdims=True))
    return (np.abs(a - b) / np.maximum(den, 1e-30)).max(axis=-1)


def top1_same_up_to_ties(a, b, tol):
    """Per position: a's top-1 is b's top-1, or b's logit there is within
    tol * max|b| of b's maximum (a tie at the precision compared)."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    ia = a.argmax(-1)
    got = np.take_along_axis(b, ia[..., None], -1)[..., 0]
    return (ia == b.argmax(-1)) | (b.max(-1) - got <= tol * np.abs(b).max(-1))


@pytest.fixture(scope="session")
def gpu_lib():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from leela_gb300 import build
    build.build()
    import leela_gb300 as lg
    lg.library()
    return lg
