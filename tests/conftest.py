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
