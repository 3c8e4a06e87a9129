"""Weight files (lg_weights_save / lg_weights_load): round trip, and the
errors a damaged file must raise.  Host-only code: runs on the CPU."""
import os

import numpy as np
import pytest


@pytest.fixture(scope="module")
def lg():
    from leela_gb300 import build
    build.build()
    import leela_gb300
    return leela_gb300


def test_round_trip(lg, weights, tmp_path):
    p = str(tmp_path / "nets.lgw")
    nets = [("policy", lg.NetDesc.config1_policy(weights["cfg_p"][1], "bf16")),
            ("value", lg.NetDesc.config1_value(weights["cfg_v"][1], "fp32")),
            ("ref_policy", lg.NetDesc.reference_policy(weights["ref_p"][1]))]
    lg.save_weights(p, nets)
    back = lg.load_weights(p)
    assert [n for n, _ in back] == ["policy", "value", "ref_policy"]
    for (_, a), (_, b) in zip(nets, back):
        assert a.shape == b.shape and a.precision == b.precision
        assert np.array_equal(a.weights, b.weights)


@pytest.mark.parametrize("damage", ["flip", "truncate", "magic"])
def test_damaged_files_are_rejected(lg, weights, tmp_path, damage):
    p = str(tmp_path / "nets.lgw")
    lg.save_weights(p, [("policy", lg.NetDesc.config1_policy(weights["cfg_p"][1]))])
    data = bytearray(open(p, "rb").read())
    if damage == "flip":
        data[1000] ^= 0x40
    elif damage == "truncate":
        data = data[: len(data) // 2]
    else:
        data[0:4] = b"XXXX"
    open(p, "wb").write(bytes(data))
    with pytest.raises(lg.LeelaGPUError) as e:
        lg.load_weights(p)
    assert e.value.code == -1


def test_missing_file(lg, tmp_path):
    with pytest.raises(lg.LeelaGPUError):
        lg.load_weights(str(tmp_path / "none.lgw"))
