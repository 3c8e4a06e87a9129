"""The C-ABI library loads and exports every entry point include/leela_gpu.h
declares; host-side argument checks work without a GPU."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import ROOT


@pytest.fixture(scope="module")
def lib():
    from leela_gb300 import build
    build.build()
    import leela_gb300 as lg
    return lg


def declared_symbols():
    with open(os.path.join(ROOT, "include", "leela_gpu.h")) as f:
        text = f.read()
    return sorted(set(re.findall(r"LG_API\s+[\w\s\*]+?\b(lg_\w+)\s*\(", text)))


def test_header_declares_the_api():
    syms = declared_symbols()
    assert "lg_create" in syms and "lg_policy" in syms and "lg_poll" in syms
    assert len(syms) >= 12


def test_library_exports_every_declared_symbol(lib):
    out = subprocess.run(["nm", "-D", "--defined-only", lib.LIB_PATH], capture_output=True,
                         text=True, check=True).stdout
    exported = set(re.findall(r"\bT (lg_\w+)", out))
    missing = [s for s in declared_symbols() if s not in exported]
    assert not missing, missing
    L = lib.library()
    for s in declared_symbols():
        assert hasattr(L, s)


def test_header_compiles_as_c(tmp_path):
    src = tmp_path / "t.c"
    src.write_text('#include "leela_gpu.h"\nint main(void){lg_net_desc d={0};(void)d;return 0;}\n')
    subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
                    "-c", str(src), "-o", str(tmp_path / "t.o")], check=True)


def test_weight_count_matches_oracle(lib, weights):
    for key, ctor in (("cfg_p", lib.NetDesc.config1_policy), ("cfg_v", lib.NetDesc.config1_value),
                      ("ref_p", lib.NetDesc.reference_policy),
                      ("ref_v", lib.NetDesc.reference_value)):
        n, w = weights[key]
        d = ctor(w)
        assert d.weight_count() == w.size


def test_bad_arguments_are_rejected(lib, weights):
    L = lib.library()
    out = ctypes.c_void_p()
    assert L.lg_create(None, None, 0, 16, ctypes.byref(out)) == -1
    assert b"bad arguments" in L.lg_last_error()
    n, w = weights["cfg_p"]
    with pytest.raises(ValueError):
        lib.NetDesc.config1_policy(w[:-1])
    # A policy description used as the value net is refused before any GPU work.
    d = lib.NetDesc.config1_policy(w)._struct()
    assert L.lg_create(None, ctypes.byref(d), 0, 16, ctypes.byref(out)) == -1
    assert L.lg_policy(None, None, 1, 1.0, None, None) == -1
    assert L.lg_poll(None, None, 1, 0) == -1


def test_no_gpu_fails_loudly(lib, weights):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    n, w = weights["cfg_p"]
    with pytest.raises(lib.LeelaGPUError):
        lib.Context(policy=lib.NetDesc.config1_policy(w), max_batch=4)
