"""The engine's own search on the GB300 backend (CPU; needs the reference
sources and g++).

leela_gb300/integration/opencl_gb300.cpp replaces the engine's OpenCL.cpp:
the engine's sources compile unmodified in their own OpenCL configuration
(USE_OPENCL in their config.h) with the stand-in CL/cl2.hpp, and its search
(UCTSearch::think, UCTNode::netscore_children -> Network::async_scored_moves
-> forward_cb -> UCTNode::scoring_cb, run_value_net, the root's
AVERAGE_ALL) runs on the backend.  Here the C ABI underneath is the CPU
stand-in tests/integration/fake_lg.cpp (the oracle), so the test checks the
backend's plumbing on a machine without a GPU: the layers it records, the
synchronous calls, asynchronous requests completed by its drain thread,
the per-thread throttle and the bounded join.
"""
import os
import re
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
REF = os.environ.get("LEELA_REF")


@pytest.fixture(scope="module")
def driver():
    if not REF or not os.path.isdir(REF) or not os.path.exists(os.path.join(REF, "UCTSearch.cpp")):
        pytest.skip("reference sources not present (set LEELA_REF)")
    if not shutil.which("g++"):
        pytest.skip("no g++")
    d = os.path.join(HERE, "integration")
    subprocess.run(["make", "-s", "-j8", "-C", d, f"REF={REF}"], check=True)
    return os.path.join(d, "_build", "search_driver")


def run(driver, playouts, threads, sync=None):
    from oracle import oracle as O
    env = dict(os.environ)
    if sync:
        env["LEELA_GB300_SYNC"] = sync
    blas = O.find_openblas()
    if blas:
        env["LEELA_OPENBLAS"] = blas
    r = subprocess.run([driver, str(playouts), str(threads)], capture_output=True, text=True, timeout=600,
                       env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    line = [ln for ln in r.stdout.splitlines() if ln.startswith("RESULT")][-1]
    return dict(re.findall(r"(\w+)=(\S+)", line))


def test_engine_search_runs_on_the_backend(driver):
    res = run(driver, 3000, 4)
    assert res["legal"] == "1"
    # DIRECT get_scored_moves through the backend: the 355 empty points of the
    # position (6 stones), the softmax mass over them
    assert int(res["direct_moves"]) == 355
    assert 0.9 < float(res["direct_sum"]) <= 1.0 + 1e-5
    assert 0.0 <= float(res["value"]) <= 1.0  # the engine's (1 + tanh) / 2 of the raw FC output
    assert int(res["submitted"]) > 0        # async_scored_moves, and the synchronous calls too,
    assert int(res["sync"]) == 0            # went through lg_submit (merged across threads)
    assert int(res["outstanding"]) == 0     # every callback ran; the join returned
    assert int(res["thread_outstanding"]) == 0


def test_engine_search_with_direct_synchronous_calls(driver):
    """LEELA_GB300_SYNC=direct: the value net and the root's synchronous
    policy calls are blocking lg_value / lg_policy calls of one position."""
    res = run(driver, 1000, 4, sync="direct")
    assert res["legal"] == "1"
    assert int(res["submitted"]) > 0        # the asynchronous policy requests
    assert int(res["sync"]) > 0             # value net, root AVERAGE_ALL
    assert int(res["outstanding"]) == 0 and int(res["thread_outstanding"]) == 0


def test_engine_search_single_thread(driver):
    res = run(driver, 500, 1)
    assert res["legal"] == "1" and int(res["outstanding"]) == 0
