"""Batching server (lg_submit / lg_poll) and host-side fault injection."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec", ["fp32", "bf16"])
def test_uneven_requests_match_direct_calls(gpu_lib, weights, positions, prec):
    """The server's merged, padded batches give each request what a direct
    call gives it.  Buckets of up to 8 positions are set to the per-layer
    kernels here (by default they take the small-batch kernel, whose FP32
    sums run in another order): BF16 results are then bit-identical whatever
    the batch, FP32 ones within the split-K order's rounding."""
    lg = gpu_lib
    with lg.Context(policy=lg.NetDesc.config1_policy(weights["cfg_p"][1], prec),
                    value=lg.NetDesc.config1_value(weights["cfg_v"][1], prec), max_batch=64) as c:
        for b in (1, 2, 4, 8):
            c.set_tuning(b, 0, 0)
        rng = np.random.default_rng(3)
        reqs = []
        start = 0
        for i in range(12):
            B = int(rng.integers(1, 40))
            net = i % 2
            src = positions["planes_p"] if net == 0 else positions["planes_v"]
            planes = np.ascontiguousarray(src[start:start + B, :24])
            start += B
            out = np.zeros((B, 361) if net == 0 else B, np.float32)
            reqs.append((net, planes, out))
            c.submit(net, planes, out, tag=i + 1, temperature=1.0)
        done = set()
        for _ in range(2000):
            done.update(c.poll(64, timeout_us=10000))
            if len(done) == len(reqs):
                break
        assert done == set(range(1, len(reqs) + 1))
        for net, planes, out in reqs:
            ref = c.policy(planes) if net == 0 else c.value(planes)
            tol = 0 if prec == "bf16" else 1e-5  # FP32 split-K order depends on the batch size
            assert np.abs(out - ref).max() <= tol
        assert c.stats()["batches"] >= 2


def test_logits_requests(gpu_lib, weights, positions):
    """LG_NET_POLICY_LOGITS: the policy net's head outputs, as lg_policy's
    logits, for callers that apply their own softmax."""
    lg = gpu_lib
    with lg.Context(policy=lg.NetDesc.config1_policy(weights["cfg_p"][1]), max_batch=16) as c:
        planes = np.ascontiguousarray(positions["planes_p"][:5, :24])
        out = np.zeros((5, 361), np.float32)
        c.submit(lg.LG_NET_POLICY_LOGITS, planes, out, tag=7)
        got = []
        for _ in range(500):
            got += c.poll(4, timeout_us=10000)
            if got:
                break
        assert got == [7]
        _, ref = c.policy(planes, 1.0, return_logits=True)
        assert np.abs(out - ref).max() <= 1e-5


def test_poll_is_bounded(gpu_lib, weights):
    lg = gpu_lib
    with lg.Context(policy=lg.NetDesc.config1_policy(weights["cfg_p"][1]), max_batch=8) as c:
        assert c.poll(4, timeout_us=20000) == []


def test_injected_fault_is_reported_and_context_survives(gpu_lib, weights, positions):
    lg = gpu_lib
    with lg.Context(policy=lg.NetDesc.config1_policy(weights["cfg_p"][1], "bf16"),
                    max_batch=8) as c:
        planes = positions["planes_p"][:4, :24]
        good = c.policy(planes)
        c.inject_fault(1)
        with pytest.raises(lg.LeelaGPUError) as e:
            c.policy(planes)
        assert e.value.code == -3
        assert np.array_equal(c.policy(planes), good)
