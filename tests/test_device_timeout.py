"""Device-side bounded waits that run out (no trap, no fault).

lg_inject_stall makes the next launch of the persistent trunk (kind 0) or
of the small-batch kernel (kind 1) wait for a flag that nothing publishes,
with its wait limits cut short.  The wait gives up, the kernel writes its
error word and unwinds (the trunk waits for its own copies in flight and
frees its tensor memory), and the blocking call returns LG_ERR_DEVICE
within a bounded time; the next call on the same context gives the same
results as before.
"""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("kind,choice,B", [(1, 4, 1), (1, 4, 5), (0, 3, 256), (0, 2, 64)])
@pytest.mark.parametrize("prec", ["bf16", "fp32"])
def test_device_wait_runs_out_and_the_context_survives(gpu_lib, weights, positions, kind, choice, B, prec):
    lg = gpu_lib
    if prec == "fp32" and kind == 0:
        pytest.skip("FP32 nets have no trunk kernel")
    idx = np.arange(B) % 1024
    pp, pv = positions["planes_p"][idx, :24], positions["planes_v"][idx, :24]
    with lg.Context(policy=lg.NetDesc.config1_policy(weights["cfg_p"][1], prec),
                    value=lg.NetDesc.config1_value(weights["cfg_v"][1], prec), max_batch=256) as c:
        c.set_tuning(B, choice, 0)
        good_p, good_v = c.policy(pp), c.value(pv)
        c.inject_stall(kind, 1 << 14)
        t0 = time.perf_counter()
        with pytest.raises(lg.LeelaGPUError) as e:
            c.policy(pp)
        elapsed = time.perf_counter() - t0
        assert e.value.code == -5, str(e.value)  # LG_ERR_DEVICE: the kernel's error word
        assert elapsed < 20.0
        # the context keeps working, with the same results
        assert np.array_equal(c.policy(pp), good_p)
        assert np.array_equal(c.value(pv), good_v)
        print(f"{prec} kind {kind} B {B}: stalled call returned after {elapsed * 1e3:.1f} ms: {e.value}")


@pytest.mark.parametrize("net", ["policy", "value"])
def test_chained_device_call_wait_runs_out(gpu_lib, weights, positions, net):
    """A device call over three chunks (each chunk's trunk, head and the next
    chunk's packing launched as programmatic dependents) whose first trunk
    gives up a wait: the chain still completes in bounded time, the later
    chunks are right, lg_device_error reports the kernel's error word once,
    and the next call gives the same results as before."""
    import torch
    lg = gpu_lib
    mb, B = 256, 3 * 256
    idx = np.arange(B) % 1024
    key = "planes_p" if net == "policy" else "planes_v"
    planes = torch.from_numpy(np.ascontiguousarray(positions[key][idx, :24])).cuda()
    with lg.Context(policy=lg.NetDesc.config1_policy(weights["cfg_p"][1], "bf16"),
                    value=lg.NetDesc.config1_value(weights["cfg_v"][1], "bf16"), max_batch=mb) as c:
        c.set_tuning(mb, 3, 0)
        s = torch.cuda.current_stream()

        def run():
            if net == "policy":
                out = torch.empty((B, 361), device="cuda")
                c.policy_device(planes.data_ptr(), B, out.data_ptr(), 1.0, None, s.cuda_stream)
            else:
                out = torch.empty(B, device="cuda")
                c.value_device(planes.data_ptr(), B, out.data_ptr(), s.cuda_stream)
            s.synchronize()
            return out.cpu().numpy()

        good = run()
        assert c.device_error() == 0
        c.inject_stall(0, 1 << 14)
        t0 = time.perf_counter()
        bad = run()
        elapsed = time.perf_counter() - t0
        assert elapsed < 20.0
        assert c.device_error() == -5
        assert b"error status" in lg.library().lg_last_error()
        assert c.device_error() == 0  # cleared
        # the stalled launch was the first chunk's trunk; the next chunks ran
        # normally (the trunk's last CTA leaves its flags at zero)
        assert np.array_equal(bad[mb:], good[mb:])
        assert np.array_equal(run(), good)
        assert c.device_error() == 0
        print(f"{net}: chained call with a stalled trunk returned after {elapsed * 1e3:.1f} ms")
