"""lg_policy_device_static: the FP32 policy forward whose scratch lives in the
library's static device array, for callers that cannot allocate device
memory when they evaluate.  Called through the C ABI and checked against
lg_policy_device (which uses the context's buffers) on two calls in a row,
within the FP32 parity tolerance of the other tests.

Kept in its own file, named to be collected last."""
import ctypes

import numpy as np
import pytest

from conftest import rel_logit_err

pytestmark = pytest.mark.gpu


def test_static_scratch_matches_context_path(gpu_lib, weights, positions, golden_config1):
    """Bit for bit the per-layer FP32 kernels' results (the same kernels run,
    only the scratch differs), on two calls in a row and on a call whose
    logits stay in the static array (logits = NULL); and within the FP32
    parity tolerance of the reference's own outputs."""
    import torch
    lg = gpu_lib
    L = lg.library()
    with lg.Context(policy=lg.NetDesc.config1_policy(weights["cfg_p"][1], "fp32"),
                    max_batch=8) as c:
        s = torch.cuda.current_stream()
        for call, (start, B, with_logits) in enumerate([(0, 4, True), (100, 3, True), (0, 4, False)]):
            c.set_tuning(B, 0, 0)  # lg_policy_device on the per-layer kernels
            planes = torch.from_numpy(
                np.ascontiguousarray(positions["planes_p"][start:start + B, :24])).cuda()
            ref_p = torch.empty((B, 361), device="cuda")
            ref_l = torch.empty((B, 361), device="cuda")
            got_p = torch.full((B, 361), -1.0, device="cuda")
            got_l = torch.full((B, 361), -1.0, device="cuda")
            assert L.lg_policy_device(c._h, planes.data_ptr(), B, 0.75, ref_p.data_ptr(),
                                      ref_l.data_ptr(), s.cuda_stream) == 0
            n0 = c.stats()["kernel_launches"]
            rc = L.lg_policy_device_static(c._h, planes.data_ptr(), B, 0.75, got_p.data_ptr(),
                                           got_l.data_ptr() if with_logits else None, s.cuda_stream)
            assert rc == 0, L.lg_last_error()
            assert c.stats()["kernel_launches"] > n0
            s.synchronize()
            rp, rl = ref_p.cpu().numpy(), ref_l.cpu().numpy()
            gp, gl = got_p.cpu().numpy(), got_l.cpu().numpy()
            assert np.array_equal(gp, rp), call
            if with_logits:
                assert np.array_equal(gl, rl), call
            else:
                assert (gl == -1.0).all(), call
            if start == 0:
                ref = golden_config1["logits_r0"][:B]
                assert rel_logit_err(rl, ref).max() <= 1e-4
                assert np.array_equal(rl.argmax(1), ref.argmax(1))


def test_static_scratch_limits(gpu_lib, weights):
    import torch
    lg = gpu_lib
    L = lg.library()
    with lg.Context(policy=lg.NetDesc.config1_policy(weights["cfg_p"][1], "fp32"),
                    max_batch=8) as c:
        planes = torch.zeros((5, 24, 361), dtype=torch.uint8, device="cuda")
        probs = torch.empty((5, 361), device="cuda")
        rc = L.lg_policy_device_static(c._h, planes.data_ptr(), 5, 1.0, probs.data_ptr(), None,
                                       None)
        assert rc == -1
        assert b"static scratch limit" in L.lg_last_error()
        # a context marked by the host-side fault injector fails the call
        c.inject_fault(1)
        rc = L.lg_policy_device_static(c._h, planes.data_ptr(), 1, 1.0, probs.data_ptr(), None,
                                       None)
        assert rc == -3
    with lg.Context(policy=lg.NetDesc.config1_policy(weights["cfg_p"][1], "bf16"),
                    max_batch=8) as c:
        rc = L.lg_policy_device_static(c._h, planes.data_ptr(), 1, 1.0, probs.data_ptr(), None,
                                       None)
        assert rc == -1
