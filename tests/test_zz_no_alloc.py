"""The allocation-free log-sum-exp entry point (emc_respons_max_expf_noalloc).

It exists for callers that cannot call cudaMalloc when they run it -- code
inside CUDA stream capture, callbacks, or a host that owns a fixed device
memory budget.  Its scratch is a fixed device array inside the library, so
this test checks, through the C ABI, that two calls in a row give the same
per-pattern sums as the allocating entry point (emc_respons_max_expf) within
the float tolerance of the other LSE tests (relative 1e-5; the two may fold
the rotation ranges in a different order), and that sizes beyond the
array are refused.  The file is named to be collected last."""
import ctypes as C

import numpy as np
import pytest
import torch

import emc_gb300 as E
from emc_gb300 import _lib

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("N,R", [(3000, 4000), (65536, 1500)])
def test_noalloc_matches_allocating_entry_point(ctx, cuda, N, R):
    lib = _lib.load()
    rng = np.random.default_rng(N + R)
    L = torch.as_tensor((rng.standard_normal((R, N)) * 20 - 100).astype(np.float32), device=cuda)
    L[3, :] = -1e12  # below the -1e10 cut
    mx = torch.empty(N, device=cuda)
    ctx.max_vector(L, N, R, mx)
    want = torch.empty(N, device=cuda)
    ctx.respons_max_expf(L, mx, N, R, want)
    ctx.sync()
    stream = torch.cuda.Stream(cuda)
    for _ in range(2):
        got = torch.full((N,), -7.0, device=cuda)
        # the fill above runs on torch's current stream: the side stream waits for it
        stream.wait_stream(torch.cuda.current_stream(cuda))
        rc = lib.emc_respons_max_expf_noalloc(L.data_ptr(), mx.data_ptr(), N, R, got.data_ptr(),
                                              stream.cuda_stream)
        assert rc == 0
        stream.synchronize()
        np.testing.assert_allclose(got.cpu().numpy(), want.cpu().numpy(), rtol=1e-5)


def test_noalloc_refuses_oversize_and_bad_arguments(cuda):
    lib = _lib.load()
    big = E._lib.load().emc_respons_max_expf_noalloc
    assert big(C.c_void_p(16), C.c_void_p(16), (1 << 20) + 1, 4, C.c_void_p(16), None) == -1
    assert lib.emc_respons_max_expf_noalloc(None, None, 10, 4, None, None) == -1
    assert lib.emc_respons_max_expf_noalloc(C.c_void_p(16), C.c_void_p(16), -1, 4,
                                            C.c_void_p(16), None) == -1
