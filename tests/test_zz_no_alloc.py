"""fo_sid_loss_noalloc: the SquaredIntensityDifference loss for callers that
cannot allocate device memory (graph captures they do not own, host pool
allocators, real-time loops).  Its partial sums live in a fixed array inside the
library; this test checks, through the C ABI, that two consecutive calls give
the same losses as the allocating metric (fo_sid_forward).

The file name sorts last so that a run stopping at the first failure has
already run every other test; it also passes when run alone.
"""

import ctypes as C

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def test_noalloc_loss_matches_metric_twice(fo):
    capi = fo._capi
    lib = capi.load()
    rng = np.random.default_rng(21)
    B, T, ny, nx = 6, 3, 96, 80
    u = torch.tensor(rng.standard_normal((B, ny, nx)) + 1j * rng.standard_normal((B, ny, nx)),
                     dtype=torch.complex64, device="cuda")
    target = torch.tensor(rng.uniform(0, 4, (T, ny, nx)), dtype=torch.float32, device="cuda")
    tidx_host = [b % T for b in range(B)]
    tidx = torch.tensor(tidx_host, dtype=torch.int32, device="cuda")

    sid = C.c_void_p()
    capi.check(lib.fo_sid_create(C.byref(sid), nx, ny, B, T, capi.ivec(tidx_host)))
    ref = torch.zeros(T, dtype=torch.float32, device="cuda")
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    capi.check(lib.fo_sid_forward(sid, C.c_void_p(u.data_ptr()), C.c_void_p(target.data_ptr()),
                                  C.c_void_p(ref.data_ptr()), stream))
    for _ in range(2):
        got = torch.full((T,), -1.0, dtype=torch.float32, device="cuda")
        capi.check(lib.fo_sid_loss_noalloc(C.c_void_p(u.data_ptr()), C.c_void_p(target.data_ptr()),
                                           C.c_void_p(tidx.data_ptr()), T, nx, ny, B,
                                           C.c_void_p(got.data_ptr()), stream))
        torch.cuda.synchronize()
        assert torch.allclose(got, ref, rtol=1e-5, atol=0.0), (got, ref)
    lib.fo_sid_destroy(sid)


def test_noalloc_rejects_too_many_slices(fo):
    capi = fo._capi
    lib = capi.load()
    one = C.c_void_p(16)
    rc = lib.fo_sid_loss_noalloc(one, one, one, 65, 8, 8, 65, one, None)
    assert rc == 2 and "at most 64" in lib.fo_last_error().decode()
