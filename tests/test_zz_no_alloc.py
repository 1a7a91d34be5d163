"""fo_sid_loss_noalloc: the SquaredIntensityDifference loss for callers that
cannot allocate device memory (host applications whose device memory belongs to
their own pool allocator, real-time loops where an allocation's implicit
synchronisation is not allowed).  Its partial sums live in a fixed array inside
the library.  These tests call it through the C ABI and check, on two
consecutive calls, its losses against the allocating metric (fo_sid_forward)
and against the FP64 oracle, including the largest accepted slice count (64), and
that a call after the first leaves the device's free memory unchanged.

The file name sorts last so that a run stopping at the first failure has
already run every other test; it also passes when run alone.
"""

import ctypes as C

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _run_case(fo, orc, B, T, ny, nx, seed):
    capi = fo._capi
    lib = capi.load()
    rng = np.random.default_rng(seed)
    u_h = (rng.standard_normal((B, ny, nx)) + 1j * rng.standard_normal((B, ny, nx))).astype(np.complex64)
    t_h = rng.uniform(0, 4, (T, ny, nx)).astype(np.float32)
    tidx_host = [b % T for b in range(B)]
    u = torch.tensor(u_h, device="cuda")
    target = torch.tensor(t_h, device="cuda")
    tidx = torch.tensor(tidx_host, dtype=torch.int32, device="cuda")
    c_ref, _ = orc.sid_value(u_h.astype(np.complex128), t_h.astype(np.float64), np.array(tidx_host))

    sid = C.c_void_p()
    capi.check(lib.fo_sid_create(C.byref(sid), nx, ny, B, T, capi.ivec(tidx_host)))
    ref = torch.zeros(T, dtype=torch.float32, device="cuda")
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    capi.check(lib.fo_sid_forward(sid, C.c_void_p(u.data_ptr()), C.c_void_p(target.data_ptr()),
                                  C.c_void_p(ref.data_ptr()), stream))
    try:
        free_before = None
        for k in range(2):
            got = torch.full((T,), -1.0, dtype=torch.float32, device="cuda")
            torch.cuda.synchronize()
            if k == 1:
                free_before = torch.cuda.mem_get_info()[0]
            capi.check(lib.fo_sid_loss_noalloc(C.c_void_p(u.data_ptr()), C.c_void_p(target.data_ptr()),
                                               C.c_void_p(tidx.data_ptr()), T, nx, ny, B,
                                               C.c_void_p(got.data_ptr()), stream))
            torch.cuda.synchronize()
            if k == 1:
                # the second call allocates no device memory
                assert torch.cuda.mem_get_info()[0] == free_before
            # same tolerance as the metric's oracle tests: 1e-4 relative per slice
            assert torch.allclose(got, ref, rtol=1e-5, atol=0.0), (got, ref)
            g = got.cpu().numpy().astype(np.float64)
            rel = np.abs(g - c_ref) / np.abs(c_ref)
            assert rel.max() <= 1e-4, rel.max()
    finally:
        lib.fo_sid_destroy(sid)


def test_noalloc_loss_matches_metric_twice(fo, orc):
    _run_case(fo, orc, B=6, T=3, ny=96, nx=80, seed=21)


def test_noalloc_loss_at_the_slice_limit(fo, orc):
    # 64 target slices (FO_SID_NOALLOC_MAX_TARGETS), two fields per slice
    _run_case(fo, orc, B=128, T=64, ny=64, nx=48, seed=22)


def test_noalloc_rejects_too_many_slices(fo):
    capi = fo._capi
    lib = capi.load()
    one = C.c_void_p(16)
    rc = lib.fo_sid_loss_noalloc(one, one, one, 65, 8, 8, 65, one, None)
    assert rc == 2 and "at most 64" in lib.fo_last_error().decode()
