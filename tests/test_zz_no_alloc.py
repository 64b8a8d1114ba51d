"""pfdd_fft_device_noalloc: the FFT entry point for callers that cannot allocate device
memory (for example code inside an OpenACC data region whose device memory belongs to
the OpenACC runtime).  It must give the same transforms as the plan-based entry point
(pfdd_fft_plan_create + pfdd_fft_forward/backward on device data) while allocating
nothing itself; its twiddle scratch is a static device array shared by all calls.

This file is collected last on purpose, and passes alone in a fresh process as well."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FP64, FP32 = 0, 1
TOL = {FP64: 1e-12, FP32: 3e-5}   # same tolerances as the FFT tests against numpy


def _lib(native_lib):
    L = native_lib
    L.pfdd_fft_device_noalloc.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                          C.c_void_p]
    return L


def _plan_transform(L, n, prec, batch, sign, dev_tensor):
    """Reference result: the existing plan-based entry point on a device buffer."""
    h = C.c_void_p()
    assert L.pfdd_fft_plan_create(C.byref(h), *n, prec, batch, 0) == 0
    fn = L.pfdd_fft_forward if sign < 0 else L.pfdd_fft_backward
    assert fn(h, C.c_void_p(dev_tensor.data_ptr()), batch, 1) == 0
    L.pfdd_fft_plan_destroy(h)


@pytest.mark.parametrize("prec", [FP64, FP32])
def test_noalloc_matches_plan_entry_point_on_two_calls(native_lib, prec):
    torch = pytest.importorskip("torch")
    L = _lib(native_lib)
    dt = torch.float64 if prec == FP64 else torch.float32
    stream = torch.cuda.current_stream()
    rng = np.random.default_rng(5)
    # two calls in a row with different sizes and directions: the second call must
    # not see anything the first left in the shared scratch array
    for n, batch, sign in [((16, 32, 64), 3, -1), ((64, 8, 128), 2, +1)]:
        N = int(np.prod(n))
        x = rng.standard_normal(batch * N * 2)
        a = torch.tensor(x, dtype=dt, device="cuda")
        b = a.clone()
        st = L.pfdd_fft_device_noalloc(C.c_void_p(a.data_ptr()), *n, batch, prec, sign,
                                       C.c_void_p(stream.cuda_stream))
        assert st == 0
        torch.cuda.synchronize()
        _plan_transform(L, n, prec, batch, sign, b)
        ra, rb = a.cpu().numpy(), b.cpu().numpy()
        scale = np.max(np.abs(rb))
        assert np.max(np.abs(ra - rb)) <= TOL[prec] * scale


def test_noalloc_rejects_sizes_beyond_its_capacity(native_lib):
    torch = pytest.importorskip("torch")
    L = _lib(native_lib)
    a = torch.zeros(16, dtype=torch.float64, device="cuda")
    ptr = C.c_void_p(a.data_ptr())
    assert L.pfdd_fft_device_noalloc(ptr, 8, 8, 1024, 1, FP64, -1, None) == 7      # PFDD_ELIMIT
    assert L.pfdd_fft_device_noalloc(ptr, 8, 6, 8, 1, FP64, -1, None) == 1         # PFDD_EINVAL
    assert L.pfdd_status_string(7) == b"size beyond a fixed capacity"
