"""pfdd_fft_device_noalloc: the FFT entry point for callers that cannot allocate device
memory (for example code inside an OpenACC data region whose device memory belongs to
the OpenACC runtime, or a process held to a fixed device-memory budget).  It must give
the same transforms as the plan-based entry point (pfdd_fft_plan_create +
pfdd_fft_forward/backward on device data) and as numpy, while allocating nothing
itself; its twiddle scratch is a static device array shared by all calls.

This file is collected last on purpose, and passes alone in a fresh process as well."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FP64, FP32 = 0, 1
TOL = {FP64: 1e-12, FP32: 3e-5}   # same tolerances as the FFT tests against numpy

# (grid, batch, sign): two sizes per precision, then a 512-long axis with a
# length-1 axis, in both directions
CASES = [((16, 32, 64), 3, -1), ((64, 8, 128), 2, +1), ((512, 4, 1), 2, -1), ((1, 8, 512), 1, +1)]


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


def _numpy_transform(x, n, batch, sign):
    z = (x[0::2] + 1j * x[1::2]).reshape((batch,) + tuple(n))
    f = np.fft.fftn(z, axes=(1, 2, 3)) if sign < 0 else np.fft.ifftn(z, axes=(1, 2, 3)) * np.prod(n)
    out = np.empty(x.shape)
    out[0::2], out[1::2] = f.real.ravel(), f.imag.ravel()
    return out


def _noalloc(L, tensor, n, batch, prec, sign, stream):
    return L.pfdd_fft_device_noalloc(C.c_void_p(tensor.data_ptr()), *n, batch, prec, sign,
                                     C.c_void_p(stream.cuda_stream))


@pytest.mark.parametrize("prec", [FP64, FP32])
def test_noalloc_matches_plan_entry_point_and_numpy(native_lib, prec):
    torch = pytest.importorskip("torch")
    L = _lib(native_lib)
    dt = torch.float64 if prec == FP64 else torch.float32
    stream = torch.cuda.current_stream()
    rng = np.random.default_rng(5)
    # calls in a row with different sizes and directions: no call may see
    # anything an earlier one left in the shared scratch array
    for n, batch, sign in CASES:
        N = int(np.prod(n))
        x = rng.standard_normal(batch * N * 2)
        a = torch.tensor(x, dtype=dt, device="cuda")
        b = a.clone()
        assert _noalloc(L, a, n, batch, prec, sign, stream) == 0
        torch.cuda.synchronize()
        _plan_transform(L, n, prec, batch, sign, b)
        ra, rb = a.cpu().numpy().astype(np.float64), b.cpu().numpy().astype(np.float64)
        rn = _numpy_transform(x, n, batch, sign)
        scale = np.max(np.abs(rn))
        assert np.max(np.abs(ra - rb)) <= TOL[prec] * scale, n
        assert np.max(np.abs(ra - rn)) <= TOL[prec] * scale, n


@pytest.mark.parametrize("prec", [FP64, FP32])
def test_noalloc_queued_calls_without_host_sync(native_lib, prec):
    """Two calls queued back to back on one stream (the second call rewrites the
    shared twiddle array while the first may still be running): both results
    match the plan-based entry point."""
    torch = pytest.importorskip("torch")
    L = _lib(native_lib)
    dt = torch.float64 if prec == FP64 else torch.float32
    stream = torch.cuda.current_stream()
    rng = np.random.default_rng(9)
    (na, ba, sa), (nb, bb, sb) = ((32, 64, 16), 4, -1), ((8, 128, 64), 2, +1)
    a = torch.tensor(rng.standard_normal(ba * int(np.prod(na)) * 2), dtype=dt, device="cuda")
    b = torch.tensor(rng.standard_normal(bb * int(np.prod(nb)) * 2), dtype=dt, device="cuda")
    ra, rb = a.clone(), b.clone()
    torch.cuda.synchronize()
    assert _noalloc(L, a, na, ba, prec, sa, stream) == 0
    assert _noalloc(L, b, nb, bb, prec, sb, stream) == 0
    torch.cuda.synchronize()
    _plan_transform(L, na, prec, ba, sa, ra)
    _plan_transform(L, nb, prec, bb, sb, rb)
    for got, ref in ((a, ra), (b, rb)):
        g, r = got.cpu().numpy().astype(np.float64), ref.cpu().numpy().astype(np.float64)
        assert np.max(np.abs(g - r)) <= TOL[prec] * np.max(np.abs(r))


def test_noalloc_allocates_no_device_memory(native_lib):
    """After a first call of each size (which may load kernel code: CUDA's lazy
    module loading), further calls leave the device's free memory and torch's
    allocator untouched."""
    torch = pytest.importorskip("torch")
    L = _lib(native_lib)
    stream = torch.cuda.current_stream()
    bufs = {prec: torch.zeros(2 * 2 * 64 * 32 * 128, dtype=torch.float64 if prec == FP64 else torch.float32,
                              device="cuda") for prec in (FP64, FP32)}
    shapes = [((64, 32, 128), 2, -1), ((128, 32, 64), 2, +1), ((8, 512, 2), 4, -1)]
    for prec, buf in bufs.items():
        for n, batch, sign in shapes:
            assert _noalloc(L, buf, n, batch, prec, sign, stream) == 0
    torch.cuda.synchronize()
    free0, used0 = torch.cuda.mem_get_info()[0], torch.cuda.memory_allocated()
    for _ in range(3):
        for prec, buf in bufs.items():
            for n, batch, sign in shapes:
                assert _noalloc(L, buf, n, batch, prec, sign, stream) == 0
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0
    assert torch.cuda.memory_allocated() == used0


def test_noalloc_rejects_sizes_beyond_its_capacity(native_lib):
    torch = pytest.importorskip("torch")
    L = _lib(native_lib)
    a = torch.zeros(16, dtype=torch.float64, device="cuda")
    ptr = C.c_void_p(a.data_ptr())
    assert L.pfdd_fft_device_noalloc(ptr, 8, 8, 1024, 1, FP64, -1, None) == 7      # PFDD_ELIMIT
    assert L.pfdd_fft_device_noalloc(ptr, 8, 6, 8, 1, FP64, -1, None) == 1         # PFDD_EINVAL
    # a batch whose launch grid would not fit 2^31 - 1 blocks: rejected before any launch
    assert L.pfdd_fft_device_noalloc(ptr, 512, 512, 512, 1 << 20, FP64, -1, None) == 1
    assert L.pfdd_status_string(7) == b"size beyond a fixed capacity"
