"""The FFT boundary (drop-in for fft_forward / fft_backward, PFDD_Final_GPU.c:209-273)
against numpy, plus size-independent properties at the full 128^3 size."""
import numpy as np
import pytest

from pfdd_gb300 import native

pytestmark = pytest.mark.gpu

SHAPES = [(8, 8, 8), (16, 8, 32), (32, 2, 32), (1, 8, 4), (2, 2, 2), (4, 1, 1), (64, 16, 8), (8, 256, 4)]


def as_interleaved(x, dt):
    a = np.empty(x.shape + (2,), dtype=dt)
    a[..., 0] = x.real
    a[..., 1] = x.imag
    return np.ascontiguousarray(a)


def from_interleaved(a):
    return a[..., 0].astype(np.float64) + 1j * a[..., 1].astype(np.float64)


@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_fft_matches_numpy(native_lib, shape, prec):
    rng = np.random.default_rng(hash(shape) % 1000)
    batch = 3
    x = rng.standard_normal((batch,) + shape) + 1j * rng.standard_normal((batch,) + shape)
    dt = np.float64 if prec == "fp64" else np.float32
    tol = 1e-12 if prec == "fp64" else 3e-5
    p = native.FFTPlan(shape, prec, max_batch=batch)
    a = as_interleaved(x, dt)
    p.forward(a, batch)
    ref = np.fft.fftn(x, axes=(1, 2, 3))
    scale = np.max(np.abs(ref))
    assert np.max(np.abs(from_interleaved(a) - ref)) <= tol * scale
    b = as_interleaved(x, dt)
    p.backward(b, batch)
    refb = np.fft.ifftn(x, axes=(1, 2, 3)) * np.prod(shape)
    assert np.max(np.abs(from_interleaved(b) - refb)) <= tol * scale
    p.close()


def test_fft_round_trip_and_linearity_full_size(native_lib):
    n = (128, 128, 128)
    rng = np.random.default_rng(7)
    x = (rng.standard_normal(n) + 1j * rng.standard_normal(n))[None]
    y = (rng.standard_normal(n) + 1j * rng.standard_normal(n))[None]
    p = native.FFTPlan(n, "fp64", max_batch=1)
    ax = as_interleaved(x, np.float64)
    p.forward(ax, 1)
    ay = as_interleaved(y, np.float64)
    p.forward(ay, 1)
    axy = as_interleaved(2.0 * x - 3.0 * y, np.float64)
    p.forward(axy, 1)
    fx, fy, fxy = from_interleaved(ax), from_interleaved(ay), from_interleaved(axy)
    assert np.max(np.abs(fxy - (2.0 * fx - 3.0 * fy))) <= 1e-9
    # Parseval
    np.testing.assert_allclose(np.sum(np.abs(fx) ** 2), np.prod(n) * np.sum(np.abs(x) ** 2), rtol=1e-12)
    p.backward(ax, 1)
    assert np.max(np.abs(from_interleaved(ax) / np.prod(n) - x)) <= 1e-12
    p.close()
