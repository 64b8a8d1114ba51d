"""ctypes front end of the CPU FP64 oracle (oracle/pfdd_cpu.c).

TEST INFRASTRUCTURE ONLY: used by tests/, ``__graft_entry__.smoke()`` and bench.py's
CPU-baseline legs to check and time the CUDA path; the product never imports it.
"""
from __future__ import annotations

import ctypes as C
import os
import platform
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
SRC = HERE / "pfdd_cpu.c"
BUILD = HERE / "_build"
LIB = BUILD / "libpfdd_oracle.so"

_lib = None


def build(force: bool = False) -> Path:
    """Compile the restatement (gcc -O2, no FP contraction so x86 and Arm agree bitwise)."""
    BUILD.mkdir(exist_ok=True)
    if LIB.exists() and not force and LIB.stat().st_mtime >= SRC.stat().st_mtime:
        return LIB
    tmp = LIB.with_suffix(f".{os.getpid()}.tmp")
    subprocess.run(["gcc", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-o", str(tmp), str(SRC),
                    "-lm", "-lpthread"], check=True)
    os.replace(tmp, LIB)
    return LIB


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(str(LIB))
        dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
        L.oracle_frec.argtypes = [C.c_int, C.c_double, dp]
        L.oracle_setfcc.argtypes = [dp, dp, C.c_double, C.c_int]
        L.oracle_setorient.argtypes = [dp]
        L.oracle_seteps.argtypes = [C.c_int, dp, dp, dp, dp, dp]
        L.oracle_resolss_uniform.argtypes = [C.c_int, dp, dp, dp]
        L.oracle_bmatrix.argtypes = [C.c_int] * 3 + [C.c_double] * 6 + [C.c_int, dp, dp, C.c_int]
        L.oracle_fft3d.argtypes = [C.c_int] * 4 + [dp, C.c_int, C.c_int]
        L.oracle_strain_stress.argtypes = ([C.c_int] * 4 + [C.c_double] * 3 + [dp] + [C.c_double] * 3 +
                                           [dp, dp, dp, dp, dp, dp, C.c_int])
        L.oracle_strain_stress.restype = None
        L.oracle_run.argtypes = ([C.c_int] * 4 + [dp, dp, dp, dp, dp, dp, C.c_double, C.c_int, dp,
                                 C.c_void_p, dp, dp, C.c_int])
        L.oracle_run.restype = C.c_int
        _lib = L
    return _lib


def nthreads() -> int:
    return max(1, min(64, os.cpu_count() or 1))


def frec(n: int, d: float = 1.0) -> np.ndarray:
    f = np.zeros(n)
    lib().oracle_frec(n, d, f)
    return f


def fcc_eps(ns: int = 12, bdiv: float = float(np.sqrt(2.0)), dslip=None, float_s3: bool = False) -> np.ndarray:
    """Eigenstrains of the first ``ns`` FCC systems in the global frame, shape [ns, 3, 3]."""
    xn = np.zeros((12, 3)); xb = np.zeros((12, 3)); th = np.zeros((3, 3))
    lib().oracle_setfcc(xn, xb, bdiv, int(float_s3))
    lib().oracle_setorient(th)
    ds = np.ones(12) if dslip is None else np.ascontiguousarray(dslip, dtype=np.float64)
    eps = np.zeros((12, 3, 3))
    lib().oracle_seteps(12, xn, xb, ds, th, eps)
    return eps[:ns].copy()


def resolved_shear(eps: np.ndarray, sigma: np.ndarray) -> np.ndarray:
    tau = np.zeros(eps.shape[0])
    lib().oracle_resolss_uniform(eps.shape[0], np.ascontiguousarray(sigma, dtype=np.float64),
                                 np.ascontiguousarray(eps), tau)
    return tau


def bmatrix(n, eps: np.ndarray, C11: float, C12: float, C44: float, d=(1.0, 1.0, 1.0)) -> np.ndarray:
    """Interaction matrix, layout [kb][ka][n1][n2][n3] like the reference's BB."""
    ns = eps.shape[0]
    B = np.zeros((ns, ns) + tuple(n))
    lib().oracle_bmatrix(n[0], n[1], n[2], d[0], d[1], d[2], C11, C12, C44, ns, np.ascontiguousarray(eps), B,
                         nthreads())
    return B


def fft3d(x: np.ndarray, sign: int) -> np.ndarray:
    """Unnormalised 3D C2C transform of complex128 fields [nf, n1, n2, n3]."""
    a = np.ascontiguousarray(np.stack([x.real, x.imag], axis=-1))
    lib().oracle_fft3d(x.shape[1], x.shape[2], x.shape[3], x.shape[0], a, int(sign), nthreads())
    return a[..., 0] + 1j * a[..., 1]


def ramp_tau(tau_max: np.ndarray, steps: int) -> np.ndarray:
    """Per-step resolved shear stress tau_max * (s+1)/K, evaluated as the patched
    reference does inside plasticevolv: tau * ((it_plastic + 1.0) / K)."""
    s = np.arange(steps, dtype=np.float64)
    return tau_max[None, :] * ((s[:, None] + 1.0) / float(steps))


def run(n, B: np.ndarray, xi: np.ndarray, bc: np.ndarray, cd2, asf, dslip, uq2: float, tau_steps: np.ndarray,
        tau_field: np.ndarray | None = None):
    """Run ``len(tau_steps)`` TDGL steps; returns (xi_final, gamma[K], gamma_a[K, ns])."""
    ns = xi.shape[0]
    K = tau_steps.shape[0]
    x = np.ascontiguousarray(np.stack([xi.real, xi.imag], axis=-1))
    b = np.ascontiguousarray(np.stack([bc, bc], axis=-1).astype(np.float64))
    g = np.zeros(K); ga = np.zeros((K, ns))
    tf = None if tau_field is None else np.ascontiguousarray(tau_field, dtype=np.float64)
    rc = lib().oracle_run(n[0], n[1], n[2], ns, np.ascontiguousarray(B), x, b,
                          np.ascontiguousarray(cd2, dtype=np.float64), np.ascontiguousarray(asf, dtype=np.float64),
                          np.ascontiguousarray(dslip, dtype=np.float64), float(uq2), K,
                          np.ascontiguousarray(tau_steps, dtype=np.float64),
                          None if tf is None else tf.ctypes.data_as(C.c_void_p), g, ga, nthreads())
    if rc != 0:
        raise MemoryError("oracle_run failed")
    return x[..., 0] + 1j * x[..., 1], g, ga


def solve(spec, steps: int | None = None, eps_bdiv: float = float(np.sqrt(2.0))):
    """Full oracle solve of a :class:`pfdd_gb300.workloads.SolveSpec` (first ``steps`` steps)."""
    from pfdd_gb300 import workloads
    K = spec.steps if steps is None else steps
    eps = fcc_eps(spec.ns, bdiv=eps_bdiv, dslip=np.full(12, spec.dslip))
    C44, C12 = spec.mu, spec.lam
    C11 = spec.C11
    B = bmatrix(spec.n, eps, C11, C12, C44, spec.d)
    sig = np.zeros((3, 3)); sig[0, 2] = sig[2, 0] = spec.sigma_max
    tau_max = resolved_shear(eps, sig)
    tau = ramp_tau(tau_max, spec.steps)[:K]
    xi, bc = workloads.initial_state(spec)
    ns = spec.ns
    return run(spec.n, B, xi, bc, np.full(ns, spec.cd2), np.full(ns, spec.asf), np.full(ns, spec.dslip), spec.uq2,
               tau)


def converge_stop(gamma: np.ndarray, gamma_prev: float = 0.0) -> int | None:
    """The inner loop's stop (plasticconverge, F:3732-3785, under the do-while of
    F:4574-4691) on a sequence of per-step gammas: the number of steps the
    reference runs, or None when it would run them all.  A step passes when
    |(g - g_last) / g| < 1e-8 or |g| < 1e-12 (g == 0: |g - g_last| < 1e-15 or
    |g| < 1e-14); a passing step from index 29 on adds one to the count when
    the last 30 steps all passed and otherwise resets it; the loop ends at a
    count of 5.  g_last of the first step is ``gamma_prev`` (F:4575)."""
    passed = np.zeros(len(gamma), dtype=bool)
    count, last = 0, float(gamma_prev)
    for it, g in enumerate(map(float, gamma)):
        if g != 0:
            ok = abs((g - last) / g) < 1e-8 or abs(g) < 1e-12
        else:
            ok = abs(g - last) < 1e-15 or abs(g) < 1e-14
        if ok:
            passed[it] = True
            if it >= 29:
                if passed[it - 29:it + 1].all():
                    count += 1
                elif count != 0:
                    count = 0
        if count == 5:
            return it + 1
        last = g
    return None


def converge_min_steps(passed, count: int) -> int:
    """The fewest further steps after which the loop of :func:`converge_stop`
    can stop, given the pass marks of the steps so far and the count: 5 - count
    with a full window of passes behind (29 or more), 34 - run otherwise, 35
    when the count is past 5 (the bound pfdd_step_converge sizes its chunks by)."""
    r = 0
    while r < 29 and r < len(passed) and passed[len(passed) - 1 - r]:
        r += 1
    if r >= 29:
        return 5 - count if count < 5 else 35
    return 34 - r


def strain_stress(n, xi: np.ndarray, eps: np.ndarray, C11: float, C12: float, C44: float, sigma_app: np.ndarray,
                  d=(1.0, 1.0, 1.0)):
    """Strain and stress fields of state ``xi`` (complex [ns, n1, n2, n3]):
    returns eps [3, 3, N], sigma [3, 3, N], aveps [3, 3], avesigma [3, 3]."""
    L = lib()
    n = tuple(int(v) for v in n)
    N = int(np.prod(n))
    ns = xi.shape[0]
    x = np.empty((ns, N, 2))
    x[..., 0] = xi.reshape(ns, N).real
    x[..., 1] = xi.reshape(ns, N).imag
    e = np.ascontiguousarray(eps[:ns], dtype=np.float64)
    sa = np.ascontiguousarray(sigma_app, dtype=np.float64)
    eo = np.zeros((9, N)); so = np.zeros((9, N)); ae = np.zeros(9); asg = np.zeros(9)
    L.oracle_strain_stress(*n, ns, C11, C12, C44, e, *map(float, d), x, sa, eo, so, ae, asg, nthreads())
    return eo.reshape(3, 3, N), so.reshape(3, 3, N), ae.reshape(3, 3), asg.reshape(3, 3)
