"""Serving form: many independent PFDD solves queued on one GPU.

Thin binding of ``include/pfdd_serve.h``; the scheduler itself (classes of
solves sharing a batched context, one worker thread and CUDA stream per class,
device-memory admission, continuous admission between step chunks) is native
code in the library (``csrc/pfdd_server.cpp``).

Each solve is one run of the reference program's TDGL loop (main,
PFDD_Final_GPU.c:4574-4691) on its own grid, slip systems, stress ramp and
initial state.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import Optional

import numpy as np

from . import native, workloads


class _Request(C.Structure):
    _fields_ = [
        ("n1", C.c_int), ("n2", C.c_int), ("n3", C.c_int), ("ns", C.c_int), ("steps", C.c_int),
        ("C11", C.c_double), ("C12", C.c_double), ("C44", C.c_double),
        ("cd2", C.c_double), ("asf", C.c_double), ("dslip", C.c_double), ("uq2", C.c_double),
        ("d1", C.c_double), ("d2", C.c_double), ("d3", C.c_double),
        ("eps", C.POINTER(C.c_double)), ("tau_max", C.POINTER(C.c_double)),
        ("xi", C.POINTER(C.c_double)), ("xi_bc", C.POINTER(C.c_double)), ("xi_out", C.POINTER(C.c_double)),
        ("converge", C.c_int), ("gamma_prev", C.c_double),
    ]


@dataclass
class Result:
    xi: Optional[np.ndarray]  # [ns, N] complex128 final order parameter (None if not requested)
    gamma: np.ndarray     # [steps]
    gamma_a: np.ndarray   # [steps, ns]
    latency_s: float      # submit -> completion
    steps_run: int = 0    # steps the solve ran (fewer than steps when a converging solve stopped)


class Server:
    """Queue of solves on one GPU (``pfdd_server_*``)."""

    def __init__(self, precision: str = "fp32", device: int = 0, hbm_budget: int = 0, max_slots: int = 16,
                 chunk_steps: int = 50):
        self.L = native.load()
        h = C.c_void_p()
        st = self.L.pfdd_server_create(C.byref(h), native.PRECISIONS[precision], device, int(hbm_budget),
                                       int(max_slots), int(chunk_steps))
        if st != native.PFDD_OK:
            raise native.PFDDError(st, f"pfdd_server_create: {self.L.pfdd_status_string(st).decode()}")
        self.h = h
        self._held = {}

    def submit_raw(self, n, ns: int, steps: int, C11: float, C12: float, C44: float, eps: np.ndarray,
                   tau_max: np.ndarray, xi: np.ndarray, bc: Optional[np.ndarray] = None, cd2: float = 0.01,
                   asf: float = 0.1, dslip: float = 1.0, uq2: float = 1.0, d=(1.0, 1.0, 1.0),
                   want_xi: bool = True, converge: bool = False, gamma_prev: float = 0.0) -> int:
        """Queues a solve from raw inputs.  xi is complex [ns, ...] or already
        interleaved float64 [ns, N, 2]; the arrays are held until :meth:`wait`."""
        n = tuple(int(v) for v in n)
        N = int(np.prod(n))
        e = native._f64(np.asarray(eps)[:ns])
        t = native._f64(tau_max)
        if isinstance(xi, np.ndarray) and xi.dtype == np.float64 and xi.size == ns * N * 2 and xi.flags.c_contiguous:
            x = xi  # already interleaved [ns][N][2]
        else:
            x = native._interleave(np.asarray(xi, dtype=np.complex128).reshape(ns, N))
        b = None
        if bc is not None:
            bb = native._f64(np.asarray(bc).reshape(ns, N))
            b = np.ascontiguousarray(np.stack([bb, bb], axis=-1))
        out = np.empty((ns, N, 2)) if want_xi else None
        q = _Request(n[0], n[1], n[2], int(ns), int(steps), C11, C12, C44, cd2, asf, dslip, uq2,
                     float(d[0]), float(d[1]), float(d[2]), native._dp(e), native._dp(t), native._dp(x),
                     native._dp(b), native._dp(out), int(bool(converge)), float(gamma_prev))
        rid = C.c_longlong()
        st = self.L.pfdd_server_submit(self.h, C.byref(q), C.byref(rid))
        if st != native.PFDD_OK:
            raise native.PFDDError(st, f"pfdd_server_submit: {self.L.pfdd_status_string(st).decode()}")
        self._held[rid.value] = (ns, steps, x, b, out)  # the server reads/writes these until wait
        return rid.value

    def submit(self, spec: workloads.SolveSpec, converge: bool = False) -> int:
        """Queues one :class:`SolveSpec` (FCC slip systems, sigma_xz ramp); with
        ``converge`` the solve also ends at the reference's convergence stop."""
        eps = native.fcc_eps(spec.ns, dslip=spec.dslip)
        sig = np.zeros((3, 3)); sig[0, 2] = sig[2, 0] = spec.sigma_max
        tau_max = native.resolved_shear(eps, sig)
        xi, bc = workloads.initial_state(spec)
        C44, C12 = spec.mu, spec.lam
        return self.submit_raw(spec.n, spec.ns, spec.steps, spec.C11, C12, C44, eps, tau_max, xi, bc,
                               cd2=spec.cd2, asf=spec.asf, dslip=spec.dslip, uq2=spec.uq2, d=spec.d,
                               converge=converge)

    def wait(self, rid: int) -> Result:
        ns, steps, _, _, out = self._held[rid]
        g = np.zeros(steps); ga = np.zeros((steps, ns)); lat = C.c_double(); ran = C.c_int()
        st = self.L.pfdd_server_wait_run(self.h, rid, native._dp(g), native._dp(ga), C.byref(lat), C.byref(ran))
        del self._held[rid]
        if st != native.PFDD_OK:
            raise native.PFDDError(st, f"pfdd_server_wait: {self.L.pfdd_status_string(st).decode()}")
        xi = None if out is None else out[..., 0] + 1j * out[..., 1]
        return Result(xi, g, ga, lat.value, ran.value)

    def stats(self) -> dict:
        a, b, c = C.c_longlong(), C.c_longlong(), C.c_longlong(); p = C.c_size_t()
        self.L.pfdd_server_stats(self.h, C.byref(a), C.byref(b), C.byref(c), C.byref(p))
        return {"steps_done": a.value, "solves_done": b.value, "classes_created": c.value, "peak_bytes": p.value}

    def close(self):
        if getattr(self, "h", None):
            self.L.pfdd_server_destroy(self.h)  # finishes every queued solve first
            self.h = None
            self._held.clear()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
