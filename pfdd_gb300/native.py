"""ctypes bindings of ``libpfdd_gb300.so`` (the C ABI in include/pfdd_gpu.h).

This is the Python mirror of the reference's operator interface for the hot path:
:class:`Solver` holds one context (a solve or a batch of replicas sharing B(k)) and
:class:`FFTPlan` is the drop-in for ``fft_forward`` / ``fft_backward``
(``PFDD_Final_GPU.c:209-273``).  There is no fallback: if the native library is
missing the import fails.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path
from typing import Optional, Sequence

import numpy as np

from . import workloads

LIB_PATH = Path(__file__).resolve().parent / "_lib" / "libpfdd_gb300.so"

PFDD_OK, PFDD_EINVAL, PFDD_ENOMEM, PFDD_ECUDA, PFDD_ETIMEOUT, PFDD_ENONFINITE, PFDD_ENOTREADY, PFDD_ELIMIT = range(8)
PRECISIONS = {"fp64": 0, "fp32": 1, "fp32_bfly": 2}

# every entry point declared in include/pfdd_gpu.h and include/pfdd_setup.h
EXPORTS = [
    "pfdd_create", "pfdd_create_batched", "pfdd_destroy", "pfdd_last_error", "pfdd_set_B", "pfdd_get_B",
    "pfdd_build_B",
    "pfdd_set_params", "pfdd_set_state", "pfdd_set_replica_state", "pfdd_set_tau_field", "pfdd_step",
    "pfdd_get_state", "pfdd_get_replica_state", "pfdd_set_replica_active", "pfdd_last_launch_count",
    "pfdd_required_bytes", "pfdd_fft_plan_create", "pfdd_fft_plan_destroy", "pfdd_fft_forward",
    "pfdd_fft_backward", "pfdd_status_string", "pfdd_frec", "pfdd_setfcc", "pfdd_setorient", "pfdd_seteps",
    "pfdd_resolve_shear", "pfdd_ramp_tau", "pfdd_get_stream", "pfdd_set_kernel_timing", "pfdd_kernel_stat",
    "pfdd_fft_device_noalloc", "pfdd_server_create", "pfdd_server_submit", "pfdd_server_wait",
    "pfdd_server_wait_run",
    "pfdd_server_stats", "pfdd_server_destroy", "pfdd_set_stream_priority", "pfdd_get_plan",
    "pfdd_strain_stress", "pfdd_set_diagnostics", "pfdd_get_diagnostics", "pfdd_state_diagnostics",
    "pfdd_converge_reset", "pfdd_step_converge", "pfdd_converge_reset_batched", "pfdd_step_converge_batched",
]

DIAG_COLUMNS = ("energy_in", "energy_in2", "energy_in3", "energy_in4", "energy_Residual", "energy_intotal")


class DiagParams(C.Structure):
    """pfdd_diag_params of include/pfdd_gpu.h."""
    _fields_ = [("ppoint", C.c_int * 3), ("interface_n", C.c_double * 3), ("sigma", C.c_double * 9),
                ("S11", C.c_double), ("S12", C.c_double), ("S44", C.c_double), ("mu", C.c_double),
                ("D", C.c_double * 4), ("ns_per_material", C.c_int)]


def reference_diag_params(n, sigma_max: float, C11: float, C12: float, C44: float, D=(0.0, 0.0, 0.0, 0.0),
                          ns_per_material: int = 0) -> DiagParams:
    """The reference program's interface-plane set-up: penetration point
    (N1/2, 0, 3 N3/4) (F:4195-4198), normal (sqrt3/3, 0, sqrt6/3) (F:4215-4217),
    the applied sigma_xz, compliances S11, S12, S44 (F:4261-4263), mu = C44."""
    p = DiagParams()
    p.ppoint[:] = [n[0] // 2, 0, n[2] * 3 // 4]
    p.interface_n[:] = [np.sqrt(3.0) / 3.0, 0.0, np.sqrt(6.0) / 3.0]
    sig = [0.0] * 9
    sig[2] = sig[6] = sigma_max
    p.sigma[:] = sig
    p.S11 = 1.0 / 3.0 * (1 / (C11 + 2 * C12) + 2 / (C11 - C12))
    p.S12 = 1.0 / 3.0 * (1 / (C11 + 2 * C12) - 1 / (C11 - C12))
    p.S44 = 1 / C44
    p.mu = C44
    p.D[:] = list(D)
    p.ns_per_material = ns_per_material
    return p

_lib = None


class PFDDError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{msg} (status {status})")
        self.status = status


def load():
    """Load the native library (built in-tree by ``pfdd_gb300.build``)."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise RuntimeError(f"native library {LIB_PATH} is missing: run pfdd_gb300.build.build()")
    L = C.CDLL(str(LIB_PATH))
    vp, i, d, sz = C.c_void_p, C.c_int, C.c_double, C.c_size_t
    dp = C.POINTER(C.c_double)
    L.pfdd_create.argtypes = [C.POINTER(vp), i, i, i, i, i, i]
    L.pfdd_create_batched.argtypes = [C.POINTER(vp), i, i, i, i, i, i, i]
    L.pfdd_destroy.argtypes = [vp]
    L.pfdd_destroy.restype = None
    L.pfdd_last_error.argtypes = [vp]
    L.pfdd_last_error.restype = C.c_char_p
    L.pfdd_set_B.argtypes = [vp, dp]
    L.pfdd_get_B.argtypes = [vp, dp]
    L.pfdd_build_B.argtypes = [vp, d, d, d, dp, d, d, d]
    L.pfdd_set_params.argtypes = [vp, dp, dp, dp, d]
    L.pfdd_set_state.argtypes = [vp, dp, dp]
    L.pfdd_set_replica_state.argtypes = [vp, i, dp, dp]
    L.pfdd_set_tau_field.argtypes = [vp, dp]
    L.pfdd_step.argtypes = [vp, i, dp, dp, dp]
    L.pfdd_converge_reset.argtypes = [vp, d]
    L.pfdd_step_converge.argtypes = [vp, i, dp, dp, dp, C.POINTER(C.c_int)]
    L.pfdd_converge_reset_batched.argtypes = [vp, dp]
    L.pfdd_step_converge_batched.argtypes = [vp, i, dp, dp, dp, C.POINTER(C.c_int)]
    L.pfdd_get_state.argtypes = [vp, dp]
    L.pfdd_get_replica_state.argtypes = [vp, i, dp]
    L.pfdd_set_replica_active.argtypes = [vp, i, i]
    L.pfdd_last_launch_count.argtypes = [vp]
    L.pfdd_last_launch_count.restype = C.c_longlong
    L.pfdd_get_stream.argtypes = [vp]
    L.pfdd_get_stream.restype = vp
    L.pfdd_set_stream_priority.argtypes = [vp, i]
    L.pfdd_get_plan.argtypes = [vp, C.c_char_p, sz]
    L.pfdd_strain_stress.argtypes = [vp, i, dp, dp, dp, dp, dp]
    L.pfdd_set_diagnostics.argtypes = [vp, C.POINTER(DiagParams)]
    L.pfdd_get_diagnostics.argtypes = [vp, i, dp]
    L.pfdd_state_diagnostics.argtypes = [vp, dp]
    L.pfdd_set_kernel_timing.argtypes = [vp, i]
    L.pfdd_kernel_stat.argtypes = [vp, i, C.POINTER(C.c_char_p), C.POINTER(C.c_longlong), C.POINTER(C.c_double)]
    L.pfdd_required_bytes.argtypes = [i, i, i, i, i, i]
    L.pfdd_required_bytes.restype = sz
    L.pfdd_fft_plan_create.argtypes = [C.POINTER(vp), i, i, i, i, i, i]
    L.pfdd_fft_plan_destroy.argtypes = [vp]
    L.pfdd_fft_plan_destroy.restype = None
    L.pfdd_fft_forward.argtypes = [vp, vp, i, i]
    L.pfdd_fft_backward.argtypes = [vp, vp, i, i]
    L.pfdd_fft_device_noalloc.argtypes = [vp, i, i, i, i, i, i, vp]
    L.pfdd_status_string.argtypes = [i]
    L.pfdd_status_string.restype = C.c_char_p
    L.pfdd_frec.argtypes = [i, d, dp]
    L.pfdd_frec.restype = None
    L.pfdd_setfcc.argtypes = [dp, dp, d]
    L.pfdd_setfcc.restype = None
    L.pfdd_setorient.argtypes = [dp]
    L.pfdd_setorient.restype = None
    L.pfdd_seteps.argtypes = [i, dp, dp, dp, dp, dp]
    L.pfdd_seteps.restype = None
    L.pfdd_resolve_shear.argtypes = [i, dp, dp, dp]
    L.pfdd_resolve_shear.restype = None
    L.pfdd_ramp_tau.argtypes = [i, dp, i, dp]
    L.pfdd_ramp_tau.restype = None
    ll = C.c_longlong
    L.pfdd_server_create.argtypes = [C.POINTER(vp), i, i, sz, i, i]
    L.pfdd_server_submit.argtypes = [vp, vp, C.POINTER(ll)]
    L.pfdd_server_wait.argtypes = [vp, ll, dp, dp, dp]
    L.pfdd_server_wait_run.argtypes = [vp, ll, dp, dp, dp, C.POINTER(C.c_int)]
    L.pfdd_server_stats.argtypes = [vp, C.POINTER(ll), C.POINTER(ll), C.POINTER(ll), C.POINTER(sz)]
    L.pfdd_server_destroy.argtypes = [vp]
    L.pfdd_server_destroy.restype = None
    _lib = L
    return L


def _dp(a: Optional[np.ndarray]):
    if a is None:
        return None
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _f64(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float64)


def _interleave(z: np.ndarray) -> np.ndarray:
    out = np.empty(z.shape + (2,), dtype=np.float64)
    out[..., 0] = z.real
    out[..., 1] = z.imag
    return out


# ---- setup helpers (host C code of the library) -------------------------------

def fcc_eps(ns: int = 12, bdiv: float = float(np.sqrt(2.0)), dslip: float = 1.0) -> np.ndarray:
    L = load()
    xn = np.zeros((12, 3)); xb = np.zeros((12, 3)); th = np.zeros((3, 3)); eps = np.zeros((12, 3, 3))
    L.pfdd_setfcc(_dp(xn), _dp(xb), bdiv)
    L.pfdd_setorient(_dp(th))
    ds = np.full(12, dslip)
    L.pfdd_seteps(12, _dp(xn), _dp(xb), _dp(ds), _dp(th), _dp(eps))
    return eps[:ns].copy()


def resolved_shear(eps: np.ndarray, sigma: np.ndarray) -> np.ndarray:
    L = load()
    e = _f64(eps); s = _f64(sigma); tau = np.zeros(e.shape[0])
    L.pfdd_resolve_shear(e.shape[0], _dp(s), _dp(e), _dp(tau))
    return tau


def ramp_tau(tau_max: np.ndarray, steps: int) -> np.ndarray:
    L = load()
    t = _f64(tau_max); out = np.zeros((steps, t.shape[0]))
    L.pfdd_ramp_tau(t.shape[0], _dp(t), steps, _dp(out))
    return out


class Solver:
    """One GPU context: ``nrep`` replicas of an ``n`` grid with ``ns`` slip systems."""

    def __init__(self, n: Sequence[int], ns: int, precision: str = "fp64", nrep: int = 1, device: int = 0):
        self.L = load()
        self.n = tuple(int(v) for v in n)
        self.ns, self.nrep, self.precision = int(ns), int(nrep), precision
        self.N = int(np.prod(self.n))
        h = C.c_void_p()
        st = self.L.pfdd_create_batched(C.byref(h), *self.n, self.ns, self.nrep, PRECISIONS[precision], device)
        self.h = h
        self._check(st, "pfdd_create_batched")

    def _check(self, st: int, what: str):
        if st != PFDD_OK:
            msg = self.L.pfdd_last_error(self.h).decode() if self.h else ""
            raise PFDDError(st, f"{what}: {self.L.pfdd_status_string(st).decode()} {msg}")

    def close(self):
        if getattr(self, "h", None):
            self.L.pfdd_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def build_B(self, C11: float, C12: float, C44: float, eps: np.ndarray, d=(1.0, 1.0, 1.0)):
        e = _f64(eps[: self.ns])
        self._check(self.L.pfdd_build_B(self.h, C11, C12, C44, _dp(e), *map(float, d)), "pfdd_build_B")

    def set_B(self, B: np.ndarray):
        b = _f64(B)
        assert b.size == self.ns * self.ns * self.N
        self._check(self.L.pfdd_set_B(self.h, _dp(b)), "pfdd_set_B")

    def get_B(self) -> np.ndarray:
        b = np.zeros((self.ns, self.ns) + self.n)
        self._check(self.L.pfdd_get_B(self.h, _dp(b)), "pfdd_get_B")
        return b

    def set_params(self, cd2, asf, dslip, uq2: float = 1.0):
        a, b, c = (_f64(np.broadcast_to(v, (self.ns,))) for v in (cd2, asf, dslip))
        self._check(self.L.pfdd_set_params(self.h, _dp(a), _dp(b), _dp(c), float(uq2)), "pfdd_set_params")

    def set_state(self, xi: np.ndarray, bc: Optional[np.ndarray] = None):
        x = _interleave(np.asarray(xi, dtype=np.complex128).reshape(self.nrep, self.ns, self.N))
        b = None
        if bc is not None:
            bb = _f64(np.asarray(bc).reshape(self.nrep, self.ns, self.N))
            b = np.ascontiguousarray(np.stack([bb, bb], axis=-1))
        self._check(self.L.pfdd_set_state(self.h, _dp(x), _dp(b)), "pfdd_set_state")

    def set_replica_state(self, r: int, xi: np.ndarray, bc: Optional[np.ndarray] = None):
        x = _interleave(np.asarray(xi, dtype=np.complex128).reshape(self.ns, self.N))
        b = None
        if bc is not None:
            bb = _f64(np.asarray(bc).reshape(self.ns, self.N))
            b = np.ascontiguousarray(np.stack([bb, bb], axis=-1))
        self._check(self.L.pfdd_set_replica_state(self.h, r, _dp(x), _dp(b)), "pfdd_set_replica_state")

    def set_tau_field(self, tf: Optional[np.ndarray]):
        t = None if tf is None else _f64(tf)
        self._check(self.L.pfdd_set_tau_field(self.h, _dp(t)), "pfdd_set_tau_field")

    def set_active(self, r: int, on: bool):
        self._check(self.L.pfdd_set_replica_active(self.h, r, int(bool(on))), "pfdd_set_replica_active")

    def step(self, tau: np.ndarray):
        """Runs len(tau) steps; tau is [K, nrep, ns] (or [K, ns] for nrep == 1).
        Returns gamma [K, nrep] and gamma_a [K, nrep, ns]."""
        t = _f64(np.asarray(tau).reshape(-1, self.nrep, self.ns))
        K = t.shape[0]
        g = np.zeros((K, self.nrep)); ga = np.zeros((K, self.nrep, self.ns))
        self._check(self.L.pfdd_step(self.h, K, _dp(t), _dp(g), _dp(ga)), "pfdd_step")
        return g, ga

    def converge_reset(self, gamma_prev: float = 0.0):
        """Starts an inner loop for step_converge (F:4567-4572); gamma_prev is
        the gamma its first step is compared with (F:4575)."""
        self._check(self.L.pfdd_converge_reset(self.h, float(gamma_prev)), "pfdd_converge_reset")

    def step_converge(self, tau: np.ndarray):
        """Runs at most len(tau) steps (tau [K, ns]; nrep == 1) and stops where
        the reference's convergence test (plasticconverge, F:3732-3785) ends the
        inner loop.  Returns gamma [k] and gamma_a [k, ns] of the k steps run."""
        t = _f64(np.asarray(tau).reshape(-1, self.ns))
        K = t.shape[0]
        g = np.zeros(K); ga = np.zeros((K, self.ns)); done = C.c_int(0)
        self._check(self.L.pfdd_step_converge(self.h, K, _dp(t), _dp(g), _dp(ga), C.byref(done)),
                    "pfdd_step_converge")
        k = done.value
        return g[:k].copy(), ga[:k].copy()

    def converge_reset_batched(self, gamma_prev):
        """Per-replica start of an inner loop: gamma_prev [nrep]."""
        gp = _f64(np.broadcast_to(np.asarray(gamma_prev, dtype=np.float64), (self.nrep,)))
        self._check(self.L.pfdd_converge_reset_batched(self.h, _dp(gp)), "pfdd_converge_reset_batched")

    def step_converge_batched(self, tau: np.ndarray):
        """Every active replica's inner loop with its own stop: tau [K, nrep, ns].
        Returns (steps run [nrep], gamma [K, nrep], gamma_a [K, nrep, ns]); a
        replica's entries past its stop are zero."""
        t = _f64(np.asarray(tau).reshape(-1, self.nrep, self.ns))
        K = t.shape[0]
        g = np.zeros((K, self.nrep)); ga = np.zeros((K, self.nrep, self.ns))
        done = (C.c_int * self.nrep)()
        self._check(self.L.pfdd_step_converge_batched(self.h, K, _dp(t), _dp(g), _dp(ga), done),
                    "pfdd_step_converge_batched")
        return np.array(list(done)), g, ga

    def get_state(self) -> np.ndarray:
        x = np.zeros((self.nrep, self.ns, self.N, 2))
        self._check(self.L.pfdd_get_state(self.h, _dp(x)), "pfdd_get_state")
        return (x[..., 0] + 1j * x[..., 1]).reshape((self.nrep, self.ns) + self.n)

    def get_replica_state(self, r: int) -> np.ndarray:
        x = np.zeros((self.ns, self.N, 2))
        self._check(self.L.pfdd_get_replica_state(self.h, r, _dp(x)), "pfdd_get_replica_state")
        return (x[..., 0] + 1j * x[..., 1]).reshape((self.ns,) + self.n)

    @property
    def launches(self) -> int:
        return int(self.L.pfdd_last_launch_count(self.h))

    @property
    def stream(self) -> int:
        """The context's cudaStream_t as an integer handle."""
        return int(self.L.pfdd_get_stream(self.h) or 0)

    def kernel_timing(self, on: bool):
        self._check(self.L.pfdd_set_kernel_timing(self.h, int(bool(on))), "pfdd_set_kernel_timing")

    def strain_stress(self, sigma_app: np.ndarray, r: int = 0, fields: bool = True):
        """Strain and stress of replica r: (eps [3,3,N], sigma [3,3,N], aveps [3,3],
        avesigma [3,3]); the fields are None with fields=False."""
        sa = _f64(sigma_app).reshape(9)
        e = np.zeros((9, self.N)) if fields else None
        s = np.zeros((9, self.N)) if fields else None
        ae = np.zeros(9); asg = np.zeros(9)
        self._check(self.L.pfdd_strain_stress(self.h, r, _dp(sa), _dp(e), _dp(s), _dp(ae), _dp(asg)),
                    "pfdd_strain_stress")
        rs = (lambda a: None if a is None else a.reshape(3, 3, self.N))
        return rs(e), rs(s), ae.reshape(3, 3), asg.reshape(3, 3)

    def set_diagnostics(self, params: "DiagParams | None"):
        """Interface-plane energy diagnostics per step (None turns them off)."""
        self._check(self.L.pfdd_set_diagnostics(self.h, C.byref(params) if params is not None else None),
                    "pfdd_set_diagnostics")

    def diagnostics(self, nsteps: int) -> np.ndarray:
        """Energies of each step of the last step() call, [nsteps, nrep, 6] (DIAG_COLUMNS)."""
        out = np.zeros((nsteps, self.nrep, 6))
        self._check(self.L.pfdd_get_diagnostics(self.h, nsteps, _dp(out)), "pfdd_get_diagnostics")
        return out

    def state_diagnostics(self) -> np.ndarray:
        """Energies of the current state of every replica, [nrep, 6] (DIAG_COLUMNS)."""
        out = np.zeros((self.nrep, 6))
        self._check(self.L.pfdd_state_diagnostics(self.h, _dp(out)), "pfdd_state_diagnostics")
        return out

    def plan(self) -> dict:
        """Launch plan (tile widths, threads, shared memory, radix plans, autotune timings)."""
        import json
        buf = C.create_string_buffer(16384)
        self._check(self.L.pfdd_get_plan(self.h, buf, len(buf)), "pfdd_get_plan")
        return json.loads(buf.value.decode())

    def kernel_stats(self) -> dict:
        """{kernel name: (timed launches, total device ms)} since timing was enabled."""
        out = {}
        idx = 0
        while True:
            nm = C.c_char_p(); cnt = C.c_longlong(); ms = C.c_double()
            st = self.L.pfdd_kernel_stat(self.h, idx, C.byref(nm), C.byref(cnt), C.byref(ms))
            if st != PFDD_OK:
                break
            if cnt.value:
                out[nm.value.decode()] = (int(cnt.value), float(ms.value))
            idx += 1
        return out


class FFTPlan:
    """In-place unnormalised 3D C2C transforms (``fft_forward`` / ``fft_backward``)."""

    def __init__(self, n: Sequence[int], precision: str = "fp32", max_batch: int = 1, device: int = 0):
        self.L = load()
        self.n = tuple(int(v) for v in n)
        self.precision = precision
        h = C.c_void_p()
        st = self.L.pfdd_fft_plan_create(C.byref(h), *self.n, PRECISIONS[precision], max_batch, device)
        if st != PFDD_OK:
            raise PFDDError(st, "pfdd_fft_plan_create")
        self.h = h

    def _run(self, fn, data: np.ndarray, batch: int):
        dt = np.float64 if self.precision == "fp64" else np.float32
        assert data.dtype == dt and data.flags.c_contiguous
        st = fn(self.h, data.ctypes.data_as(C.c_void_p), batch, 0)
        if st != PFDD_OK:
            raise PFDDError(st, "pfdd_fft")

    def forward(self, data: np.ndarray, batch: int):
        self._run(self.L.pfdd_fft_forward, data, batch)

    def backward(self, data: np.ndarray, batch: int):
        self._run(self.L.pfdd_fft_backward, data, batch)

    def close(self):
        if getattr(self, "h", None):
            self.L.pfdd_fft_plan_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def solver_for(spec: workloads.SolveSpec, precision: str = "fp64", nrep: int = 1, device: int = 0) -> Solver:
    """Context for a :class:`SolveSpec`: B(k) built on the device, parameters set."""
    s = Solver(spec.n, spec.ns, precision, nrep, device)
    eps = fcc_eps(spec.ns, dslip=spec.dslip)
    C44, C12 = spec.mu, spec.lam
    s.build_B(spec.C11, C12, C44, eps, spec.d)
    s.set_params(spec.cd2, spec.asf, spec.dslip, spec.uq2)
    return s


def spec_tau(spec: workloads.SolveSpec) -> np.ndarray:
    """Per-step resolved shear stress [K, ns] of the sigma_xz ramp 0 -> sigma_max."""
    eps = fcc_eps(spec.ns, dslip=spec.dslip)
    sig = np.zeros((3, 3)); sig[0, 2] = sig[2, 0] = spec.sigma_max
    return ramp_tau(resolved_shear(eps, sig), spec.steps)
