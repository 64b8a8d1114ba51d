"""Generate the golden vectors in tests/golden/ by running the patched reference program.

Run here (where the reference checkout exists): ``python tests/golden/make_golden.py``.
For every case it builds the patched reference (oracle/build_ref.py) in FP64
(``-Dfloat=double``, the reference's own double-precision run) and in its stock FP32
spectral precision, writes the seeded inputs as xi.dat / xi_bc.dat (the reference is
built with 12 FCC systems; systems beyond the case's ``ns`` are zero and pinned), runs
it, and stores per-step gamma / gamma_a (full precision) and the final xi (full field
for small grids, a seeded sample of points otherwise) in ``<case>.npz``.  The
``strain_*`` cases hold the reference's strain and stress fields of an initial state.
"""
from __future__ import annotations

import json
import shutil
import sys
import tempfile
from concurrent.futures import ThreadPoolExecutor
from dataclasses import asdict
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "oracle"))

import build_ref  # noqa: E402
from pfdd_gb300 import refio, workloads  # noqa: E402

OUT = Path(__file__).resolve().parent
FULL_LIMIT = 8192  # grids up to this many points store the full final field


def cases():
    c0 = workloads.config0()
    yield "config0_32c_ns3_k200", c0
    yield "fcc12_8x16x32_k40", workloads.SolveSpec(
        n=(8, 16, 32), ns=12, steps=40, sigma_max=0.05,
        loops=workloads.random_loops((8, 16, 32), 4, 2.0, 5.0, 12, seed=7), noise_seed=7)
    yield "quasi2d_32x2x32_ns3_k50", workloads.SolveSpec(
        n=(32, 2, 32), ns=3, steps=50, sigma_max=0.03,
        loops=[workloads.Loop(0, (16, 0, 16), 6.0), workloads.Loop(1, (10, 1, 8), 4.0)], noise_seed=3)
    yield "fcc12_8c_k30", workloads.SolveSpec(
        n=(8, 8, 8), ns=12, steps=30, sigma_max=0.08,
        loops=workloads.random_loops((8, 8, 8), 3, 1.5, 3.0, 12, seed=11), noise_seed=11)
    yield "config1_64c_ns12_k10", workloads.config1(steps=10, n=64)
    # anisotropic grid spacing (frec divides by d per axis, so B(k) changes) with
    # material and kinetic constants other than the defaults
    yield "fcc12_32x8x16_aniso_k30", workloads.SolveSpec(
        n=(32, 8, 16), ns=12, steps=30, sigma_max=0.05,
        loops=workloads.random_loops((32, 8, 16), 3, 2.0, 4.0, 12, seed=21), noise_seed=21,
        nu=0.25, asf=0.15, cd2=0.02, d=(1.0, 0.5, 2.0))
    # a tenth of every field's points held fixed (xi_bc = 1), some inside the loops
    yield "fcc12_16c_pinned_k30", workloads.SolveSpec(
        n=(16, 16, 16), ns=12, steps=30, sigma_max=0.06,
        loops=workloads.random_loops((16, 16, 16), 4, 2.5, 5.0, 12, seed=31), noise_seed=31,
        pin_frac=0.1, pin_seed=31)
    # slip-plane spacing 2 (the eigenstrains b n / dslip and the update's tau / dslip)
    yield "fcc12_16x32x8_dslip2_k30", workloads.SolveSpec(
        n=(16, 32, 8), ns=12, steps=30, sigma_max=0.1,
        loops=workloads.random_loops((16, 32, 8), 3, 2.0, 4.0, 12, seed=41), noise_seed=41, dslip=2.0)
    # the update's factor of the elastic force (Re and Im) at 0.6
    yield "fcc12_32x16x8_uq2_k30", workloads.SolveSpec(
        n=(32, 16, 8), ns=12, steps=30, sigma_max=0.05,
        loops=workloads.random_loops((32, 16, 8), 3, 2.0, 4.0, 12, seed=51), noise_seed=51, uq2=0.6)
    # a cubic material (C11 != 2 mu + lambda) with mu = 1.5
    yield "fcc12_16x16x32_cubic_k30", workloads.SolveSpec(
        n=(16, 16, 32), ns=12, steps=30, sigma_max=0.08,
        loops=workloads.random_loops((16, 16, 32), 3, 2.0, 4.0, 12, seed=61), noise_seed=61,
        mu=1.5, nu=0.3, c11=6.0)


def spec_json(spec: workloads.SolveSpec) -> str:
    d = asdict(spec)
    return json.dumps(d)


def run_case(name: str, spec: workloads.SolveSpec, fp64: bool, krun: int | None = None):
    b = build_ref.compile_ref(n=spec.n, k=spec.steps, sigma=spec.sigma_max, fp64=fp64,
                              asf=spec.asf, cd2=spec.cd2, mu=spec.mu, lam=spec.lam, d=spec.d,
                              dslip=spec.dslip, uq2=spec.uq2, c11=spec.c11)
    d = Path(tempfile.mkdtemp(prefix=f"golden_{name}_"))
    try:
        xi, bc = workloads.initial_state(spec)
        refio.write_xi_files(d, xi, bc, ns_ref=12)
        build_ref.run_ref(b, d, krun=krun)
        g = refio.read_gamma_full(d / "gamma_full.dat")
        xf = refio.read_xi_file(d / "xi.dat", spec.n, 12 + refio.NV)
        return g, xf[:spec.ns]
    finally:
        shutil.rmtree(d, ignore_errors=True)


def sample_points(npts: int, count: int, seed: int) -> np.ndarray:
    rng = np.random.Generator(np.random.PCG64(seed))
    return np.sort(rng.choice(npts, size=min(count, npts), replace=False))


def make(name: str, spec: workloads.SolveSpec, krun: int | None = None):
    """krun: the reference runs only the first ``krun`` steps of the spec's K-step
    ramp (a prefix of the full solve; the ramp divisor stays K)."""
    with ThreadPoolExecutor(2) as ex:
        f64 = ex.submit(run_case, name, spec, True, krun)
        f32 = ex.submit(run_case, name, spec, False, krun)
        (g64, x64), (g32, x32) = f64.result(), f32.result()
    K = spec.steps if krun is None else krun
    assert g64.shape[0] == K, f"{name}: reference stopped after {g64.shape[0]} steps"
    npts = spec.npts
    xi0, _ = workloads.initial_state(spec)
    out = dict(spec=spec_json(spec), steps_run=np.array(K), gamma=g64[:, 1], gamma_a=g64[:, 2:2 + spec.ns],
               gamma_fp32ref=g32[:, 1], gamma_a_fp32ref=g32[:, 2:2 + spec.ns],
               xi0_checksum=np.array([xi0.real.sum(), (xi0.real ** 2).sum()]),
               xi_final_checksum=np.array([x64.real.sum(), x64.imag.sum(), (np.abs(x64) ** 2).sum()]),
               fp32ref_max_dxi=np.array(np.max(np.abs(x32 - x64))))
    flat = x64.reshape(spec.ns, -1)
    if npts <= FULL_LIMIT:
        out["xi_final"] = flat
    else:
        idx = sample_points(npts, 2048, seed=12345)
        out["sample_idx"] = idx
        out["xi_final_sample"] = flat[:, idx]
    np.savez_compressed(OUT / f"{name}.npz", **out)
    print(f"{name}: K={K} gamma[-1]={g64[-1, 1]:.6e} fp32-ref max|dxi|={float(out['fp32ref_max_dxi']):.2e}")


def prefix_cases():
    """Prefixes of full-size solves: (name, spec, steps run).  The 128^3 x 12
    config-1 solve (8 seeded loops, sigma_xz ramp 0 -> 0.05 over K = 1000
    steps): its first 5 steps, so the reference's setup (Bmatrix at 128^3)
    dominates the generation time."""
    yield "config1_128c_ns12_prefix5", workloads.config1(), 5


def make_oracle_long(name: str = "oracle_config1_128c_ns12_k1000", every: int = 100, keep=(100, 1000)):
    """The whole 1000-step config-1 solve (128^3 x 12) run by the CPU FP64
    restatement (oracle/pfdd_cpu.c), which the reference-generated cases pin to the
    reference itself (at 128^3 through config1_128c_ns12_prefix5): gamma and gamma_a
    of every step and a seeded sample of xi at the steps ``keep``.  The reference
    at this size runs for hours on one core; the restatement on all cores in
    minutes."""
    import oracle as orc
    spec = workloads.config1()
    eps = orc.fcc_eps(spec.ns, dslip=np.full(12, spec.dslip))
    C44, C12 = spec.mu, spec.lam
    B = orc.bmatrix(spec.n, eps, spec.C11, C12, C44, spec.d)
    sig = np.zeros((3, 3)); sig[0, 2] = sig[2, 0] = spec.sigma_max
    tau = orc.ramp_tau(orc.resolved_shear(eps, sig), spec.steps)
    xi, bc = workloads.initial_state(spec)
    idx = sample_points(spec.npts, 1024, seed=4242)
    gs, gas, samples = [], [], []
    ns = spec.ns
    for s0 in range(0, spec.steps, every):
        xi, g, ga = orc.run(spec.n, B, xi, bc, np.full(ns, spec.cd2), np.full(ns, spec.asf),
                            np.full(ns, spec.dslip), 1.0, tau[s0:s0 + every])
        gs.append(g); gas.append(ga)
        if s0 + every in keep:
            samples.append(xi.reshape(ns, -1)[:, idx])
        print(f"{name}: step {s0 + every} gamma={g[-1]:.9e}", flush=True)
    out = dict(spec=spec_json(spec), gamma=np.concatenate(gs), gamma_a=np.concatenate(gas), sample_idx=idx,
               sample_steps=np.array(keep), xi_samples=np.stack(samples),
               generator=np.array("oracle/pfdd_cpu.c (FP64 restatement)"))
    np.savez_compressed(OUT / f"{name}.npz", **out)


def converge_cases():
    """Solves the reference stops early by its convergence test (plasticconverge,
    F:3732-3785): noise relaxing under no stress with the reference's own
    kinetic coefficient CD2 = 0.1; K = 300 steps allowed."""
    yield "converge_16c_ns3_cd01", workloads.SolveSpec(n=(16, 16, 16), ns=3, steps=300, sigma_max=0.0,
                                                       noise_seed=5, cd2=0.1)


def make_converge(name: str, spec: workloads.SolveSpec):
    g, x = run_case(name, spec, True)
    out = dict(spec=spec_json(spec), steps_run=np.array(g.shape[0]), gamma=g[:, 1], gamma_a=g[:, 2:2 + spec.ns],
               xi_final=x.reshape(spec.ns, -1),
               xi_final_checksum=np.array([x.real.sum(), x.imag.sum(), (np.abs(x) ** 2).sum()]))
    xi0, _ = workloads.initial_state(spec)
    out["xi0_checksum"] = np.array([xi0.real.sum(), (xi0.real ** 2).sum()])
    np.savez_compressed(OUT / f"{name}.npz", **out)
    print(f"{name}: the reference stopped after {g.shape[0]} of {spec.steps} steps")


def diag_cases():
    """Interface-plane energy diagnostics (patch 13 of oracle/build_ref.py): the
    reference's full-precision copies of checkEnergy.dat (one line per outer
    step) and checkEbarrier.dat's energies (one line per inner TDGL step)."""
    c0 = workloads.config0()
    c0.steps = 40
    yield "diag_config0_32c_ns3_k40", c0
    yield "diag_fcc12_16x8x32_k12", workloads.SolveSpec(
        n=(16, 8, 32), ns=12, steps=12, sigma_max=0.06,
        loops=workloads.random_loops((16, 8, 32), 4, 2.0, 5.0, 12, seed=41), noise_seed=41)
    # mu = 1.5, nu = 0.25, slip-plane spacing 2, Asf and CD2 off their defaults
    yield "diag_fcc12_16x8x16_mu15_k10", workloads.SolveSpec(
        n=(16, 8, 16), ns=12, steps=10, sigma_max=0.05,
        loops=workloads.random_loops((16, 8, 16), 3, 2.0, 4.0, 12, seed=81), noise_seed=81,
        mu=1.5, nu=0.25, dslip=2.0, asf=0.12, cd2=0.015)


def make_diag(name: str, spec: workloads.SolveSpec):
    import re
    b = build_ref.compile_ref(n=spec.n, k=spec.steps, sigma=spec.sigma_max, fp64=True, diag=True,
                              asf=spec.asf, cd2=spec.cd2, mu=spec.mu, lam=spec.lam, d=spec.d,
                              dslip=spec.dslip, uq2=spec.uq2, c11=spec.c11)
    d = Path(tempfile.mkdtemp(prefix=f"golden_{name}_"))
    try:
        xi, bc = workloads.initial_state(spec)
        refio.write_xi_files(d, xi, bc, ns_ref=12)
        build_ref.run_ref(b, d)
        outer = np.loadtxt(d / "energy_full.dat", ndmin=2)
        inner = np.loadtxt(d / "ebarrier_full.dat", ndmin=2)
        g = refio.read_gamma_full(d / "gamma_full.dat")
        log = (d / "stdout.log").read_text()
    finally:
        shutil.rmtree(d, ignore_errors=True)
    m = re.search(r"^D00 = (\S+), D11 = (\S+), D10 = (\S+), D01 = (\S+)", log, re.M)
    D = np.array([float(m.group(1)), float(m.group(4)), float(m.group(3)), float(m.group(2))])  # D00 D01 D10 D11
    out = dict(spec=spec_json(spec), energy_outer=outer, energy_inner=inner, gamma=g[:, 1], D=D,
               columns=np.array("step energy_in energy_in2 energy_in3 energy_in4 energy_Residual energy_intotal"))
    np.savez_compressed(OUT / f"{name}.npz", **out)
    print(f"{name}: {inner.shape[0]} inner lines, D = {D}")


def strain_cases():
    """Strain/stress of an initial state (patch 12 of oracle/build_ref.py): the
    reference dumps both fields in full precision and writes strain.txt,
    stress.txt and the averages of stress-strain.dat for the state it starts from."""
    yield "strain_fcc12_8x16x16", workloads.SolveSpec(
        n=(8, 16, 16), ns=12, steps=2, sigma_max=0.05,
        loops=workloads.random_loops((8, 16, 16), 4, 2.0, 5.0, 12, seed=31), noise_seed=31)
    c0 = workloads.config0()
    c0.steps = 2
    yield "strain_config0_32c_ns3", c0
    # anisotropic grid spacing, slip-plane spacing 2, mu = 1.5, nu = 0.25
    yield "strain_fcc12_16x8x16_aniso", workloads.SolveSpec(
        n=(16, 8, 16), ns=12, steps=2, sigma_max=0.05,
        loops=workloads.random_loops((16, 8, 16), 3, 2.0, 4.0, 12, seed=71), noise_seed=71,
        mu=1.5, nu=0.25, dslip=2.0, d=(2.0, 1.0, 0.5))


def make_strain(name: str, spec: workloads.SolveSpec):
    b = build_ref.compile_ref(n=spec.n, k=spec.steps, sigma=spec.sigma_max, fp64=True, strain=True,
                              asf=spec.asf, cd2=spec.cd2, mu=spec.mu, lam=spec.lam, d=spec.d,
                              dslip=spec.dslip, uq2=spec.uq2, c11=spec.c11)
    d = Path(tempfile.mkdtemp(prefix=f"golden_{name}_"))
    try:
        xi, bc = workloads.initial_state(spec)
        refio.write_xi_files(d, xi, bc, ns_ref=12)
        build_ref.run_ref(b, d)
        N = spec.npts
        # dumps: [component i + 3 j][point][re, im]; stored as [3 i + j][point], real parts
        e = np.fromfile(d / "eps_full.bin").reshape(9, N, 2)[..., 0]
        s = np.fromfile(d / "sigma_full.bin").reshape(9, N, 2)[..., 0]
        order = [i + 3 * j for i in range(3) for j in range(3)]
        e, s = e[order], s[order]
        ss = np.loadtxt(d / "stress-strain.dat")
        strain_txt = (d / "strain.txt").read_text().splitlines()
        stress_txt = (d / "stress.txt").read_text().splitlines()
    finally:
        shutil.rmtree(d, ignore_errors=True)
    out = dict(spec=spec_json(spec), aveps_txt=ss[0:18:2], avesigma_over_mu_txt=ss[1:18:2],
               strain_txt_head=np.array(strain_txt[:6]), strain_txt_lines=np.array(len(strain_txt)),
               stress_txt_head=np.array(stress_txt[:6]), stress_txt_lines=np.array(len(stress_txt)))
    if N <= FULL_LIMIT:
        out["eps"], out["sigma"] = e, s
    else:
        idx = sample_points(N, 2048, seed=777)
        out["sample_idx"], out["eps_sample"], out["sigma_sample"] = idx, e[:, idx], s[:, idx]
    np.savez_compressed(OUT / f"{name}.npz", **out)
    print(f"{name}: max|eps|={np.abs(e).max():.3e} max|sigma|={np.abs(s).max():.3e}")


if __name__ == "__main__":
    want = set(sys.argv[1:])
    for nm, sp in cases():
        if not want or nm in want:
            make(nm, sp)
    for nm, sp, kr in prefix_cases():
        if not want or nm in want:
            make(nm, sp, krun=kr)
    if not want or "oracle_config1_128c_ns12_k1000" in want:
        make_oracle_long()
    for nm, sp in strain_cases():
        if not want or nm in want:
            make_strain(nm, sp)
    for nm, sp in diag_cases():
        if not want or nm in want:
            make_diag(nm, sp)
    for nm, sp in converge_cases():
        if not want or nm in want:
            make_converge(nm, sp)
