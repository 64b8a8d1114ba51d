"""The C host driver (reads xi.dat/xi_bc.dat, writes phasefield.dat / xi.dat like the
reference program) reproduces the reference's FP64 run of config 0."""
import subprocess

import numpy as np
import pytest

from conftest import load_golden
from pfdd_gb300 import build, refio, workloads

pytestmark = pytest.mark.gpu


def test_host_driver_reproduces_reference_run(native_lib, tmp_path):
    spec, z = load_golden("config0_32c_ns3_k200")
    xi, bc = workloads.initial_state(spec)
    refio.write_xi_files(tmp_path, xi, bc, ns_ref=12)
    r = subprocess.run([str(build.RUNNER), *map(str, spec.n), str(spec.ns), str(spec.steps), repr(spec.sigma_max),
                        "--nsfile", "12"], cwd=tmp_path, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    g = np.loadtxt(tmp_path / "gamma_full.dat", ndmin=2)
    assert g.shape[0] == spec.steps
    np.testing.assert_allclose(g[:, 1], z["gamma"], rtol=1e-9)
    lines = (tmp_path / "phasefield.dat").read_text().splitlines()
    assert len(lines) == spec.steps and lines[0].split()[:2] == ["1", "1"]
    xf = refio.read_xi_file(tmp_path / "xi.dat", spec.n, 21)
    flat = xf[:3].reshape(3, -1)
    assert np.max(np.abs(flat[:, z["sample_idx"]] - z["xi_final_sample"])) <= 1e-10
    assert np.all(xf[3:] == 0)


def test_host_driver_fp32_form(native_lib, tmp_path):
    spec, z = load_golden("config0_32c_ns3_k200")
    xi, bc = workloads.initial_state(spec)
    refio.write_xi_files(tmp_path, xi, bc, ns_ref=12)
    r = subprocess.run([str(build.RUNNER), *map(str, spec.n), str(spec.ns), str(spec.steps), repr(spec.sigma_max),
                        "--nsfile", "12", "--fp32"], cwd=tmp_path, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    g = np.loadtxt(tmp_path / "gamma_full.dat", ndmin=2)
    np.testing.assert_allclose(g[:, 1], z["gamma"], rtol=1e-5)


def test_host_driver_converge_stops_where_the_reference_stopped(native_lib, tmp_path):
    """--converge: the reference's inner-loop stop (plasticconverge,
    F:3732-3785); the reference's own run stopped after 112 of 300 steps."""
    spec, z = load_golden("converge_16c_ns3_cd01")
    xi, bc = workloads.initial_state(spec)
    refio.write_xi_files(tmp_path, xi, bc, ns_ref=12)
    r = subprocess.run([str(build.RUNNER), *map(str, spec.n), str(spec.ns), str(spec.steps), repr(spec.sigma_max),
                        "--nsfile", "12", "--cd2", repr(spec.cd2), "--converge"], cwd=tmp_path,
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    k = int(z["steps_run"])
    g = np.loadtxt(tmp_path / "gamma_full.dat", ndmin=2)
    assert g.shape[0] == k
    assert np.max(np.abs(g[:, 1] - z["gamma"])) <= 1e-9 * np.max(np.abs(z["gamma"]))  # gamma decays to 1e-16
    assert len((tmp_path / "phasefield.dat").read_text().splitlines()) == k
    xf = refio.read_xi_file(tmp_path / "xi.dat", spec.n, 21)
    assert np.max(np.abs(xf[:3].reshape(3, -1) - z["xi_final"])) <= 1e-10 * np.max(np.abs(z["xi_final"]))


def _spec_flags(spec):
    """pfdd_run options that carry a workload spec's constants."""
    f = ["--asf", repr(spec.asf), "--cd2", repr(spec.cd2), "--mu", repr(spec.mu), "--lambda", repr(spec.lam),
         "--dslip", repr(spec.dslip), "--uq2", repr(spec.uq2), "--d", *map(repr, spec.d)]
    return f + (["--c11", repr(spec.c11)] if spec.c11 is not None else [])


@pytest.mark.parametrize("name", ["fcc12_32x8x16_aniso_k30", "fcc12_16c_pinned_k30", "fcc12_16x32x8_dslip2_k30",
                                  "fcc12_32x16x8_uq2_k30", "fcc12_16x16x32_cubic_k30"])
def test_host_driver_with_reference_constants(native_lib, tmp_path, name):
    """The driver's options for the reference's constants (grid spacing,
    slip-plane spacing, uq2, a cubic C11, nu, Asf, CD2) and a pinned xi_bc:
    the reference's own FP64 run of each parameter golden."""
    spec, z = load_golden(name)
    xi, bc = workloads.initial_state(spec)
    refio.write_xi_files(tmp_path, xi, bc, ns_ref=12)
    r = subprocess.run([str(build.RUNNER), *map(str, spec.n), str(spec.ns), str(spec.steps), repr(spec.sigma_max),
                        "--nsfile", "12", *_spec_flags(spec)], cwd=tmp_path, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    g = np.loadtxt(tmp_path / "gamma_full.dat", ndmin=2)
    np.testing.assert_allclose(g[:, 1], z["gamma"], rtol=1e-9)
    xf = refio.read_xi_file(tmp_path / "xi.dat", spec.n, 21)
    assert np.max(np.abs(xf[:spec.ns].reshape(spec.ns, -1) - z["xi_final"])) <= 1e-10
