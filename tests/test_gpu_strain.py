"""Strain and stress fields on the GPU (pfdd_strain_stress) against the reference's
own full-precision dump of the initial state's fields, the oracle on an evolved
state, and the reference's text formats (strain.txt, stress.txt, stress-strain.dat)
through the C host driver.  FP64 throughout: max |difference| <= 1e-10."""
import subprocess

import numpy as np
import pytest

from conftest import load_golden, strain_golden_cases
from oracle import oracle
from pfdd_gb300 import build, native, refio, workloads

pytestmark = pytest.mark.gpu

TOL = 1e-10


def applied(spec):
    sig = np.zeros((3, 3)); sig[0, 2] = sig[2, 0] = spec.sigma_max
    return sig


@pytest.mark.parametrize("name", strain_golden_cases())
def test_strain_stress_matches_reference(native_lib, name):
    spec, z = load_golden(name)
    x0, b0 = workloads.initial_state(spec)
    res = {}
    for prec in ("fp64", "fp32"):
        s = native.solver_for(spec, prec)
        s.set_state(x0, b0)
        res[prec] = s.strain_stress(applied(spec))
        s.close()
    e, sg, ae, asg = res["fp64"]
    e, sg = e.reshape(9, -1), sg.reshape(9, -1)
    if "eps" in z:
        re, rs = z["eps"], z["sigma"]
    else:
        idx = z["sample_idx"]
        e, sg, re, rs = e[:, idx], sg[:, idx], z["eps_sample"], z["sigma_sample"]
    assert np.max(np.abs(e - re)) <= TOL
    assert np.max(np.abs(sg - rs)) <= TOL
    np.testing.assert_allclose(ae.ravel(), z["aveps_txt"], rtol=1e-6, atol=1e-12)
    np.testing.assert_allclose(asg.ravel() / spec.mu, z["avesigma_over_mu_txt"], rtol=1e-6, atol=1e-12)
    # computed in FP64 from the FP64 state whatever the context's precision
    for a, b in zip(res["fp64"], res["fp32"]):
        np.testing.assert_array_equal(a, b)


def test_strain_stress_of_evolved_state_and_replica(native_lib):
    spec = workloads.SolveSpec(n=(16, 8, 32), ns=12, steps=15, sigma_max=0.06, noise_seed=5,
                               loops=workloads.random_loops((16, 8, 32), 3, 2.0, 5.0, 12, seed=5))
    s = native.solver_for(spec, "fp32", nrep=2)
    x0, b0 = workloads.initial_state(spec)
    s.set_state(np.stack([0.3 * x0, x0]), np.stack([b0, b0]))
    s.step(np.stack([native.spec_tau(spec)] * 2, axis=1))
    xf = s.get_state()[1]
    e, sg, ae, asg = s.strain_stress(applied(spec), r=1)
    e_only, _, ae2, _ = s.strain_stress(applied(spec), r=1, fields=False)
    s.close()
    eps = native.fcc_eps(12)
    C44, C12 = spec.mu, spec.lam
    eo, so, aeo, asgo = oracle.strain_stress(spec.n, xf, eps, 2 * C44 + C12, C12, C44, applied(spec))
    assert np.max(np.abs(e - eo)) <= TOL
    assert np.max(np.abs(sg - so)) <= TOL
    assert np.max(np.abs(ae - aeo)) <= TOL and np.max(np.abs(asg - asgo)) <= TOL
    assert e_only is None and np.array_equal(ae2, ae)
    assert np.allclose(e, np.swapaxes(e, 0, 1))  # the strain is symmetric


def test_strain_needs_elastic_constants(native_lib):
    spec = workloads.SolveSpec(n=(8, 8, 8), ns=3, steps=1, sigma_max=0.0, noise_seed=1)
    s = native.Solver(spec.n, spec.ns)
    s.set_B(np.zeros((3, 3) + spec.n))
    s.set_state(*workloads.initial_state(spec))
    with pytest.raises(native.PFDDError) as ei:
        s.strain_stress(np.zeros((3, 3)))
    assert ei.value.status == native.PFDD_ENOTREADY
    s.close()


def test_host_driver_strain_files(native_lib, tmp_path):
    spec, z = load_golden("strain_fcc12_8x16x16")
    xi, bc = workloads.initial_state(spec)
    refio.write_xi_files(tmp_path, xi, bc, ns_ref=12)
    r = subprocess.run([str(build.RUNNER), *map(str, spec.n), str(spec.ns), str(spec.steps), repr(spec.sigma_max),
                        "--nsfile", "12", "--strain"], cwd=tmp_path, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    st = (tmp_path / "strain.txt").read_text().splitlines()
    ss = (tmp_path / "stress.txt").read_text().splitlines()
    assert len(st) == int(z["strain_txt_lines"]) and len(ss) == int(z["stress_txt_lines"])
    for ours, ref in ((st, z["strain_txt_head"]), (ss, z["stress_txt_head"])):
        assert ours[0] == str(ref[0])
        for a, b in zip(ours[1:], ref[1:]):
            va = np.array(a.split(","), dtype=float); vb = np.array(str(b).split(","), dtype=float)
            assert np.max(np.abs(va - vb)) <= 1.5e-6  # %lf rounding
    row = np.loadtxt(tmp_path / "stress-strain.dat")
    assert row.shape == (36 + 12 + 1,)
    np.testing.assert_allclose(row[0:18:2], z["aveps_txt"], rtol=2e-6, atol=1e-12)
    np.testing.assert_allclose(row[1:18:2], z["avesigma_over_mu_txt"], rtol=2e-6, atol=1e-12)
    g = np.loadtxt(tmp_path / "gamma_full.dat", ndmin=2)
    np.testing.assert_allclose(row[-1], g[-1, 1], rtol=1e-6)
