"""Interface-plane energy diagnostics through the C ABI (pfdd_set_diagnostics,
pfdd_get_diagnostics, pfdd_state_diagnostics) against the reference's own FP64
runs (full-precision checkEnergy.dat / checkEbarrier.dat energies, patch 13 of
oracle/build_ref.py): the initial state's line, every inner step's energy_in3
and energy_in4, the final state's line; in both forms and in a batch."""
import numpy as np
import pytest

from conftest import check_residual, diag_golden_cases, load_golden
from oracle import diag, oracle
from pfdd_gb300 import native, workloads

pytestmark = pytest.mark.gpu


def run(spec, z, precision, nrep=1):
    C44, C12 = spec.mu, spec.lam
    p = native.reference_diag_params(spec.n, spec.sigma_max, spec.C11, C12, C44, D=z["D"])
    s = native.solver_for(spec, precision, nrep=nrep)
    try:
        x0, b0 = workloads.initial_state(spec)
        tau = native.spec_tau(spec)
        if nrep > 1:
            x0, b0, tau = np.stack([x0] * nrep), np.stack([b0] * nrep), np.stack([tau] * nrep, axis=1)
        s.set_state(x0, b0)
        s.set_diagnostics(p)
        e0 = s.state_diagnostics()
        s.step(tau)
        e = s.diagnostics(spec.steps)
        ef = s.state_diagnostics()
        return e0, e, ef, s.launches
    finally:
        s.close()


@pytest.mark.parametrize("name", diag_golden_cases())
def test_diagnostics_match_reference(native_lib, name):
    spec, z = load_golden(name)
    outer, inner = z["energy_outer"], z["energy_inner"]
    scale3 = np.max(np.abs(inner[:, 3]))
    e0, e, ef, launches = run(spec, z, "fp64")
    assert launches == 5 * spec.steps + 1 or launches >= 5 * spec.steps  # the gather runs every step
    np.testing.assert_allclose(e0[0, 2:4], outer[0, 3:5], rtol=1e-13)
    assert e0[0, 0] == 0.0 and e0[0, 1] == 0.0
    check_residual(outer[0, 5:7], e0[0, 4:6])
    assert np.max(np.abs(e[:, 0, 2] - inner[:, 3])) <= 1e-12 * scale3
    np.testing.assert_allclose((np.arange(spec.steps) + 2) * e[:, 0, 3], inner[:, 4], rtol=1e-12)
    check_residual(inner[:, 5], e[:, 0, 4])
    assert abs(ef[0, 2] - outer[-1, 3]) <= 1e-12 * scale3
    # the FP32-FFT form: within its tolerance; a batch of identical replicas: the same bits
    _, e32, _, _ = run(spec, z, "fp32")
    assert np.max(np.abs(e32[:, 0, 2] - inner[:, 3])) <= 1e-5 * scale3
    _, eb, _, _ = run(spec, z, "fp64", nrep=2)
    np.testing.assert_array_equal(eb[:, 0, 2:4], e[:, 0, 2:4])
    np.testing.assert_array_equal(eb[:, 1, 2:4], e[:, 0, 2:4])


def test_diagnostics_with_finite_coefficients_match_restatement(native_lib):
    """energy_Residual with finite D coefficients and two materials' worth of
    systems, against the numpy restatement on the oracle's final state."""
    spec = workloads.SolveSpec(n=(16, 8, 32), ns=4, steps=6, sigma_max=0.05, noise_seed=43,
                               loops=workloads.random_loops((16, 8, 32), 3, 2.0, 5.0, 4, seed=43))
    C44, C12 = spec.mu, spec.lam
    p = native.reference_diag_params(spec.n, spec.sigma_max, 2.0 * C44 + C12, C12, C44, D=(0.5, -0.25, 0.75, 2.0),
                                     ns_per_material=2)
    s = native.solver_for(spec, "fp64")
    try:
        x0, b0 = workloads.initial_state(spec)
        s.set_state(x0, b0)
        s.set_diagnostics(p)
        s.step(native.spec_tau(spec))
        e = s.diagnostics(spec.steps)
    finally:
        s.close()
    xo, _, _ = oracle.solve(spec)
    want = diag.energies(xo.real, oracle.fcc_eps(spec.ns), p)
    np.testing.assert_allclose(e[-1, 0, 2:], want[2:], rtol=1e-10)
    assert want[4] > 0
