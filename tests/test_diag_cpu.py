"""The interface-plane energies (checkEnergy.dat / checkEbarrier.dat) restated in
numpy (oracle/diag.py) against the reference's own FP64 runs: every inner step's
energy_in3 and energy_in4 and the outer lines, from the oracle's states."""
import numpy as np
import pytest

from conftest import check_residual, diag_golden_cases, load_golden
from oracle import diag, oracle
from pfdd_gb300 import native, workloads


@pytest.mark.parametrize("name", diag_golden_cases())
def test_restated_energies_match_reference(name):
    spec, z = load_golden(name)
    outer, inner, D = z["energy_outer"], z["energy_inner"], z["D"]
    C44, C12 = spec.mu, spec.lam
    p = native.reference_diag_params(spec.n, spec.sigma_max, spec.C11, C12, C44, D=D)
    eps = oracle.fcc_eps(spec.ns, dslip=np.full(12, spec.dslip))
    xi, bc = workloads.initial_state(spec)
    B = oracle.bmatrix(spec.n, eps, spec.C11, C12, C44, spec.d)
    tau = oracle.ramp_tau(oracle.resolved_shear(eps, np.array([[0, 0, spec.sigma_max], [0, 0, 0],
                                                               [spec.sigma_max, 0, 0]])), spec.steps)
    ns = spec.ns
    e0 = diag.energies(xi.real, eps, p)
    # energy_in3 sums plane terms that cancel: its error is held to the run's scale
    scale3 = np.max(np.abs(inner[:, 3]))
    # outer line of the initial state (before the inner loop): one call's energy_in4
    np.testing.assert_allclose(outer[0, 3:5], e0[2:4], rtol=1e-13)
    assert outer[0, 1] == 0.0 and outer[0, 2] == 0.0
    # energy_Residual and the total from the reference's D coefficients
    check_residual(outer[0, 5:7], e0[4:6])
    for s in range(spec.steps):
        xi, _, _ = oracle.run(spec.n, B, xi, bc, np.full(ns, spec.cd2), np.full(ns, spec.asf),
                              np.full(ns, spec.dslip), spec.uq2, tau[s:s + 1])
        e = diag.energies(xi.real, eps, p)
        assert abs(inner[s, 3] - e[2]) <= 1e-12 * scale3, s
        # the reference adds one call's energy_in4 per call, from the outer
        # step's call on: s + 2 calls by inner step s
        np.testing.assert_allclose(inner[s, 4], (s + 2) * e[3], rtol=1e-12)
        assert inner[s, 1] == 0.0 and inner[s, 2] == 0.0
        check_residual(inner[s, 5], e[4])
    # the outer line after the inner loop: the final state's energy_in3
    np.testing.assert_allclose(outer[-1, 3], diag.energies(xi.real, eps, p)[2], rtol=1e-12)


def test_residual_energy_with_finite_coefficients():
    """ResidualEnergy's line sum with finite D coefficients and two materials'
    worth of systems (ism = is / NS1): a hand-computed case."""
    n = (4, 3, 4)
    rng = np.random.default_rng(3)
    re_xi = rng.uniform(-1, 1, size=(4,) + n)
    p = native.reference_diag_params(n, 0.0, 3.5, 1.5, 1.0, D=(0.5, -0.25, 0.75, 2.0), ns_per_material=2)
    eps = oracle.fcc_eps(4)
    e = diag.energies(re_xi, eps, p)
    pp = list(p.ppoint)
    want = 0.0
    for j in range(n[1]):
        x0 = re_xi[0, pp[0], j, pp[2]] + re_xi[1, pp[0], j, pp[2]]
        x1 = re_xi[2, pp[0], j, pp[2]] + re_xi[3, pp[0], j, pp[2]]
        want += abs(-2.0 * x1 * x1 + (0.75 - 0.25) * x1 * x0 - 0.5 * x0 * x0)
    assert abs(e[4] - want) <= 1e-14 * want
    assert e[2] == 0.0 and e[3] == 0.0  # sigma = 0
