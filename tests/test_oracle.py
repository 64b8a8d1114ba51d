"""The CPU FP64 oracle against the reference program's own FP64 run (golden vectors)."""
import numpy as np
import pytest

from conftest import golden_cases, golden_steps, load_golden, strain_golden_cases
from oracle import oracle
from pfdd_gb300 import workloads


@pytest.mark.parametrize("name", golden_cases())
def test_oracle_matches_patched_reference(name):
    spec, z = load_golden(name)
    xi0, _ = workloads.initial_state(spec)
    # the inputs regenerate bit-identically from the spec
    np.testing.assert_array_equal(z["xi0_checksum"], [xi0.real.sum(), (xi0.real ** 2).sum()])
    xf, g, ga = oracle.solve(spec, steps=golden_steps(spec, z))
    assert g.shape == z["gamma"].shape
    rel = np.max(np.abs(g - z["gamma"]) / np.maximum(np.abs(z["gamma"]), 1e-300))
    assert rel <= 1e-12, rel
    assert np.max(np.abs(ga - z["gamma_a"])) <= 1e-13
    flat = xf.reshape(spec.ns, -1)
    ref = z["xi_final"] if "xi_final" in z else z["xi_final_sample"]
    got = flat if "xi_final" in z else flat[:, z["sample_idx"]]
    assert np.max(np.abs(got - ref)) <= 1e-12
    # full-field checksums cover the unsampled points
    cs = np.array([xf.real.sum(), xf.imag.sum(), (np.abs(xf) ** 2).sum()])
    np.testing.assert_allclose(cs[[0, 2]], z["xi_final_checksum"][[0, 2]], rtol=1e-12)
    assert abs(cs[1] - z["xi_final_checksum"][1]) <= 1e-10


def test_oracle_fft_matches_numpy():
    rng = np.random.default_rng(0)
    for n in [(8, 4, 16), (2, 2, 2), (1, 8, 4), (16, 16, 16)]:
        x = rng.standard_normal((2,) + n) + 1j * rng.standard_normal((2,) + n)
        f = oracle.fft3d(x, -1)
        np.testing.assert_allclose(f, np.fft.fftn(x, axes=(1, 2, 3)), atol=1e-12)
        b = oracle.fft3d(x, +1)
        np.testing.assert_allclose(b, np.fft.ifftn(x, axes=(1, 2, 3)) * np.prod(n), atol=1e-12)


def test_frec_nyquist_convention():
    # F:2711-2736: Nyquist index maps to -1/2, no 2*pi
    np.testing.assert_array_equal(oracle.frec(8), [0, 0.125, 0.25, 0.375, -0.5, -0.375, -0.25, -0.125])
    np.testing.assert_array_equal(oracle.frec(2), [0.0, -0.5])


def test_bmatrix_properties():
    n = (8, 4, 16)
    eps = oracle.fcc_eps(12)
    B = oracle.bmatrix(n, eps, 3.5, 1.5, 1.0)
    assert np.all(B[:, :, 0, 0, 0] == 0.0)            # B(0) = 0
    np.testing.assert_allclose(B, B.transpose(1, 0, 2, 3, 4), atol=1e-15)  # symmetric in (a, b)
    # degree-0 homogeneity: B depends on the direction of f only
    Bs = oracle.bmatrix(n, eps, 3.5, 1.5, 1.0, d=(2.0, 2.0, 2.0))
    np.testing.assert_allclose(Bs, B, atol=1e-13)


def test_bmatrix_closed_form_matches_loop():
    """The closed form used on the device, B = (E - t^T G t)/mu, restated in numpy,
    agrees with the reference's 81x27x3 loop (oracle_bmatrix)."""
    n = (4, 8, 8)
    eps = oracle.fcc_eps(12)
    mu, lam = 1.0, 1.5
    for C11 in (2 * mu + lam, 4.2):  # isotropic and cubic (mu' != 0)
        C12, C44 = lam, mu
        B = oracle.bmatrix(n, eps, C11, C12, C44)
        mup = C11 - C12 - 2 * C44
        d = np.eye(3)
        Cc = (mu * (np.einsum("ik,jm->ijkm", d, d) + np.einsum("im,jk->ijkm", d, d))
              + lam * np.einsum("ij,km->ijkm", d, d))
        for i in range(3):
            Cc[i, i, i, i] += mup
        sig = np.einsum("ijmn,amn->aij", Cc, eps)
        E = np.einsum("aij,bij->ab", eps, sig)
        f = np.stack(np.meshgrid(oracle.frec(n[0]), oracle.frec(n[1]), oracle.frec(n[2]), indexing="ij"), -1)
        for idx in [(1, 2, 3), (2, 4, 4), (3, 7, 1), (0, 0, 5)]:
            fk = f[idx]
            f2 = fk @ fk
            z = fk * fk / f2
            den = mu + mup * z
            kk = 1 + (mu + lam) * np.sum(z / den)
            G = (np.diag(1 / den) - np.outer(fk, fk) / f2 / np.outer(den, den) * (mu + lam) / kk) / f2
            t = sig @ fk
            Bc = (E - t @ G @ t.T) / mu
            np.testing.assert_allclose(B[(slice(None), slice(None)) + idx], Bc.T, atol=1e-13)


def test_update_uses_truncated_pi():
    """plasticevolv's sin(2*pi*xi) uses pi = 3.141592654 (F:95): one step on a
    uniform state with zero force shows it."""
    n = (2, 2, 2)
    B = np.zeros((1, 1) + n)
    xi = np.full((1,) + n, 0.3 + 0j)
    bc = np.zeros((1,) + n)
    xf, g, _ = oracle.run(n, B, xi, bc, [0.01], [0.1], [1.0], 1.0, np.zeros((1, 1)))
    pt = 3.141592654
    expect = 0.3 - 0.01 * (0.1 * pt * np.sin(2.0 * pt * 0.3))
    assert xf.real.flat[0] == expect
    assert g[0] == expect


def test_pinned_points_do_not_move():
    spec = workloads.SolveSpec(n=(8, 8, 8), ns=3, steps=5, sigma_max=0.05,
                               loops=[workloads.Loop(0, (4, 4, 4), 3.0)], noise_seed=5)
    eps = oracle.fcc_eps(3)
    B = oracle.bmatrix(spec.n, eps, 3.5, 1.5, 1.0)
    xi, bc = workloads.initial_state(spec)
    bc[1, :4] = 1.0
    sig = np.zeros((3, 3)); sig[0, 2] = sig[2, 0] = 0.05
    tau = oracle.ramp_tau(oracle.resolved_shear(eps, sig), 5)
    xf, _, _ = oracle.run(spec.n, B, xi, bc, [0.01] * 3, [0.1] * 3, [1.0] * 3, 1.0, tau)
    np.testing.assert_array_equal(xf[1, :4], xi[1, :4])
    assert np.max(np.abs(xf[1, 4:] - xi[1, 4:])) > 0


def strain_inputs(spec):
    """Initial state, eigenstrains, constants and applied stress of a strain golden case."""
    xi, _ = workloads.initial_state(spec)
    eps = oracle.fcc_eps(12, dslip=np.full(12, spec.dslip))[:spec.ns]
    sig = np.zeros((3, 3)); sig[0, 2] = sig[2, 0] = spec.sigma_max
    return xi, eps, spec.C11, spec.lam, spec.mu, sig


@pytest.mark.parametrize("name", strain_golden_cases())
def test_oracle_strain_stress_matches_reference(name):
    """Strain and stress fields (strain F:752-835, stress F:837-972) of the initial
    state: the restatement against the reference's own full-precision dump, and its
    averages against the reference's stress-strain.dat (printed with %e)."""
    spec, z = load_golden(name)
    xi, eps, C11, C12, C44, sig = strain_inputs(spec)
    e, s, ae, asg = oracle.strain_stress(spec.n, xi, eps, C11, C12, C44, sig, spec.d)
    e, s = e.reshape(9, -1), s.reshape(9, -1)
    if "eps" in z:
        re, rs = z["eps"], z["sigma"]
    else:
        idx = z["sample_idx"]
        e, s, re, rs = e[:, idx], s[:, idx], z["eps_sample"], z["sigma_sample"]
    assert np.max(np.abs(e - re)) <= 1e-12
    assert np.max(np.abs(s - rs)) <= 1e-12
    np.testing.assert_allclose(ae.ravel(), z["aveps_txt"], rtol=1e-6, atol=1e-12)
    np.testing.assert_allclose(asg.ravel() / C44, z["avesigma_over_mu_txt"], rtol=1e-6, atol=1e-12)
    # the applied stress is the average stress
    np.testing.assert_allclose(asg, sig * C44, atol=1e-12)
