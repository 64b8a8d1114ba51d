"""CUDA path (through the C ABI) against the CPU FP64 oracle and the reference's golden
vectors.

Tolerances: plain FP64 form max|dxi| <= 1e-10 and gamma relative error <= 1e-9
(the plain-form parity bar); FP32-FFT form gamma relative error <= 1e-5 against the
FP64 oracle."""
import numpy as np
import pytest

from conftest import GOLDEN, golden_cases, golden_steps, load_golden
from oracle import oracle
from pfdd_gb300 import native, workloads

pytestmark = pytest.mark.gpu

XI_TOL = 1e-10
GAMMA_RTOL = 1e-9
FP32_GAMMA_RTOL = 1e-5


def run_gpu(spec, precision="fp64", steps=None, bc=None, xi=None):
    K = spec.steps if steps is None else steps
    s = native.solver_for(spec, precision)
    try:
        x0, b0 = workloads.initial_state(spec)
        s.set_state(x0 if xi is None else xi, b0 if bc is None else bc)
        tau = native.spec_tau(spec)[:K]
        g, ga = s.step(tau)
        return s.get_state()[0], g[:, 0], ga[:, 0], s.launches
    finally:
        s.close()


def rel(a, b):
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), 1e-300)))


@pytest.mark.parametrize("name", golden_cases())
def test_fp64_matches_reference_golden(native_lib, name):
    spec, z = load_golden(name)
    K = golden_steps(spec, z)
    xf, g, ga, launches = run_gpu(spec, steps=K)
    assert launches >= K * 4
    assert rel(g, z["gamma"]) <= GAMMA_RTOL
    assert np.max(np.abs(ga - z["gamma_a"])) <= GAMMA_RTOL * max(1e-3, np.max(np.abs(z["gamma_a"])))
    flat = xf.reshape(spec.ns, -1)
    if "xi_final" in z:
        err = np.max(np.abs(flat - z["xi_final"]))
    else:
        err = np.max(np.abs(flat[:, z["sample_idx"]] - z["xi_final_sample"]))
    assert err <= XI_TOL, err


def test_fp64_matches_oracle_config0_full_field(native_lib):
    spec = workloads.config0()
    xo, go, gao = oracle.solve(spec)
    xf, g, ga, _ = run_gpu(spec)
    assert np.max(np.abs(xf - xo)) <= XI_TOL
    assert rel(g, go) <= GAMMA_RTOL
    assert np.max(np.abs(xo.imag)) > 1e-4  # Im(xi) really evolves (Nyquist planes)


def test_device_B_matches_reference_formula(native_lib):
    for n in [(8, 16, 4), (32, 32, 32), (2, 8, 1)]:
        eps = oracle.fcc_eps(12)
        for C11 in (3.5, 4.2):
            Bo = oracle.bmatrix(n, eps, C11, 1.5, 1.0)
            s = native.Solver(n, 12, "fp64")
            s.build_B(C11, 1.5, 1.0, eps)
            Bg = s.get_B()
            s.close()
            assert np.max(np.abs(Bg - Bo)) <= 1e-13 * max(1.0, np.max(np.abs(Bo)))


@pytest.mark.parametrize("n", [(8, 16, 4), (32, 32, 32), (2, 8, 1), (1, 16, 8), (16, 1, 2), (128, 8, 16)])
def test_fp32_tile_table_B_matches_reference_formula(native_lib, n):
    """The FP32 stored-table form keeps one of each pair of mirrored points
    (B(-k) = B(k)); every point read back equals the formula rounded to FP32."""
    eps = oracle.fcc_eps(12)
    Bo = oracle.bmatrix(n, eps, 3.5, 1.5, 1.0)
    s = native.Solver(n, 12, "fp32")
    s.build_B(3.5, 1.5, 1.0, eps)
    Bg = s.get_B()
    xp = s.plan()["x_pass"]
    s.close()
    assert np.max(np.abs(Bg - Bo)) <= 1.2e-7 * max(1.0, np.max(np.abs(Bo)))
    assert xp["b_mirrored"] == 1 and xp["b_tiles"] <= n[1] * n[2]


def test_fp32_tile_table_with_asymmetric_B(native_lib):
    """A caller's B(k) without the mirror symmetry switches the FP32 table
    form to single tiles: the step still matches the FP64 form given the
    same B(k), and a symmetric B(k) through the host path gives the device
    build's bits."""
    spec = workloads.SolveSpec(n=(16, 8, 16), ns=12, steps=8, sigma_max=0.05,
                               loops=workloads.random_loops((16, 8, 16), 3, 2.0, 5.0, 12, seed=5), noise_seed=5)
    eps = oracle.fcc_eps(12)
    Bo = oracle.bmatrix(spec.n, eps, 3.5, 1.5, 1.0)
    x0, b0 = workloads.initial_state(spec)
    tau = native.spec_tau(spec)

    def run(prec, B=None):
        s = native.Solver(spec.n, 12, prec)
        if B is None:
            s.build_B(3.5, 1.5, 1.0, eps)
        else:
            s.set_B(B)
        s.set_params(0.01, 0.1, 1.0)
        s.set_state(x0, b0)
        g, _ = s.step(tau)
        xp = s.plan()["x_pass"]
        out = (g[:, 0], s.get_state()[0], (xp["b_tiles"], xp["b_mirrored"]), s.get_B())
        s.close()
        return out

    g_dev, x_dev, lay_dev, B_dev = run("fp32")
    assert lay_dev[1] == 1 and lay_dev[0] < 8 * 16
    # the device-built values through the host path: the same table, the same bits
    g_host, x_host, lay_host, _ = run("fp32", B_dev)
    np.testing.assert_array_equal(g_host, g_dev)
    np.testing.assert_array_equal(x_host, x_dev)
    assert lay_host == lay_dev
    Ba = Bo.copy()
    Ba[0, 0, 3, 2, 5] *= 1.01  # one point no longer equals its mirror
    g_a, x_a, lay_a, B_back = run("fp32", Ba)
    g_64, x_64, _, _ = run("fp64", Ba)
    assert lay_a == (8 * 16, 0)  # one tile per line
    assert np.max(np.abs(B_back - Ba)) <= 1.2e-7 * np.max(np.abs(Ba))
    assert np.max(np.abs(x_a - x_64)) <= 1e-6
    assert rel(g_a, g_64) <= 1e-5


def test_set_B_host_path_equals_device_build(native_lib):
    spec = workloads.SolveSpec(n=(16, 8, 16), ns=12, steps=6, sigma_max=0.05,
                               loops=workloads.random_loops((16, 8, 16), 3, 2.0, 5.0, 12, seed=3), noise_seed=3)
    eps = oracle.fcc_eps(12)
    Bo = oracle.bmatrix(spec.n, eps, 3.5, 1.5, 1.0)
    s = native.Solver(spec.n, 12, "fp64")
    s.set_B(Bo)
    s.set_params(0.01, 0.1, 1.0)
    x0, b0 = workloads.initial_state(spec)
    s.set_state(x0, b0)
    g, _ = s.step(native.spec_tau(spec))
    xs = s.get_state()[0]
    s.close()
    xo, go, _ = oracle.solve(spec)
    assert np.max(np.abs(xs - xo)) <= XI_TOL and rel(g[:, 0], go) <= GAMMA_RTOL


def test_pinned_points_and_non_cubic(native_lib):
    spec = workloads.SolveSpec(n=(16, 4, 32), ns=12, steps=12, sigma_max=0.06,
                               loops=workloads.random_loops((16, 4, 32), 4, 2.0, 6.0, 12, seed=9), noise_seed=9)
    x0, bc = workloads.initial_state(spec)
    rng = np.random.default_rng(1)
    bc = (rng.random(bc.shape) < 0.2).astype(np.float64) * rng.choice([1.0, 2.0], size=bc.shape)
    xf, g, _, _ = run_gpu(spec, bc=bc)
    eps = oracle.fcc_eps(12)
    B = oracle.bmatrix(spec.n, eps, 3.5, 1.5, 1.0)
    tau = native.spec_tau(spec)
    xo, go, _ = oracle.run(spec.n, B, x0, bc, [0.01] * 12, [0.1] * 12, [1.0] * 12, 1.0, tau)
    assert np.max(np.abs(xf - xo)) <= XI_TOL and rel(g, go) <= GAMMA_RTOL
    pinned = bc != 0
    np.testing.assert_array_equal(xf[pinned], x0[pinned])


def test_tau_field_mode(native_lib):
    spec = workloads.SolveSpec(n=(8, 16, 16), ns=3, steps=8, sigma_max=0.0,
                               loops=[workloads.Loop(1, (4, 8, 8), 4.0)], noise_seed=2)
    rng = np.random.default_rng(4)
    tf = rng.uniform(-0.1, 0.1, size=(spec.npts, 3))  # [i][j][k][ns]
    mult = np.linspace(0.1, 1.0, spec.steps)[:, None] * np.ones((1, 3))
    s = native.solver_for(spec)
    x0, b0 = workloads.initial_state(spec)
    s.set_state(x0, b0)
    s.set_tau_field(tf)
    g, _ = s.step(mult)
    xs = s.get_state()[0]
    s.close()
    eps = oracle.fcc_eps(3)
    B = oracle.bmatrix(spec.n, eps, 3.5, 1.5, 1.0)
    xo, go, _ = oracle.run(spec.n, B, x0, b0, [0.01] * 3, [0.1] * 3, [1.0] * 3, 1.0, mult, tau_field=tf)
    assert np.max(np.abs(xs - xo)) <= XI_TOL and rel(g[:, 0], go) <= GAMMA_RTOL


def test_step_chunks_and_restart_are_seamless(native_lib):
    spec = workloads.SolveSpec(n=(16, 16, 16), ns=3, steps=20, sigma_max=0.05,
                               loops=[workloads.Loop(0, (8, 8, 8), 5.0)], noise_seed=4)
    xa, ga_, _, _ = run_gpu(spec)
    s = native.solver_for(spec)
    x0, b0 = workloads.initial_state(spec)
    s.set_state(x0, b0)
    tau = native.spec_tau(spec)
    g1, _ = s.step(tau[:7])
    g2, _ = s.step(tau[7:])
    xb = s.get_state()[0]
    s.close()
    np.testing.assert_array_equal(xa, xb)
    np.testing.assert_array_equal(ga_, np.concatenate([g1[:, 0], g2[:, 0]]))


def test_batched_replicas_equal_individual_runs(native_lib):
    base = workloads.SolveSpec(n=(16, 8, 32), ns=12, steps=10, sigma_max=0.05,
                               loops=workloads.random_loops((16, 8, 32), 3, 2.0, 5.0, 12, seed=5))
    specs = []
    for r, sig in enumerate([0.01, 0.05, 0.08]):
        sp = workloads.SolveSpec(**{**base.__dict__, "noise_seed": 50 + r, "sigma_max": sig})
        specs.append(sp)
    for prec in ("fp64", "fp32"):
        s = native.solver_for(specs[0], prec, nrep=3)
        xs = np.stack([workloads.initial_state(sp)[0] for sp in specs])
        bcs = np.stack([workloads.initial_state(sp)[1] for sp in specs])
        s.set_state(xs, bcs)
        tau = np.stack([native.spec_tau(sp) for sp in specs], axis=1)
        g, ga = s.step(tau)
        xb = s.get_state()
        s.close()
        for r, sp in enumerate(specs):
            xr, gr, _, _ = run_gpu(sp, prec)
            np.testing.assert_array_equal(xb[r], xr)
            np.testing.assert_array_equal(g[:, r], gr)


def test_idle_replica_keeps_state(native_lib):
    spec = workloads.SolveSpec(n=(8, 8, 8), ns=3, steps=5, sigma_max=0.05,
                               loops=[workloads.Loop(0, (4, 4, 4), 3.0)], noise_seed=1)
    s = native.solver_for(spec, "fp64", nrep=2)
    x0, b0 = workloads.initial_state(spec)
    s.set_state(np.stack([x0, x0]), np.stack([b0, b0]))
    s.set_active(1, False)
    s.step(np.stack([native.spec_tau(spec)] * 2, axis=1))
    xb = s.get_state()
    s.close()
    np.testing.assert_array_equal(xb[1], x0)
    assert np.max(np.abs(xb[0] - x0)) > 0


def test_fp32_form_error_vs_fp64_oracle(native_lib):
    spec = workloads.config0()
    xo, go, _ = oracle.solve(spec)
    xf, g, _, _ = run_gpu(spec, "fp32")
    assert rel(g, go) <= FP32_GAMMA_RTOL
    assert np.max(np.abs(xf - xo)) <= 1e-5


@pytest.mark.parametrize("precision", ["fp32", "fp32_bfly"])
def test_fp32_forms_with_anisotropic_spacing(native_lib, precision):
    """Grid spacing d = (1, 0.5, 2) (frec divides each axis's frequency by its
    spacing, so B(k) changes) with nu, Asf and CD2 off their defaults: the FP32
    table form (B(k) built in FP64, rounded) and the closed-form one (B(k)
    evaluated in FP32 from the frequencies) against the reference's own FP64
    run of the same solve, at the FP32-form bar."""
    spec, z = load_golden("fcc12_32x8x16_aniso_k30")
    assert spec.d == (1.0, 0.5, 2.0)
    xf, g, _, _ = run_gpu(spec, precision)
    assert rel(g, z["gamma"]) <= FP32_GAMMA_RTOL
    assert np.max(np.abs(xf.reshape(spec.ns, -1) - z["xi_final"])) <= 1e-5


def test_nonfinite_state_is_reported(native_lib):
    spec = workloads.SolveSpec(n=(8, 8, 8), ns=3, steps=3, sigma_max=0.0, noise_seed=0)
    s = native.solver_for(spec)
    x0, b0 = workloads.initial_state(spec)
    x0[0, 1, 2, 3] = np.nan
    s.set_state(x0, b0)
    with pytest.raises(native.PFDDError) as ei:
        s.step(np.zeros((3, 3)))
    assert ei.value.status == native.PFDD_ENONFINITE
    s.close()


def test_missing_inputs_are_reported(native_lib):
    s = native.Solver((8, 8, 8), 3)
    with pytest.raises(native.PFDDError) as ei:
        s.step(np.zeros((1, 3)))
    assert ei.value.status == native.PFDD_ENOTREADY
    s.close()


def test_fp32_bfly_form_error_vs_fp64_oracle(native_lib):
    """FP32 form with B(k) evaluated in the x-pass (no stored table): same error class
    as the stored-table FP32 form against the FP64 oracle, and close to it."""
    spec = workloads.config0()
    xo, go, _ = oracle.solve(spec)
    xb, gb, _, _ = run_gpu(spec, "fp32_bfly")
    xs, gs, _, _ = run_gpu(spec, "fp32")
    assert rel(gb, go) <= FP32_GAMMA_RTOL
    assert np.max(np.abs(xb - xo)) <= 1e-5
    assert rel(gb, gs) <= 1e-6


def test_fp32_bfly_noncubic_and_batched(native_lib):
    base = workloads.SolveSpec(n=(32, 8, 16), ns=12, steps=8, sigma_max=0.05,
                               loops=workloads.random_loops((32, 8, 16), 3, 2.0, 5.0, 12, seed=21))
    specs = [workloads.SolveSpec(**{**base.__dict__, "noise_seed": 60 + r, "sigma_max": 0.02 * (r + 1)})
             for r in range(2)]
    s = native.solver_for(specs[0], "fp32_bfly", nrep=2)
    s.set_state(np.stack([workloads.initial_state(sp)[0] for sp in specs]),
                np.stack([workloads.initial_state(sp)[1] for sp in specs]))
    g, _ = s.step(np.stack([native.spec_tau(sp) for sp in specs], axis=1))
    xb = s.get_state()
    with pytest.raises(native.PFDDError):
        s.get_B()
    s.close()
    for r, sp in enumerate(specs):
        xr, gr, _, _ = run_gpu(sp, "fp32_bfly")
        np.testing.assert_array_equal(xb[r], xr)
        xo, go, _ = oracle.solve(sp)
        assert rel(gr, go) <= FP32_GAMMA_RTOL


@pytest.mark.parametrize("n", [(16, 1, 16), (1, 16, 32), (16, 16, 1), (2, 4, 8), (512, 2, 2), (2, 2, 512)])
def test_degenerate_and_long_axes_match_oracle(native_lib, n):
    """Axes of length 1 (quasi-2D and 1-D grids), tiny grids and 512-long lines, in both forms."""
    spec = workloads.SolveSpec(n=n, ns=3, steps=12, sigma_max=0.04, noise_seed=13, noise_amp=0.05)
    xo, go, _ = oracle.solve(spec)
    x64, g64, _, _ = run_gpu(spec, "fp64")
    assert np.max(np.abs(x64 - xo)) <= XI_TOL
    assert rel(g64, go) <= GAMMA_RTOL
    x32, g32, _, _ = run_gpu(spec, "fp32")
    assert np.max(np.abs(x32 - xo)) <= 1e-5


@pytest.mark.parametrize("n", [(512, 2, 4), (256, 4, 4), (8, 4, 2)])
def test_fp32_table_form_twelve_systems_long_and_short_lines(native_lib, n):
    """The FP32 stored-table form with 12 systems on 512-long x lines (the
    line-pair tile does not fit: a CTA per line), 256-long ones, and lines
    shorter than the warp-team range, against the FP64 oracle."""
    spec = workloads.SolveSpec(n=n, ns=12, steps=8, sigma_max=0.04, noise_seed=14, noise_amp=0.05)
    xo, go, _ = oracle.solve(spec)
    x32, g32, _, _ = run_gpu(spec, "fp32")
    assert np.max(np.abs(x32 - xo)) <= 1e-5
    assert rel(g32, go) <= FP32_GAMMA_RTOL


@pytest.mark.parametrize("ns", [1, 2, 7])
def test_small_and_odd_system_counts_match_oracle(native_lib, ns):
    """Slip-system counts away from 3 and 12 (every count has its own compiled
    x-pass, and the gamma reduction sizes its block by it), all three forms,
    with a pinned point, against the FP64 oracle."""
    n = (32, 8, 16)
    spec = workloads.SolveSpec(n=n, ns=ns, steps=10, sigma_max=0.05, noise_seed=40 + ns,
                               loops=workloads.random_loops(n, 2, 1.5, 3.0, ns, seed=40 + ns))
    x0, b0 = workloads.initial_state(spec)
    bc = b0.copy()
    bc[0, 3, 2, 1] = 1.0  # one pinned point
    eps = oracle.fcc_eps(ns, bdiv=float(np.sqrt(2.0)), dslip=np.full(12, spec.dslip))
    B = oracle.bmatrix(spec.n, eps, 2.0 * spec.mu + spec.lam, spec.lam, spec.mu, spec.d)
    xo, go, gao = oracle.run(spec.n, B, x0, bc, np.full(ns, spec.cd2), np.full(ns, spec.asf),
                             np.full(ns, spec.dslip), 1.0, native.spec_tau(spec))
    x64, g64, ga64, _ = run_gpu(spec, "fp64", bc=bc)
    assert np.max(np.abs(x64 - xo)) <= XI_TOL
    assert rel(g64, go) <= GAMMA_RTOL
    assert np.max(np.abs(ga64 - gao)) <= GAMMA_RTOL * max(1e-3, np.max(np.abs(gao)))
    for form in ("fp32", "fp32_bfly"):
        x32, g32, _, _ = run_gpu(spec, form, bc=bc)
        assert np.max(np.abs(x32 - xo)) <= 1e-5
        assert rel(g32, go) <= FP32_GAMMA_RTOL


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_trailing_idle_replicas_are_skipped(native_lib, prec):
    """A step's grids cover the replicas up to the last active one: with the
    last two of four idle, the active two equal their own runs bit for bit and
    the idle ones keep their state; activating the last one widens the grids
    again (the graphs are recaptured) with the same per-replica results."""
    base = workloads.SolveSpec(n=(16, 16, 32), ns=3, steps=8, sigma_max=0.05,
                               loops=[workloads.Loop(0, (8, 8, 16), 4.0)])
    specs = [workloads.SolveSpec(**{**base.__dict__, "noise_seed": 70 + r}) for r in range(4)]
    xs = np.stack([workloads.initial_state(sp)[0] for sp in specs])
    bcs = np.stack([workloads.initial_state(sp)[1] for sp in specs])
    tau = np.stack([native.spec_tau(sp) for sp in specs], axis=1)
    s = native.solver_for(specs[0], prec, nrep=4)
    try:
        s.set_state(xs, bcs)
        s.set_active(2, False)
        s.set_active(3, False)
        g1, _ = s.step(tau[:4])
        x1 = s.get_state()
        s.set_active(3, True)
        g2, _ = s.step(tau[4:])
        x2 = s.get_state()
    finally:
        s.close()
    np.testing.assert_array_equal(x1[2], xs[2])
    np.testing.assert_array_equal(x1[3], xs[3])
    np.testing.assert_array_equal(x2[2], xs[2])
    for r in (0, 1):
        xr, gr, _, _ = run_gpu(specs[r], prec)
        np.testing.assert_array_equal(x2[r], xr)
        np.testing.assert_array_equal(np.concatenate([g1[:, r], g2[:, r]]), gr)
    # replica 3 ran the last 4 steps of its ramp from its initial state
    s3 = native.solver_for(specs[3], prec)
    try:
        s3.set_state(xs[3], bcs[3])
        g3, _ = s3.step(native.spec_tau(specs[3])[4:])
        np.testing.assert_array_equal(x2[3], s3.get_state()[0])
        np.testing.assert_array_equal(g2[:, 3], g3[:, 0])
    finally:
        s3.close()
