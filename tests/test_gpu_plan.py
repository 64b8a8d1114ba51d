"""Launch plan and autotuning: the plan is reported, every tile width tried by the
autotuner is one that fits, and the tuned context gives the same bits as the
default plan (tile widths do not change any result)."""
import os

import numpy as np
import pytest

from oracle import oracle
from pfdd_gb300 import native, workloads

pytestmark = pytest.mark.gpu


def run(spec, precision, tune):
    old = os.environ.get("PFDD_NO_TUNE")
    os.environ["PFDD_NO_TUNE"] = "0" if tune else "1"
    try:
        s = native.solver_for(spec, precision)
    finally:
        if old is None:
            del os.environ["PFDD_NO_TUNE"]
        else:
            os.environ["PFDD_NO_TUNE"] = old
    x0, b0 = workloads.initial_state(spec)
    s.set_state(x0, b0)
    g, ga = s.step(native.spec_tau(spec))
    out = (g, s.get_state(), s.plan())
    s.close()
    return out


@pytest.mark.parametrize("precision", ["fp64", "fp32", "fp32_bfly"])
def test_tuned_plan_gives_same_bits(native_lib, precision):
    spec = workloads.SolveSpec(n=(32, 16, 64), ns=12, steps=12, sigma_max=0.05, noise_seed=21,
                               loops=workloads.random_loops((32, 16, 64), 4, 2.0, 6.0, 12, seed=21))
    g1, x1, p1 = run(spec, precision, True)
    g0, x0, p0 = run(spec, precision, False)
    if p1["radix_plan"] == p0["radix_plan"]:
        np.testing.assert_array_equal(g1, g0)
        np.testing.assert_array_equal(x1, x0)
    else:  # the tuner chose another radix plan: other rounding, same result within the form's tolerance
        tol = 1e-10 if precision == "fp64" else 1e-5
        assert np.max(np.abs(x1 - x0)) <= tol
        assert np.max(np.abs(g1 - g0) / np.abs(g0)) <= (1e-9 if precision == "fp64" else 1e-5)
    assert p0["autotune"] is None
    tune = p1["autotune"]
    if tune.get("cached"):  # an earlier context of this shape was tuned in this process
        tune = tune["timings"]
    tried = tune["x_pass_us_by_tile"]
    assert len(tried) >= 1 and all(v > 0 for v in tried.values())
    assert str(p1["x_pass"]["tile_columns"]) in tried
    assert p0["radix_plan"] == ["8x4", "16", "8x8"]  # 16 values a thread for the 16-long y lines
    assert p1["radix_plan"][1] in ("16", "8x2") and p1["radix_plan"][2] in ("8x8", "16x4")
    assert any("/16" in k for k in tune["z_pass_us_by_lines"]) and any("/8" in k for k in tune["z_pass_us_by_lines"])


def test_pinned_plan(native_lib):
    spec = workloads.SolveSpec(n=(32, 16, 64), ns=12, steps=6, sigma_max=0.05, noise_seed=22,
                               loops=workloads.random_loops((32, 16, 64), 3, 2.0, 6.0, 12, seed=22))
    os.environ["PFDD_PLAN"] = "z=8,x=2,y=8"
    try:
        g1, x1, p1 = run(spec, "fp32", True)
    finally:
        del os.environ["PFDD_PLAN"]
    g0, x0, _ = run(spec, "fp32", False)
    assert p1["autotune"] == "pinned"
    assert (p1["z_pass"]["lines"], p1["x_pass"]["tile_columns"], p1["y_pass"]["tile_columns"]) == (8, 2, 8)
    np.testing.assert_array_equal(g1, g0)
    np.testing.assert_array_equal(x1, x0)


def test_plan_is_tuned_once_per_shape(native_lib):
    spec = workloads.SolveSpec(n=(16, 32, 16), ns=3, steps=3, sigma_max=0.02, noise_seed=23)
    g1, x1, p1 = run(spec, "fp32", True)
    g2, x2, p2 = run(spec, "fp32", True)
    assert p2["autotune"]["cached"] is True
    assert (p2["z_pass"], p2["x_pass"], p2["y_pass"]) == (p1["z_pass"], p1["x_pass"], p1["y_pass"])
    np.testing.assert_array_equal(g1, g2)
    np.testing.assert_array_equal(x1, x2)


def pinned(spec, precision, plan, nrep=1, prepare=None):
    old = os.environ.get("PFDD_PLAN")
    if plan is None:
        os.environ.pop("PFDD_PLAN", None)
        os.environ["PFDD_NO_TUNE"] = "1"
    else:
        os.environ["PFDD_PLAN"] = plan
    try:
        s = native.solver_for(spec, precision, nrep=nrep)
    finally:
        os.environ.pop("PFDD_NO_TUNE", None)
        if old is None:
            os.environ.pop("PFDD_PLAN", None)
        else:
            os.environ["PFDD_PLAN"] = old
    x0, b0 = workloads.initial_state(spec)
    tau = native.spec_tau(spec)
    if nrep > 1:
        s.set_state(np.stack([x0 * (1.0 - 0.3 * i) for i in range(nrep)]), np.stack([b0] * nrep))
        tau = np.stack([tau] * nrep, axis=1)
    else:
        s.set_state(x0, b0)
    if prepare:
        prepare(s, b0)
    g, ga = s.step(tau)
    out = (g, s.get_state(), s.plan())
    s.close()
    return out


@pytest.mark.parametrize("precision", ["fp32_bfly"])
def test_warp_team_xpass_batched_pinned_and_idle(native_lib, precision):
    """The warp-team x-pass on a batch: an idle replica whose tiles are
    skipped, pinned points, N1 = 128."""
    spec = workloads.SolveSpec(n=(128, 8, 16), ns=3, steps=12, sigma_max=0.05, noise_seed=32,
                               loops=workloads.random_loops((128, 8, 16), 3, 2.0, 5.0, 3, seed=32))

    def prep(s, b0):
        bc = np.zeros((3,) + b0.shape); bc[:, :, 0, 0, :] = 1.0
        s.set_state(s.get_state(), bc)
        s.set_active(1, False)

    res = [pinned(spec, precision, plan, nrep=3, prepare=prep) for plan in ("x=2,w=1", None)]
    live = [0, 2]
    np.testing.assert_array_equal(res[0][0][:, live], res[1][0][:, live])
    np.testing.assert_array_equal(res[0][1], res[1][1])
    assert res[0][2]["x_pass"]["warp_teams"] == 1


@pytest.mark.parametrize("precision", ["fp32_bfly"])
@pytest.mark.parametrize("n1,plan", [(32, "x=1,w=1"), (64, "x=2,w=1"), (128, "x=1,w=1"), (128, "x=4,w=1"),
                                     (256, "x=1,w=1")])
def test_warp_team_xpass_gives_same_bits(native_lib, precision, n1, plan):
    """The warp-team x-pass (lines straight between global memory and
    registers, warp-local FFT stages, swizzled shared-memory lines) computes
    the block-team x-pass's bits (B(k) in registers; the stored-table form
    runs the block-team kernel on its tile table)."""
    n = (n1, 8, 16)
    spec = workloads.SolveSpec(n=n, ns=12, steps=6, sigma_max=0.05, noise_seed=33,
                               loops=workloads.random_loops(n, 3, 1.5, 3.0, 12, seed=33))
    g1, x1, p1 = pinned(spec, precision, plan)
    g0, x0, p0 = pinned(spec, precision, None)
    assert p1["x_pass"]["warp_teams"] == 1 and p0["x_pass"]["warp_teams"] == 0
    assert p1["x_pass"]["tile_columns"] == int(plan.split(",")[0][2:])
    np.testing.assert_array_equal(g1, g0)
    np.testing.assert_array_equal(x1, x0)


@pytest.mark.parametrize("n", [(128, 8, 16), (32, 16, 8), (16, 2, 4), (64, 4, 2)])
@pytest.mark.parametrize("plan", ["x=1", "x=1,w=1", "x=2,w=1"])
def test_table_form_line_and_pair_ctas_same_bits(native_lib, n, plan):
    """The FP32 stored-table form's x-pass shapes on the mirrored B(k) tile
    table -- a CTA per line or per mirrored pair, block or warp teams -- give
    the same bits."""
    spec = workloads.SolveSpec(n=n, ns=12, steps=6, sigma_max=0.05, noise_seed=34,
                               loops=workloads.random_loops(n, 2, 1.0, 2.0, 12, seed=34))
    g1, x1, p1 = pinned(spec, "fp32", plan)
    g2, x2, p2 = pinned(spec, "fp32", "x=2")
    warp = "w=1" in plan and n[0] >= 32
    assert p1["x_pass"]["tile_columns"] == int(plan.split(",")[0][2:]) and p2["x_pass"]["tile_columns"] == 2
    assert p1["x_pass"]["warp_teams"] == int(warp) and p2["x_pass"]["warp_teams"] == 0
    assert p1["x_pass"]["b_mirrored"] == p2["x_pass"]["b_mirrored"] == 1
    np.testing.assert_array_equal(g1, g2)
    np.testing.assert_array_equal(x1, x2)


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_y_field_order_same_bits(native_lib, precision):
    """The step's y passes take the fields from the last down (so each starts
    on what the pass before it wrote last); the ascending order (f=0) gives the
    same bits, one solve and a batch."""
    spec = workloads.SolveSpec(n=(32, 16, 8), ns=5, steps=6, sigma_max=0.05, noise_seed=36,
                               loops=workloads.random_loops((32, 16, 8), 2, 1.0, 3.0, 5, seed=36))
    for nrep in (1, 3):
        g1, x1, _ = pinned(spec, precision, "f=1", nrep=nrep)
        g0, x0, _ = pinned(spec, precision, "f=0", nrep=nrep)
        np.testing.assert_array_equal(g1, g0)
        np.testing.assert_array_equal(x1, x0)


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_every_radix_plan_matches_oracle(native_lib, precision):
    """The z-pass and y-pass radix plans the autotuner chooses from (8 or 16
    values a thread: 128-long y lines as 8x8x2 or 16x8, 256-long z lines as
    8x8x4 or 16x16), each pinned, against the FP64 oracle within the form's
    tolerance (the plans round differently, so they are not bitwise equal)."""
    spec = workloads.SolveSpec(n=(16, 128, 256), ns=3, steps=6, sigma_max=0.05, noise_seed=38,
                               loops=workloads.random_loops((16, 128, 256), 3, 3.0, 8.0, 3, seed=38))
    xo, go, _ = oracle.solve(spec)
    tol, gtol = (1e-10, 1e-9) if precision == "fp64" else (1e-5, 1e-5)
    want = {8: ("8x8x2", "8x8x4"), 16: ("16x8", "16x16")}
    seen = set()
    for zn in (8, 16):
        for yn in (8, 16):
            g, x, p = pinned(spec, precision, f"n={zn},m={yn}")
            assert p["radix_plan"][1] == want[yn][0] and p["radix_plan"][2] == want[zn][1]
            assert np.max(np.abs(x - xo)) <= tol, (zn, yn)
            assert np.max(np.abs(g[:, 0] - go) / np.abs(go)) <= gtol, (zn, yn)
            seen.add(x.tobytes())
    assert len(seen) >= 2  # the plans really differ in rounding


@pytest.mark.parametrize("n,ns,plan", [((32, 16, 8), 12, "x=2,w=2"), ((64, 8, 16), 12, "x=1,w=2"),
                                       ((128, 8, 16), 12, "x=2,w=2"), ((256, 8, 16), 12, "x=1,w=2"),
                                       ((128, 16, 8), 3, "x=1,w=2"), ((256, 4, 8), 5, "x=1,w=2")])
def test_split_b_block_same_bits(native_lib, n, ns, plan):
    """The warp-team x-pass on the mirrored B(k) tile table with the tile's B
    block in two halves of its pair rows through one buffer (the second half
    loaded once every thread is past the first) gives the bits of the
    whole-block kernel: mirrored pairs, Nyquist single lines, a CTA per pair
    and per line, odd pair counts (5 systems: 15 pairs), 3 and 12 systems."""
    spec = workloads.SolveSpec(n=n, ns=ns, steps=6, sigma_max=0.05, noise_seed=35,
                               loops=workloads.random_loops(n, 3, 1.0, 3.0, ns, seed=35))
    whole = plan.replace("w=2", "w=1")
    g1, x1, p1 = pinned(spec, "fp32", plan)
    g0, x0, p0 = pinned(spec, "fp32", whole)
    assert p1["x_pass"]["b_split"] == 1 and p0["x_pass"]["b_split"] == 0
    assert p1["x_pass"]["warp_teams"] == p0["x_pass"]["warp_teams"] == 1
    assert p1["x_pass"]["smem"] < p0["x_pass"]["smem"]
    np.testing.assert_array_equal(g1, g0)
    np.testing.assert_array_equal(x1, x0)


def test_split_b_block_batched_pinned_and_idle(native_lib):
    """The split B block on a batch of three with an idle replica (its CTAs
    leave before the buffer swap) and pinned points: the bits of the
    whole-block kernel."""
    n = (256, 4, 8)
    spec = workloads.SolveSpec(n=n, ns=12, steps=6, sigma_max=0.05, noise_seed=37,
                               loops=workloads.random_loops(n, 3, 1.0, 3.0, 12, seed=37))

    def prep(s, b0):
        bc = np.zeros((3,) + b0.shape); bc[:, :, 0, 0, :] = 1.0
        s.set_state(s.get_state(), bc)
        s.set_active(1, False)

    res = [pinned(spec, "fp32", plan, nrep=3, prepare=prep) for plan in ("x=1,w=2", "x=1,w=1")]
    assert res[0][2]["x_pass"]["b_split"] == 1 and res[1][2]["x_pass"]["b_split"] == 0
    live = [0, 2]
    np.testing.assert_array_equal(res[0][0][:, live], res[1][0][:, live])
    np.testing.assert_array_equal(res[0][1], res[1][1])
