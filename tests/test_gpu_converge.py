"""pfdd_step_converge: the inner loop with the reference's convergence stop
(plasticconverge, F:3732-3785), against the reference's own run of a solve
that stops after 112 of its 300 allowed steps (converge_16c_ns3_cd01)."""
import numpy as np
import pytest

from conftest import load_golden
from oracle import oracle
from pfdd_gb300 import native, workloads

pytestmark = pytest.mark.gpu

CASE = "converge_16c_ns3_cd01"
GAMMA_RTOL = 1e-9


def _run(spec, form, pieces=None, plain=None):
    """Converge (in calls of the given sizes) or, with ``plain``, step that many
    steps with pfdd_step.  Returns gamma, gamma_a, final xi."""
    x0, b0 = workloads.initial_state(spec)
    tau = native.spec_tau(spec)
    s = native.solver_for(spec, form)
    try:
        s.set_state(x0, b0)
        if plain is not None:
            g, ga = s.step(tau[:plain])
            g, ga = g[:, 0], ga[:, 0]
        else:
            s.converge_reset(0.0)
            gs, gas, at = [], [], 0
            for p in pieces or [len(tau)]:
                g, ga = s.step_converge(tau[at:at + p])
                gs.append(g); gas.append(ga); at += len(g)
                if len(g) < p:
                    break
            g, ga = np.concatenate(gs), np.concatenate(gas)
        x = s.get_state()[0].reshape(spec.ns, -1)
    finally:
        s.close()
    return g, ga, x


def test_fp64_stops_where_the_reference_stopped():
    spec, z = load_golden(CASE)
    k = int(z["steps_run"])
    g, ga, x = _run(spec, "fp64")
    assert len(g) == k
    # gamma decays to 1e-16 here, so the bound is relative to its largest value:
    # the exact fixed-point sums round each point to 2^-44 (|error| <= ns 2^-45)
    assert np.max(np.abs(g - z["gamma"])) <= GAMMA_RTOL * np.max(np.abs(z["gamma"]))
    assert np.max(np.abs(ga - z["gamma_a"])) <= GAMMA_RTOL * np.max(np.abs(z["gamma_a"]))
    assert np.max(np.abs(x - z["xi_final"])) <= 1e-10 * np.max(np.abs(z["xi_final"]))
    # the state is the state after the stop step: the same bits as k plain steps
    gp, gap, xp = _run(spec, "fp64", plain=k)
    np.testing.assert_array_equal(g, gp)
    np.testing.assert_array_equal(ga, gap)
    np.testing.assert_array_equal(x, xp)


@pytest.mark.parametrize("form", ["fp64", "fp32"])
def test_loop_run_in_pieces_gives_the_same_stop_and_bits(form):
    """The pass marks carry over between calls: 50 + 50 + the rest stops at the
    same step with the same bits as one call, and the stop agrees with the
    restated rule on the form's own gammas."""
    spec, z = load_golden(CASE)
    g1, ga1, x1 = _run(spec, form)
    g2, ga2, x2 = _run(spec, form, pieces=[50, 50, spec.steps - 100])
    assert oracle.converge_stop(g1) == len(g1) < spec.steps
    np.testing.assert_array_equal(g1, g2)
    np.testing.assert_array_equal(ga1, ga2)
    np.testing.assert_array_equal(x1, x2)


def test_nonconverging_loop_runs_every_step_and_reset_restarts_the_count():
    spec, z = load_golden(CASE)
    x0, b0 = workloads.initial_state(spec)
    tau = native.spec_tau(spec)
    k = int(z["steps_run"])
    s = native.solver_for(spec, "fp64")
    try:
        s.set_state(x0, b0)
        s.converge_reset(0.0)
        g, _ = s.step_converge(tau[:k - 1])  # one step short of the stop: all run
        assert len(g) == k - 1
        s.converge_reset(float(g[-1]))  # a new loop: 30 more passing steps before any count
        g2, _ = s.step_converge(tau[k - 1:])
        assert len(g2) == oracle.converge_stop(g2, float(g[-1]))
        assert len(g2) >= 34
    finally:
        s.close()


def test_batched_context_is_rejected(native_lib):
    spec, _ = load_golden(CASE)
    s = native.solver_for(spec, "fp64", nrep=2)
    try:
        with pytest.raises(native.PFDDError) as ei:
            s.step_converge(np.zeros((4, 2, spec.ns)))
        assert ei.value.status == native.PFDD_EINVAL
    finally:
        s.close()


def test_batched_loops_stop_each_at_its_own_step(native_lib, monkeypatch):
    """Three replicas in one context, each with its own convergence test: two
    of the golden solve (the reference stops it at 112 steps) and one with
    ten times its noise, which stops later. Each replica stops where a
    one-solve context stops on its input, with the same bits; the replica that
    stops first leaves the batch at its stop while the other runs on."""
    spec, z = load_golden(CASE)
    loud = workloads.SolveSpec(**{**spec.__dict__, "noise_amp": spec.noise_amp * 10})
    monkeypatch.setenv("PFDD_NO_TUNE", "1")  # one launch plan in every context: the same rounding
    singles = [_run(sp, "fp64") for sp in (spec, loud)]
    assert len(singles[0][0]) == int(z["steps_run"]) < len(singles[1][0]) < spec.steps
    x0, b0 = workloads.initial_state(spec)
    x1, _ = workloads.initial_state(loud)
    tau = native.spec_tau(spec)
    s = native.solver_for(spec, "fp64", nrep=3)
    try:
        s.set_state(np.stack([x0, x1, x0]), np.stack([b0] * 3))
        s.converge_reset(0.0)
        done, g, ga = s.step_converge_batched(np.stack([tau] * 3, axis=1))
        x = s.get_state().reshape(3, spec.ns, -1)
    finally:
        s.close()
    for r, (sg, sga, sx) in zip((0, 1, 2), (singles[0], singles[1], singles[0])):
        k = len(sg)
        assert done[r] == k, (r, done)
        np.testing.assert_array_equal(g[:k, r], sg)
        np.testing.assert_array_equal(ga[:k, r], sga)
        assert not g[k:, r].any()
        np.testing.assert_array_equal(x[r], sx)
