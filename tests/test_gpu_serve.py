"""Serving form (include/pfdd_serve.h): a solve's result is the same, bit for bit,
whether it runs alone in its own context or among other solves of mixed sizes in
the server (continuous admission into freed slots, chunked steps, classes created
and released under a device-memory budget)."""
import numpy as np
import pytest

from pfdd_gb300 import native, serve, workloads

pytestmark = pytest.mark.gpu


def mixed_requests():
    out = []
    shapes = [((16, 16, 16), 3), ((16, 16, 16), 12), ((32, 8, 16), 3), ((16, 16, 16), 3), ((32, 8, 16), 3),
              ((16, 16, 16), 3), ((16, 16, 16), 12), ((16, 16, 16), 3)]
    for q, ((n, ns), steps) in enumerate(zip(shapes, [23, 40, 17, 9, 31, 50, 12, 28])):
        loops = workloads.random_loops(n, 2, 2.0, 5.0, ns, seed=300 + q)
        out.append(workloads.SolveSpec(n=n, ns=ns, steps=steps, sigma_max=0.01 + 0.007 * q, loops=loops,
                                       noise_seed=400 + q))
    return out


def solo(spec, precision):
    s = native.solver_for(spec, precision)
    try:
        x0, b0 = workloads.initial_state(spec)
        s.set_state(x0, b0)
        g, ga = s.step(native.spec_tau(spec))
        return s.get_state()[0].reshape(spec.ns, -1), g[:, 0], ga[:, 0]
    finally:
        s.close()


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_solves_identical_alone_and_in_the_mix(native_lib, precision):
    specs = mixed_requests()
    with serve.Server(precision, max_slots=3, chunk_steps=7) as srv:
        ids = [srv.submit(sp) for sp in specs]
        res = [srv.wait(i) for i in ids]
        st = srv.stats()
    assert st["solves_done"] == len(specs)
    assert st["steps_done"] == sum(sp.steps for sp in specs)
    assert st["classes_created"] >= 3
    for sp, r in zip(specs, res):
        x, g, ga = solo(sp, precision)
        np.testing.assert_array_equal(r.xi, x)
        np.testing.assert_array_equal(r.gamma, g)
        np.testing.assert_array_equal(r.gamma_a, ga)
        assert r.latency_s > 0


def test_budget_serialises_classes_and_rejects_oversize(native_lib):
    specs = mixed_requests()[:5]
    one = max(native.load().pfdd_required_bytes(*sp.n, sp.ns, 1, native.PRECISIONS["fp32"]) for sp in specs)
    with serve.Server("fp32", hbm_budget=one, max_slots=4, chunk_steps=5) as srv:
        ids = [srv.submit(sp) for sp in specs]
        res = [srv.wait(i) for i in ids]
        big = workloads.SolveSpec(n=(64, 64, 64), ns=12, steps=2, sigma_max=0.01)
        with pytest.raises(native.PFDDError) as ei:
            srv.wait(srv.submit(big))
        assert ei.value.status == native.PFDD_ENOMEM
        st = srv.stats()
    assert st["peak_bytes"] <= one
    assert st["classes_created"] >= 3
    for sp, r in zip(specs, res):
        x, g, _ = solo(sp, "fp32")
        np.testing.assert_array_equal(r.xi, x)
        np.testing.assert_array_equal(r.gamma, g)


def test_converging_solves_stop_where_the_reference_stops(native_lib):
    """Solves submitted with the convergence stop end where the reference's test
    ends the inner loop: the golden solve (the reference stops it after 112 of
    its 300 steps) and the same with ten times its noise (it stops later), beside
    a fixed-length solve of the same class. Each has the bits of a one-solve
    context on its input (pfdd_step_converge for the two, pfdd_step for the
    other), and the converging ones hold zeros past their stop."""
    from conftest import load_golden
    spec, z = load_golden("converge_16c_ns3_cd01")
    loud = workloads.SolveSpec(**{**spec.__dict__, "noise_amp": spec.noise_amp * 10})
    fixed = workloads.SolveSpec(**{**spec.__dict__, "steps": 60, "noise_seed": 11})
    with serve.Server("fp64", max_slots=3, chunk_steps=7) as srv:
        ids = [srv.submit(spec, converge=True), srv.submit(fixed), srv.submit(loud, converge=True)]
        res = [srv.wait(i) for i in ids]
        st = srv.stats()
    assert st["classes_created"] == 1
    for sp, r in ((spec, res[0]), (loud, res[2])):
        s = native.solver_for(sp, "fp64")
        try:
            x0, b0 = workloads.initial_state(sp)
            s.set_state(x0, b0)
            s.converge_reset(0.0)
            g, ga = s.step_converge(native.spec_tau(sp))
            x = s.get_state()[0].reshape(sp.ns, -1)
        finally:
            s.close()
        k = len(g)
        assert r.steps_run == k < sp.steps
        np.testing.assert_array_equal(r.gamma[:k], g)
        np.testing.assert_array_equal(r.gamma_a[:k], ga)
        assert not r.gamma[k:].any()
        np.testing.assert_array_equal(r.xi, x)
    assert res[0].steps_run == int(z["steps_run"]) < res[2].steps_run
    x, g, ga = solo(fixed, "fp64")
    assert res[1].steps_run == fixed.steps
    np.testing.assert_array_equal(res[1].gamma, g)
    np.testing.assert_array_equal(res[1].xi, x)
