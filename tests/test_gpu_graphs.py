"""Replayed CUDA graphs of steps give the same bits as direct launches.

A context runs its first step with direct launches, then replays captured
graphs of 16 steps and of one step; the step index inside a chunk comes from a
device counter.  Changing a captured argument (the kinetic coefficients, the
pinned mask) must rebuild the graphs."""
import os

import numpy as np
import pytest

from pfdd_gb300 import native, workloads

pytestmark = pytest.mark.gpu


def make(spec, precision, graphs, nrep=1):
    old = os.environ.get("PFDD_NO_GRAPHS")
    os.environ["PFDD_NO_GRAPHS"] = "0" if graphs else "1"
    try:
        return native.solver_for(spec, precision, nrep=nrep)
    finally:
        if old is None:
            del os.environ["PFDD_NO_GRAPHS"]
        else:
            os.environ["PFDD_NO_GRAPHS"] = old


def trajectory(spec, precision, graphs):
    s = make(spec, precision, graphs)
    x0, b0 = workloads.initial_state(spec)
    s.set_state(x0, b0)
    tau = native.spec_tau(spec)
    out = []
    g, _ = s.step(tau[:37])          # 1 direct step + 2 graphs of 16 + 4 single-step graphs
    out.append(g)
    launches = s.launches
    g, _ = s.step(tau[37:53])        # graphs reused
    out.append(g)
    s.set_params(spec.cd2 * 1.5, spec.asf, spec.dslip, 1.0)   # captured coefficients change
    g, _ = s.step(tau[53:70])
    out.append(g)
    bc = np.zeros_like(b0); bc[:, 0, 0, :] = 1.0               # a pinned row: mask now read
    s.set_state(s.get_state()[0], bc)
    g, _ = s.step(tau[70:90])
    out.append(g)
    xf = s.get_state()
    s.close()
    return np.concatenate(out), xf, launches


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_graph_replay_matches_direct_launches(native_lib, precision):
    spec = workloads.SolveSpec(n=(16, 16, 32), ns=3, steps=90, sigma_max=0.04,
                               loops=workloads.random_loops((16, 16, 32), 3, 2.0, 5.0, 3, seed=9), noise_seed=9)
    g1, x1, l1 = trajectory(spec, precision, graphs=True)
    g0, x0, l0 = trajectory(spec, precision, graphs=False)
    np.testing.assert_array_equal(g1, g0)
    np.testing.assert_array_equal(x1, x0)
    assert l1 == l0 == 37 * 4 + 2  # + the spectral prologue and the chunk's gamma reduction


def test_graph_replay_batched(native_lib):
    spec = workloads.SolveSpec(n=(16, 8, 16), ns=12, steps=40, sigma_max=0.05, noise_seed=3,
                               loops=workloads.random_loops((16, 8, 16), 4, 2.0, 4.0, 12, seed=3))
    res = []
    for graphs in (True, False):
        s = make(spec, "fp32", graphs, nrep=3)
        x0, b0 = workloads.initial_state(spec)
        s.set_state(np.stack([x0, 0.5 * x0, -x0]), np.stack([b0] * 3))
        s.set_active(1, False)
        tau = np.stack([native.spec_tau(spec)] * 3, axis=1)
        g, _ = s.step(tau)
        res.append((g, s.get_state()))
        s.close()
    live = [0, 2]  # replica 1 is idle: its gamma slots are not written
    np.testing.assert_array_equal(res[0][0][:, live], res[1][0][:, live])
    np.testing.assert_array_equal(res[0][1], res[1][1])
