"""The inner loop's convergence stop (plasticconverge, F:3732-3785): the
oracle's restatement of the rule, pinned on the reference's own run of a solve
that stops early (tests/golden/converge_16c_ns3_cd01.npz: the compiled
reference with its stop left in, 112 of 300 steps).  The GPU test then checks
pfdd_step_converge against the same golden and this restatement."""
import numpy as np
import pytest

from conftest import load_golden
from oracle import oracle

CASE = "converge_16c_ns3_cd01"


def test_restated_rule_stops_where_the_reference_stopped():
    spec, g = load_golden(CASE)
    k = int(g["steps_run"])
    assert k < spec.steps  # the golden is an early stop
    # on the reference's own gammas: the stop falls on the last step it ran
    assert oracle.converge_stop(g["gamma"]) == k
    assert oracle.converge_stop(g["gamma"][:k - 1]) is None


def test_oracle_trajectory_stops_at_the_same_step():
    spec, g = load_golden(CASE)
    k = int(g["steps_run"])
    x, gam, ga = oracle.solve(spec)
    assert oracle.converge_stop(gam) == k
    np.testing.assert_allclose(gam[:k], g["gamma"], rtol=1e-10, atol=1e-16)
    np.testing.assert_allclose(ga[:k], g["gamma_a"], rtol=1e-10, atol=1e-16)
    xk = oracle.solve(spec, steps=k)[0].reshape(spec.ns, -1)
    assert np.max(np.abs(xk - g["xi_final"])) <= 1e-10 * np.max(np.abs(g["xi_final"]))


@pytest.mark.parametrize("seq,prev,want", [
    # 30 steps of no change from the start: the counts reach 5 at index 33
    (np.full(40, 1e-3), 1e-3, 34),
    # gamma zero throughout (the second test form): the same
    (np.zeros(40), 0.0, 34),
    # first step fails (gamma jumps from prev), then no change: window full at index 30
    (np.full(40, 1e-3), 0.0, 35),
    # a failing step leaves the count alone, and the window keeps it from growing
    # until 30 passing steps follow it
    (np.concatenate([np.full(32, 1e-3), [2e-3], np.full(40, 2e-3)]), 1e-3, 33 + 29 + 5),
    # never converges
    (np.arange(1, 60) * 1e-3, 0.0, None),
])
def test_rule_cases(seq, prev, want):
    assert oracle.converge_stop(seq, prev) == want


def _rule_states(seq, prev):
    """(pass marks so far, count, stopped) before each step of the rule."""
    passed, count, last, out = [], 0, float(prev), []
    for it, g in enumerate(map(float, seq)):
        out.append((list(passed), count))
        ok = (abs((g - last) / g) < 1e-8 or abs(g) < 1e-12) if g != 0 else (abs(g - last) < 1e-15 or abs(g) < 1e-14)
        passed.append(ok)
        if ok and it >= 29:
            if all(passed[it - 29:it + 1]):
                count += 1
            elif count != 0:
                count = 0
        if count == 5:
            count += 1
        last = g
    return out


def test_chunks_never_pass_the_stop():
    """pfdd_step_converge runs chunks no longer than the fewest steps to the next
    possible stop: on random pass patterns (runs of constant gamma between jumps,
    and the reference golden's gammas) no stop ever falls before that bound."""
    rng = np.random.default_rng(7)
    seqs = [load_golden(CASE)[1]["gamma"]]
    for _ in range(300):
        seq, g = [], 1e-3
        for _ in range(int(rng.integers(20, 200))):
            if rng.random() < rng.uniform(0.0, 0.15):
                g *= 1.0 + rng.uniform(1e-6, 1e-2)
            seq.append(g)
        seqs.append(np.array(seq))
    for seq in seqs:
        states = _rule_states(seq, 0.0)
        stop = oracle.converge_stop(seq, 0.0)
        for i, (passed, count) in enumerate(states):
            if stop is not None and i >= stop:
                break
            k = oracle.converge_min_steps(passed, count)
            assert k >= 1
            if stop is not None:
                assert i + k <= stop, (i, k, stop)


def _rule_trace(seq, prev):
    """(min_steps before the step, 1 if the loop stops after it) for every
    step of the rule, which is not reset at a stop (its count goes on past 5)."""
    out, passed, count, last = [], [], 0, float(prev)
    for it, g in enumerate(map(float, seq)):
        k = oracle.converge_min_steps(passed, count)
        ok = (abs((g - last) / g) < 1e-8 or abs(g) < 1e-12) if g != 0 else (abs(g - last) < 1e-15 or abs(g) < 1e-14)
        passed.append(ok)
        if ok and it >= 29:
            if all(passed[it - 29:it + 1]):
                count += 1
            elif count != 0:
                count = 0
        stop = count == 5
        if stop:
            count += 1
        out.append((k, int(stop)))
        last = g
    return out


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    """tests/converge_harness.cpp built with the host compiler against the
    library's own tracker header (pfdd_gb300/csrc/pfdd_converge.h)."""
    import shutil
    import subprocess
    from pathlib import Path
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        pytest.skip("no host C++ compiler")
    here = Path(__file__).resolve().parent
    exe = tmp_path_factory.mktemp("converge") / "converge_harness"
    subprocess.run([cxx, "-std=c++17", "-O1", "-Wall", "-Werror", "-I", str(here.parent / "pfdd_gb300" / "csrc"),
                    str(here / "converge_harness.cpp"), "-o", str(exe)], check=True)
    return exe


def _run_harness(exe, seq, prev):
    import subprocess
    text = " ".join([float(prev).hex(), str(len(seq))] + [float(g).hex() for g in seq])
    r = subprocess.run([str(exe)], input=text, capture_output=True, text=True, check=True)
    return [tuple(map(int, line.split())) for line in r.stdout.splitlines()]


def _random_sequences(rng, n):
    """Runs of constant gamma between jumps (of every size, including jumps
    below the 1e-8 threshold), sign changes, zeros, values below the absolute
    thresholds, and IEEE specials."""
    seqs = []
    for _ in range(n):
        seq, g = [], float(rng.choice([1e-3, -2e-5, 0.0, 5e-13, 3e-15]))
        p_jump = rng.uniform(0.0, 0.2)
        for _ in range(int(rng.integers(1, 260))):
            u = rng.random()
            if u < p_jump:
                g = g * (1.0 + rng.choice([1e-9, 3e-8, 1e-6, 1e-2, -2.0])) if g != 0 else float(rng.choice([1e-16, 1e-13, 1e-3]))
            elif u < p_jump + 0.01:
                g = float(rng.choice([0.0, -0.0, 1e-300, 5e-324, np.inf, -np.inf, np.nan]))
            elif u < p_jump + 0.02:
                g = float(rng.choice([1e-3, -1e-3]))
            seq.append(g)
        seqs.append(np.array(seq))
    return seqs


def test_host_tracker_follows_the_rule(harness):
    """The library's C++ tracker (every whole-step context and the server use
    it) gives, step by step, the restated rule's chunk bound and stops,
    including after a stop when the caller does not reset it."""
    rng = np.random.default_rng(11)
    cases = [(load_golden(CASE)[1]["gamma"], 0.0), (np.full(120, 1e-3), 1e-3), (np.zeros(100), 0.0),
             (np.full(100, 1e-3), 0.0)]
    cases += [(s, float(rng.choice([0.0, 1e-3]))) for s in _random_sequences(rng, 400)]
    nstop = 0
    for seq, prev in cases:
        got = _run_harness(harness, seq, prev)
        want = _rule_trace(seq, prev)
        assert got == want, (list(seq[:8]), prev)
        stops = [i for i, (_, s) in enumerate(got) if s]
        first = oracle.converge_stop(seq, prev)
        assert (stops[0] + 1 if stops else None) == first
        nstop += len(stops)
    assert nstop > 50  # the sequences do reach stops, and some go on past them
