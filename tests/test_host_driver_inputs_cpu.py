"""The C host driver (pfdd_run) rejects malformed input files before it touches a
GPU: a short xi.dat, a missing xi_bc.dat, state in the slip systems beyond NS,
unknown options.  It reads xi.dat / xi_bc.dat (F:4366-4382) whole and checks the
read counts, where the reference's own fread calls go unchecked."""
import subprocess

import numpy as np

from pfdd_gb300 import build, refio, workloads


def _spec():
    return workloads.SolveSpec(n=(8, 8, 8), ns=3, steps=4, sigma_max=0.02,
                               loops=[workloads.Loop(0, (4, 4, 4), 2.0)], noise_seed=1)


def _run(cwd, *extra):
    sp = _spec()
    return subprocess.run([str(build.RUNNER), *map(str, sp.n), str(sp.ns), str(sp.steps), "0.02", "--nsfile", "12",
                           *extra], cwd=cwd, capture_output=True, text=True, timeout=60)


def _write(tmp_path):
    xi, bc = workloads.initial_state(_spec())
    refio.write_xi_files(tmp_path, xi, bc, ns_ref=12)


def test_short_xi_file_is_rejected(native_lib, tmp_path):
    _write(tmp_path)
    raw = (tmp_path / "xi.dat").read_bytes()
    (tmp_path / "xi.dat").write_bytes(raw[: len(raw) - 8])  # one double short
    r = _run(tmp_path)
    assert r.returncode == 1
    assert "cannot read xi.dat" in r.stderr
    assert not (tmp_path / "phasefield.dat").exists()


def test_missing_bc_file_is_rejected(native_lib, tmp_path):
    _write(tmp_path)
    (tmp_path / "xi_bc.dat").unlink()
    r = _run(tmp_path)
    assert r.returncode == 1 and "cannot read" in r.stderr


def test_state_beyond_ns_is_rejected(native_lib, tmp_path):
    sp = _spec()
    xi, bc = workloads.initial_state(sp)
    refio.write_xi_files(tmp_path, xi, bc, ns_ref=12)
    raw = np.fromfile(tmp_path / "xi.dat")
    raw[2 * sp.ns * sp.npts + 6] = 0.5  # a value in system ns (unevolved, must stay zero)
    raw.tofile(tmp_path / "xi.dat")
    r = _run(tmp_path)
    assert r.returncode == 1 and "must be zero and pinned" in r.stderr


def test_bad_arguments_are_rejected(native_lib, tmp_path):
    _write(tmp_path)
    r = _run(tmp_path, "--bogus")
    assert r.returncode == 2 and "unknown option" in r.stderr
    r = subprocess.run([str(build.RUNNER), "8", "8"], cwd=tmp_path, capture_output=True, text=True, timeout=60)
    assert r.returncode == 2 and "usage" in r.stderr


def test_bad_spacing_and_force_factor_are_rejected(native_lib, tmp_path):
    _write(tmp_path)
    for extra in (["--dslip", "0"], ["--d", "1", "0", "1"], ["--d", "1", "-2", "1"], ["--uq2", "nan"],
                  ["--d", "1", "inf", "1"]):
        r = _run(tmp_path, *extra)
        assert r.returncode == 2 and "bad spacing or force factor" in r.stderr, extra
        assert not (tmp_path / "phasefield.dat").exists()
    r = _run(tmp_path, "--d", "1", "1")  # three values or none
    assert r.returncode == 2 and "unknown option" in r.stderr
