"""Host-side checks that need no GPU: the C-ABI library loads and exports every declared
entry point, the product's setup code agrees with the oracle, argument validation, the
seeded workloads and the reference file formats."""
import re
import subprocess
from pathlib import Path

import numpy as np
import pytest

from oracle import oracle
from pfdd_gb300 import native, refio, workloads

ROOT = Path(__file__).resolve().parents[1]


def declared_functions():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = h.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"\b(pfdd_\w+)\s*\(", text):
            names.add(m.group(1))
    return sorted(names)


def test_library_exports_every_declared_symbol(native_lib):
    out = subprocess.run(["nm", "-D", "--defined-only", str(native.LIB_PATH)], capture_output=True, text=True,
                         check=True).stdout
    exported = {ln.split()[-1] for ln in out.splitlines() if " T " in ln}
    decl = declared_functions()
    assert len(decl) >= 25
    missing = [d for d in decl if d not in exported]
    assert not missing, missing
    for d in decl:  # and ctypes resolves each of them
        getattr(native_lib, d)
    assert set(native.EXPORTS) <= set(decl)


def test_setup_matches_oracle(native_lib):
    np.testing.assert_array_equal(native.fcc_eps(12), oracle.fcc_eps(12))
    eps = native.fcc_eps(12)
    sig = np.zeros((3, 3)); sig[0, 2] = sig[2, 0] = 0.05
    np.testing.assert_array_equal(native.resolved_shear(eps, sig), oracle.resolved_shear(eps, sig))
    tm = native.resolved_shear(eps, sig)
    np.testing.assert_array_equal(native.ramp_tau(tm, 7), oracle.ramp_tau(tm, 7))
    import ctypes as C
    for n in (1, 2, 8, 128):
        f = np.zeros(n)
        native_lib.pfdd_frec(n, 1.0, f.ctypes.data_as(C.POINTER(C.c_double)))
        np.testing.assert_array_equal(f, oracle.frec(n))


def test_schmid_factors_of_config0():
    # (111) systems 0-2 glide on x-normal planes; sigma_xz resolves to 0, +-sqrt(3)/2*sigma/... (nonzero on 1, 2)
    eps = native.fcc_eps(3)
    sig = np.zeros((3, 3)); sig[0, 2] = sig[2, 0] = 1.0
    tau = native.resolved_shear(eps, sig)
    assert abs(tau[0]) < 1e-15
    assert abs(tau[1] + tau[2]) < 1e-15 and abs(tau[1]) > 0.5


def test_argument_validation_before_any_device_call(native_lib):
    import ctypes as C
    h = C.c_void_p()
    for args in [(3, 8, 8, 3, 0, 0), (8, 8, 8, 0, 0, 0), (8, 8, 8, 13, 0, 0), (8, 8, 1024, 3, 0, 0),
                 (8, 8, 8, 3, 7, 0)]:
        assert native_lib.pfdd_create(C.byref(h), *args) == native.PFDD_EINVAL
        assert not h.value
    assert native_lib.pfdd_fft_plan_create(C.byref(h), 6, 8, 8, 1, 1, 0) == native.PFDD_EINVAL
    assert native_lib.pfdd_status_string(native.PFDD_ENONFINITE) == b"state became non-finite"
    # serving form: rejected before the device is touched
    for args in [(0, 0, 0, 0, 1), (0, 0, 0, 1, 0), (9, 0, 0, 4, 10)]:
        assert native_lib.pfdd_server_create(C.byref(h), *args) == native.PFDD_EINVAL
        assert not h.value
    cnt = C.c_longlong()
    assert native_lib.pfdd_server_submit(None, None, C.byref(cnt)) == native.PFDD_EINVAL
    assert native_lib.pfdd_server_stats(None, None, None, None, None) == native.PFDD_EINVAL
    assert native_lib.pfdd_server_wait(None, 1, None, None, None) == native.PFDD_EINVAL
    assert native_lib.pfdd_server_wait_run(None, 1, None, None, None, None) == native.PFDD_EINVAL
    native_lib.pfdd_server_destroy(None)
    # convergence stop: no context
    ran = (C.c_int * 1)()
    assert native_lib.pfdd_converge_reset(None, 0.0) == native.PFDD_EINVAL
    assert native_lib.pfdd_converge_reset_batched(None, None) == native.PFDD_EINVAL
    assert native_lib.pfdd_step_converge(None, 1, None, None, None, ran) == native.PFDD_EINVAL
    assert native_lib.pfdd_step_converge_batched(None, 1, None, None, None, ran) == native.PFDD_EINVAL


def test_required_bytes_scale():
    b1 = native.load().pfdd_required_bytes(128, 128, 128, 12, 1, 0)
    b32 = native.load().pfdd_required_bytes(128, 128, 128, 12, 1, 1)
    N = 128 ** 3
    assert b1 >= N * 12 * 32 + N * 78 * 8
    assert b32 >= N * 12 * 24 + N * 78 * 4 and b32 < b1


def test_workloads_deterministic_and_loops():
    s = workloads.config0()
    xi, bc = workloads.initial_state(s)
    xi2, _ = workloads.initial_state(s)
    np.testing.assert_array_equal(xi, xi2)
    m = workloads.loop_mask(s.n, s.loops[0])
    assert m[16].sum() == m.sum()            # one-voxel slab i == 16
    assert 190 <= m.sum() <= 210              # disc of radius 8 (~pi*64)
    assert np.all(bc == 0)
    assert np.max(np.abs(xi.real - np.where(m, 1.0, 0.0)[None] * (np.arange(3) == 0)[:, None, None, None])) <= 1e-3
    c1 = workloads.config1()
    assert len(c1.loops) == 8 and all(8 <= lp.radius <= 20 for lp in c1.loops)
    reps = workloads.config3_replicas(16)
    assert reps[0].loops == reps[15].loops and reps[0].noise_seed != reps[1].noise_seed
    assert abs(reps[0].sigma_max - 0.005) < 1e-15 and abs(reps[-1].sigma_max - 0.08) < 1e-15
    reqs = workloads.config4_requests(96)
    assert len(reqs) == 96 and {r.n[0] for r in reqs} <= {32, 64, 128, 256}


def test_rotated_normals_of_111_systems_are_x():
    nn = workloads.rotated_normals()
    for s in range(3):
        np.testing.assert_allclose(np.abs(nn[s]), [1, 0, 0], atol=1e-12)


def test_refio_round_trip(tmp_path):
    s = workloads.SolveSpec(n=(4, 2, 8), ns=3, steps=1, sigma_max=0.0, noise_seed=1)
    xi, bc = workloads.initial_state(s)
    xi = xi + 1j * 0.25
    refio.write_xi_files(tmp_path, xi, bc, ns_ref=12)
    back = refio.read_xi_file(tmp_path / "xi.dat", s.n, 21)
    np.testing.assert_array_equal(back[:3], xi)
    assert np.all(back[3:] == 0)
    bcb = refio.read_xi_file(tmp_path / "xi_bc.dat", s.n, 21)
    assert np.all(bcb[:3] == 0) and np.all(bcb[3:] == 1 + 1j)
    line = refio.format_phasefield_line(1, 3, 1.5e-3, -2e-4, 6.0e-3)
    assert line == "1       3         1.500000e-03           -2.000000e-04           6.000000e-03\n"


def test_reference_patch_recipe_applies():
    import oracle.build_ref as br
    if not br.REF_SRC.exists():
        pytest.skip("reference checkout not present")
    out = br.write_patched_source(dst=ROOT / "oracle" / "_ref" / "pfdd_ref_patched.c")
    text = out.read_text(encoding="latin-1")
    assert "#define NS1 12" in text and "if(0) {" in text and "PFDD_LOG_STEP" in text


def test_every_context_call_rejects_a_null_handle(native_lib):
    """Each entry point that takes a context or plan returns PFDD_EINVAL for a
    null one before touching the device (its first check), with every other
    argument null or zero."""
    import ctypes as C
    names = ["pfdd_set_B", "pfdd_get_B", "pfdd_build_B", "pfdd_set_params", "pfdd_set_state",
             "pfdd_set_replica_state", "pfdd_set_tau_field", "pfdd_set_replica_active", "pfdd_step",
             "pfdd_converge_reset", "pfdd_converge_reset_batched", "pfdd_step_converge",
             "pfdd_step_converge_batched", "pfdd_get_plan", "pfdd_set_diagnostics", "pfdd_get_diagnostics",
             "pfdd_state_diagnostics", "pfdd_get_state", "pfdd_get_replica_state", "pfdd_set_stream_priority",
             "pfdd_set_kernel_timing", "pfdd_kernel_stat", "pfdd_fft_forward", "pfdd_fft_backward",
             "pfdd_strain_stress"]
    for name in names:
        fn = getattr(native_lib, name)
        assert fn.argtypes, name
        args = [0.0 if t is C.c_double else 0 if t in (C.c_int, C.c_size_t, C.c_longlong) else None
                for t in fn.argtypes]
        assert fn(*args) == native.PFDD_EINVAL, name
