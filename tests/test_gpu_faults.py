"""Failure detection, with every failure made on the host (no GPU fault):

- a bounded device wait that runs out: with PFDD_TEST_DROP_BULK=1 the x-pass's
  first CTA announces its B(k) tile's bytes on its mbarrier but issues no copy,
  so its wait gives up after a short limit; nothing is left in flight, the kernel
  returns, pfdd_step reports PFDD_ETIMEOUT and the context stays usable;
- an allocation failure: with PFDD_TEST_FAIL_ALLOC=k the k-th allocation of
  pfdd_create fails as on an exhausted device; pfdd_create returns PFDD_ENOMEM
  and pfdd_destroy of the partial context releases what it had allocated."""
import ctypes as C

import numpy as np
import pytest

from pfdd_gb300 import native, workloads

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("form,plan", [("fp64", None), ("fp32", None), ("fp32", "x=2,w=1"),
                                       ("fp32", "x=2,w=0"), ("fp32", "x=2,w=2")])
def test_bounded_wait_timeout_is_reported_and_context_recovers(native_lib, monkeypatch, form, plan):
    """Every x-pass kernel that waits on a bulk copy: the block-team (FP64 and
    FP32 table form) and the warp-team (FP32 table form, whole and split B
    block: with the first half's wait run out, no second half is loaded)
    kernels."""
    spec = workloads.SolveSpec(n=(32, 16, 16), ns=3, steps=6, sigma_max=0.05,
                               loops=[workloads.Loop(1, (16, 8, 8), 5.0)], noise_seed=8)
    x0, b0 = workloads.initial_state(spec)
    tau = native.spec_tau(spec)
    if plan:
        monkeypatch.setenv("PFDD_PLAN", plan)
    s = native.solver_for(spec, form)
    if plan:
        monkeypatch.delenv("PFDD_PLAN")
        assert s.plan()["x_pass"]["warp_teams"] == int(not plan.endswith("w=0"))
        assert s.plan()["x_pass"]["b_split"] == int(plan.endswith("w=2"))
    try:
        s.set_state(x0, b0)
        monkeypatch.setenv("PFDD_TEST_DROP_BULK", "1")
        with pytest.raises(native.PFDDError) as ei:
            s.step(tau[:3])
        assert ei.value.status == native.PFDD_ETIMEOUT
        monkeypatch.delenv("PFDD_TEST_DROP_BULK")
        # the same context, its state set again, gives a fresh context's bits
        s.set_state(x0, b0)
        g, _ = s.step(tau)
        xs = s.get_state()[0]
    finally:
        s.close()
    if plan:  # the same launch plan (an autotuned one may pick another radix plan: other rounding)
        monkeypatch.setenv("PFDD_PLAN", plan)
    r = native.solver_for(spec, form)
    if plan:
        monkeypatch.delenv("PFDD_PLAN")
    try:
        r.set_state(x0, b0)
        gr, _ = r.step(tau)
        xr = r.get_state()[0]
    finally:
        r.close()
    np.testing.assert_array_equal(xs, xr)
    np.testing.assert_array_equal(g, gr)


def test_allocation_failure_in_create_reports_enomem_without_leak(native_lib, monkeypatch):
    import torch
    L = native.load()
    shape = (128, 64, 64, 12, 1, native.PRECISIONS["fp32"], 0)  # 100 MB of xi: a leak would show
    h = C.c_void_p()
    assert L.pfdd_create_batched(C.byref(h), *shape) == native.PFDD_OK  # context and modules loaded
    L.pfdd_destroy(h)
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for k in (1, 2, 3, 8, 13, 14, 17, 20):
        monkeypatch.setenv("PFDD_TEST_FAIL_ALLOC", str(k))
        h = C.c_void_p()
        st = L.pfdd_create_batched(C.byref(h), *shape)
        assert st == native.PFDD_ENOMEM, (k, st)
        assert b"out of memory" in L.pfdd_last_error(h), k
        L.pfdd_destroy(h)
    monkeypatch.delenv("PFDD_TEST_FAIL_ALLOC")
    torch.cuda.synchronize()
    assert abs(torch.cuda.mem_get_info()[0] - free0) <= 8 << 20
    # and the next context is whole
    h = C.c_void_p()
    assert L.pfdd_create_batched(C.byref(h), *shape) == native.PFDD_OK
    L.pfdd_destroy(h)
