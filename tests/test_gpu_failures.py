"""Failure detection without a GPU fault.

The reference prints and resets every device on any error (fullResetDMR, gDMR.cu:409-429).
Here every failure becomes a status, and the process's GPU context stays usable:

* a bounded device wait that runs out: the wait limit (gdmrWaitLimit) is set to zero, so the
  first grid-wide barrier of the fused small-system Krylov kernel gives up at once (nothing in
  flight there but plain loads and stores); the kernel returns, the solve reports
  GDMR_ETIMEOUT, and the next solve at the normal limit matches the oracle;
* a device allocation that fails, injected on the host (gdmrInjectAllocFailure): creation
  reports GDMR_ENOMEM and frees what it had allocated;
* a right-hand side holding NaN: GDMR_ENONFINITE, where the reference's loop test (NaN >
  tol is false) would return NaN as if converged.
"""
import numpy as np
import pytest

import gdmr
import problems

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_wait_limit_runs_out_then_the_next_solve_is_correct(oracle_mod):
    A, rhs, cfg = problems.config_2d64()
    s = gdmr.System(A, cfg["m"], cfg["k"], capacity=1, precision="fp64")   # n = 4096: fused Krylov loop
    before = gdmr.async_timeouts()
    prev = gdmr.wait_limit(0.0)
    try:
        with pytest.raises(gdmr.GDMRError) as e:
            s.solve(rhs[0], mode=0, tol=1e-10, mat_rank=2000)
    finally:
        gdmr.wait_limit(prev)
    assert e.value.status == 8 and "wait" in str(e.value)
    assert gdmr.async_timeouts() > before
    assert gdmr.wait_limit() == prev
    x, st = s.solve(rhs[0], mode=0, tol=1e-10, mat_rank=2000)
    r = oracle_mod.Oracle(A, cfg["m"], cfg["k"], fuse_deflation=True).solve(rhs[0], mode=0, tol=1e-10,
                                                                             mat_rank=2000)
    assert st["status"] == 0 and st["cycles"] == r["cycles"]
    assert _rel(x, r["x"]) < 1e-8


def test_batched_solve_reports_a_wait_that_ran_out():
    A, rhs, cfg = problems.config_2d64()
    s = gdmr.System(A, cfg["m"], cfg["k"], capacity=1, precision="fp64")
    prev = gdmr.wait_limit(0.0)
    try:
        X, stats = s.solve_batch(np.array(rhs[:1]), tol=1e-10, max_cycles=50)
        raised = None
    except gdmr.GDMRError as err:
        raised = err
    finally:
        gdmr.wait_limit(prev)
    assert raised is not None and raised.status == 8
    X, stats = s.solve_batch(np.array(rhs[:1]), tol=1e-10, max_cycles=2000)
    assert stats[0]["status"] == 0 and stats[0]["true_rel_res"] <= 1e-10


@pytest.mark.parametrize("nth", [1, 5, 30])
def test_injected_allocation_failure_reports_enomem_and_leaks_nothing(nth):
    import torch
    A, rhs, cfg = problems.config_2d64()
    ok = gdmr.System(A, cfg["m"], cfg["k"], capacity=4, precision="mixed")   # warms the context
    ok.close()
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    gdmr.inject_alloc_failure(nth)
    try:
        with pytest.raises(gdmr.GDMRError) as e:
            gdmr.System(A, cfg["m"], cfg["k"], capacity=4, precision="mixed")
    finally:
        gdmr.inject_alloc_failure(0)
    assert e.value.status == 2 and "injected" in str(e.value)
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free0 - free1 < 8 << 20, (free0, free1)
    s = gdmr.System(A, cfg["m"], cfg["k"], capacity=4, precision="mixed")
    X, stats = s.solve_batch(np.array(rhs[:2]), tol=1e-10, max_cycles=2000)
    assert all(t["status"] == 0 for t in stats)


def test_nan_right_hand_side_reports_nonfinite():
    A, rhs, cfg = problems.config_2d64()
    s = gdmr.System(A, cfg["m"], cfg["k"], capacity=1, precision="fp64")
    b = rhs[0].copy()
    b[17] = np.nan
    with pytest.raises(gdmr.GDMRError) as e:
        s.solve(b, mode=0, tol=1e-10, mat_rank=100)
    assert e.value.status == 9
    x, st = s.solve(rhs[0], mode=0, tol=1e-10, mat_rank=2000)
    assert st["status"] == 0 and st["true_rel_res"] <= 2e-10
