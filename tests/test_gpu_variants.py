"""Every Gram-Schmidt kernel variant gives a correct batched solve.

The tuner picks one projection and one update variant per shape class, so a
normal run exercises only the winners.  Here each variant is pinned in turn
(gdmrTuneForce) for a batch of 20 right-hand sides of the 64x64 Helmholtz
problem (m=40, k=10, tol 1e-10) that shares one deflation basis, and the
answers are checked against a sparse direct solve (relative 1e-8) and the
true FP64 residual (<= 1.5e-10).  The last index of each list is the batched
shared-basis pair (split-K projection of W for the whole batch, update with
W in registers for 16 systems at a time), which only runs while 8 or more
systems are active; complex64 projection variant 10 is the same shared-W
projection on the tensor cores (tcgen05, TF32 operands split big + small), and
complex64 update variant 9 applies W c on the tensor cores into the next Krylov
vector's slot before the per-system update, and variant 10 does the whole update in one kernel
(W c on the tensor cores, subtracted from TMEM by the warps that stream w and V), and variant 11
takes every system of the batch in one CTA with its rows of W in registers; complex128 / fp64e projection 8 and
update 7 prefetch the next group of basis vectors; projection 9 / 10 and update 8 / 9 are
the persistent forms (each CTA strides over many element chunks and reduces once), projection
12 / 13 and update 11 / 12 the same with the next loads issued before the arithmetic; double-float
projection 11 and update 10 are the bulk-copy pipelines (cp.async.bulk tiles behind mbarriers),
after which no bounded pipeline wait may have run out.
"""
import numpy as np
import pytest

import gdmr
import problems

pytestmark = pytest.mark.gpu

NRHS = 20
PAIRS = {
    "mixed": [(i, i) for i in range(9)] + [(9, 8), (10, 0), (10, 8), (0, 9), (10, 9), (0, 10), (10, 10),
              (0, 11), (10, 11)],
    "fp64": [(i, i) for i in range(7)] + [(7, 6), (8, 7), (9, 8), (10, 9), (12, 11), (13, 12)],
    "fp64e": [(0, 0), (1, 1), (2, 2), (6, 5), (8, 7), (9, 8), (10, 9), (11, 10), (12, 11), (13, 12)],
}


@pytest.fixture(scope="module")
def batch20():
    import scipy.sparse.linalg as spl
    A, _, cfg = problems.config_2d64()
    rhs = np.array([problems.unit_gaussian_rhs(A.n, 50 + s) for s in range(NRHS)])
    lu = spl.splu(A.to_scipy().tocsc())
    return A, rhs, cfg, np.array([lu.solve(b) for b in rhs])


@pytest.mark.parametrize("precision,pair", [(p, v) for p in PAIRS for v in PAIRS[p]])
def test_pinned_variant_solves_the_batch(batch20, precision, pair):
    A, rhs, cfg, direct = batch20
    timeouts0 = gdmr.async_timeouts()    # process-wide counter: only this test's waits count
    gdmr.tune_force(*pair)
    try:
        s = gdmr.System(A, cfg["m"], cfg["k"], capacity=NRHS, precision=precision)
        X, stats = s.solve_batch(rhs, tol=1e-10, max_cycles=2000)
    finally:
        gdmr.tune_force(-1, -1)
    for i, st in enumerate(stats):
        assert st["status"] == 0, (pair, i, st)
        assert st["true_rel_res"] <= 1.5e-10, (pair, i, st)
    err = np.linalg.norm(X - direct, axis=1) / np.linalg.norm(direct, axis=1)
    assert err.max() < 1e-8, (pair, err.max())
    rel = s.true_residual(rhs, X)
    assert np.all(rel <= 1.5e-10)
    assert gdmr.async_timeouts() == timeouts0


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_grouped_combination_matches_one_system_a_cta(batch20, precision):
    """The cycle-end combination four systems a CTA (W and Z loaded once for the four) against
    one system a CTA: the same per-element operations, so both batches converge alike and to
    the direct solution.  The Gram-Schmidt variants are pinned for both runs: with the tuner,
    the first run's launches before its tuning take variant 0 and the second run's the tuned
    one, and complex64 cycle counts follow such rounding differences by several cycles."""
    A, rhs, cfg, direct = batch20
    out = {}
    for grouped in (True, False):
        gdmr.combine_group(grouped)
        gdmr.tune_force(0, 0)
        try:
            s = gdmr.System(A, cfg["m"], cfg["k"], capacity=NRHS, precision=precision)
            out[grouped] = s.solve_batch(rhs, tol=1e-10, max_cycles=2000)
        finally:
            gdmr.combine_group(True)
            gdmr.tune_force(-1, -1)
    for grouped, (X, stats) in out.items():
        assert all(st["status"] == 0 and st["true_rel_res"] <= 1.5e-10 for st in stats), grouped
        err = np.linalg.norm(X - direct, axis=1) / np.linalg.norm(direct, axis=1)
        assert err.max() < 1e-8, (grouped, err.max())
    cg = [st["cycles"] for st in out[True][1]]
    cs = [st["cycles"] for st in out[False][1]]
    assert max(abs(a - b) for a, b in zip(cg, cs)) <= 2, (cg, cs)




@pytest.mark.parametrize("precision", ["mixed", "fp64", "fp64e"])
def test_residual_beside_the_deflation_loop_changes_nothing(batch20, precision):
    """The FP64 residual on its own stream beside the next cycle's deflation loop against the
    residual before the loop (eager cycles: graphs off, so the overlap runs from the third
    cycle on).  The same kernels read the same data, and the residual's smaller grid sums the
    same virtual blocks in the same order, so answers and cycle counts agree bit for bit."""
    A, rhs, cfg, direct = batch20
    out = {}
    for on in (2, 0):
        prev = gdmr.overlap_residual(on)
        gdmr.tune_force(0, 0)
        try:
            s = gdmr.System(A, cfg["m"], cfg["k"], capacity=NRHS, precision=precision)
            s.set_graphs(False)
            out[on] = s.solve_batch(rhs, tol=1e-10, max_cycles=2000)
            s.close()
        finally:
            gdmr.overlap_residual(prev)
            gdmr.tune_force(-1, -1)
    (X1, st1), (X0, st0) = out[2], out[0]
    assert [st["cycles"] for st in st1] == [st["cycles"] for st in st0]
    assert max(st["cycles"] for st in st1) >= 3
    assert np.array_equal(X1, X0)
    assert all(st["status"] == 0 and st["true_rel_res"] <= 1.5e-10 for st in st1)
    err = np.linalg.norm(X1 - direct, axis=1) / np.linalg.norm(direct, axis=1)
    assert err.max() < 1e-8
