"""Many operators of uneven size in lockstep, the Krylov loops of every right-hand side in flight
in one cooperative launch a cycle (gdmr_multi_solve, k_krylov_multi).

Three operators of different n (a 3D Helmholtz cube, a 3D Helmholtz box, a variable-coefficient
-div(a grad u) box), two or three right-hand sides each, more right-hand sides than slots for one
of them (refill between cycles), complex64 inner cycles with the FP64 true residual: every
solution meets its tolerance by the true FP64 residual and matches a sparse direct solve
(SuperLU) to 1e-8; the same systems solved one operator at a time (gdmr_solve_batch, the
step-by-step kernels) give the same solutions within the tolerance; no bounded wait ran out.
These run the lockstep to the end (gdmrMultiTail 0); one more test hands the last three systems
to the engines' own cycles, as the default tail does for the last eight.
"""
import numpy as np
import pytest

import gdmr
import problems

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def three():
    import scipy.sparse.linalg as spl
    mats = [problems.helmholtz((20, 20, 20), 6.0, 0.1),
            problems.helmholtz((24, 16, 12), 5.0, 0.1),
            problems.variable_helmholtz((30, 22, 18), 4.0, 0.1, seed=3)]
    rhs = [np.array([problems.unit_gaussian_rhs(A.n, 300 + 10 * i + j) for j in range(2 + (i == 2))])
           for i, A in enumerate(mats)]
    direct = [np.array([spl.splu(A.to_scipy().tocsc()).solve(b) for b in B]) for A, B in zip(mats, rhs)]
    return mats, rhs, direct


@pytest.fixture
def lockstep_to_the_end():
    prev = gdmr.multi_tail(0)      # no hand-over: every cycle in the lockstep launch
    yield
    gdmr.multi_tail(prev)


def test_three_operators_in_one_launch_match_a_direct_solve(three, lockstep_to_the_end):
    mats, rhs, direct = three
    t0 = gdmr.async_timeouts()
    systems = [gdmr.System(A, 30, 8, capacity=2, precision="mixed") for A in mats]
    out = gdmr.multi_solve(systems, rhs, tol=1e-10, max_cycles=2000)
    for A, B, D, (X, stats) in zip(mats, rhs, direct, out):
        S = A.to_scipy()
        for i, st in enumerate(stats):
            assert st["status"] == 0 and st["true_rel_res"] <= 1e-10, (A.n, i, st)
            assert np.linalg.norm(B[i] - S @ X[i]) / np.linalg.norm(B[i]) <= 1.5e-10
            assert np.linalg.norm(X[i] - D[i]) / np.linalg.norm(D[i]) < 1e-8
    assert gdmr.async_timeouts() == t0
    # the same right-hand sides one operator at a time, on the step-by-step kernels
    for A, B, (X, stats) in zip(mats, rhs, out):
        s = gdmr.System(A, 30, 8, capacity=2, precision="mixed")
        Xs, ss = s.solve_batch(B, tol=1e-10, max_cycles=2000)
        for i in range(B.shape[0]):
            assert ss[i]["status"] == 0
            assert np.linalg.norm(X[i] - Xs[i]) / np.linalg.norm(Xs[i]) < 2e-8


def test_tail_hands_the_last_systems_to_the_engines(three):
    """With the tail at 3, the lockstep runs while more than three systems are in flight, then the
    engines' own batched cycles finish the rest: the same solutions (SuperLU to 1e-8)."""
    mats, rhs, direct = three
    prev = gdmr.multi_tail(3)
    try:
        systems = [gdmr.System(A, 30, 8, capacity=2, precision="mixed") for A in mats]
        out = gdmr.multi_solve(systems, rhs, tol=1e-10, max_cycles=2000)
    finally:
        gdmr.multi_tail(prev)
    for A, B, D, (X, stats) in zip(mats, rhs, direct, out):
        S = A.to_scipy()
        for i, st in enumerate(stats):
            assert st["status"] == 0 and st["true_rel_res"] <= 1e-10, (A.n, i, st)
            assert np.linalg.norm(B[i] - S @ X[i]) / np.linalg.norm(B[i]) <= 1.5e-10
            assert np.linalg.norm(X[i] - D[i]) / np.linalg.norm(D[i]) < 1e-8


@pytest.mark.parametrize("precision", ["fp64", "fp64e"])
def test_many_operator_launch_in_the_fp64_forms(three, precision, lockstep_to_the_end):
    mats, rhs, direct = three
    systems = [gdmr.System(A, 30, 8, capacity=3, precision=precision) for A in mats]
    out = gdmr.multi_solve(systems, rhs, tol=1e-10, max_cycles=2000)
    for A, D, (X, stats) in zip(mats, direct, out):
        for i, st in enumerate(stats):
            assert st["status"] == 0 and st["true_rel_res"] <= 1e-10, (A.n, i, st)
            assert np.linalg.norm(X[i] - D[i]) / np.linalg.norm(D[i]) < 1e-8


def test_mixed_precisions_are_refused(three):
    mats, rhs, _ = three
    a = gdmr.System(mats[0], 30, 8, capacity=2, precision="mixed")
    b = gdmr.System(mats[1], 30, 8, capacity=2, precision="fp64")
    with pytest.raises(gdmr.GDMRError) as e:
        gdmr.multi_solve([a, b], rhs[:2])
    assert e.value.status == 1
