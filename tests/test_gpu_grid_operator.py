"""The structured-grid operator kernel (k_grid_spmm) against the SELL-32 kernels.

A CSR matrix on a 5- or 7-point grid stencil is also kept as coefficient planes, and its
products run on the grid kernel (gdmrGridOperator, on by default).  The kernel adds a row's
terms in the order the SELL kernels do and leaves out only terms whose neighbour lies outside
the grid (where SELL adds a stored zero times x), so for a matrix with sorted, duplicate-free
CSR rows every product, and with it every solve, must come out identical:
  * mixed batched solves of 7 and 5 right-hand sides, with the batched products on the grid
    kernel at 1, 2 and 4 systems a thread (the last group partial; batches that shrink as
    systems converge) and on SELL (the default, where only single-vector products take the grid
    kernel), on a 3D grid whose x and y edges leave partial tiles and whose z edge a partial
    chunk of planes, and on a 2D grid with variable coefficients;
  * plain complex128 and double-float solves of one right-hand side (step-by-step Krylov loop).
The tuner is settled by a first solve, so both runs take the same Gram-Schmidt variants.
"""
import numpy as np
import pytest

import gdmr
import problems

pytestmark = pytest.mark.gpu


def _batch(A, B, m, k, precision, grid, sg=0):
    gdmr.grid_operator(grid)
    gdmr.grid_batch(sg)
    try:
        s = gdmr.System(A, m, k, capacity=B.shape[0], precision=precision)
        try:
            shape = s.grid_shape()
            X, stats = s.solve_batch(B, tol=1e-10, max_cycles=3000)
        finally:
            s.close()
    finally:
        gdmr.grid_operator(True)
        gdmr.grid_batch(0)
    return shape, X, stats


def _plain(A, b, m, k, precision, grid):
    gdmr.grid_operator(grid)
    try:
        s = gdmr.System(A, m, k, capacity=1, precision=precision)
        try:
            s.set_fused(False)
            x, st = s.solve(b, mode=0, tol=1e-10, mat_rank=4000)
        finally:
            s.close()
    finally:
        gdmr.grid_operator(True)
    return x, st


CASES = {
    "3d": (lambda: problems.helmholtz((40, 36, 30), 10.0, 0.1), (40, 36, 30), 7),
    "2d_variable": (lambda: problems.variable_helmholtz((70, 45, 1), 12.0, 0.1, seed=5), (70, 45, 1), 5),
}


@pytest.mark.parametrize("sgt", [0, 1, 2, 4])
@pytest.mark.parametrize("case", sorted(CASES))
def test_mixed_batch_is_identical_on_both_kernels(case, sgt):
    make, shape, nrhs = CASES[case]
    A = make()
    B = np.array([problems.unit_gaussian_rhs(A.n, 40 + i) for i in range(nrhs)])
    _batch(A, B, 30, 10, "mixed", True, sgt)                 # settles the tuner
    g_shape, Xg, sg = _batch(A, B, 30, 10, "mixed", True, sgt)
    s_shape, Xs, ss = _batch(A, B, 30, 10, "mixed", False)
    assert g_shape == shape and s_shape == shape
    for i in range(nrhs):
        assert sg[i]["status"] == 0 and sg[i]["true_rel_res"] <= 1e-10, (i, sg[i])
        assert sg[i]["cycles"] == ss[i]["cycles"], (i, sg[i]["cycles"], ss[i]["cycles"])
    assert np.array_equal(Xg, Xs)


@pytest.mark.parametrize("precision", ["fp64", "fp64e"])
def test_plain_solve_is_identical_on_both_kernels(precision):
    A = problems.helmholtz((40, 36, 30), 10.0, 0.1)
    b = problems.unit_gaussian_rhs(A.n, 9)
    _plain(A, b, 30, 10, precision, True)
    xg, sg = _plain(A, b, 30, 10, precision, True)
    xs, ss = _plain(A, b, 30, 10, precision, False)
    assert sg["status"] == 0 and sg["true_rel_res"] <= 2e-10, sg
    assert sg["cycles"] == ss["cycles"]
    assert np.array_equal(xg, xs)


@pytest.mark.parametrize("case", sorted(CASES))
def test_fp64_true_residual_is_identical_on_both_kernels(case):
    """The FP64 true residual b - A x (real coefficients skip their zero imaginary products) is
    the same with the grid operator kernel on and off, and matches SciPy's FP64 product."""
    make, shape, nrhs = CASES[case]
    A = make()
    rng = np.random.default_rng(11)
    B = np.array([problems.unit_gaussian_rhs(A.n, 70 + i) for i in range(nrhs)])
    X = rng.standard_normal(B.shape) + 1j * rng.standard_normal(B.shape)
    out = {}
    for grid in (True, False):
        gdmr.grid_operator(grid)
        try:
            s = gdmr.System(A, 30, 10, capacity=nrhs, precision="mixed")
            out[grid] = s.true_residual(B, X)
            s.close()
        finally:
            gdmr.grid_operator(True)
    assert np.array_equal(out[True], out[False])
    S = A.to_scipy()
    ref = np.linalg.norm(B - (S @ X.T).T, axis=1) / np.linalg.norm(B, axis=1)
    assert np.allclose(out[True], ref, rtol=1e-12)
