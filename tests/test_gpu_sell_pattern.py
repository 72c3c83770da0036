"""The SELL-32 operator store, with and without its offset pattern, and the structured-grid
kernel, against scipy.

A matrix whose column offsets (column - row) take at most 8 values is stored with the offsets
as a pattern: the operator kernels form the columns as row + offset instead of loading them, and
entries the pattern has but a row lacks are stored as zeros.  Through the plugin operator
(impCsrLS_z, then linOptLS_z: x <- A x on the device, complex128), y must equal scipy's A x to
1e-13 relative for:
  * a 2D 5-point operator whose CSR rows are shuffled and carry split (duplicate) entries;
  * a 3D 7-point operator, whose first and last planes' slices cannot use the pattern;
  * an unstructured random matrix (more than 8 offsets: no pattern at all).
The two stencil matrices also have the structured-grid form: each case runs with the grid
kernel on (the default) and off.
"""
import numpy as np
import pytest

import gdmr
import problems
from problems import CSR

pytestmark = pytest.mark.gpu


@pytest.fixture(params=[True, False], ids=["grid", "sell"])
def grid(request):
    gdmr.grid_operator(request.param)
    yield request.param
    gdmr.grid_operator(True)


def _apply(A, x):
    ls = gdmr.LinearSystem(A.n, 10, 2, precision="c128")
    try:
        ls.imp_csr(A)
        ls.imp_src(x)
        ls.lin_opt()
        return ls.exp_src()
    finally:
        ls.close()


def _shuffled_with_duplicates(A, seed):
    rng = np.random.default_rng(seed)
    indptr, indices, data = [0], [], []
    for r in range(A.n):
        beg, end = A.indptr[r], A.indptr[r + 1]
        cols = list(A.indices[beg:end])
        vals = list(A.data[beg:end])
        j = int(rng.integers(len(cols)))       # split one entry into two that sum to it
        w = complex(rng.standard_normal(), rng.standard_normal())
        cols.append(cols[j])
        vals.append(w)
        vals[j] = vals[j] - w
        order = rng.permutation(len(cols))
        indices += [cols[i] for i in order]
        data += [vals[i] for i in order]
        indptr.append(len(indices))
    return CSR(A.n, np.array(indptr), np.array(indices), np.array(data, dtype=complex))


def _check(A, seed):
    rng = np.random.default_rng(seed)
    x = rng.standard_normal(A.n) + 1j * rng.standard_normal(A.n)
    y = _apply(A, x)
    ref = A.to_scipy() @ x
    assert np.linalg.norm(y - ref) / np.linalg.norm(ref) < 1e-13


def test_2d_pattern_with_shuffled_rows_and_duplicates(grid):
    A = problems.helmholtz((37, 29), 12.0, 0.05)
    _check(_shuffled_with_duplicates(A, 3), 4)


def test_3d_pattern_with_boundary_slices(grid):
    _check(problems.helmholtz((12, 10, 9), 6.0, 0.1), 5)


def test_unstructured_matrix_has_no_pattern():
    rng = np.random.default_rng(6)
    n, per_row = 1500, 9
    indptr = np.arange(0, (n + 1) * per_row, per_row)
    indices = np.concatenate([np.sort(rng.choice(n, per_row, replace=False)) for _ in range(n)])
    data = rng.standard_normal(n * per_row) + 1j * rng.standard_normal(n * per_row)
    _check(CSR(n, indptr, indices, data), 7)


def _with_complex_entry(A, row, col, value):
    S = A.to_scipy().tolil()
    S[row, col] = value
    S = S.tocsr()
    S.sort_indices()
    return CSR(A.n, S.indptr.astype(np.int32), S.indices.astype(np.int32), S.data.astype(np.complex128))


@pytest.mark.parametrize("case", ["helmholtz3d", "one_complex_offdiag", "all_complex", "helmholtz2d"])
def test_fp64_residual_real_pattern_entries(case):
    """The FP64 true residual takes two FMAs instead of four for pattern entries that are real in
    every pattern-stored slice (the Helmholtz off-diagonals), decided on the host.  Against numpy
    ||b - A x|| / ||b|| to 1e-13: a 3D 7-point operator (one complex entry, the diagonal), the same
    with one complex off-diagonal value in one interior row (that entry is then complex in every
    slice), a 7-point operator with complex values everywhere (the plain loop), and a 2D 5-point
    operator."""
    rng = np.random.default_rng(11)
    if case == "helmholtz2d":
        A = problems.helmholtz((40, 33), 9.0, 0.1)
    else:
        A = problems.helmholtz((14, 12, 11), 6.0, 0.1)
    if case == "one_complex_offdiag":
        r = A.n // 2
        A = _with_complex_entry(A, r, r + 1, -1.0 + 0.25j)
    if case == "all_complex":
        S = A.to_scipy().tocsr()
        S.data = S.data + 1j * rng.uniform(0.1, 0.5, S.nnz)
        A = CSR(A.n, S.indptr.astype(np.int32), S.indices.astype(np.int32), S.data.astype(np.complex128))
    s = gdmr.System(A, 10, 2, capacity=3, precision="mixed")
    try:
        B = rng.standard_normal((3, A.n)) + 1j * rng.standard_normal((3, A.n))
        X = rng.standard_normal((3, A.n)) + 1j * rng.standard_normal((3, A.n))
        rel = s.true_residual(B, X)
    finally:
        s.close()
    S = A.to_scipy()
    ref = np.array([np.linalg.norm(b - S @ x) / np.linalg.norm(b) for b, x in zip(B, X)])
    assert np.max(np.abs(rel - ref) / ref) < 1e-13, (rel, ref)
