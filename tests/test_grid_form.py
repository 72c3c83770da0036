"""Host-side detection of the structured-grid operator form (gdmr_csr_grid_form, no GPU).

A CSR matrix gets coefficient planes for the grid operator kernel when its non-zeros lie on
the 5- or 7-point offsets of a lexicographic grid and none couples two rows across the grid's
edge.  The kernel tests each neighbour against the grid's edges instead of reading a column
index, so a wrap-around entry (periodic coupling) must keep a matrix off that kernel, while an
explicit zero there contributes nothing and may stay.
"""
import numpy as np
import pytest

import gdmr
import problems
from problems import CSR


def _with_entry(A, r, c, v):
    """A copy of A with v added as one more stored entry (r, c)."""
    indptr = np.asarray(A.indptr, dtype=np.int64).copy()
    indices = list(A.indices)
    data = list(A.data)
    at = int(indptr[r + 1])
    indices.insert(at, c)
    data.insert(at, v)
    indptr[r + 1:] += 1
    return CSR(A.n, indptr, np.array(indices), np.array(data, dtype=complex))


def test_3d_and_2d_helmholtz_are_grids():
    assert gdmr.csr_grid_form(problems.helmholtz((12, 10, 9), 6.0, 0.1)) == (12, 10, 9)
    assert gdmr.csr_grid_form(problems.helmholtz((37, 29), 12.0, 0.05)) == (37, 29, 1)


def test_variable_coefficients_are_a_grid():
    A = problems.variable_helmholtz((20, 17, 11), 16.0, 0.1, seed=3)
    assert gdmr.csr_grid_form(A) == (20, 17, 11)


def test_shuffled_rows_with_duplicates_stay_a_grid():
    A = problems.helmholtz((16, 8, 5), 6.0, 0.1)
    rng = np.random.default_rng(1)
    indptr, indices, data = [0], [], []
    for r in range(A.n):
        cols = list(A.indices[A.indptr[r]:A.indptr[r + 1]])
        vals = list(A.data[A.indptr[r]:A.indptr[r + 1]])
        cols.append(cols[0])
        vals.append(0.5 + 0.25j)
        order = rng.permutation(len(cols))
        indices += [cols[i] for i in order]
        data += [vals[i] for i in order]
        indptr.append(len(indices))
    B = CSR(A.n, np.array(indptr), np.array(indices), np.array(data, dtype=complex))
    assert gdmr.csr_grid_form(B) == (16, 8, 5)


@pytest.mark.parametrize("where", ["x+", "x-", "y+", "y-"])
def test_a_wrap_around_entry_is_not_a_grid(where):
    nx, ny, nz = 8, 6, 5
    A = problems.helmholtz((nx, ny, nz), 6.0, 0.1)
    r = {"x+": nx - 1,                  # last point of an x line -> first point of the next line
         "x-": 2 * nx,                  # first point of a line -> last point of the previous line
         "y+": (ny - 1) * nx + 2,       # last line of plane 0 -> first line of plane 1
         "y-": nx * ny + 2}[where]      # first line of plane 1 -> last line of plane 0
    c = r + {"x+": 1, "x-": -1, "y+": nx, "y-": -nx}[where]
    assert gdmr.csr_grid_form(_with_entry(A, r, c, -1.0 + 0.0j)) is None
    # the same entry stored as an explicit zero changes nothing the kernel computes
    assert gdmr.csr_grid_form(_with_entry(A, r, c, 0.0)) == (nx, ny, nz)


def test_other_patterns_are_not_grids():
    n = 50
    # tridiagonal (three offsets)
    rows = np.repeat(np.arange(n), 3)
    cols = np.clip(rows + np.tile([-1, 0, 1], n), 0, n - 1)
    T = problems._assemble(n, [rows], [cols], [np.ones(3 * n, dtype=complex)])
    assert gdmr.csr_grid_form(T) is None
    # unstructured
    rng = np.random.default_rng(2)
    per = 6
    indptr = np.arange(0, (n + 1) * per, per)
    indices = np.concatenate([np.sort(rng.choice(n, per, replace=False)) for _ in range(n)])
    U = CSR(n, indptr, indices, rng.standard_normal(n * per) + 0j)
    assert gdmr.csr_grid_form(U) is None


def test_malformed_csr_is_rejected():
    A = problems.helmholtz((6, 5, 4), 6.0, 0.1)
    bad = CSR(A.n, A.indptr, np.where(np.arange(A.nnz) == 7, A.n, A.indices), A.data)
    with pytest.raises(gdmr.GDMRError):
        gdmr.csr_grid_form(bad)


def test_column_check_covers_rows_after_the_pattern_overflows():
    # an unstructured matrix has more than 8 offsets by its first rows; a bad column in the
    # last row must still be caught (the operator kernels would gather through it)
    rng = np.random.default_rng(4)
    n, per = 300, 6
    indptr = np.arange(0, (n + 1) * per, per)
    indices = np.concatenate([np.sort(rng.choice(n, per, replace=False)) for _ in range(n)])
    indices[-1] = n + 5
    U = CSR(n, indptr, indices, rng.standard_normal(n * per) + 0j)
    with pytest.raises(gdmr.GDMRError):
        gdmr.csr_grid_form(U)
    indices[-1] = -1
    with pytest.raises(gdmr.GDMRError):
        gdmr.csr_grid_form(CSR(n, indptr, indices, U.data))
