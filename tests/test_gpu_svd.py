"""The deflation update's SVD (gdmr_hessenberg_svd) against LAPACK.

k_svd gives the right singular vectors of the k smallest singular values of the (m+1) x m
Hessenberg: FP32 pivoted QR and one-sided Jacobi, then a double-float polar correction and a
double-float Jacobi polish restricted to those k columns.  The vectors must match LAPACK's to
1e-12, or to 1e-13 ||H|| / gap where the gap to the next singular value is small (up to a unit
phase); they must be orthonormal to 1e-13 m, their singular values must match to 1e-13 ||H||, and
the other singular values, which only the FP32 phase refines, to 2 m eps32 ||H||.  Cases: Arnoldi Hessenbergs of the 64 x 64
Helmholtz operator (first cycle and after five restarts), a graded random Hessenberg (singular
values over six decades), a near-degenerate pair at the boundary of the k smallest, and the
largest basis the kernel takes in shared memory (m = 64) and in global memory (m = 96).
"""
import numpy as np
import pytest

import gdmr
import problems

pytestmark = pytest.mark.gpu


def _arnoldi_h(m, restarts, seed=1):
    A, rhs, _ = problems.config_2d64()
    S = A.to_scipy().tocsr()
    b = rhs[seed - 1]
    x = np.zeros(S.shape[0], complex)
    for _ in range(restarts + 1):
        r = b - S @ x
        V = np.zeros((S.shape[0], m + 1), complex)
        H = np.zeros((m + 1, m), complex)
        V[:, 0] = r / np.linalg.norm(r)
        for j in range(m):
            w = S @ V[:, j]
            for _ in range(2):
                c = V[:, :j + 1].conj().T @ w
                w -= V[:, :j + 1] @ c
                H[:j + 1, j] += c
            H[j + 1, j] = np.linalg.norm(w)
            V[:, j + 1] = w / H[j + 1, j]
        e = np.zeros(m + 1, complex)
        e[0] = np.linalg.norm(r)
        x = x + V[:, :m] @ np.linalg.lstsq(H, e, rcond=None)[0]
    return H


def _graded(m, seed, decades=6.0, gap=None):
    rng = np.random.default_rng(seed)
    Q1 = np.linalg.qr(rng.standard_normal((m + 1, m + 1)) + 1j * rng.standard_normal((m + 1, m + 1)))[0]
    Q2 = np.linalg.qr(rng.standard_normal((m, m)) + 1j * rng.standard_normal((m, m)))[0]
    s = np.logspace(0, -decades, m)
    if gap is not None:                 # two nearly equal values straddling the k-th boundary
        s[-gap - 1] = s[-gap] * (1 + 1e-6)
    return Q1[:, :m] @ np.diag(s) @ Q2.conj().T


def _check(H, k):
    """Errors are bounded the way LAPACK's own are: eps ||H|| absolute for the values and
    eps ||H|| / gap for the vectors, with eps = 2^-48 (double-float) times a small factor."""
    m = H.shape[1]
    sigma, vs, sweeps = gdmr.hessenberg_svd(H, k, with_sweeps=True)
    U, s, Vh = np.linalg.svd(H)
    V = Vh.conj().T
    err = np.abs(sigma - s)
    print("m", m, "k", k, "sweeps", sweeps, "sigma err flagged", err[m - k:].max(), "others", err[:m - k].max(),
          "at", int(np.argmax(err[:m - k])))
    assert np.all(np.diff(sigma) <= 0)
    assert np.all(np.abs(sigma[m - k:] - s[m - k:]) <= 1e-13 * s[0] + 1e-12 * s[m - k:])
    assert np.all(err <= 2 * m * 6e-8 * s[0])             # the others: FP32-refined
    assert sweeps[1] < 24                                  # the polish converged
    # orthonormal to double-float rounding, which grows with the rotations each column takes
    assert np.linalg.norm(vs.conj().T @ vs - np.eye(k)) < 1e-13 * m
    for t in range(k):
        j = m - k + t
        c = V.conj().T @ vs[:, t]       # component outside LAPACK's vector, phase-free
        c[j] = 0
        gap = np.min(np.abs(np.delete(s, j) - s[j])) / s[0]
        assert np.linalg.norm(c) < max(1e-12, 1e-13 / gap), (t, np.linalg.norm(c), gap)


@pytest.mark.parametrize("restarts", [0, 5])
def test_helmholtz_arnoldi_hessenberg(restarts):
    _check(_arnoldi_h(40, restarts), 10)


@pytest.mark.parametrize("m,k", [(40, 10), (64, 20), (96, 24)])
def test_graded_random(m, k):
    _check(_graded(m, 7 + m, decades=6.0), k)


def test_near_degenerate_pair_at_the_boundary():
    # the 10th and 11th smallest values differ by 1e-6 relative: the flagged block still
    # has to come out right, the two vectors only up to their mixing
    m, k = 40, 10
    H = _graded(m, 3, decades=4.0, gap=k)
    sigma, vs = gdmr.hessenberg_svd(H, k)
    U, s, Vh = np.linalg.svd(H)
    V = Vh.conj().T
    assert np.all(np.abs(sigma - s) <= 2 * m * 6e-8 * s[0])
    assert np.linalg.norm(vs.conj().T @ vs - np.eye(k)) < 1e-12
    # the span of the nine well-separated smallest vectors is exact, to 1e-13 ||H|| / gap
    P = V[:, m - k + 1:]
    gap = (s[m - k] - s[m - k + 1]) / s[0]
    for t in range(1, k):
        assert np.linalg.norm(vs[:, t] - P @ (P.conj().T @ vs[:, t])) < 1e-13 / gap


@pytest.mark.parametrize("m", [40, 96])
def test_non_finite_hessenberg_returns_without_fault(m):
    # a Hessenberg holding a NaN (an inner cycle that overflowed) must give NaN singular values
    # and in-range output, not an out-of-range gather: the ranking keeps NaN in a total order
    # and every output slot written; the next call on a finite matrix is still right
    k = 10
    H = _graded(m, 5, decades=3.0)
    H[3, 2] = np.nan
    sigma, vs = gdmr.hessenberg_svd(H, k)
    assert sigma.shape == (m,) and vs.shape == (m, k)
    assert np.isnan(sigma).any()
    _check(_graded(m, 7 + m, decades=6.0), k if m == 40 else 24)


def test_rejects_bad_sizes():
    with pytest.raises(gdmr.GDMRError):
        gdmr.hessenberg_svd(np.zeros((162, 161), complex), 4)
    with pytest.raises(ValueError):
        gdmr.hessenberg_svd(np.zeros((5, 5), complex), 2)
