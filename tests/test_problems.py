"""Synthetic workload generators (CPU)."""
import os

import numpy as np
import pytest

import problems

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def _splitmix_scalar(seed, count):
    out, state = [], seed & (2**64 - 1)
    for _ in range(count):
        state = (state + 0x9E3779B97F4A7C15) & (2**64 - 1)
        z = state
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & (2**64 - 1)
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & (2**64 - 1)
        out.append(z ^ (z >> 31))
    return out


def test_splitmix_matches_scalar_definition():
    for seed in (0, 1, 12345, 2**63 + 7):
        assert [int(v) for v in problems.splitmix64(seed, 16)] == _splitmix_scalar(seed, 16)


def test_rng_stream_is_pinned():
    d = np.load(os.path.join(GOLDEN, "rng.npz"))
    assert np.array_equal(problems.splitmix64(0, 8), d["sm0"])
    assert np.array_equal(problems.splitmix64(12345, 8), d["sm12345"])
    assert np.array_equal(problems.complex_gaussian(7, 6), d["g7"])


def test_complex_gaussian_moments():
    g = problems.complex_gaussian(3, 200000)
    assert abs(np.mean(g.real)) < 0.01 and abs(np.mean(g.imag)) < 0.01
    assert abs(np.var(g.real) - 0.5) < 0.01 and abs(np.var(g.imag) - 0.5) < 0.01


def test_helmholtz_2d64_shape_and_values():
    A = problems.helmholtz((64, 64), 20.0, 0.05)
    assert A.n == 4096 and A.nnz == 20224
    S = A.to_scipy()
    assert np.isclose(S[0, 0], 4 * 65**2 - 400 * (1 + 0.05j))
    assert S[0, 1] == -65**2 and S[0, 64] == -65**2 and S[0, 2] == 0
    assert (S - S.T).nnz == 0          # complex symmetric


def test_helmholtz_3d_counts():
    A = problems.helmholtz((16, 12, 10), 5.0, 0.1)
    n = 16 * 12 * 10
    assert A.n == n
    # 7-point stencil with dropped Dirichlet neighbours
    assert A.nnz == n + 2 * (15 * 12 * 10 + 16 * 11 * 10 + 16 * 12 * 9)
    assert np.isclose(A.to_scipy()[0, 0], 2 * (17**2 + 13**2 + 11**2) - 25 * (1 + 0.1j))


def test_variable_helmholtz_row_sums():
    A = problems.variable_helmholtz((16, 9, 8), 4.0, 0.1, seed=5)
    S = A.to_scipy()
    assert S.shape == (16 * 9 * 8,) * 2
    # interior rows: off-diagonals sum to -(diag + kappa^2 (1+0.1i)) only at the boundary; symmetric
    assert abs(S - S.T).max() < 1e-9


def test_gaussian_source_noise_level():
    s = problems.gaussian_source_rhs((24, 24, 24), 101)
    assert s.shape == (24**3,)
    assert np.abs(s).max() > 0.5


def _stencil_apply(shape, coef, x):
    """y = d x + w_axis (x[-1] + x[+1]) along every axis, Dirichlet (the k_stencil formula)."""
    d, wx, wy, wz = coef
    X = x.reshape(tuple(reversed(shape)))          # numbering i + nx (j + ny l): x fastest
    Y = d * X
    for axis, w in zip(range(X.ndim - 1, -1, -1), (wx, wy, wz)):
        sl_lo = [slice(None)] * X.ndim
        sl_hi = [slice(None)] * X.ndim
        sl_lo[axis] = slice(0, -1)
        sl_hi[axis] = slice(1, None)
        Y[tuple(sl_lo)] += w * X[tuple(sl_hi)]
        Y[tuple(sl_hi)] += w * X[tuple(sl_lo)]
    return Y.reshape(-1)


@pytest.mark.parametrize("shape,kappa,damping", [((64, 64), 20.0, 0.05), ((7, 5, 6), 3.0, 0.1)])
def test_helmholtz_stencil_matches_csr(shape, kappa, damping):
    A = problems.helmholtz(shape, kappa, damping)
    coef = problems.helmholtz_stencil(shape, kappa, damping)
    x = problems.complex_gaussian(3, A.n)
    y_csr = A.to_scipy() @ x
    y_st = _stencil_apply(shape, coef, x)
    assert np.max(np.abs(y_csr - y_st)) <= 1e-12 * np.max(np.abs(y_csr))
