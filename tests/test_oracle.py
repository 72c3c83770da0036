"""The host oracle (oracle/dmr_oracle.cpp) against the golden fixtures, LAPACK
and a sparse direct solve.  CPU only."""
import os

import numpy as np
import pytest

import problems
from problems import CSR

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def _load(name):
    d = np.load(os.path.join(GOLDEN, name))
    A = CSR(int(d["indptr"].size - 1), d["indptr"], d["indices"], d["data"])
    return A, d


def test_ls_matches_lapack(oracle_mod):
    rng = np.random.default_rng(0)
    for rows, cols in ((5, 4), (41, 40), (61, 60)):
        H = rng.standard_normal((rows, cols)) + 1j * rng.standard_normal((rows, cols))
        g = rng.standard_normal(rows) + 1j * rng.standard_normal(rows)
        y = oracle_mod.ls(H, g)
        y_ref = np.linalg.lstsq(H, g, rcond=None)[0]
        assert np.allclose(y, y_ref, rtol=1e-12, atol=1e-12)


def test_svd_matches_lapack(oracle_mod):
    rng = np.random.default_rng(1)
    H = rng.standard_normal((49, 48)) + 1j * rng.standard_normal((49, 48))
    s, V = oracle_mod.svd(H)
    assert np.allclose(s, np.linalg.svd(H, compute_uv=False), rtol=1e-12)
    assert np.allclose(V.conj().T @ V, np.eye(48), atol=1e-12)
    # right singular vectors: ||H v_i|| = sigma_i, descending
    assert np.allclose(np.linalg.norm(H @ V, axis=0), s, rtol=1e-10)
    assert np.all(np.diff(s) <= 0)


@pytest.mark.parametrize("fuse", [False, True])
def test_oracle_matches_golden_sequence(oracle_mod, fuse):
    A, d = _load("helmholtz10.npz")
    o = oracle_mod.Oracle(A, int(d["m"]), int(d["k"]), fuse_deflation=fuse, threads=1)
    for i in range(int(d["nrhs"])):
        r = o.solve(d[f"b{i}"], mode=0 if i == 0 else 1, tol=float(d["tol"]), mat_rank=int(d["mat_rank"]))
        assert r["status"] == 0
        assert abs(r["cycles"] - int(d[f"cycles{i}"])) <= 2
        if i == 0:
            # the first solve tracks the golden run cycle by cycle; later solves start from a
            # recycled space built from residual directions that carry rounding of order
            # eps / (relative residual), so only their cycle counts and solutions are compared
            # cycle c works on a residual direction accurate to about eps / ||r_c||/||b||
            rel_before = np.concatenate([[1.0], np.cumprod(d[f"rho{i}"])[:-1]])
            assert np.all(np.abs(r["rho"] - d[f"rho{i}"]) <= 1e-12 / rel_before + 1e-12)
        x_ref = d[f"x{i}"]
        assert np.linalg.norm(r["x"] - x_ref) / np.linalg.norm(x_ref) < 1e-9
        xd = d[f"direct{i}"]
        assert np.linalg.norm(r["x"] - xd) / np.linalg.norm(xd) < 1e-8


def test_oracle_breakdown_identity_tail(oracle_mod):
    A, d = _load("breakdown30.npz")
    o = oracle_mod.Oracle(A, int(d["m"]), int(d["k"]), threads=1)
    r = o.solve(d["b0"], mode=0, tol=float(d["tol"]), mat_rank=int(d["mat_rank"]))
    assert r["status"] == 0 and r["cycles"] == int(d["cycles0"]) == 1
    assert np.linalg.norm(r["x"] - d["direct0"]) / np.linalg.norm(d["direct0"]) < 1e-12


def test_oracle_2d64_first_rhs_matches_direct(oracle_mod):
    import scipy.sparse.linalg as spl
    A, rhs, cfg = problems.config_2d64()
    o = oracle_mod.Oracle(A, cfg["m"], cfg["k"])
    r = o.solve(rhs[0], mode=0, tol=1e-13, mat_rank=2000)
    assert r["status"] == 0
    xd = spl.splu(A.to_scipy().tocsc()).solve(rhs[0])
    assert np.linalg.norm(r["x"] - xd) / np.linalg.norm(xd) < 1e-11
    true = np.linalg.norm(rhs[0] - A.to_scipy() @ r["x"]) / np.linalg.norm(rhs[0])
    assert true < 1e-12   # the recursive residual drifts from the true one near 1e-13


def test_oracle_complex64_emulation_converges(oracle_mod):
    A, rhs, cfg = problems.config_2d64()
    o = oracle_mod.Oracle(A, cfg["m"], cfg["k"], precision="c64")
    r = o.solve(rhs[0], mode=0, tol=1e-5, mat_rank=2000)
    assert r["status"] == 0 and r["ret"] < 1e-5
    true = np.linalg.norm(rhs[0] - A.to_scipy() @ r["x"]) / np.linalg.norm(rhs[0])
    assert true < 1e-3   # complex64 recursion: the true residual trails the recursive one


def test_oracle_rejects_bad_sizes(oracle_mod):
    A, rhs, cfg = problems.config_2d64()
    with pytest.raises(ValueError):
        oracle_mod.Oracle(A, 10, 9)


def test_oracle_deflation_roundtrip(oracle_mod):
    A, d = _load("helmholtz10.npz")
    o = oracle_mod.Oracle(A, 12, 4, threads=1)
    o.solve(d["b0"], mode=0, tol=1e-10, mat_rank=500)
    Z = o.get_Z()
    assert np.allclose(np.linalg.norm(Z, axis=1), 1.0)
    o2 = oracle_mod.Oracle(A, 12, 4, threads=1)
    o2.set_Z(Z)
    r1 = o.solve(d["b1"], mode=1, tol=1e-10, mat_rank=500)
    r2 = o2.solve(d["b1"], mode=1, tol=1e-10, mat_rank=500)
    assert r1["cycles"] == r2["cycles"]
    assert np.allclose(r1["x"], r2["x"], rtol=0, atol=1e-12)
