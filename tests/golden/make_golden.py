"""Generates the golden fixtures in tests/golden/ (committed; rerun only on purpose).

The reference (seanMolesky/gDMR-solver) ships no tests, fixtures or golden
vectors, and its CUDA implementation cannot run without a GPU, so the fixtures
are produced by the numpy restatement of its algorithm (oracle/dmr_numpy.py)
and by SciPy's SuperLU direct solver.  The C++ oracle and the GPU library are
then checked against them.

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "gdmr-solver_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import problems  # noqa: E402
from dmr_numpy import DMRNumpy  # noqa: E402


def run_sequence(A, rhs, m, k, tol, mat_rank, compat_eye=True):
    import scipy.sparse.linalg as spl
    S = A.to_scipy()
    solver = DMRNumpy(A.n, m, k, lambda v: S @ v, compat_eye=compat_eye)
    lu = spl.splu(S.tocsc())
    out = {}
    for i, b in enumerate(rhs):
        res = solver.solve(b, np.zeros(A.n, np.complex128), 0 if i == 0 else 1, tol, mat_rank)
        out[f"x{i}"] = res["x"]
        out[f"ret{i}"] = np.float64(res["ret"])
        out[f"its{i}"] = np.int64(res["its"])
        out[f"cycles{i}"] = np.int64(res["cycles"])
        out[f"rho{i}"] = np.array([c["rho"] for c in solver.cycle_log])
        out[f"broke{i}"] = np.array([c["broke"] or 0 for c in solver.cycle_log])
        out[f"direct{i}"] = lu.solve(b)
        out[f"b{i}"] = b
    return out


def main():
    # 1. 2D Helmholtz 10x10, kappa 8, damping 0.05, m 12, k 4, three RHS with recycling
    A = problems.helmholtz((10, 10), 8.0, 0.05)
    rhs = [problems.unit_gaussian_rhs(A.n, s) for s in (1, 2, 3)]
    d = run_sequence(A, rhs, 12, 4, 1e-10, 500)
    np.savez_compressed(os.path.join(HERE, "helmholtz10.npz"), indptr=A.indptr, indices=A.indices, data=A.data,
                        m=12, k=4, tol=1e-10, mat_rank=500, nrhs=3, **d)
    # 2. breakdown: diagonal operator with three distinct eigenvalues, the Krylov space is invariant
    n = 30
    diag = np.array([0.1, 0.2, 0.3] * 10, dtype=np.complex128) * (1 + 0.1j)
    from problems import CSR
    B = CSR(n, np.arange(n + 1, dtype=np.int32), np.arange(n, dtype=np.int32), diag)
    rhs2 = [problems.unit_gaussian_rhs(n, 7)]
    d2 = run_sequence(B, rhs2, 8, 2, 1e-10, 50)
    np.savez_compressed(os.path.join(HERE, "breakdown30.npz"), indptr=B.indptr, indices=B.indices, data=B.data,
                        m=8, k=2, tol=1e-10, mat_rank=50, nrhs=1, **d2)
    # 3. SplitMix64 / Box-Muller stream of the generator (first outputs of two seeds)
    np.savez_compressed(os.path.join(HERE, "rng.npz"), sm0=problems.splitmix64(0, 8),
                        sm12345=problems.splitmix64(12345, 8), g7=problems.complex_gaussian(7, 6))
    print("wrote", sorted(os.listdir(HERE)))


if __name__ == "__main__":
    main()
