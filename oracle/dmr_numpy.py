"""Numpy restatement of the reference DMR iteration (test infrastructure only).

This is the oracle's second, independent restatement, written with numpy and
LAPACK (QR and SVD through numpy.linalg).  The tests use it to cross-check the
C++ oracle (dmr_oracle.cpp) cycle by cycle; the product never imports it.

Parity status: unpinned.  The reference (seanMolesky/gDMR-solver) ships no
tests, fixtures or golden vectors, and its only implementation is CUDA, which
cannot run in a container without a GPU.  What pins this file instead is a
sparse direct solve (SciPy SuperLU) of the same systems and the invariants of
the iteration (orthonormal bases, the Arnoldi relation A[Z V] = [W V] H).

The iteration follows gDMR.cu step for step (one device, natural Krylov order):

* solverDMR         gDMR.cu:2638-2900  outer loop, runaway/cycle-cap tests,
                                       returned relative residual, numIts = cycles-1
* arnoldiSetupDMR   gDMR.cu:2586-2632  restart vector (residual, or the stored
                                       Krylov vector (m-k)/2 after stagnation)
* arnoldiDMR        gDMR.cu:1790-2332  deflation loop (A z_i -> W, H[:, :k]),
                                       CGS1 Krylov loop, absolute breakdown test
* deflatorDMR       gDMR.cu:1710-1787  w -= W W^H w (coefficients into H[:k])
* updateTrgCoeffsDMR gDMR.cu:2334-2408 g = [W V]^H r
* updateAppResDMR   gDMR.cu:2411-2582  y = argmin ||H y - g||, r -= [W V] H y,
                                       0.995 stagnation flag, x += rho [Z V] y
* genDeflatDMR      gDMR.cu:1583-1704  Z <- [Z V] (right singular vectors of the
                                       k smallest singular values), normalised
* innerProdKerDMR   gDMR.cu:268-326    <a, b> = sum conj(a_i) b_i
"""
from __future__ import annotations

import numpy as np


class DMRNumpy:
    """One solver instance: the state that outlives a solve (Z, the stagnation counter,
    the last basis) lives here, as the reference keeps it in globals (gDMR.cu:18-96)."""

    def __init__(self, n: int, m: int, k: int, matvec, dtype=np.complex128, compat_eye: bool = True):
        if m - k < 2:
            raise ValueError("basisDim - deflatDim must be >= 2 (gDMR.cu:856-860)")
        self.n, self.m, self.k = n, m, k
        self.matvec = matvec
        self.dtype = np.dtype(dtype)
        self.rdtype = np.float64 if self.dtype == np.complex128 else np.float32
        self.compat_eye = compat_eye
        self.Z = np.zeros((k, n), dtype=self.dtype)        # defBasisDMR
        self.basis = np.zeros((m + 1, n), dtype=self.dtype)  # itrBasisDMR: [W | V]
        self.flag_count = 0                                   # kryFlagCountDMR (never reset by a solve)
        self.loop_flag = 0
        self.cycle_log = []

    # -- building blocks -------------------------------------------------
    def _norm(self, v):
        return self.rdtype(np.sqrt(np.vdot(v, v).real))

    def _arnoldi(self, kk: int, tol: float):
        m, n = self.m, self.n
        H = np.zeros((m + 1, m), dtype=self.dtype)
        B = self.basis
        # deflation loop, gDMR.cu:1823-2030
        for i in range(kk):
            w = self.matvec(self.Z[i].copy())
            w_orig = w.copy()
            if i > 0:
                c = B[:i].conj() @ w
                w = w - c @ B[:i]
                H[:i, i] = c
            w = w / self._norm(w)
            B[i] = w
            H[i, i] = np.vdot(w, w_orig)
        # orthogonalise the starting vector against W, gDMR.cu:2033-2059
        if kk > 0:
            v0 = B[kk]
            c = B[:kk].conj() @ v0
            v0 = v0 - c @ B[:kk]
            B[kk] = v0 / self._norm(v0)
        # Krylov loop, gDMR.cu:2069-2328
        steps = m - kk
        broke = None
        for j in range(1, steps + 1):
            w = self.matvec(B[kk + j - 1].copy())
            w_orig = w.copy()
            col = kk + j - 1
            if kk > 0:
                c = B[:kk].conj() @ w
                H[:kk, col] = c
                w = w - c @ B[:kk]
            V = B[kk:kk + j]
            c = V.conj() @ w
            w = w - c @ V
            H[kk:kk + j, col] = c
            nrm = self._norm(w)
            if nrm < tol:
                # breakdown, gDMR.cu:2256-2289: zero the remaining basis and give H
                # an identity tail; the reference starts the tail at column j,
                # which overwrites valid diagonals when kk > 0 (kept as compat)
                B[kk + j:] = 0
                start = j if self.compat_eye else kk + j
                for cc in range(start, m):
                    H[cc, cc] = 1.0
                broke = j
                break
            v = w / nrm
            B[kk + j] = v
            H[kk + j, col] = np.vdot(v, w_orig)
        return H, broke

    def _svd_smallest(self, H):
        # gesvdj order: singular values descending; columns m-k..m-1 of V
        _, s, Vh = np.linalg.svd(H.astype(np.complex128), full_matrices=True)
        V = Vh.conj().T
        return V[:, self.m - self.k:self.m].astype(self.dtype), s

    # -- one solve -------------------------------------------------------
    def solve(self, b, x0, mode: int, tol: float, mat_rank: int):
        m, k = self.m, self.k
        rd = self.rdtype
        self.cycle_log = []
        self.loop_flag = 0
        b = np.asarray(b, dtype=self.dtype)
        x = np.asarray(x0, dtype=self.dtype).copy()
        bnorm = self._norm(b)
        r = b - self.matvec(x.copy())
        rho_abs = self._norm(r)
        if rho_abs < bnorm * tol:
            return dict(x=x, ret=float(rho_abs), its=mat_rank * mat_rank, cycles=0, status="initial")
        r = r / rho_abs
        cycle = 0
        first_def = 0 if mode == 0 else k
        status = "converged"
        while rho_abs > rd(tol) * bnorm:
            if cycle > mat_rank:
                return dict(x=x, ret=float(rho_abs / bnorm), its=cycle, cycles=cycle, status="maxcycles")
            if rho_abs / bnorm > 1.0:
                return dict(x=x, ret=float(rho_abs / bnorm), its=cycle, cycles=cycle, status="runaway")
            kk = 0 if (cycle == 0 and first_def == 0) else k
            # restart vector, gDMR.cu:2600-2621
            period = (2 * mat_rank) // (m - k)
            if self.loop_flag == 0 or (period != 0 and self.flag_count % period == 0):
                self.basis[kk] = r
            else:
                self.basis[kk] = self.basis[kk + (m - k) // 2].copy()
            H, broke = self._arnoldi(kk, tol)
            B = self.basis
            g = B.conj() @ r                                   # gDMR.cu:2334-2408
            Hq = H.astype(np.complex128)
            y = np.linalg.lstsq(Hq, g.astype(np.complex128), rcond=None)[0]
            t = (Hq @ y).astype(self.dtype)
            y = y.astype(self.dtype)
            r = r - t @ B                                      # gDMR.cu:2470-2482
            rho = self._norm(r)
            if rho > 0.995:                                    # gDMR.cu:2506-2514
                self.loop_flag = 1
                self.flag_count += 1
            else:
                self.loop_flag = 0
            r = r / rho
            S = np.concatenate([self.Z[:kk], B[kk:m]]) if kk > 0 else B[:m]
            x = x + (y @ S) * rho_abs                          # gDMR.cu:2557-2571
            rho_abs = rd(rho * rho_abs)
            if k > 0:                                          # gDMR.cu:2853-2871
                Vs, _ = self._svd_smallest(H)
                Znew = Vs.T @ S
                nz = np.sqrt(np.einsum("ij,ij->i", Znew.conj(), Znew).real)
                self.Z = (Znew / nz[:, None]).astype(self.dtype)
            self.cycle_log.append(dict(kk=kk, rho=float(rho), rho_abs=float(rho_abs), broke=broke))
            cycle += 1
        return dict(x=x, ret=float(rho_abs / bnorm), its=cycle - 1, cycles=cycle, status=status)
