"""The fused Krylov loop of one small system (k_krylov_small, one cooperative launch a cycle)
against the step-by-step kernels.

On the 64 x 64 Helmholtz sequence (m = 40, k = 10, tol 1e-10), complex128 and fp64e, with and
without CUDA graphs.  Every solve of the sequence starts both forms from the same state: the
first from none, each later one from the step-by-step engine's recycled deflation space,
imported into the fused engine.  (Left to recycle their own spaces, the two forms drift apart:
each space is built from residual directions that carry rounding of order eps / 1e-10, and in
fp64e's 48-bit arithmetic that moved one later solve 15 cycles.)  The first solve must end
within one restart cycle of the step-by-step path with the solution within 1e-9.  A later solve
updates its deflation space every cycle for some 95 cycles, each update built from the last, so
the two reduction orders' rounding grows along the solve: in complex128 the counts still agree
within one cycle, in fp64e (2^-48 against 2^-53) they agree within 2 + 5% (measured 94 against 98).
Every solve meets the true FP64 residual and the direct solution to 1e-8; repeated fused solves
are bitwise identical (fixed-order reductions); and no bounded grid-barrier wait ran out.
"""
import numpy as np
import pytest

import gdmr
import problems

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def c1():
    import scipy.sparse.linalg as spl
    A, rhs, cfg = problems.config_2d64()
    lu = spl.splu(A.to_scipy().tocsc())
    return A, rhs[:3], cfg, [lu.solve(b) for b in rhs[:3]]


def _sequence(A, rhs, cfg, precision, fused, graphs):
    s = gdmr.System(A, cfg["m"], cfg["k"], capacity=1, precision=precision)
    s.set_fused(fused)
    s.set_graphs(graphs)
    out = [s.solve(b, mode=0 if i == 0 else 1, tol=1e-10, mat_rank=2000) for i, b in enumerate(rhs)]
    s.close()
    return out


@pytest.mark.parametrize("graphs", [False, True])
@pytest.mark.parametrize("precision", ["fp64", "fp64e"])
def test_fused_matches_step_by_step(c1, precision, graphs):
    timeouts0 = gdmr.async_timeouts()    # process-wide counter: only this test's waits count
    A, rhs, cfg, direct = c1
    ref = gdmr.System(A, cfg["m"], cfg["k"], capacity=1, precision=precision)
    fus = gdmr.System(A, cfg["m"], cfg["k"], capacity=1, precision=precision)
    ref.set_fused(False)
    fus.set_fused(True)
    for s in (ref, fus):
        s.set_graphs(graphs)
    for i, b in enumerate(rhs):
        if i > 0:
            fus.import_deflation(ref.export_deflation())      # the same recycled space for both
        xr, sr = ref.solve(b, mode=0 if i == 0 else 1, tol=1e-10, mat_rank=2000)
        xf, sf = fus.solve(b, mode=0 if i == 0 else 1, tol=1e-10, mat_rank=2000)
        assert sf["status"] == 0 and sf["true_rel_res"] <= 2e-10, (i, sf)
        slack = 1 if i == 0 or precision == "fp64" else 2 + sr["cycles"] // 20
        assert abs(sf["cycles"] - sr["cycles"]) <= slack, (i, sr["cycles"], sf["cycles"])
        if slack == 1:
            assert np.linalg.norm(xf - xr) / np.linalg.norm(xr) < 1e-9, i
        assert np.linalg.norm(xf - direct[i]) / np.linalg.norm(direct[i]) < 1e-8
    ref.close()
    fus.close()
    assert gdmr.async_timeouts() == timeouts0


def test_fused_is_deterministic(c1):
    A, rhs, cfg, _ = c1
    a = _sequence(A, rhs[:2], cfg, "fp64", True, True)
    b = _sequence(A, rhs[:2], cfg, "fp64", True, True)
    for (xa, sa), (xb, sb) in zip(a, b):
        assert sa["cycles"] == sb["cycles"]
        assert np.array_equal(xa, xb)


@pytest.mark.parametrize("precision", ["fp64", "fp64e"])
def test_breakdown_after_a_full_cycle_clears_the_rest_of_the_basis(precision):
    """A breakdown leaves v_j and the rest of the basis zero (gDMR.cu:2256-2289), also in an
    engine whose basis still holds the previous solve's vectors: the cycle-end projection
    g = [W V]^H r and the identity-tail least squares read all of it.  A diagonal operator with
    distinct values; the first right-hand side fills the whole basis, the second lives on six
    eigenvalues and breaks down at step 6 of 8 in its first cycle."""
    import scipy.sparse as sp
    from problems import CSR
    n, m, k = 512, 8, 2
    lam = np.array([0.4, 3 + 1j, -0.6 + 0.5j, 4 - 1j, 1.5 + 2j, -2 - 1j])
    d = np.where(np.arange(n) < n // 2, lam[np.arange(n) % 6], 1.0 + 0.002 * np.arange(n) + 0.3j)
    S = sp.diags([d], [0], format="csr")
    A = CSR(n, S.indptr.astype(np.int32), S.indices.astype(np.int32), S.data.astype(np.complex128))
    b1 = problems.unit_gaussian_rhs(n, 21)
    b2 = problems.unit_gaussian_rhs(n, 22)
    b2[n // 2:] = 0
    out = {}
    for fused in (True, False):
        s = gdmr.System(A, m, k, capacity=1, precision=precision)
        s.set_fused(fused)
        s.solve(b1, mode=0, tol=1e-10, mat_rank=300)
        x, st = s.solve(b2, mode=0, tol=1e-10, mat_rank=300)
        hist = gdmr.last_history()
        assert hist[0]["breakdown"] == 6 and st["status"] == 0
        out[fused] = x
        s.close()
    exact = b2 / d
    for fused, x in out.items():
        assert np.linalg.norm(x - exact) / np.linalg.norm(exact) < 1e-9, fused
