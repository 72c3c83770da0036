"""The fused Krylov loop of one small system (k_krylov_small, one cooperative launch a cycle)
against the step-by-step kernels.

On the 64 x 64 Helmholtz sequence (m = 40, k = 10, tol 1e-10), complex128 and fp64e, with and
without CUDA graphs: the first solve ends within one restart cycle of the step-by-step path
with the solution within 1e-9; later solves of the recycled sequence within 2 + 10% cycles
(the slack of the oracle parity tests); every solve meets the true FP64 residual; repeated
fused solves are bitwise identical (fixed-order reductions); and no bounded grid-barrier wait
ran out.
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
    ref = _sequence(A, rhs, cfg, precision, False, graphs)
    fus = _sequence(A, rhs, cfg, precision, True, graphs)
    for i, ((xr, sr), (xf, sf)) in enumerate(zip(ref, fus)):
        assert sf["status"] == 0 and sf["true_rel_res"] <= 2e-10, (i, sf)
        slack = 1 if i == 0 else 2 + sr["cycles"] // 10
        assert abs(sf["cycles"] - sr["cycles"]) <= slack, (i, sr["cycles"], sf["cycles"])
        if i == 0:
            assert np.linalg.norm(xf - xr) / np.linalg.norm(xr) < 1e-9
        assert np.linalg.norm(xf - direct[i]) / np.linalg.norm(direct[i]) < 1e-8
    assert gdmr.async_timeouts() == timeouts0


def test_fused_is_deterministic(c1):
    A, rhs, cfg, _ = c1
    a = _sequence(A, rhs[:2], cfg, "fp64", True, True)
    b = _sequence(A, rhs[:2], cfg, "fp64", True, True)
    for (xa, sa), (xb, sb) in zip(a, b):
        assert sa["cycles"] == sb["cycles"]
        assert np.array_equal(xa, xb)
