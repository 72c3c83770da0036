"""Full-size checks through size-independent properties.

The 128^3 drifting-sequence configuration (n = 2,097,152, 14.6M non-zeros, kappa 30,
damping 0.1, m = 60, k = 20) is too large for the oracle to run here in seconds, so these
tests check what does not depend on size:
  * every batched mixed-precision solve reaches the requested 1e-10 on the true FP64
    residual, as certified on the GPU and recomputed independently on the host (SciPy);
  * a right-hand side gives the same solution (to 1e-8 relative) solved alone and inside a
    batch that shares the recycled deflation space.
"""
import numpy as np
import pytest

import gdmr
import problems

pytestmark = pytest.mark.gpu

NRHS = 4


@pytest.fixture(scope="module")
def c2():
    A, seq, cfg = problems.config_3d128()
    return A, np.array(seq(NRHS)), cfg


def _host_rel(As, b, x):
    return float(np.linalg.norm(b - As @ x) / np.linalg.norm(b))


def test_c2_batched_mixed_reaches_fp64_tolerance(c2):
    A, B, cfg = c2
    s = gdmr.System(A, cfg["m"], cfg["k"], capacity=NRHS, precision="mixed")
    X, stats = s.solve_batch(B, tol=1e-10, max_cycles=3000)
    As = A.to_scipy()
    for i, st in enumerate(stats):
        assert st["status"] == 0, (i, st)
        assert st["true_rel_res"] <= 1e-10, (i, st)
        assert _host_rel(As, B[i], X[i]) <= 1.05e-10, i
    # alone vs in the batch: one right-hand side again, with a fresh deflation space
    alone = gdmr.System(A, cfg["m"], cfg["k"], capacity=1, precision="mixed")
    Xa, sa = alone.solve_batch(B[2:3], tol=1e-10, max_cycles=3000)
    assert sa[0]["status"] == 0
    assert float(np.linalg.norm(Xa[0] - X[2]) / np.linalg.norm(X[2])) < 1e-8
