"""gdmr_true_residual_noalloc through the C ABI.

The allocation-free residual check exists for callers that cannot call cudaMalloc: hosts
whose own allocator owns the device-memory pool (a library allocation would fail or fragment
it) and latency-critical loops (an allocation can synchronise the device).  It must give what the allocating entry point gdmr_true_residual gives, on two calls
in a row (the static scratch keeps state between calls), and refuse sizes beyond its static
scratch.  This file is collected last so a stop-at-first-failure run has already run
everything else; it also passes alone in a fresh process.
"""
import numpy as np
import pytest

import gdmr
import problems

pytestmark = pytest.mark.gpu


def test_noalloc_residual_matches_allocating_entry_point():
    import torch
    A, rhs, cfg = problems.config_2d64()
    sys_ = gdmr.System(A, cfg["m"], cfg["k"], capacity=4, precision="fp64")
    B = np.array(rhs[:3])
    Xs, _ = sys_.solve_batch(B, tol=1e-10, max_cycles=2000)       # converged solutions
    rng = np.random.default_rng(3)
    Xr = Xs + 1e-3 * (rng.standard_normal(Xs.shape) + 1j * rng.standard_normal(Xs.shape))
    for X in (Xs, Xr, np.zeros_like(Xs)):
        expected = sys_.true_residual(B, X)                       # allocating entry point
        Bd = torch.from_numpy(np.ascontiguousarray(B)).cuda()
        Xd = torch.from_numpy(np.ascontiguousarray(X)).cuda()
        stream = torch.cuda.current_stream().cuda_stream
        for call in range(2):                                     # two calls in a row
            out = torch.full((B.shape[0],), -1.0, dtype=torch.float64, device="cuda")
            sys_.true_residual_noalloc(Bd.data_ptr(), Xd.data_ptr(), out.data_ptr(), B.shape[0], stream)
            torch.cuda.synchronize()
            got = out.cpu().numpy()
            assert np.allclose(got, expected, rtol=1e-12, atol=0), (call, got, expected)
    # ||b - A 0|| / ||b|| is exactly 1 in both
    assert np.allclose(expected, 1.0, rtol=1e-15)


def test_noalloc_rejects_more_rhs_than_its_scratch():
    A, rhs, cfg = problems.config_2d64()
    sys_ = gdmr.System(A, cfg["m"], cfg["k"], capacity=1, precision="fp64")
    with pytest.raises(gdmr.GDMRError) as e:
        sys_.true_residual_noalloc(1, 1, 1, 65)                   # rejected before any launch
    assert e.value.status == 1 and "64" in str(e.value)
