"""Parity of libgDMR's CUDA path with the oracle, through the C ABI.

Every test here runs the sm_103a kernels (SELL SpMV, fused Gram-Schmidt,
Givens least squares, Jacobi SVD, deflation update) via ctypes and compares
with the host oracle (oracle/dmr_oracle.cpp), the golden fixtures, or a
sparse direct solve.  Tolerances:
  * complex128 forms: same restart-cycle count as the oracle on a first solve
    (+-2 later in a recycled sequence, whose deflation space is sensitive to
    rounding), x within 1e-8 relative of the oracle, true FP64 residual
    <= 2x the requested tolerance;
  * complex64 (reference precision) forms: cycles +-2, x within 1e-3;
  * fp64e (the complex128 iteration in double-float arithmetic on the FP32
    pipes, about 48 significant bits): as complex128, with one cycle of slack
    on a first solve and 1e-11 on the breakdown fixture.
"""
import os

import numpy as np
import pytest

import gdmr
import problems
from problems import CSR

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def _golden(name):
    d = np.load(os.path.join(GOLDEN, name))
    return CSR(int(d["indptr"].size - 1), d["indptr"], d["indices"], d["data"]), d


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _true(A, b, x):
    return float(np.linalg.norm(b - A.to_scipy() @ x) / np.linalg.norm(b))


@pytest.fixture(scope="module")
def c1():
    import scipy.sparse.linalg as spl
    A, rhs, cfg = problems.config_2d64()
    lu = spl.splu(A.to_scipy().tocsc())
    return A, rhs, cfg, [lu.solve(b) for b in rhs]


# fp64e: the same iteration in double-float arithmetic (about 48 significant bits), so the
# first solve may end one cycle apart from the oracle; everything else holds as for fp64.
CYCLE_SLACK = {"fp64": 0, "fp64e": 1}


@pytest.mark.parametrize("precision", ["fp64", "fp64e"])
def test_fp64_first_solve_matches_oracle(c1, oracle_mod, precision):
    A, rhs, cfg, direct = c1
    sys_ = gdmr.System(A, cfg["m"], cfg["k"], capacity=1, precision=precision)
    x, st = sys_.solve(rhs[0], mode=0, tol=1e-10, mat_rank=2000)
    o = oracle_mod.Oracle(A, cfg["m"], cfg["k"], fuse_deflation=True)
    r = o.solve(rhs[0], mode=0, tol=1e-10, mat_rank=2000)
    assert st["status"] == 0
    assert abs(st["cycles"] - r["cycles"]) <= CYCLE_SLACK[precision]
    assert st["its"] == st["cycles"] - 1 and r["its"] == r["cycles"] - 1
    # the last cycle works near 1e-10, where the recursive residual carries rounding of
    # order eps / (relative residual): two correct implementations differ by ~1% there
    if st["cycles"] == r["cycles"]:
        assert abs(st["rel_res"] - r["ret"]) <= 5e-2 * r["ret"]
    assert _rel(x, r["x"]) < 1e-8
    assert st["true_rel_res"] <= 2e-10
    assert _true(A, rhs[0], x) <= 2e-10
    assert _rel(x, direct[0]) < 1e-8


@pytest.mark.parametrize("precision", ["fp64", "fp64e"])
def test_fp64_recycled_sequence(c1, oracle_mod, precision):
    A, rhs, cfg, direct = c1
    sys_ = gdmr.System(A, cfg["m"], cfg["k"], capacity=1, precision=precision)
    o = oracle_mod.Oracle(A, cfg["m"], cfg["k"], fuse_deflation=True)
    total_gpu = total_orc = 0
    for i, b in enumerate(rhs):
        x, st = sys_.solve(b, mode=0 if i == 0 else 1, tol=1e-10, mat_rank=2000)
        r = o.solve(b, mode=0 if i == 0 else 1, tol=1e-10, mat_rank=2000)
        assert st["status"] == 0
        assert abs(st["cycles"] - r["cycles"]) <= 2 + r["cycles"] // 10, (i, st["cycles"], r["cycles"])
        assert _true(A, b, x) <= 2e-10
        assert _rel(x, direct[i]) < 1e-8
        total_gpu += st["cycles"]
        total_orc += r["cycles"]
    assert abs(total_gpu - total_orc) <= 2 * len(rhs)


@pytest.mark.parametrize("precision", ["fp64", "fp64e"])
def test_fp64_golden_sequence(precision):
    A, d = _golden("helmholtz10.npz")
    sys_ = gdmr.System(A, int(d["m"]), int(d["k"]), capacity=1, precision=precision)
    for i in range(int(d["nrhs"])):
        x, st = sys_.solve(d[f"b{i}"], mode=0 if i == 0 else 1, tol=float(d["tol"]), mat_rank=int(d["mat_rank"]))
        assert st["status"] == 0
        assert abs(st["cycles"] - int(d[f"cycles{i}"])) <= 2
        assert _rel(x, d[f"x{i}"]) < 1e-9
        assert _rel(x, d[f"direct{i}"]) < 1e-8


@pytest.mark.parametrize("precision,xtol", [("fp64", 1e-12), ("fp64e", 1e-11)])
def test_fp64_breakdown_identity_tail(precision, xtol):
    A, d = _golden("breakdown30.npz")
    sys_ = gdmr.System(A, int(d["m"]), int(d["k"]), capacity=1, precision=precision)
    x, st = sys_.solve(d["b0"], mode=0, tol=float(d["tol"]), mat_rank=int(d["mat_rank"]))
    assert st["status"] == 0 and st["cycles"] == 1 and st["breakdowns"] == 1
    assert _rel(x, d["direct0"]) < xtol


def test_legacy_complex64_plugin_csr(c1, oracle_mod):
    """gDMRC.h in the reference's precision with a CSR operator (impCsrLS).

    The first solve (no deflation space yet) matches the oracle's cycle count within 2.  Later
    solves run on a recycled space built from complex64 residual directions, which carry
    rounding of order eps32 / tol = 6e-8 / 1e-5, about 6e-3 relative (1e-6 for the FP64 form
    at 1e-10); carried from solve to solve, the two implementations' spaces drift apart (one
    clean run: 27 cycles against the oracle's 33 on the third solve).  So each later solve starts
    the oracle from the library's own space (expSVDMR, then the oracle's set_Z), and the two
    agree on the cycle count within 2 + 10% and on x within 1e-3.
    """
    A, rhs, cfg, direct = c1
    ls = gdmr.LinearSystem(A.n, cfg["m"], cfg["k"], precision="c64")
    try:
        ls.imp_csr(A)
        o = oracle_mod.Oracle(A, cfg["m"], cfg["k"], precision="c64", fuse_deflation=True)
        for i, b in enumerate(rhs[:3]):
            if i > 0:
                o.set_Z(ls.exp_sv())      # the same recycled space for both
            ls.imp_img(b)
            ls.imp_src(np.zeros(A.n))
            ret, its = ls.solve(0 if i == 0 else 1, 1e-5, 2000)
            x = ls.exp_src()
            r = o.solve(b, mode=0 if i == 0 else 1, tol=1e-5, mat_rank=2000)
            assert ret < 1e-5
            assert abs(its - r["its"]) <= (2 if i == 0 else 2 + r["its"] // 10), (i, its, r["its"])
            assert _rel(x, direct[i]) < 1e-3
            assert _rel(x, r["x"]) < 1e-3
        Z = ls.exp_sv()
        assert Z.shape == (cfg["k"], A.n)
        assert np.allclose(np.linalg.norm(Z, axis=1), 1.0, atol=1e-4)
    finally:
        ls.close()


def _dense_tridiag(n):
    # indefinite (eigenvalues 0.5 - 2 cos t + 0.02i): a 127-vector cycle does not converge, so
    # the Krylov loop never runs on rounding noise (where the reference's sub-diagonal
    # <v_j, A v_{j-1}> breaks the Arnoldi relation and the recursion runs away)
    main = np.full(n, 0.5 + 0.02j, np.complex64)
    off = np.full(n - 1, -1.0 + 0.0j, np.complex64)
    return np.diag(main) + np.diag(off, 1) + np.diag(off, -1)


def test_legacy_complex64_plugin_dense_like_control_program(oracle_mod):
    """The reference control program's set-up: dense 1024 x 1024 operator,
    basis 127, no deflation, tolerance 1e-5, five right-hand sides."""
    n = 1024
    Ad = _dense_tridiag(n)
    import scipy.sparse as sp
    S = sp.csr_matrix(Ad.astype(np.complex128))
    A = CSR(n, S.indptr.astype(np.int32), S.indices.astype(np.int32), S.data)
    ls = gdmr.LinearSystem(n, 127, 0, precision="c64")
    try:
        ls.imp_opt(Ad)
        o = oracle_mod.Oracle(A, 127, 0, precision="c64", fuse_deflation=True)
        for i in range(5):
            b = problems.unit_gaussian_rhs(n, 40 + i)
            ls.imp_img(b)
            ls.imp_src(np.zeros(n))
            ret, its = ls.solve(i, 1e-5, n)
            x = ls.exp_src()
            r = o.solve(b, mode=i, tol=1e-5, mat_rank=n)
            assert ret < 1e-5
            assert abs(its - r["its"]) <= 2
            assert _rel(x, r["x"]) < 1e-3
        # linOptLS applies the dense operator in place
        v = problems.unit_gaussian_rhs(n, 99).astype(np.complex64)
        ls.imp_src(v)
        ls.lin_opt()
        assert _rel(ls.exp_src(), Ad @ v) < 1e-5
    finally:
        ls.close()


def test_legacy_complex128_plugin(c1, oracle_mod):
    A, rhs, cfg, direct = c1
    ls = gdmr.LinearSystem(A.n, cfg["m"], cfg["k"], precision="c128")
    try:
        ls.imp_csr(A)
        o = oracle_mod.Oracle(A, cfg["m"], cfg["k"], fuse_deflation=True)
        ls.imp_img(rhs[0])
        ls.imp_src(np.zeros(A.n))
        ret, its = ls.solve(0, 1e-10, 2000)
        x = ls.exp_src()
        r = o.solve(rhs[0], mode=0, tol=1e-10, mat_rank=2000)
        assert its == r["its"]
        assert _rel(x, r["x"]) < 1e-8
        assert _true(A, rhs[0], x) <= 2e-10
        assert gdmr.last_stats()["cycles"] == r["cycles"]
    finally:
        ls.close()


@pytest.mark.parametrize("precision", ["mixed", "fp64", "fp64e"])
def test_refined_batch_reaches_fp64_tolerance(c1, precision):
    A, rhs, cfg, direct = c1
    sys_ = gdmr.System(A, cfg["m"], cfg["k"], capacity=8, precision=precision)
    X, stats = sys_.solve_batch(np.array(rhs), tol=1e-10, max_cycles=2000)
    for i, st in enumerate(stats):
        assert st["status"] == 0, st
        assert st["true_rel_res"] <= 1e-10
        assert _true(A, rhs[i], X[i]) <= 1.5e-10
        assert _rel(X[i], direct[i]) < 1e-8
    rel = sys_.true_residual(np.array(rhs), X)
    assert np.all(rel <= 1.5e-10)


def test_batch_result_is_the_same_alone_and_in_the_mix(c1):
    """Continuous batching does not change answers beyond the tolerance: each
    right-hand side solved alone equals its solution inside a mixed batch."""
    A, rhs, cfg, direct = c1
    batch = gdmr.System(A, cfg["m"], cfg["k"], capacity=4, precision="mixed")
    Xb, _ = batch.solve_batch(np.array(rhs[:6]), tol=1e-10, max_cycles=2000)   # 6 > capacity: refills
    for i in (0, 3, 5):
        alone = gdmr.System(A, cfg["m"], cfg["k"], capacity=1, precision="mixed")
        Xa, st = alone.solve_batch(np.array(rhs[i:i + 1]), tol=1e-10, max_cycles=2000)
        assert st[0]["status"] == 0
        # both are within the tolerance of the exact solution, hence of each other
        assert _rel(Xa[0], Xb[i]) < 2e-8
        assert _rel(Xb[i], direct[i]) < 1e-8


def test_repeat_solves_are_bitwise_identical(c1):
    A, rhs, cfg, direct = c1
    xs = []
    for _ in range(2):
        s = gdmr.System(A, cfg["m"], cfg["k"], capacity=1, precision="fp64")
        x, st = s.solve(rhs[1], mode=0, tol=1e-10, mat_rank=2000)
        xs.append(x)
    assert np.array_equal(xs[0], xs[1])


def test_deflation_export_import_roundtrip(c1):
    A, rhs, cfg, direct = c1
    s1 = gdmr.System(A, cfg["m"], cfg["k"], capacity=1, precision="fp64")
    s1.solve(rhs[0], mode=0, tol=1e-10, mat_rank=2000)
    Z = s1.export_deflation()
    assert np.allclose(np.linalg.norm(Z, axis=1), 1.0)
    s2 = gdmr.System(A, cfg["m"], cfg["k"], capacity=1, precision="fp64")
    s2.import_deflation(Z)
    x1, st1 = s1.solve(rhs[1], mode=1, tol=1e-10, mat_rank=2000)
    x2, st2 = s2.solve(rhs[1], mode=1, tol=1e-10, mat_rank=2000)
    assert st1["cycles"] == st2["cycles"]
    assert _rel(x1, x2) < 1e-12


def test_initial_guess_within_tolerance_returns_absolute_norm(c1):
    A, rhs, cfg, direct = c1
    s = gdmr.System(A, cfg["m"], cfg["k"], capacity=1, precision="fp64")
    x, st = s.solve(rhs[0], x0=direct[0], mode=0, tol=1e-6, mat_rank=10)
    assert st["cycles"] == 0
    assert st["rel_res"] < 1e-6 * np.linalg.norm(rhs[0])
    assert np.array_equal(x, direct[0])


def test_cycle_cap_reports_no_convergence(c1):
    A, rhs, cfg, direct = c1
    s = gdmr.System(A, cfg["m"], cfg["k"], capacity=1, precision="fp64")
    x, st = s.solve(rhs[0], mode=0, tol=1e-10, mat_rank=3)
    assert st["status"] == 3 and st["cycles"] == 4
    assert "converge" in gdmr.last_error()


@pytest.mark.parametrize("precision", ["fp64", "mixed", "fp64e"])
def test_graph_replay_matches_eager_launches(c1, precision):
    """Restart cycles replayed as CUDA graphs give the same iterates as eager launches."""
    A, rhs, cfg, direct = c1
    res = []
    for graphs in (False, True):
        s = gdmr.System(A, cfg["m"], cfg["k"], capacity=2, precision=precision)
        s.set_graphs(graphs)
        if precision in ("fp64", "fp64e"):
            x0, st0 = s.solve(rhs[0], mode=0, tol=1e-10, mat_rank=2000)
            x1, st1 = s.solve(rhs[1], mode=1, tol=1e-10, mat_rank=2000)
            res.append((np.stack([x0, x1]), [st0["cycles"], st1["cycles"]]))
        else:
            X, st = s.solve_batch(np.array(rhs[:2]), tol=1e-10, max_cycles=2000)
            res.append((X, [t["cycles"] for t in st]))
    (xe, ce), (xg, cg) = res
    assert ce == cg
    assert np.array_equal(xe, xg)


def test_deflation_space_survives_the_process_through_a_file(c1, tmp_path):
    """save -> load through the versioned file gives the same next solve as keeping the
    space resident (the reference can only move Z between host and device)."""
    A, rhs, cfg, direct = c1
    s1 = gdmr.System(A, cfg["m"], cfg["k"], capacity=1, precision="fp64")
    s1.solve(rhs[0], mode=0, tol=1e-10, mat_rank=2000)
    path = str(tmp_path / "z.gdmr")
    s1.save_deflation(path)
    s2 = gdmr.System(A, cfg["m"], cfg["k"], capacity=1, precision="fp64")
    s2.load_deflation(path)
    x1, st1 = s1.solve(rhs[1], mode=1, tol=1e-10, mat_rank=2000)
    x2, st2 = s2.solve(rhs[1], mode=1, tol=1e-10, mat_rank=2000)
    assert st1["cycles"] == st2["cycles"]
    assert _rel(x1, x2) < 1e-12
