"""Serving layer through the C ABI (gdmr_server_*): resident operators, admission by a
device-memory budget, continuous batching across requests of several operators, and the
result-invariance property (a request's answer is the same alone and in the mix, within
the stated tolerance)."""
import numpy as np
import pytest

import gdmr
import problems

pytestmark = pytest.mark.gpu


def _direct(A, b):
    import scipy.sparse.linalg as spl
    return spl.splu(A.to_scipy().tocsc()).solve(b)


@pytest.fixture(scope="module")
def ops():
    A1 = problems.helmholtz((48, 48), 14.0, 0.05)
    A2 = problems.helmholtz((16, 16, 16), 6.0, 0.1)
    return [A1, A2]


def test_budget_limits_capacity(ops):
    A1, _ = ops
    per = gdmr.load().gdmr_server_slot_bytes(A1.n, 30, 1)
    srv = gdmr.Server(budget_bytes=200 * 1024 * 1024 + 5 * per)
    op = srv.add_operator(A1, 30, 8, capacity=0, precision="mixed")
    cap = srv.capacity(op)
    assert 1 <= cap <= 200
    assert srv.device_bytes <= 200 * 1024 * 1024 + 5 * per
    with pytest.raises(gdmr.GDMRError):
        srv.add_operator(A1, 30, 8, capacity=10**6, precision="mixed")
    srv.close()


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_mixed_requests_meet_their_tolerances(ops, precision):
    srv = gdmr.Server(budget_bytes=8 << 30)
    ids = [srv.add_operator(A, 30, 8, capacity=3, precision=precision) for A in ops]
    srv.start()
    reqs = []
    tols = [1e-6, 1e-8, 1e-10]
    for i in range(10):   # more requests than slots: the queue refills slots as they free
        j = i % 2
        A = ops[j]
        b = problems.unit_gaussian_rhs(A.n, 500 + i)
        tol = tols[i % 3]
        reqs.append((j, b, tol, srv.submit(ids[j], b, tol=tol)))
    for j, b, tol, t in reqs:
        x, st = srv.wait(t, timeout=120)
        A = ops[j]
        assert st["status"] == 0, st
        assert st["true_rel_res"] <= tol
        r = np.linalg.norm(b - A.to_scipy() @ x) / np.linalg.norm(b)
        assert r <= 1.5 * tol
        assert st["latency_ms"] > 0
    srv.close()


def test_result_same_alone_and_in_the_mix(ops):
    A1, A2 = ops
    b = problems.unit_gaussian_rhs(A1.n, 777)
    alone = gdmr.Server(budget_bytes=4 << 30)
    o = alone.add_operator(A1, 30, 8, capacity=1)
    alone.start()
    xa, sa = alone.wait(alone.submit(o, b, tol=1e-10), timeout=120)
    alone.close()
    mix = gdmr.Server(budget_bytes=8 << 30)
    o1 = mix.add_operator(A1, 30, 8, capacity=4)
    o2 = mix.add_operator(A2, 30, 8, capacity=4)
    mix.start()
    others = [mix.submit(o1 if i % 2 else o2, problems.unit_gaussian_rhs((A1 if i % 2 else A2).n, 900 + i), tol=1e-8)
              for i in range(6)]
    t = mix.submit(o1, b, tol=1e-10)
    xm, sm = mix.wait(t, timeout=120)
    for q in others:
        mix.wait(q, timeout=120)
    mix.close()
    assert sa["status"] == 0 and sm["status"] == 0
    xd = _direct(A1, b)
    assert np.linalg.norm(xa - xd) / np.linalg.norm(xd) < 1e-8
    assert np.linalg.norm(xm - xd) / np.linalg.norm(xd) < 1e-8
    assert np.linalg.norm(xa - xm) / np.linalg.norm(xd) < 2e-8


def test_operators_spread_over_a_device_list_and_solve_correctly(ops):
    """A server over two budgets (the device list names device 0 twice, as the reference's
    device lists may): operators go to the budget with the most room left, requests of both
    run and meet their tolerance, and no budget is exceeded."""
    A1, A2 = ops
    per_dev = 3 << 30
    srv = gdmr.Server(budget_bytes=per_dev, devices=[0, 0])
    ids = [srv.add_operator(A, 30, 8, capacity=4, precision="mixed") for A in (A1, A2, A1, A2)]
    placed = [srv.device_of(i) for i in ids]
    assert sorted(placed) == [0, 0, 1, 1] and placed[0] != placed[1]
    assert srv.device_bytes <= 2 * per_dev
    srv.start()
    reqs = [(j, problems.unit_gaussian_rhs((A1 if j % 2 == 0 else A2).n, 1300 + j)) for j in range(4)]
    tickets = [srv.submit(ids[j], b, tol=1e-10) for j, b in reqs]
    for (j, b), t in zip(reqs, tickets):
        x, st = srv.wait(t, timeout=120)
        A = A1 if j % 2 == 0 else A2
        assert st["status"] == 0 and st["true_rel_res"] <= 1e-10
        assert np.linalg.norm(b - A.to_scipy() @ x) / np.linalg.norm(b) <= 1.5e-10
    srv.close()
