"""The serving layer's placement of operators across devices by memory budget (host-only).

gdmr_place_operator is the rule gdmr_server_add_operator applies: an operator (fixed bytes for
its matrix and deflation space, plus bytes per request slot) goes to the device that keeps the
most budget free after taking it, so operators spread over the devices and no device is asked
for more than its budget.  With capacity 0 the operator takes as many slots as fit (at most
256) on the device with the most room.
"""
import gdmr

GB = 1 << 30


def test_worst_fit_spreads_operators_over_devices():
    budget = [10 * GB, 10 * GB]
    used = [0, 0]
    placed = []
    for _ in range(4):
        d, cap = gdmr.place_operator(budget, used, 2 * GB, GB // 2, capacity=4)
        assert cap == 4
        used[d] += 2 * GB + 4 * (GB // 2)
        placed.append(d)
    assert placed == [0, 1, 0, 1]
    # a fifth operator of 4 GB does not fit on either device (2 GB left each)
    assert gdmr.place_operator(budget, used, 2 * GB, GB // 2, capacity=4) == (-1, 0)
    # one slot still fits
    d, cap = gdmr.place_operator(budget, used, GB, GB // 2, capacity=1)
    assert d in (0, 1) and cap == 1


def test_capacity_zero_takes_the_roomiest_device_and_fills_it():
    budget = [8 * GB, 16 * GB, 12 * GB]
    used = [0, 2 * GB, 0]
    d, cap = gdmr.place_operator(budget, used, GB, GB, capacity=0)
    assert d == 1 and cap == 13                 # 16 - 2 - 1 = 13 slots of 1 GB
    d, cap = gdmr.place_operator(budget, used, GB, GB // 1024, capacity=0)
    assert cap == 256                           # at most 256 slots


def test_unequal_budgets_and_an_operator_too_large_for_all():
    budget = [4 * GB, 6 * GB]
    used = [0, 0]
    d, cap = gdmr.place_operator(budget, used, 5 * GB, GB // 2, capacity=1)
    assert (d, cap) == (1, 1)                   # only the larger device holds it
    assert gdmr.place_operator(budget, used, 7 * GB, 1, capacity=1) == (-1, 0)
    assert gdmr.place_operator(budget, used, 0, 7 * GB, capacity=0) == (-1, 0)
