"""Host-side scheduling logic of the g2 service (no GPU)."""
import numpy as np
import pytest

from dynamix_gb300.serving import Arena, ArenaFull, admit_order, plan_slice


def test_arena_first_fit_and_merge():
    a = Arena(100)
    x = a.alloc(30)
    y = a.alloc(30)
    z = a.alloc(40)
    assert (x, y, z) == (0, 30, 60) and a.used == 100
    with pytest.raises(ArenaFull):
        a.alloc(1)
    a.release(y, 30)
    assert a.alloc(10) == 30
    a.release(x, 30)
    a.release(30, 10)
    assert a.free == [(0, 60)]              # neighbours merged
    a.release(z, 40)
    assert a.free == [(0, 100)] and a.used == 0


def test_plan_slice_shortest_first_and_no_starvation():
    ops = [np.full(100, 10.0), np.full(3, 10.0), np.full(50, 10.0)]
    rem = [o.sum() for o in ops]
    plan = plan_slice(rem, ops, [0, 0, 0], slice_ops=120.0)
    order = [j for j, _, _ in plan]
    assert order == [1, 2, 0]                # shortest remaining first
    got = {j: k for j, k, _ in plan}
    assert got[1] == 3                       # the short job finishes in this launch
    assert all(k >= 1 for k in got.values())  # every job advances (floor share)
    assert got[0] >= 2                       # floor: 120 / (2 * 3) = 20 ops = 2 items


def test_plan_slice_drains_every_job():
    rng = np.random.default_rng(0)
    ops = [rng.integers(1, 50, n).astype(float) for n in (7, 300, 41, 1)]
    nxt = [0] * 4
    rem = [o.sum() for o in ops]
    launches = 0
    while any(n < o.size for n, o in zip(nxt, ops)):
        for j, k, o in plan_slice(rem, ops, nxt, slice_ops=500.0):
            assert k >= 1 and nxt[j] + k <= ops[j].size
            assert np.isclose(o, ops[j][nxt[j]:nxt[j] + k].sum())
            nxt[j] += k
            rem[j] -= o
        launches += 1
        assert launches < 1000
    assert np.allclose(rem, 0)


def test_admit_order_budget_slots_and_too_large():
    needs = [50, 80, 10, 500, 30]
    admit, big = admit_order(needs, used=20, budget=100, free_slots=8)
    assert admit == [0, 2]                   # 20+50 = 70; 80 does not fit; 10 does; 30 does not
    assert big == [3]
    admit, big = admit_order(needs, used=0, budget=100, free_slots=1)
    assert admit == [0]
    assert admit_order([], 0, 100, 4) == ([], [])
