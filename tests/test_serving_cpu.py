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


def test_plan_slice_fifo_oldest_first_and_fill():
    ops = [np.full(100, 10.0), np.full(3, 10.0), np.full(50, 10.0)]
    rem = [o.sum() for o in ops]
    age = [2.0, 1.0, 3.0]                    # job 1 is the oldest, then 0, then 2
    plan = plan_slice(rem, ops, [0, 0, 0], slice_ops=120.0, policy="fifo", age=age)
    assert [j for j, _, _ in plan] == [1, 0]  # the oldest ends inside the slice, the next fills it
    got = {j: k for j, k, _ in plan}
    assert got[1] == 3 and got[0] == 9       # 30 + 90 = 120 ops; nothing left for job 2
    # a job that needs more than the slice takes all of it, alone
    plan = plan_slice(rem, ops, [0, 0, 0], slice_ops=120.0, policy="fifo", age=[0.0, 1.0, 2.0])
    assert plan == [(0, 12, 120.0)]
    # an item larger than the slice still advances the oldest job
    plan = plan_slice([500.0], [np.array([500.0])], [0], slice_ops=100.0, policy="fifo", age=[0.0])
    assert plan == [(0, 1, 500.0)]
    with pytest.raises(ValueError):
        plan_slice(rem, ops, [0, 0, 0], 120.0, policy="lifo")


@pytest.mark.parametrize("policy", ["fifo", "srpt"])
def test_plan_slice_policies_drain(policy):
    rng = np.random.default_rng(1)
    ops = [rng.integers(1, 50, n).astype(float) for n in (7, 300, 41, 1, 90)]
    nxt = [0] * len(ops)
    rem = [o.sum() for o in ops]
    age = list(rng.random(len(ops)))
    finish = {}
    launches = 0
    while any(n < o.size for n, o in zip(nxt, ops)):
        for j, k, o in plan_slice(rem, ops, nxt, slice_ops=400.0, policy=policy, age=age):
            assert k >= 1 and nxt[j] + k <= ops[j].size
            assert np.isclose(o, ops[j][nxt[j]:nxt[j] + k].sum())
            nxt[j] += k
            rem[j] -= o
            if nxt[j] == ops[j].size:
                finish[j] = launches
        launches += 1
        assert launches < 1000
    assert np.allclose(rem, 0)
    if policy == "fifo":                     # jobs finish in age order
        order = sorted(range(len(ops)), key=lambda j: age[j])
        assert [finish[j] for j in order] == sorted(finish[j] for j in order)


def test_slice_policy_switches_with_backlog():
    from dynamix_gb300.serving import slice_policy
    assert slice_policy(1, 4) == "fifo"
    assert slice_policy(4, 4) == "fifo"
    assert slice_policy(5, 4) == "srpt"
    assert slice_policy(3, 0) == "srpt"
