"""bench.budget_groups: consecutive calibration instances packed into batch groups whose adjoint
step records fit a device-memory budget together (so that no group replays a step)."""
import os
import sys

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
import bench  # noqa: E402


def _per(n, steps):
    return int(1.02 * n * (80 * steps + 400)) + (64 << 20)


def test_groups_cover_every_instance_in_order_and_fit_the_budget():
    nelts = [2 * (250 + (i * 37) % 300) * (100 + (i * 23) % 180) for i in range(64)]
    budget = 120 << 30
    groups = bench.budget_groups(nelts, 3000, budget)
    assert [i for g in groups for i in g] == list(range(64))
    for g in groups:
        assert len(g) >= 1
        if len(g) > 1:
            assert sum(_per(nelts[i], 3000) for i in g) <= budget
    # greedy: the next instance did not fit into the group before it
    for g, nxt in zip(groups, groups[1:]):
        assert sum(_per(nelts[i], 3000) for i in g) + _per(nelts[nxt[0]], 3000) > budget


def test_small_run_is_one_group():
    assert bench.budget_groups([20000, 30000, 40000], 400, 120 << 30) == [[0, 1, 2]]


def test_an_instance_larger_than_the_budget_forms_its_own_group():
    groups = bench.budget_groups([1000, 10 ** 9, 1000], 3000, 1 << 30)
    assert groups == [[0], [1], [2]]
