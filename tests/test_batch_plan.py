"""Host side of the batched-request path: the chain assignment (longest
processing time first onto the least loaded chain) the batch graph uses."""
import numpy as np


def test_plan_balances_longest_first(native_lib):
    from vulkanpbrt_gb300 import batch

    rng = np.random.default_rng(0)
    costs = rng.lognormal(0, 1.5, 64)
    for branches in (1, 2, 4, 8, 16):
        a = batch.plan(costs, branches, order=1)
        assert a.min() >= 0 and a.max() < branches
        loads = np.bincount(a, weights=costs, minlength=branches)
        # LPT bound: makespan <= 4/3 OPT, and OPT >= max(mean load, largest job)
        opt_lb = max(costs.sum() / branches, costs.max())
        assert loads.max() <= 4.0 / 3.0 * opt_lb + 1e-9
        # replay the rule in Python
        load = np.zeros(branches)
        want = np.zeros(64, np.uint32)
        for i in sorted(range(64), key=lambda i: -costs[i]):
            k = int(np.argmin(load))
            want[i] = k
            load[k] += costs[i]
        assert np.array_equal(a, want)


def test_plan_in_given_order_and_rejects_bad_input(native_lib):
    import pytest

    from vulkanpbrt_gb300 import batch
    from vulkanpbrt_gb300._abi import PbrtError

    a = batch.plan([5.0, 1.0, 1.0, 1.0], 2, order=0)
    assert list(a) == [0, 1, 1, 1]
    with pytest.raises(PbrtError):
        batch.plan([1.0], 0)
