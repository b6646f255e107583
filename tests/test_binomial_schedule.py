"""The binomial (revolve) checkpoint schedule of sse_rk_record_binomial,
host arithmetic only: its extra forward steps against a brute-force search
over every split of the Griewank-Walther recursion on small horizons, the
limiting cases, and monotonicity in the number of checkpoints."""
import functools

import pytest


@functools.lru_cache(maxsize=None)
def best(n, c):
    """Fewest extra forward steps reversing n steps with c free slots."""
    if n == 1:
        return 0
    if c == 0:
        return n * (n - 1) // 2
    return min(m + best(n - m, c - 1) + best(m, c) for m in range(1, n))


@pytest.fixture(scope="module")
def sched(pkg):
    pkg.build.build()
    return pkg.gb300.binomial_schedule


@pytest.mark.parametrize("n", [1, 2, 3, 7, 16, 40, 61])
@pytest.mark.parametrize("c", [0, 1, 2, 3, 5, 10])
def test_matches_exhaustive_search(sched, n, c):
    extra, first = sched(n, c)
    assert extra == best(n, min(c, n - 1))
    if n > 1 and c > 0:
        assert 1 <= first < n


def test_limits(sched):
    # a checkpoint for every step: only the descent is extra
    assert sched(50, 49)[0] == 49
    assert sched(50, 500)[0] == 49
    assert sched(2048, 2047)[0] == 2047
    # no checkpoint: every step is recomputed from the start
    assert sched(50, 0)[0] == 50 * 49 // 2
    # 200 stages of the C5 workload as 40 steps with 4 checkpoints
    extra, _ = sched(40, 4)
    assert extra == best(40, 4)


def test_more_checkpoints_never_cost_more(sched):
    for n in (10, 40, 200, 1000):
        costs = [sched(n, c)[0] for c in range(0, 12)]
        assert all(b <= a for a, b in zip(costs, costs[1:]))
        # each checkpoint at least halves the recomputation while it is quadratic
        assert costs[1] < costs[0] / 2


def test_rejects_invalid(pkg, sched):
    with pytest.raises(pkg.SSEError):
        sched(0, 3)
