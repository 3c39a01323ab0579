"""Host logic of simplify_batch(streams=k): the split of a batch into k runs
of consecutive instances with about equal clause counts."""
import random

from parafrost_gb300.simplifier import split_runs


def check(sizes, k):
    runs = split_runs(sizes, k)
    kk = max(1, min(k, len(sizes)))
    assert len(runs) == kk
    assert runs[0][0] == 0 and runs[-1][1] == len(sizes)
    assert all(b < e for b, e in runs)
    assert all(runs[i][1] == runs[i + 1][0] for i in range(kk - 1))
    return runs


def test_equal_sizes_split_evenly():
    assert check([10] * 8, 4) == [(0, 2), (2, 4), (4, 6), (6, 8)]
    assert check([5] * 9, 3) == [(0, 3), (3, 6), (6, 9)]


def test_runs_cover_the_batch_in_order():
    rng = random.Random(3)
    for _ in range(5000):
        n = rng.randint(1, 40)
        k = rng.randint(1, 9)
        sizes = [int(rng.expovariate(1.0) * rng.choice([1, 10, 1000])) for _ in range(n)]
        check(sizes, k)


def test_balance_of_uneven_sizes():
    rng = random.Random(5)
    sizes = [rng.randint(1000, 200000) for _ in range(512)]
    runs = check(sizes, 4)
    loads = [sum(sizes[b:e]) for b, e in runs]
    assert max(loads) - min(loads) <= 2 * max(sizes)


def test_skewed_batch_still_gets_k_runs():
    assert check([1, 1, 1, 1, 1, 1, 1, 100], 4) == [(0, 5), (5, 6), (6, 7), (7, 8)]
    assert check([100, 1, 1, 1], 4) == [(0, 1), (1, 2), (2, 3), (3, 4)]
    assert check([7], 3) == [(0, 1)]
