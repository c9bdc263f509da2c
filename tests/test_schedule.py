"""The binomial checkpoint schedule of swc_backward (restated in
smaiso_wcomp_gb300/schedule.py, which the GPU adjoint tests hold the library to): its
split is optimal against a brute-force search over every split, and its cost is
Griewank's closed form."""
from functools import lru_cache

from smaiso_wcomp_gb300 import schedule


@lru_cache(maxsize=None)
def _best(n, s):
    """Minimum advances over all schedules (exhaustive search of the first split)."""
    if n <= 1:
        return 0
    if s == 0:
        return n * (n - 1) // 2
    return min(m + _best(n - m, s - 1) + _best(m, s) for m in range(1, n))


def test_split_is_optimal_against_exhaustive_search():
    for s in range(0, 7):
        for n in range(1, 71):
            assert schedule.binomial_advances(n, s) == _best(n, s) == schedule.optimal_advances(n, s), (n, s)


def test_split_meets_the_closed_form_at_larger_sizes():
    for s in (1, 2, 5, 11, 30, 62):
        for n in (2, 3, 17, 100, 257, 1000, 2000):
            assert schedule.binomial_advances(n, s) == schedule.optimal_advances(n, s), (n, s)


def test_long_horizon_configuration():
    # 2000 steps: 59 snapshot slots (the mixed 256^3 engine under a 40 GB cap) and 50
    assert schedule.forward_steps(2000, 59) == 4047 + 2000
    assert schedule.forward_steps(2000, 50) == 4569 + 2000
    assert schedule.forward_steps(5, 0) == 10 + 5
