"""The binomial checkpoint schedule of swc_backward (adjoint_ckpt = -1), restated for
planning: how many forward steps a reversal of n steps costs with a given number of
snapshot slots (the library reports the count it ran as swc_grad.forward_steps).

The reversal of steps l+1 .. l+n from a held state l with s free slots (Griewank's
binomial checkpointing): advance m steps, snapshot, reverse the right part n - m with
s - 1 slots, then the left part m with s slots; one step is reversed by a taped rerun;
with no free slot every step is rerun from l. With S = s + 1 states held (the loaded
one counts) and t the least integer with C(S + t, t) >= n, the split
m = max(n - C(S - 1 + t, t), C(S + t - 2, t - 2)), within [1, n - 1], is optimal, and
the reversal advances t n - C(S + t, t - 1) steps in all.
"""
from functools import lru_cache
from math import comb

__all__ = ["binomial_split", "binomial_advances", "optimal_advances", "forward_steps"]


def _reach(s, t):
    """C(s + t, t): the steps S = s checkpoints reverse with each step advanced <= t times."""
    return comb(s + t, t) if t >= 0 else 0


def _reps(n, nfree):
    t = 0
    while _reach(nfree + 1, t) < n:
        t += 1
    return t


def binomial_split(n, nfree):
    """Steps advanced before the first snapshot (n >= 2, nfree >= 1 free slots)."""
    t = _reps(n, nfree)
    m = n - min(n, _reach(nfree, t))
    if t >= 2:
        m = max(m, _reach(nfree + 1, t - 2))
    return min(max(m, 1), n - 1)


@lru_cache(maxsize=None)
def binomial_advances(n, nfree):
    """Forward steps the schedule advances (taped reruns excluded) to reverse n steps."""
    if n <= 1:
        return 0
    if nfree == 0:
        return n * (n - 1) // 2
    m = binomial_split(n, nfree)
    return m + binomial_advances(n - m, nfree - 1) + binomial_advances(m, nfree)


def optimal_advances(n, nfree):
    """Griewank's minimum over all schedules: t n - C(S + t, t - 1), S = nfree + 1."""
    if n <= 1:
        return 0
    t = _reps(n, nfree)
    return t * n - _reach(nfree + 2, t - 1)


def forward_steps(n, nfree):
    """swc_grad.forward_steps of a binomial swc_backward over n steps: the advances plus
    one taped rerun per step."""
    return binomial_advances(n, nfree) + n
