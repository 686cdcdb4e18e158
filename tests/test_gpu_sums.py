"""The PT2 map-reduce (sum and sum of squares of the per-det contributions) is a compensated,
fixed-order reduction: checked through the C ABI on an ill-conditioned vector against an
exactly rounded sum (math.fsum)."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def ill_conditioned(n, seed):
    """Large terms that cancel in pairs plus small ones, shuffled; every value has at most
    25 significant bits, so squares are exact in FP64 and fsum of them is exactly rounded."""
    rng = np.random.default_rng(seed)
    big = rng.integers(-(1 << 25), 1 << 25, n // 4).astype(np.float64) * 2.0 ** -10
    small = rng.integers(-(1 << 25), 1 << 25, n - 2 * (n // 4)).astype(np.float64) * 2.0 ** -30
    x = np.concatenate([big, -big, small])
    rng.shuffle(x)
    return x


@pytest.mark.parametrize("n", [1, 1000, 1 << 22, (1 << 22) + 12345])
def test_mapreduce_sum_compensated(n):
    import shci_gb300 as S
    c = S.Context()
    x = ill_conditioned(n, 5 + n)
    s, s2 = c.mapreduce_sum(x)
    exact = math.fsum(x.tolist())
    exact2 = math.fsum((x * x).tolist())
    assert abs(s - exact) <= 1e-12 * max(abs(exact), 1e-300)
    assert abs(s2 - exact2) <= 4e-16 * exact2
    # plain FP64 summation loses the small terms on the large cancelling ones
    if n >= 1 << 22:
        assert abs(float(np.sum(x)) - exact) > 1e3 * abs(s - exact)
    # deterministic: the same call gives the same bits
    assert c.mapreduce_sum(x) == (s, s2)


def test_mapreduce_sum_empty():
    import shci_gb300 as S
    c = S.Context()
    assert c.mapreduce_sum(np.zeros(0)) == (0.0, 0.0)
