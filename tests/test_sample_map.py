"""The value order's sample map i -> (a*i + b) mod n (host side): the
multiplier keeps it a permutation of the level for every level size,
including sizes that share a factor with some of the candidate primes."""
import math

import numpy as np
import pytest

from pca_gb300.guided import _MAP_PRIMES, map_multiplier


def _is_permutation(a, b, n):
    i = np.arange(n, dtype=np.uint64)
    img = (np.uint64(a) * i + np.uint64(b)) % np.uint64(n)
    return np.unique(img).size == n


@pytest.mark.parametrize("n", [1, 2, 3, 7, 64, 4096, 4097, 99991, 1000003, 2 * 1000033])
def test_map_is_a_permutation(n):
    rng = np.random.default_rng(n)
    for start in range(len(_MAP_PRIMES)):
        a = map_multiplier(n, start)
        assert 0 <= a < n and math.gcd(a, n) == 1 or n == 1
        assert _is_permutation(a, int(rng.integers(0, n)), n)


def test_sizes_sharing_listed_primes_wrap_to_another():
    # a level size divisible by the first three primes takes the fourth
    big = _MAP_PRIMES[0] * _MAP_PRIMES[1] * _MAP_PRIMES[2]
    assert map_multiplier(big, 0) == _MAP_PRIMES[3]
    # starting at the last prime, wrapping past the end
    n = _MAP_PRIMES[-1] * _MAP_PRIMES[0]
    assert map_multiplier(n, len(_MAP_PRIMES) - 1) == _MAP_PRIMES[1]


def test_empty_level_is_refused():
    with pytest.raises(ValueError):
        map_multiplier(0)
