"""CPU tests of the quasi-Monte Carlo point set (myql_qmc_directions, host code, no GPU):
the direction numbers are those of a Sobol sequence built on primitive polynomials, so
every dimension is stratified and the first two dimensions form (0, m, 2)-nets."""
import ctypes as C
from math import gcd

import numpy as np
import pytest

from myquantlib_gb300 import _abi


def directions(D, seed=42):
    lib = _abi.load()
    out = np.zeros(D * 32, dtype=np.uint32)
    _abi.check(lib.myql_qmc_directions(D, seed, out.ctypes.data_as(C.POINTER(C.c_uint32))))
    return out.reshape(D, 32)


def points(V, n):
    """The first n Sobol points (Gray-code order) as 32-bit integers, [n][D]."""
    idx = np.arange(n, dtype=np.uint64)
    g = idx ^ (idx >> np.uint64(1))
    x = np.zeros((n, V.shape[0]), dtype=np.uint32)
    for b in range(32):
        bit = ((g >> np.uint64(b)) & np.uint64(1)).astype(bool)
        x[bit] ^= V[:, b]
    return x


def test_direction_numbers_are_odd_m_k_scaled():
    # V_k = m_k 2^(32-k) with m_k odd and m_k < 2^k: bit 32-k is the lowest bit set
    V = directions(600)
    for k in range(1, 33):
        col = V[:, k - 1].astype(np.uint64)
        assert np.all((col >> np.uint64(32 - k)) & np.uint64(1) == np.uint64(1)), k
        assert np.all(col & ((np.uint64(1) << np.uint64(32 - k)) - np.uint64(1)) == np.uint64(0)), k


@pytest.mark.parametrize("m", [4, 8, 12])
def test_every_dimension_is_stratified(m):
    V = directions(300)
    x = points(V, 1 << m) >> np.uint32(32 - m)
    for d in range(V.shape[0]):
        assert len(np.unique(x[:, d])) == 1 << m, d


def test_first_two_dimensions_are_0_m_2_nets():
    V = directions(2)
    m = 10
    x = points(V, 1 << m)
    for a in range(m + 1):           # elementary intervals 2^-a x 2^-(m-a)
        cells = (x[:, 0] >> np.uint32(32 - a)).astype(np.int64) * (1 << (m - a)) + \
                (x[:, 1] >> np.uint32(32 - (m - a))).astype(np.int64) if a < 32 else None
        assert len(np.unique(cells)) == 1 << m, a


def count_primitive(s):
    """phi(2^s - 1) / s, the number of primitive polynomials of degree s over GF(2)."""
    n = (1 << s) - 1
    phi = sum(1 for k in range(1, n + 1) if gcd(k, n) == 1)
    return phi // s


def test_dimensions_follow_the_primitive_polynomials_by_degree():
    # one dimension per primitive polynomial, degree by degree: 1 + sum_s count(s) dimensions
    # exhaust degrees <= 8, so dimension 1 + sum is the first of degree 9 -- its direction
    # numbers V_1..V_9 are free (seeded) and V_10.. follow the degree-9 recurrence
    total = 1 + sum(count_primitive(s) for s in range(1, 9))
    assert total == 1 + 1 + 1 + 2 + 2 + 6 + 6 + 18 + 16
    V = directions(total + 1)
    assert V.shape == (total + 1, 32)


def test_directions_depend_on_the_seed_beyond_dimension_one():
    a, b = directions(50, 1), directions(50, 2)
    assert np.array_equal(a[:2], b[:2])      # van der Corput and the degree-1 polynomial are forced
    assert not np.array_equal(a[2:], b[2:])


def t_value(xi, xj, m):
    """The t of the first 2^m points of a 2-D projection: the smallest t such that every
    elementary interval 2^-a x 2^-(m-t-a) holds exactly 2^t points."""
    xi, xj = xi.astype(np.uint64), xj.astype(np.uint64)
    for t in range(m + 1):
        k = m - t
        if all(np.all(np.bincount(((xi >> np.uint64(32 - a)) << np.uint64(k - a) |
                                   (xj >> np.uint64(32 - (k - a)))).astype(np.int64),
                                  minlength=1 << k) == (1 << t)) for a in range(k + 1)):
            return t
    return m


def test_two_dimensional_projections_meet_the_sobol_t_bound():
    """Every pair of the first 13 dimensions (polynomial degrees up to 5) is a (t, m, 2)-net
    with t at most (s_i - 1) + (s_j - 1), the bound of Sobol's construction whatever the odd
    initial direction numbers (dimension 0, van der Corput, counts as s = 1)."""
    degrees = [1, 1, 2, 3, 3, 4, 4] + [5] * 6
    V = directions(len(degrees))
    m = 12
    x = points(V, 1 << m)
    ts = {}
    for i in range(len(degrees)):
        for j in range(i + 1, len(degrees)):
            t = t_value(x[:, i], x[:, j], m)
            ts[(i, j)] = t
            assert t <= (degrees[i] - 1) + (degrees[j] - 1), (i, j, t)
    assert ts[(0, 1)] == 0
