"""The index division of the element and node kernels (csrc/common.cuh: fast_div, fdiv,
unflatten3): n / d as (umulhi(n, m) + n) >> l with l = ceil(log2 d) and
m = floor(2^32 (2^l - d) / d) + 1 (Granlund and Montgomery 1994). The kernels rely on it being
exact for every divisor and index their grids allow (d, n < 2^31); this checks the method over
edge and random cases, in the 32-bit arithmetic the device performs."""
import numpy as np


def fast_div(d):
    l = 0
    while l < 31 and (1 << l) < d:
        l += 1
    m = ((1 << 32) * ((1 << l) - d)) // d + 1
    assert 0 < m < (1 << 32) or d == 1
    return m, l


def fdiv(n, m, l):
    s = ((n * m) >> 32) + n
    assert s < (1 << 32)  # the device sum is 32-bit
    return s >> l


def test_fast_division_is_exact():
    rng = np.random.default_rng(0)
    divisors = list(range(1, 300)) + [2**k + o for k in range(9, 31) for o in (-1, 0, 1) if 2**k + o < 2**31]
    divisors += [int(v) for v in rng.integers(1, 2**31, 300)]
    for d in divisors:
        m, l = fast_div(d)
        ns = {0, 1, d - 1, d, d + 1, 2**31 - 1, (2**31 - 1) // d * d, (2**31 - 1) // d * d - 1}
        ns |= {int(v) for v in rng.integers(0, 2**31, 64)}
        ns |= {q * d + r for q in (1, 2, 1000, (2**31 - 1) // d) for r in (0, d - 1) if q * d + r < 2**31}
        for n in ns:
            if 0 <= n < 2**31:
                assert fdiv(n, m, l) == n // d, (n, d)


def test_unflatten_matches_row_major_order():
    for a, b, c in [(1, 1, 1), (3, 5, 2), (33, 7, 5), (65, 65, 65), (193, 97, 97), (6, 40, 3)]:
        mb, lb = fast_div(b)
        mc, lc = fast_div(c)
        for n in range(0, a * b * c, max(1, a * b * c // 5000)):
            q = fdiv(n, mc, lc)
            k = n - q * c
            i = fdiv(q, mb, lb)
            j = q - i * b
            assert (i * b + j) * c + k == n and 0 <= j < b and 0 <= k < c and 0 <= i < a
