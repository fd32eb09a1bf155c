"""The ConstantStepSize grid fraction of the kernels (grid_fraction in
diffrax_gb300/csrc/gbdx_common.cuh) restated with exact rational arithmetic:
from inv = RN(1 / n), q = RN(s inv), r = s - q n (exact under an FMA) and
RN(q + r inv) must be the correctly rounded quotient RN(s / n) that the
reference's grid t0 + (t1 - t0) (s / n) uses (constant.py:84-86), for every
integer 0 < s <= n < 2^31 (Markstein's theorem on the final correction step
of Newton-Raphson division).  Exhaustive for small n, sampled above."""
import random
from fractions import Fraction

import pytest


def grid_fraction(s: int, n: int):
    inv = 1.0 / n                                  # RN(1 / n)
    q = float(Fraction(s) * Fraction(inv))         # RN(s * inv)
    r_exact = Fraction(s) - Fraction(q) * n        # fma(-q, n, s) before rounding
    r = float(r_exact)
    assert Fraction(r) == r_exact, "the remainder is exact"
    return float(Fraction(q) + Fraction(r) * Fraction(inv))  # fma(r, inv, q)


def test_grid_fraction_exhaustive_small_n():
    for n in range(1, 260):
        for s in range(1, n + 1):
            assert grid_fraction(s, n) == s / n, (s, n)


@pytest.mark.parametrize("seed", [0, 1])
def test_grid_fraction_random_and_edge_n(seed):
    rng = random.Random(seed)
    cases = [(rng.randrange(1, n + 1), n) for n in (rng.randrange(1, 2**31) for _ in range(20000))]
    for k in range(31):
        for n in {2**k, 2**k + 1, max(2**k - 1, 1), 3 * 2**k if 3 * 2**k < 2**31 else 2**30 + 1}:
            cases += [(s, n) for s in {1, max(n // 3, 1), max(n // 2, 1), max(n - 1, 1), n}]
    for s, n in cases:
        assert grid_fraction(s, n) == s / n, (s, n)
