"""Host helpers with the reference's names (utils.py of ali-ramadhan/lagrangian-microbes).

Only the lattice-shape helpers sit on the hot path: they decide the particle lattice of
uniform_particle_locations.
"""

from __future__ import annotations

import math


def factor(n: int) -> list[int]:
    """All positive divisors of n in ascending order (utils.py:7-22)."""
    n = int(n)
    if n < 1:
        raise ValueError("factor() needs a positive integer")
    small, large = [], []
    for d in range(1, math.isqrt(n) + 1):
        if n % d == 0:
            small.append(d)
            if d != n // d:
                large.append(n // d)
    return small + large[::-1]


def most_symmetric_integer_factorization(N: int) -> tuple[int, int]:
    """The divisor pair (a, N // a) of N with a closest to sqrt(N) (utils.py:25-42).

    Among divisors, the one nearest sqrt(N) is always the largest divisor a with a * a <= N (its
    cofactor N // a lies farther above sqrt(N) than a lies below it), so a is returned first.
    """
    N = int(N)
    a = max(d for d in factor(N) if d * d <= N)
    return a, N // a
