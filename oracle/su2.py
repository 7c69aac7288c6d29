"""SU(2) recoupling coefficients in doubled-integer arguments.

Restates the Racah single-sum formula used by ``W6JS`` (code/update.f90:1665-1716)
and the factorial table of ``FACTRL`` (code/update.f90:1610-1618).  All angular
momenta are passed doubled (2j), exactly as the reference passes ``num_down``.
"""
import math
from functools import lru_cache

_NFAC = 301
FACT = [1.0] * (_NFAC + 1)
for _i in range(1, _NFAC + 1):
    FACT[_i] = FACT[_i - 1] * float(_i)


def _tri_ok(a, b, c):
    """Triangle condition for doubled momenta a, b, c with integer sum."""
    return c <= a + b and c >= abs(a - b) and (a + b + c) % 2 == 0


def _delta(a, b, c):
    """Triangle coefficient Delta(abc) for doubled momenta."""
    return (FACT[(a + b - c) // 2] * FACT[(a - b + c) // 2] * FACT[(-a + b + c) // 2]
            / FACT[(a + b + c) // 2 + 1])


@lru_cache(maxsize=None)
def w6j(j1, j2, j3, l1, l2, l3):
    """Wigner 6j symbol {j1 j2 j3; l1 l2 l3}, arguments doubled.

    Racah's formula: the triads (j1 j2 j3), (j1 l2 l3), (l1 j2 l3), (l1 l2 j3)
    must satisfy the triangle rule, otherwise the symbol is 0 (code/update.f90:1673-1695).
    """
    if min(j1, j2, j3, l1, l2, l3) < 0:
        return 0.0
    if not (_tri_ok(j1, j2, j3) and _tri_ok(j1, l2, l3) and _tri_ok(l1, j2, l3)
            and _tri_ok(l1, l2, j3)):
        return 0.0
    a1 = j1 + j2 + j3
    a2 = j1 + l2 + l3
    a3 = l1 + j2 + l3
    a4 = l1 + l2 + j3
    b1 = j1 + j2 + l1 + l2
    b2 = j2 + j3 + l2 + l3
    b3 = j3 + j1 + l3 + l1
    tmin = max(a1, a2, a3, a4)
    tmax = min(b1, b2, b3)
    s = 0.0
    for t in range(tmin, tmax + 1, 2):
        den = (FACT[(t - a1) // 2] * FACT[(t - a2) // 2] * FACT[(t - a3) // 2]
               * FACT[(t - a4) // 2] * FACT[(b1 - t) // 2] * FACT[(b2 - t) // 2]
               * FACT[(b3 - t) // 2])
        term = FACT[t // 2 + 1] / den
        if (t // 2) % 2:
            term = -term
        s += term
    return s * math.sqrt(_delta(j1, j2, j3) * _delta(j1, l2, l3)
                         * _delta(l1, j2, l3) * _delta(l1, l2, j3))


def w3j(j1, j2, j3, m1, m2, m3):
    """Wigner 3j symbol, doubled arguments (Racah formula)."""
    if m1 + m2 + m3 != 0 or not _tri_ok(j1, j2, j3):
        return 0.0
    if abs(m1) > j1 or abs(m2) > j2 or abs(m3) > j3:
        return 0.0
    if (j1 - m1) % 2 or (j2 - m2) % 2 or (j3 - m3) % 2:
        return 0.0
    kmin = max(0, (j2 - j3 - m1) // 2, (j1 - j3 + m2) // 2)
    kmax = min((j1 + j2 - j3) // 2, (j1 - m1) // 2, (j2 + m2) // 2)
    s = 0.0
    for k in range(kmin, kmax + 1):
        den = (FACT[k] * FACT[(j1 + j2 - j3) // 2 - k] * FACT[(j1 - m1) // 2 - k]
               * FACT[(j2 + m2) // 2 - k] * FACT[(j3 - j2 + m1) // 2 + k]
               * FACT[(j3 - j1 - m2) // 2 + k])
        s += (-1.0) ** k / den
    pre = math.sqrt(_delta(j1, j2, j3) * FACT[(j1 + m1) // 2] * FACT[(j1 - m1) // 2]
                    * FACT[(j2 + m2) // 2] * FACT[(j2 - m2) // 2]
                    * FACT[(j3 + m3) // 2] * FACT[(j3 - m3) // 2])
    sign = -1.0 if ((j1 - j2 - m3) // 2) % 2 else 1.0
    return sign * pre * s


def cg(j1, m1, j2, m2, j, m):
    """Clebsch-Gordan <j1 m1 j2 m2 | j m>, doubled arguments."""
    ph = -1.0 if ((j1 - j2 + m) // 2) % 2 else 1.0
    return ph * math.sqrt(j + 1.0) * w3j(j1, j2, j, m1, m2, -m)


def parity_sign(n):
    """(-1)**(n//2) for a non-negative doubled sum n (Fortran integer division)."""
    return -1.0 if (n // 2) % 2 else 1.0
