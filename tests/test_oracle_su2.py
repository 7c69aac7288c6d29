"""6j symbols of the oracle: tabulated values, symmetries, orthogonality."""
import math

import pytest

from oracle.su2 import w6j, w3j


def test_known_values():
    # {1/2 1/2 1; 1/2 1/2 0} = 1/2 ; {1 1 1; 1 1 1} = 1/6 ; {1/2 1/2 0; 1/2 1/2 1} = 1/2
    assert w6j(1, 1, 2, 1, 1, 0) == pytest.approx(0.5)
    assert w6j(2, 2, 2, 2, 2, 2) == pytest.approx(1.0 / 6.0)
    assert w6j(1, 1, 0, 1, 1, 2) == pytest.approx(0.5)
    # {1/2 1/2 0; 1/2 1/2 0} = -1/2
    assert w6j(1, 1, 0, 1, 1, 0) == pytest.approx(-0.5)


def test_triangle_rule_zero():
    assert w6j(1, 1, 4, 1, 1, 0) == 0.0
    assert w6j(1, 2, 2, 1, 1, 1) == 0.0  # odd triad sum


@pytest.mark.parametrize("args", [(1, 2, 3, 2, 1, 3), (3, 2, 1, 2, 3, 2), (4, 3, 1, 2, 3, 4), (5, 4, 3, 2, 3, 4)])
def test_symmetries(args):
    j1, j2, j3, l1, l2, l3 = args
    v = w6j(j1, j2, j3, l1, l2, l3)
    # column permutations and upper/lower swaps of two columns
    assert w6j(j2, j1, j3, l2, l1, l3) == pytest.approx(v)
    assert w6j(j1, j3, j2, l1, l3, l2) == pytest.approx(v)
    assert w6j(l1, l2, j3, j1, j2, l3) == pytest.approx(v)


def test_orthogonality():
    # sum_x (2x+1)(2e+1) {a b x; c d e}{a b x; c d f} = delta_ef
    a, b, c, d = 3, 2, 3, 2
    for e in range(0, 8):
        for f in range(0, 8):
            s = 0.0
            for x in range(0, 12):
                s += (x + 1) * (e + 1) * w6j(a, b, x, c, d, e) * w6j(a, b, x, c, d, f)
            tri_e = all(((p + q + e) % 2 == 0 and abs(p - q) <= e <= p + q) for p, q in ((a, d), (c, b)))
            expect = 1.0 if (e == f and tri_e) else 0.0
            assert s == pytest.approx(expect, abs=1e-12)


def test_3j_against_half_integer_cg():
    # <1/2 1/2 1/2 -1/2 | 0 0> = 1/sqrt2  via 3j
    v = w3j(1, 1, 0, 1, -1, 0)
    assert abs(v) == pytest.approx(1 / math.sqrt(2))
