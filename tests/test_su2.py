"""Spin-coupling coefficients of the host code (host/su2.cpp, the Racah
formulas of new_anglib.C:19-316 in the reference's operation order) against
exact rational values from sympy.physics.wigner: Clebsch-Gordan
coefficients for every 2j <= 6, and 6j, 9j and normalised 9j symbols
(couplingCoeffs.h:88-97: sqrt((2g+1)(2h+1)(2c+1)(2f+1)) times the 9j) over
seeded samples of admissible arguments, to 1e-13; symbols whose triangle
conditions fail are 0; Transposeview::get_scaling (BaseOperator.C:56-91)
against the same ratio of exact Clebsch-Gordan coefficients."""
import itertools
import math
import random

import pytest

sympy = pytest.importorskip("sympy")
from sympy import Rational  # noqa: E402
from sympy.physics.wigner import clebsch_gordan, wigner_6j, wigner_9j  # noqa: E402

TOL = 1e-13


def h(n2):
    return Rational(n2, 2)


def tri(a, b, c):
    return abs(a - b) <= c <= a + b and (a + b + c) % 2 == 0


def test_clebsch_exact(oracle):
    n = 0
    for j1, j2 in itertools.product(range(7), repeat=2):
        for j3 in range(abs(j1 - j2), j1 + j2 + 1, 2):
            for m1 in range(-j1, j1 + 1, 2):
                for m2 in range(-j2, j2 + 1, 2):
                    m3 = m1 + m2
                    if abs(m3) > j3:
                        continue
                    ref = float(clebsch_gordan(h(j1), h(j2), h(j3), h(m1), h(m2), h(m3)))
                    got = oracle.su2("clebsch", j1, m1, j2, m2, j3, m3)
                    assert abs(got - ref) <= TOL, (j1, m1, j2, m2, j3, m3, got, ref)
                    n += 1
    assert n > 1000
    # m's that do not add up, or a broken triangle, give 0
    assert oracle.su2("clebsch", 2, 2, 2, 0, 2, 0) == 0.0
    assert oracle.su2("clebsch", 1, 1, 1, 1, 6, 2) == 0.0


def test_six_j_exact(oracle):
    rng = random.Random(6)
    n = 0
    while n < 300:
        a, b, c, d, e, f = (rng.randint(0, 6) for _ in range(6))
        ok = tri(a, b, c) and tri(a, e, f) and tri(d, b, f) and tri(d, e, c)
        got = oracle.su2("six_j", a, b, c, d, e, f)
        if not ok:
            assert got == 0.0
            continue
        ref = float(wigner_6j(h(a), h(b), h(c), h(d), h(e), h(f)))
        assert abs(got - ref) <= TOL, ((a, b, c, d, e, f), got, ref)
        n += 1


def test_nine_j_exact(oracle):
    rng = random.Random(9)
    n = 0
    while n < 150:
        a, b, d, e = (rng.randint(0, 4) for _ in range(4))
        cs = [c for c in range(abs(a - b), a + b + 1, 2)]
        fs = [f for f in range(abs(d - e), d + e + 1, 2)]
        gs = [g for g in range(abs(a - d), a + d + 1, 2)]
        hs = [x for x in range(abs(b - e), b + e + 1, 2)]
        c, f, g, hh = rng.choice(cs), rng.choice(fs), rng.choice(gs), rng.choice(hs)
        iis = [i for i in range(abs(c - f), c + f + 1, 2) if tri(g, hh, i)]
        if not iis:
            continue
        i = rng.choice(iis)
        args = (a, b, c, d, e, f, g, hh, i)
        ref = float(wigner_9j(*(h(x) for x in args), prec=None))
        got = oracle.su2("nine_j", *args)
        assert abs(got - ref) <= TOL, (args, got, ref)
        norm = math.sqrt((g + 1) * (hh + 1) * (c + 1) * (f + 1))
        assert abs(oracle.su2("ninej", *args) - norm * ref) <= TOL * max(1.0, norm), args
        n += 1
    # a broken row triangle gives 0
    assert oracle.su2("nine_j", 0, 0, 2, 0, 0, 0, 0, 0, 2) == 0.0


def test_transpose_scaling(oracle):
    for l2, r2, k2 in itertools.product(range(5), range(5), (0, 2)):
        if not tri(l2, k2, r2):
            continue
        got = oracle.su2("transpose_scaling", l2, r2, k2)
        ref = None
        if k2 == 0:
            ref = 1.0
        else:
            for lz in range(-l2, l2 + 1, 2):
                for rz in range(-r2, r2 + 1, 2):
                    num = float(clebsch_gordan(h(l2), h(k2), h(r2), h(lz), h(-k2), h(rz)))
                    den = float(clebsch_gordan(h(r2), h(k2), h(l2), h(rz), h(k2), h(lz)))
                    if abs(num) > 1e-10 and abs(den) > 1e-10:
                        ref = (-1) ** k2 * num / den
                        break
                if ref is not None:
                    break
        assert ref is not None and abs(got - ref) <= TOL, (l2, r2, k2, got, ref)
