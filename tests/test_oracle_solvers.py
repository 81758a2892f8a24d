"""The oracle's root solvers against the convergence patterns of test/test_solvers.jl:27-121."""
import math

import oracle as O

X1, X2, X3, X4 = 0.0, (-math.sqrt(2), math.sqrt(2)), 6.907755278982137, (-1.0, 1.0)


def approx(a, b):   # Julia's isapprox default: rtol = sqrt(eps)
    return abs(a - b) <= math.sqrt(2.220446049250313e-16) * max(abs(a), abs(b))


def test_newton_raphson():
    s = O.NEWTON
    assert [O.solve(s, 1, x) == X1 for x in (-10, -1, 0, 1, 10, 100)] == [False, True, True, True, False, False]
    got = [approx(O.solve(s, 2, x), X2[0]) for x in (-5, -1, -0.1, 0)] + \
          [approx(O.solve(s, 2, x), X2[1]) for x in (0.1, 1, 5)]
    assert got == [True, True, True, False, True, True, True]
    assert [O.solve(s, 3, x) == X3 for x in (-1, 0, 1, 5, 7, 10)] == [False, False, True, True, True, True]
    got = [approx(O.solve(s, 4, x), X4[0]) for x in (-10, -1.5, -1, 0)] + \
          [approx(O.solve(s, 4, x), X4[1]) for x in (1, 1.5, 5)]
    assert got == [False, True, True, False, True, True, False]
    assert approx(O.solve(s, 5, -5, pa=1, pb=-2), -math.sqrt(2))


def test_newton_raphson_safe():
    s = O.NEWTON_SAFE
    for a, b in ((-1000, 1000), (-100, 1), (-10, 0)):
        assert abs(O.solve(s, 1, a, b) - X1) <= 1e-10
    assert abs(O.solve(s, 2, -1000, 0) - X2[0]) <= 1e-10
    assert abs(O.solve(s, 2, -10, math.sqrt(2) - 0.1) - X2[0]) <= 1e-10
    assert abs(O.solve(s, 2, 0, 1000) - X2[1]) <= 1e-10
    assert O.solve(s, 3, -10000, 10000) == X3
    assert abs(O.solve(s, 4, -1000, 0) - X4[0]) <= 1e-10
    assert abs(O.solve(s, 4, -10, 0.9) - X4[0]) <= 1e-10
    assert abs(O.solve(s, 4, 0, 1000) - X4[1]) <= 1e-10
    assert approx(O.solve(s, 5, -100, 0, pa=1, pb=-2), -math.sqrt(2))


def test_damped_newton():
    s = O.DAMPED
    assert all(O.solve(s, 1, x, damping=0.1) == X1 for x in (-10, -1, 0, 1, 10))
    got = [approx(O.solve(s, 2, x, damping=0.1), X2[0]) for x in (-5, -1, -0.1, 0)] + \
          [approx(O.solve(s, 2, x, damping=0.1), X2[1]) for x in (0.1, 1, 5)]
    assert got == [True, True, True, False, True, True, True]
    assert all(O.solve(s, 3, x, damping=0.1) == X3 for x in (-1, 0, 1, 5, 7, 10))
    got = [approx(O.solve(s, 4, x, damping=0.1), X4[0]) for x in (-10, -1.5, -1, 0)] + \
          [approx(O.solve(s, 4, x, damping=0.1), X4[1]) for x in (1, 1.5, 5)]
    assert got == [True, True, True, False, True, True, True]
    assert approx(O.solve(s, 5, -5, damping=0.1, pa=1, pb=-2), -math.sqrt(2))


def test_bisection():
    s = O.BISECTION
    for a, b in ((-1000, 1000), (-100, 1), (-10, 0)):
        assert abs(O.solve(s, 1, a, b) - X1) <= 1e-10
    assert abs(O.solve(s, 2, -1000, 0) - X2[0]) <= 1e-10
    assert abs(O.solve(s, 2, -10, math.sqrt(2) - 0.1) - X2[0]) <= 1e-10
    assert abs(O.solve(s, 2, 0, 1000) - X2[1]) <= 1e-10
    assert approx(O.solve(s, 3, -10000, 10000), X3)
    for a, b in ((-1000, 0), (-10, 0.9), (0, 1000)):
        x = O.solve(s, 4, a, b)
        assert abs(1 / (1 + x * x) - 0.5) <= 1e-10
    assert approx(O.solve(s, 5, -100, 0, pa=1, pb=-2), -math.sqrt(2))
