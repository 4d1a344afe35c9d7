"""Oracle helpers the GPU parity tests rely on (test infrastructure)."""

import numpy as np

from oracle import interp


def test_window_of_a_contiguous_program():
    text = "ccir 1 ew\no 1 6\np 1 6 00000000\nx 0 2 1 0\nu exp 1\nr 2\n"
    x = np.linspace(0.1, 2, 6).astype(np.float32)
    full = interp.evaluate(text, [x])
    part = interp.evaluate(interp.window_text(text, 3), [x[2:5]])
    assert np.array_equal(part, full[2:5])


def test_supplied_transcendentals_replace_the_correctly_rounded_ones():
    """A device's exp/log/tanh values can stand in for the correctly rounded
    ones; every other operation keeps the oracle's rounding."""
    text = "ccir 1 ew\no 1 4\np 1 4 00000000\nx 0 2 1 0\nu log 1\nb mul 2 1\nr 3\n"
    x = np.array([0.5, 1.0, 2.7182817, 4.0], np.float32)
    up = lambda op, a: np.nextafter(getattr(np, op)(a.astype(np.float64)).astype(np.float32), np.float32(np.inf))
    got = interp.evaluate(text, [x], transcendental=up)
    want = (up("log", x) * x).astype(np.float32)
    assert np.array_equal(got.view(np.int32), want.view(np.int32))
    assert not np.array_equal(got, interp.evaluate(text, [x]))


def test_fma32_is_correctly_rounded():
    """The oracle's fused multiply-add against exact rational arithmetic,
    including sums that cancel and sums whose binary64 rounding lands on a
    binary32 midpoint."""
    from fractions import Fraction
    r = np.random.RandomState(0)
    n = 4000
    a = (r.standard_normal(n) * np.exp2(r.randint(-30, 30, n))).astype(np.float32)
    b = (r.standard_normal(n) * np.exp2(r.randint(-30, 30, n))).astype(np.float32)
    c = np.where(r.rand(n) < 0.5, (-(a.astype(np.float64) * b)).astype(np.float32),
                 (r.standard_normal(n) * np.exp2(r.randint(-60, 60, n))).astype(np.float32))
    got = interp.fma32(a, b, c)
    for i in range(n):
        exact = Fraction(float(a[i])) * Fraction(float(b[i])) + Fraction(float(c[i]))
        f = np.float32(float(exact))
        near = [np.nextafter(f, np.float32(-np.inf)), f, np.nextafter(f, np.float32(np.inf))]
        want = min(near, key=lambda x: (abs(Fraction(float(x)) - exact), int(np.array(x, np.float32).view(np.int32)) & 1))
        assert got[i] == want, i


def test_fma_mode_contracts_product_operands():
    """p*q + c, c - p*q and p*q - r*s fuse the (left) product; a product that is
    not an operand of + or - rounds on its own."""
    text = ("ccir 1 ew\no 1 3\np 1 3 00000000\np 1 3 00000000\nx 0 2 1 0\nx 1 2 1 0\n"
            "b mul 2 3\nb add 4 2\nb sub 3 4\nb mul 2 2\nb sub 4 7\nb mul 5 6\nb add 9 8\nr 10\n")
    r = np.random.RandomState(3)
    x, y = r.standard_normal(3).astype(np.float32), r.standard_normal(3).astype(np.float32)
    got = interp.evaluate(text, [x, y], fma=True)
    f = interp.fma32
    n5 = f(x, y, x)                  # x*y + x
    n6 = f(-x, y, y)                 # y - x*y
    n8 = f(x, y, -(x * x))           # x*y - x*x (left product fused, right rounded)
    want = f(n5, n6, n8)             # (n5*n6) + n8: the product operand fuses
    assert np.array_equal(got.view(np.int32), want.view(np.int32))
