"""The double-float arithmetic of the mixed-precision integrator and thermostat chain
(moltwister_gb300/csrc/md_device.cuh: two_sum, fast_two_sum, df_add, df_addq, df_mul, df_fix,
frac32_df, df_exp_chain, df_exp_tiny), restated operation for operation in IEEE binary32 on the
CPU (numpy float32 with correctly rounded operations; FMA through exact rationals), against exact
arithmetic.  Pins the error bounds the design relies on: about 2^-47 relative for sums and products,
exact conversion of fixed-point forces, box fractions within one unit of round(x 2^32 / L) modulo
2^32, exponentials within 1e-14 relative.  No GPU."""
from fractions import Fraction as Fr

import numpy as np
import pytest

f32 = np.float32


def fadd(a, b): return f32(f32(a) + f32(b))
def fsub(a, b): return f32(f32(a) - f32(b))
def fmul(a, b): return f32(f32(a) * f32(b))
def fma(a, b, c): return f32(float(Fr(float(a)) * Fr(float(b)) + Fr(float(c))))   # see note below
# float(Fraction) rounds the exact value to binary64 and f32 then to binary32; the double rounding
# differs from a single rounding only when the binary64 result lies exactly halfway between two
# floats, which the random operands below do not produce.


def two_sum(a, b):
    s = fadd(a, b)
    bb = fsub(s, a)
    return s, fadd(fsub(a, fsub(s, bb)), fsub(b, bb))


def fast_two_sum(a, b):
    s = fadd(a, b)
    return s, fsub(b, fsub(s, a))


def df_add(a, b):
    s = two_sum(a[0], b[0])
    t = two_sum(a[1], b[1])
    u = fast_two_sum(s[0], fadd(s[1], t[0]))
    return fast_two_sum(u[0], fadd(u[1], t[1]))


def df_addq(a, b):
    s = two_sum(a[0], b[0])
    return fast_two_sum(s[0], fadd(s[1], fadd(a[1], b[1])))


def df_mul(a, b):
    p = fmul(a[0], b[0])
    c = fma(a[1], b[0], fmul(a[0], b[1]))
    e = fma(a[0], b[0], -p)
    return fast_two_sum(p, fadd(e, c))


def df_mul_f(a, b):
    p = fmul(a[0], b)
    return fast_two_sum(p, fma(a[1], b, fma(a[0], b, -p)))


def df_of(x):
    h = f32(x)
    return h, f32(x - float(h))


def exact(a):
    return Fr(float(a[0])) + Fr(float(a[1]))


def df_fix(q):
    a, b = q >> 22, q & 0x3FFFFF
    return two_sum(fmul(f32(a), f32(0.0625)), fmul(f32(b), f32(2.0 ** -26)))


def frac32_df(x, conv):
    y = df_mul(x, conv)
    k = np.rint(fmul(y[0], f32(2.0 ** -32)))
    t = fsub(y[0], fmul(k, f32(2.0 ** 32)))
    ti = np.rint(t)
    r = fadd(fsub(t, ti), y[1])
    return (int(ti) + int(np.rint(r))) % 2 ** 32


SIXTH = (f32(float.fromhex("0x1.555556p-3")), f32(-float.fromhex("0x1.555556p-28")))


def df_exp_chain(x):
    xf = x[0]
    t = fma(xf, f32(1 / 40320), f32(1 / 5040))
    t = fma(t, xf, f32(1 / 720))
    t = fma(t, xf, f32(1 / 120))
    t = fma(t, xf, f32(1 / 24))
    x2f = fmul(xf, xf)
    tail = fmul(t, fmul(x2f, x2f))
    a = df_addq(df_mul(x, SIXTH), (f32(0.5), f32(0)))
    b = df_addq(df_mul(df_mul(x, x), a), (tail, f32(0)))
    return df_addq(df_addq((f32(1), f32(0)), x), b)


def df_exp_tiny(x):
    xf = x[0]
    tail = fmul(fmul(xf, xf), fmul(xf, fma(xf, f32(1 / 24), f32(1 / 6))))
    x2h = df_mul(x, (fmul(f32(0.5), x[0]), fmul(f32(0.5), x[1])))
    return df_addq(df_addq((f32(1), f32(0)), x), df_addq(x2h, (tail, f32(0))))


RNG = np.random.default_rng(12)


@pytest.mark.parametrize("op", ["add", "addq", "mul"])
def test_sums_and_products(op):
    worst = 0.0
    for _ in range(600):
        a = df_of(RNG.uniform(-50, 50))
        b = df_of(RNG.uniform(-1, 1) * 10.0 ** RNG.integers(-4, 2))
        if op == "mul":
            got, ref, scale = df_mul(a, b), exact(a) * exact(b), abs(exact(a) * exact(b))
        else:
            got = df_add(a, b) if op == "add" else df_addq(a, b)
            ref = exact(a) + exact(b)
            scale = abs(exact(a) + exact(b)) if op == "add" else abs(exact(a)) + abs(exact(b))
        worst = max(worst, float(abs(exact(got) - ref) / scale))
        assert abs(float(got[1])) <= abs(float(np.spacing(got[0]))) / 2 * (1 + 1e-6)   # normalised
    assert worst < 2.0 ** -46, worst


def test_fixed_point_forces_convert_exactly():
    for _ in range(2000):
        q = int(RNG.integers(-(2 ** 45), 2 ** 45))
        assert exact(df_fix(q)) == Fr(q, 2 ** 26)


def test_box_fractions_within_one_unit():
    L = 95.63
    conv = df_of(2.0 ** 32 / L)
    for _ in range(2000):
        x = RNG.uniform(-0.6 * L, 0.6 * L)
        X = df_of(x)
        want = round(exact(X) * 2 ** 32 / Fr(L)) % 2 ** 32
        d = (frac32_df(X, conv) - want + 2 ** 31) % 2 ** 32 - 2 ** 31
        assert abs(d) <= 1


@pytest.mark.parametrize("fn,r", [(df_exp_chain, 2.0 ** -5), (df_exp_tiny, 2.0 ** -10)])
def test_exponentials(fn, r):
    import math
    worst = 0.0
    for x in np.concatenate([RNG.uniform(-r, r, 400), [r, -r, 1e-9, -1e-9, 0.0]]):
        X = df_of(x)
        v = exact(fn(X))
        xe = float(exact(X))
        # e^x to ~1e-30 from the Taylor series in exact rationals
        ref = sum(Fr(xe) ** k / math.factorial(k) for k in range(16))
        worst = max(worst, float(abs(v - ref) / ref))
    assert worst < 1e-14, worst
