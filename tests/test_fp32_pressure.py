"""The FP32 path's pressure recovery (cons2prim_cell<float> in
amr2d_mhd_gb300/csrc/stage.cuh), restated with numpy on the CPU: the sums of
squares and |m|^2/rho as FP32 hi + lo pairs (Dekker's exact product through
an FMA, Knuth's TwoSum, the reciprocal corrected by its FMA residual), then
E - (|m|^2/rho + |B|^2)/2 and gamma - 1 in FP64.  An FP32 FMA is emulated
exactly: the product of two FP32 values is exact in FP64, and so is its sum
with an FP32 value of the same magnitude, so one rounding to FP32 gives the
FMA's result.  The test bounds the error of the recovered pressure against
an exact rational evaluation on states from gas- to magnetically dominated
and at high Mach numbers."""
from fractions import Fraction

import numpy as np

F = np.float32


def fma32(a, b, c):
    return F(np.float64(a) * np.float64(b) + np.float64(c))


def two_sum(a, b):
    s = F(a + b)
    v = F(s - a)
    return s, F(F(a - F(s - v)) + F(b - v))


def sum_sq3(a, b, c):
    pa, pb, pc = F(a * a), F(b * b), F(c * c)
    ea, eb, ec = fma32(a, a, -pa), fma32(b, b, -pb), fma32(c, c, -pc)
    s1, t1 = two_sum(pa, pb)
    s2, t2 = two_sum(s1, pc)
    return s2, F(F(F(ea + eb) + ec) + F(t1 + t2))


def pressure_df(u, g):
    """Mode 2 of cons2prim_cell<float> (the default)."""
    ir = F(F(1) / u[0])
    rl = F(fma32(-u[0], ir, F(1)) * ir)
    mh, ml = sum_sq3(u[1], u[2], u[3])
    bh, bl = sum_sq3(u[5], u[6], u[7])
    kh = F(mh * ir)
    kl = F(fma32(mh, ir, -kh) + F(F(mh * rl) + F(ml * ir)))
    return (g - 1) * (np.float64(u[4]) - 0.5 * ((np.float64(kh) + np.float64(kl)) +
                                                (np.float64(bh) + np.float64(bl))))


def pressure_exact(u, g):
    q = [Fraction(float(x)) for x in u]
    m2 = q[1] ** 2 + q[2] ** 2 + q[3] ** 2
    b2 = q[5] ** 2 + q[6] ** 2 + q[7] ** 2
    return Fraction(g) - 1, q[4] - (m2 / q[0] + b2) / 2, q[4] + (m2 / q[0] + b2) / 2


def test_pressure_recovery_error_bound():
    rng = np.random.default_rng(5)
    g = 5.0 / 3.0
    worst = 0.0
    for n in range(3000):
        rho = 10.0 ** rng.uniform(-3, 3)
        v = rng.standard_normal(3) * 10.0 ** rng.uniform(-2, 2)     # up to Mach ~100
        B = rng.standard_normal(3) * 10.0 ** rng.uniform(-3, 1.5)
        p = 10.0 ** rng.uniform(-4, 2)
        u = np.array([rho, *(rho * v), 0.0, *B], dtype=F)
        ke = 0.5 * float(sum(float(x) ** 2 for x in u[1:4])) / float(u[0])
        me = 0.5 * float(sum(float(x) ** 2 for x in u[5:8]))
        u[4] = F(p / (g - 1) + ke + me)
        gm1, diff, scale = pressure_exact(u, g)
        got = pressure_df(u, np.float64(g))
        ref = float(gm1 * diff)
        # error relative to the magnitude of the subtracted terms, where the
        # FP64 recovery rounds as well
        err = abs(got - ref) / float(gm1 * scale)
        worst = max(worst, err)
    assert worst < 2.0 ** -43, worst
