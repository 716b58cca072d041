"""The exact BF16 slice representation on the CPU: the digit arithmetic of the staging slicer
(FP32 pairs cut into balanced base-64 digits in FP32 arithmetic) restated with numpy float32,
its reconstruction error, the digit ranges that keep the group sums exact, and the truncation
bounds of the correction precisions (3 and 4 slices).  No GPU: these are the bounds the
exact-slice contractions rely on."""
from fractions import Fraction

import numpy as np
import pytest

KMAX = 3072  # K terms of one CTA's range in the exact-slice contractions


def digits_pair(hi, lo, e, ns=6):
    """Balanced base-64 digits q_t of F ~ (hi + lo) 2^(36 - e), in float32 arithmetic, as the
    slicer computes them: the scale as two powers of two, the low part joining at t = 3."""
    f32 = np.float32
    sc = 36 - e
    s1 = sc >> 1
    s2 = sc - s1
    f1, f2 = f32(2.0 ** s1), f32(2.0 ** s2)
    r = f32(f32(f32(hi) * f1) * f2)
    l = f32(f32(f32(lo) * f1) * f2)
    q = []
    for t in range(ns):
        if t == 3:
            r = f32(r + l)
        sh = 30 - 6 * t
        qt = f32(np.rint(f32(r * f32(2.0 ** -sh))))
        r = f32(r - f32(qt * f32(2.0 ** sh)))  # exact: q 2^sh is exact and |r - q 2^sh| <= 2^(sh-1)
        q.append(int(qt))
    return q


def value(q, e, ns=None):
    """sum_t q_t 2^(-6(t+1)) 2^e, exactly."""
    ns = len(q) if ns is None else ns
    return sum(Fraction(q[t]) * Fraction(2) ** (e - 6 * (t + 1)) for t in range(ns))


def random_pairs(rng, n):
    """FP32 pairs hi + lo (|lo| below half an ulp of hi) spread over a row's dynamic range,
    with the row exponent e: max |hi + lo| < 2^e."""
    e = int(rng.integers(-40, 40))
    mags = 2.0 ** rng.uniform(-45, 0, n) * rng.choice([-1.0, 1.0], n)
    hi = (mags * 2.0 ** e * 0.999).astype(np.float32)
    ulp = np.spacing(np.abs(hi)).astype(np.float64)
    lo = (rng.uniform(-0.5, 0.5, n) * ulp).astype(np.float32)
    hi[:3] = [0.0, np.float32(2.0 ** e * 0.9999), -np.float32(2.0 ** e * 0.75)]
    lo[:3] = 0.0
    return hi, lo, e


@pytest.mark.parametrize("seed", range(6))
def test_digits_reconstruct_to_the_fixed_point_grid(seed):
    rng = np.random.default_rng(seed)
    hi, lo, e = random_pairs(rng, 400)
    for h, l in zip(hi, lo):
        q = digits_pair(h, l, e)
        exact = Fraction(float(h)) + Fraction(float(l))
        # |F - v 2^(36 - e)| <= 1/2 + 2^-6 in units of 2^(e - 36)
        assert abs(value(q, e) - exact) <= (Fraction(1, 2) + Fraction(1, 64)) * Fraction(2) ** (e - 36)
        # balanced digits: the leading one within 64, the rest within 32 (the group-sum bounds)
        assert abs(q[0]) <= 64 and all(abs(x) <= 32 for x in q[1:])


@pytest.mark.parametrize("ns,bound_exp", [(3, -19), (4, -25)])
def test_correction_precision_truncation(ns, bound_exp):
    """Reading only the leading ns slices cuts each operand at 2^(e - 6 ns - 1) (plus the last
    digit's rounding of the full representation, 2^(e - 36))."""
    rng = np.random.default_rng(100 + ns)
    hi, lo, e = random_pairs(rng, 300)
    for h, l in zip(hi, lo):
        q = digits_pair(h, l, e)
        exact = Fraction(float(h)) + Fraction(float(l))
        err = abs(value(q, e, ns) - exact)
        assert err <= Fraction(2) ** (e + bound_exp) + Fraction(2) ** (e - 35)


def test_group_sums_stay_exact_in_fp32():
    """Products of the same digit weight g = t + u are integers times one power of two; with
    |q_0| <= 64, |q_t| <= 32 and at most KMAX terms per CTA, the sums of groups 0, 1, 2 stay
    below 2^24, so the FP32 accumulators of those groups are exact."""
    q0, qt = 64, 32
    g0 = q0 * q0 * KMAX
    g1 = 2 * q0 * qt * KMAX
    g2 = (2 * q0 * qt + qt * qt) * KMAX
    assert max(g0, g1, g2) < 2 ** 24
    assert KMAX % 32 == 0  # whole K blocks of 32 per CTA range
