"""The split assembly's arithmetic, emulated exactly on the CPU.

The tensor-core kernel (cdet_split.cu) evaluates G = sum_ab C[a][b] T_a(u)
T_b(v) of one coefficient block as eight balanced 8-bit digits of C (the
block scaled by 2^-E) against seven of the Q56 basis T_b(v), accumulates the
digit products of each level tau = t + t' in FP32, and finishes in 64- and
128-bit integers. These tests restate that arithmetic with Python integers
(the FP32 steps rounded as the kernel rounds them) and check the claims the
design rests on:

* every accumulator level tau = 2..7 stays within 2^24 in magnitude for any
  coefficients and any v, so its FP32 sums are exact integers;
* the digits reconstruct the coefficients and the basis values exactly;
* the result is within 1e-15 of the block's largest coefficient of the exact
  series (50-digit evaluation), at or below the FP64 Clenshaw sum's error,
  including a degree above 128 cut into sub-blocks of 128 columns.
"""
import math
from fractions import Fraction

import numpy as np
import pytest

KSUB = 128  # K columns of one sub-block
M64 = (1 << 64) - 1
DIGIT_BIAS = 0x0100808080808080


def s64(x):
    x &= M64
    return x - (1 << 64) if x >> 63 else x


def fixed(x, frac):
    """round(|x| 2^frac) with halves away from zero, signed (fixed_from_double)."""
    v = abs(Fraction(x)) * (1 << frac)
    r = math.floor(v + Fraction(1, 2))
    return -r if x < 0 else r


def cheb_step(w, t, tprev):
    """round(2 w t) in Q62 minus tprev, modulo 2^64 (cheb_step_q62)."""
    return s64(((w * t + (1 << 60)) >> 61) - tprev)


def basis_stride2(x, n):
    """T_0..T_{n-1}(x) in Q62 by the stride-2 recurrence of the basis producers."""
    xf = fixed(x, 62)
    w = cheb_step(xf, xf, 1 << 62)
    out = [0] * n
    for h in (0, 1):
        prev, cur = (w, 1 << 62) if h == 0 else (xf, xf)
        for b in range(h, n, 2):
            out[b] = cur
            prev, cur = cur, cheb_step(w, cur, prev)
    return out


def basis_stride4(x, n):
    """T_0..T_{n-1}(x) in Q62 by the stride-4 recurrence of the epilogue."""
    one = 1 << 62
    xf = fixed(x, 62)
    t2 = cheb_step(xf, xf, one)
    t3 = cheb_step(xf, t2, xf)
    t4 = cheb_step(xf, t3, t2)
    starts = {0: (t4, one), 1: (t3, xf), 2: (t2, t2), 3: (xf, t3)}
    out = [0] * n
    for r in range(4):
        prev, cur = starts[r]
        for a in range(r, n, 4):
            out[a] = cur
            prev, cur = cur, cheb_step(t4, cur, prev)
    return out


def coefficient_digits(c, e):
    """The eight balanced digits of c 2^-e (slice_blocks): q_1 in [-256, 256],
    q_2..q_8 in [-128, 128]; c 2^-e = sum_t q_t 2^-8t + remainder."""
    r = math.ldexp(float(c), -e)
    q = []
    for _ in range(8):
        scaled = r * 256.0
        d = float(np.rint(scaled))
        r = scaled - d
        q.append(int(d))
    return q


def basis_digits(x56):
    """The seven digits of a Q56 basis value (digit_pair): the top field minus
    256, then six bytes minus 128; x56 = sum_t d_t 2^(56 - 8t)."""
    y = x56 + DIGIT_BIAS
    return [(y >> 48) - 256] + [((y >> (8 * (7 - t))) & 255) - 128 for t in range(2, 8)]


def fp32(x):
    return float(np.float32(x))


def split_eval(C, u, v):
    """The kernel's value of one lookup: per K chunk of 128 columns the levels
    P_tau (tau = 2..7 exact, tau = 8 with the pre-scaled eighth coefficient
    digit, rounded to FP32), their 64-bit fixed-point combination, the Q62 u
    basis products rounded to 2^-55, the exact sum over rows and chunks, one
    final rounding."""
    nu, nv = C.shape
    mx = float(np.max(np.abs(C)))
    e = math.frexp(mx)[1] if mx > 0 else 0
    A = [[coefficient_digits(C[a, b], e) for b in range(nv)] for a in range(nu)]
    tv = basis_stride2(v, nv)
    B = [basis_digits((tv[b] + 32) >> 6) for b in range(nv)]
    tu = basis_stride4(u, nu)
    total = 0
    levels_max = [0] * 6
    for k0 in range(0, nv, KSUB):
        cols = range(k0, min(nv, k0 + KSUB))
        for a in range(nu):
            P = [0] * 7
            P8 = Fraction(0)
            for b in cols:
                qa, qb = A[a][b], B[b]
                for t in range(1, 8):
                    for tp in range(1, 9 - t):
                        P[t + tp - 2] += qa[t - 1] * qb[tp - 1]
                P8 += Fraction(qa[7] * qb[0], 256)
            for lev in range(6):
                levels_max[lev] = max(levels_max[lev], abs(P[lev]))
            p7 = fp32(P[5])
            p8 = fp32(Fraction(P[6]) + P8)
            w = sum(P[lev] << (39 - 8 * lev) for lev in range(5))
            w += int(np.rint(fp32(fp32(p8 * 2.0 ** -9) + p7 * 0.5)))
            total += (w * tu[a] + (1 << 61)) >> 62
    return float(Fraction(total) * Fraction(2) ** (e - 55)), mx, levels_max


def clenshaw(c, x):
    b1 = b2 = 0.0
    for k in range(len(c) - 1, 0, -1):
        b1, b2 = c[k] + 2.0 * x * b1 - b2, b1
    return c[0] + b1 * x - b2


def test_level_bounds_hold_for_any_digits():
    """Worst case over all digit values: |P_tau| <= K * sum over the level's
    pairs of |q_t| |q'_t'| with K = 128."""
    amax = [256] + [128] * 7
    bmax = [256] + [128] * 6
    for tau in range(2, 8):
        bound = KSUB * sum(amax[t - 1] * bmax[tau - t - 1] for t in range(1, tau))
        assert bound <= 1 << 24, (tau, bound)


def test_digits_reconstruct():
    rng = np.random.default_rng(5)
    for c in rng.standard_normal(200) * 10.0 ** rng.integers(-6, 6, 200):
        e = math.frexp(abs(c))[1]
        q = coefficient_digits(c, e)
        assert abs(q[0]) <= 256 and max(abs(d) for d in q[1:]) <= 128
        approx = sum(Fraction(d, 256 ** (t + 1)) for t, d in enumerate(q))
        assert abs(approx - Fraction(math.ldexp(c, -e))) <= Fraction(1, 2 ** 65)
    for x in list(rng.uniform(-1, 1, 200)) + [-1.0, 1.0, 0.0]:
        x56 = (fixed(x, 62) + 32) >> 6
        d = basis_digits(x56)
        assert abs(d[0]) <= 256 and max(abs(t) for t in d[1:]) <= 128
        assert sum(dt << (56 - 8 * (t + 1)) for t, dt in enumerate(d)) == x56


@pytest.mark.parametrize("d", [16, 64, 160])
def test_split_matches_exact_series(d):
    mpmath = pytest.importorskip("mpmath")
    mpmath.mp.dps = 50
    rng = np.random.default_rng(100 + d)
    worst_split = worst_fp64 = 0.0
    for trial in range(3 if d > 100 else 6):
        # decaying like a smooth function's expansion, with random signs
        decay = np.exp(-0.08 * np.add.outer(np.arange(d), np.arange(d)))
        C = rng.standard_normal((d, d)) * decay * 10.0 ** rng.uniform(-3, 1)
        u = float(rng.uniform(-1, 1)) if trial % 3 else 0.9999
        v = 1.0 if trial % 2 == 0 else float(rng.uniform(-1, 1))
        val, mx, levels_max = split_eval(C, u, v)
        assert max(levels_max) <= 1 << 24
        tu = [mpmath.cos(a * mpmath.acos(u)) for a in range(d)]
        tv = [mpmath.cos(b * mpmath.acos(v)) for b in range(d)]
        exact = mpmath.fsum(tu[a] * mpmath.fsum(mpmath.mpf(float(C[a, b])) * tv[b] for b in range(d))
                            for a in range(d))
        fp64 = clenshaw([clenshaw(list(C[a]), v) for a in range(d)], u)
        worst_split = max(worst_split, abs(val - float(exact)) / mx)
        worst_fp64 = max(worst_fp64, abs(fp64 - float(exact)) / mx)
    print(f"degree {d}: split {worst_split:.2e}, FP64 Clenshaw {worst_fp64:.2e} (of max |C|)")
    assert worst_split <= 1e-15
    assert worst_split <= max(worst_fp64, 5e-16)
