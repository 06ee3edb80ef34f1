"""The split assembly's arithmetic, emulated exactly on the CPU.

The tensor-core kernel (cdet_split.cu) evaluates G = sum_ab C[a][b] T_a(u)
T_b(v) of one coefficient block as eight balanced 8-bit digits of C (the
block scaled by 2^-E) against seven of the Q56 basis T_b(v), accumulates the
digit products of each level tau = t + t' in FP32, and finishes in 64- and
128-bit integers. These tests restate that arithmetic with Python integers
(the FP32 steps rounded as the kernel rounds them; the level-8 accumulator,
which sums fractional products, modelled as one rounding of its exact sum)
and check the claims the design rests on:

* every accumulator level tau = 2..7 stays within 2^24 in magnitude for any
  coefficients and any v, so its FP32 sums are exact integers;
* the digits reconstruct the coefficients and the basis values exactly;
* the products the kernel does not issue (a coefficient digit before its K
  step's lead, or a row beyond its level's rows) are zero;
* with the kernel's arithmetic paths, chosen from the same slicing marks (Q62
  chains of stride 8; Q30 chains where only basis digits 1 and 2, or only
  the levels 7 and 8, are read), the result is within 1e-15 of the block's
  largest coefficient of the exact series (50-digit evaluation) and at or
  below the FP64 Clenshaw sum's error, for slowly and for quickly decaying
  coefficients (the latter with a round-off floor, as the Green tables
  have), including degrees above 128 cut into sub-blocks.
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


def q62_table(x):
    """T_0..T_8(x) in Q62 by the stride-1 recurrence (cheb_table8)."""
    xf = fixed(x, 62)
    t = [1 << 62, xf]
    for k in range(1, 8):
        t.append(cheb_step(xf, t[k], t[k - 1]))
    return t


def q30(x):
    """Q62 -> Q30, rounded (q62_to_q30)."""
    return (x + (1 << 31)) >> 32


def chain30_step(w30, cur, prev):
    """round(2 T_8 T_m / 2^30) - T_{m-8} in Q30 (ChebChain30)."""
    return ((w30 * cur + (1 << 28)) >> 29) - prev


def basis_chains(x, n, switch=None):
    """T_0..T_{n-1}(x) as the kernel's chains of stride 8 give them: chain r
    holds degrees r, r + 8, ..., started from (T_{8-r}, T_r), each step
    T_{m+8} = 2 T_8 T_m - T_{m-8} in Q62. From degree `switch` on (a multiple
    of 8) each chain continues in Q30 from its converted state. Returns
    [(value, is_q30)]."""
    t = q62_table(x)
    w30 = q30(t[8])
    out = [None] * n
    for r in range(8):
        prev, cur = t[8 - r], t[r]
        in30 = False
        for m in range(r, n, 8):
            if switch is not None and not in30 and m >= switch:
                prev, cur, in30 = q30(prev), q30(cur), True
            out[m] = (cur, in30)
            if in30:
                prev, cur = cur, chain30_step(w30, cur, prev)
            else:
                prev, cur = cur, cheb_step(t[8], cur, prev)
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


def slicing_marks(C, e):
    """slice_blocks' marks of one sub-block: the first nonzero digit of every
    coefficient, each 16-column K step's lead (first nonzero digit over the
    step) and the level rows (per level tau = 2..8, 1 + the last row with a
    digit t <= tau - 1; at tau = 8 any digit)."""
    nu, nv = C.shape
    first = np.full((nu, nv), 9)
    for a in range(nu):
        for b in range(nv):
            q = coefficient_digits(C[a, b], e)
            nz = [t + 1 for t, d in enumerate(q) if d != 0]
            if nz:
                first[a, b] = nz[0]
    leads = [int(first[:, 16 * k:16 * k + 16].min()) for k in range((nv + 15) // 16)]
    row_lead = first.min(axis=1)
    rows = []
    for tau in range(2, 9):
        reach = 8 if tau == 8 else tau - 1
        hit = [a for a in range(nu) if row_lead[a] <= reach]
        rows.append(max(hit) + 1 if hit else 0)
    return first, leads, rows


def step_lead(leads, ks):
    return 1 if ks == 0 else min(leads[ks], 8)


def tail_kstep(leads):
    """The first K step from which every lead is 6 or more (tail_kstep)."""
    first = len(leads)
    for ks in range(len(leads) - 1, 0, -1):
        if step_lead(leads, ks) < 6:
            break
        first = ks
    return first


def pass_geometry(rows):
    """pass_geom: one pass when the levels' 16-rounded rows fit 496 columns,
    else two over rows 0..63 and 64..127; per pass (row0, n per level)."""
    up = [(r + 15) // 16 * 16 for r in rows]
    if sum(up) <= 496:
        return [(0, up)]
    return [(p * 64, [(min(max(r - p * 64, 0), 64) + 15) // 16 * 16 for r in rows]) for p in (0, 1)]


def split_eval(C, u, v, paths=None):
    """The kernel's value of one lookup: per sub-block of 128 rows x 128
    columns the levels P_tau (tau = 2..7 exact, tau = 8 with the pre-scaled
    eighth coefficient digit, rounded to FP32), then per row either the 64-bit
    fixed-point combination times the Q62 T_a(u), rounded to 2^-55, or (rows
    only levels 7 and 8 reach) the folded FP32 value times the Q30 T_a(u),
    the exact sum over rows and sub-blocks, one final rounding. The basis
    T_b(v) is Q62 before the sub-block's tail K step and Q30 from it on. Every
    digit product is formed; the ones the kernel leaves out are zero
    (test_skipped_products_are_zero). `paths`, when given, counts the rows
    and basis values each path takes."""
    nu, nv = C.shape
    mx = float(np.max(np.abs(C)))
    e = math.frexp(mx)[1] if mx > 0 else 0
    A = [[coefficient_digits(C[a, b], e) for b in range(nv)] for a in range(nu)]
    total = 0
    levels_max = [0] * 6
    for r0 in range(0, nu, 128):
        for k0 in range(0, nv, KSUB):
            rows_rng = range(r0, min(nu, r0 + 128))
            cols = range(k0, min(nv, k0 + KSUB))
            _, leads, lrows = slicing_marks(C[r0:r0 + 128, k0:k0 + KSUB], e)
            ks_tail = tail_kstep(leads)
            tv = basis_chains(v, k0 + 16 * len(leads), switch=k0 + 16 * ks_tail)
            B = {}
            for b in cols:
                val, in30 = tv[b]
                B[b] = basis_digits(val << 26 if in30 else (val + 32) >> 6)
                if paths is not None:
                    paths["basis_q30" if in30 else "basis_q62"] += 1
            P = {}
            for a in rows_rng:
                lev = [0] * 7
                p8 = Fraction(0)
                for b in cols:
                    qa, qb = A[a][b], B[b]
                    for t in range(1, 8):
                        for tp in range(1, 9 - t):
                            lev[t + tp - 2] += qa[t - 1] * qb[tp - 1]
                    p8 += Fraction(qa[7] * qb[0], 256)
                for l in range(6):
                    levels_max[l] = max(levels_max[l], abs(lev[l]))
                P[a] = (lev, fp32(lev[5]), fp32(Fraction(lev[6]) + p8))
            for row0, n in pass_geometry(lrows):
                c_tail = n[4]
                tu = basis_chains(u, r0 + row0 + 128, switch=r0 + row0 + c_tail)
                for c in range(max(n)):
                    a = r0 + row0 + c
                    if a not in P:
                        continue
                    lev, p7, p8 = P[a]
                    fold = int(np.rint(fp32(fp32(p8 * 2.0 ** -9) + p7 * 0.5)))
                    val, in30 = tu[a]
                    if c >= c_tail:  # only levels 7 and 8 reach this row
                        assert in30 and all(lev[l] == 0 for l in range(5))
                        total += (fold * val + (1 << 29)) >> 30
                    else:
                        w = sum(lev[l] << (39 - 8 * l) for l in range(5)) + fold
                        total += (w * val + (1 << 61)) >> 62
                    if paths is not None:
                        paths["rows_q30" if c >= c_tail else "rows_q62"] += 1
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


def green_like(rng, d, fast):
    """Coefficients decaying like a smooth function's expansion with random
    signs: slowly, or quickly down to a round-off floor of 1e-16 of the
    largest (the shape of the Green tables' blocks)."""
    if not fast:
        decay = np.exp(-0.08 * np.add.outer(np.arange(d), np.arange(d)))
        return rng.standard_normal((d, d)) * decay * 10.0 ** rng.uniform(-3, 1)
    decay = np.exp(-0.9 * np.add.outer(np.arange(d), np.arange(d)))
    return (rng.standard_normal((d, d)) * decay + 1e-16 * rng.standard_normal((d, d))) * 10.0 ** rng.uniform(-3, 1)


@pytest.mark.parametrize("d,fast", [(16, False), (64, False), (160, False), (64, True), (160, True)])
def test_split_matches_exact_series(d, fast):
    mpmath = pytest.importorskip("mpmath")
    mpmath.mp.dps = 50
    rng = np.random.default_rng(100 + d + 7 * fast)
    worst_split = worst_fp64 = 0.0
    paths = {"basis_q62": 0, "basis_q30": 0, "rows_q62": 0, "rows_q30": 0}
    for trial in range(3 if d > 100 else 6):
        C = green_like(rng, d, fast)
        u = float(rng.uniform(-1, 1)) if trial % 3 else 0.9999
        v = 1.0 if trial % 2 == 0 else float(rng.uniform(-1, 1))
        val, mx, levels_max = split_eval(C, u, v, paths)
        assert max(levels_max) <= 1 << 24
        tu = [mpmath.cos(a * mpmath.acos(u)) for a in range(d)]
        tv = [mpmath.cos(b * mpmath.acos(v)) for b in range(d)]
        exact = mpmath.fsum(tu[a] * mpmath.fsum(mpmath.mpf(float(C[a, b])) * tv[b] for b in range(d))
                            for a in range(d))
        fp64 = clenshaw([clenshaw(list(C[a]), v) for a in range(d)], u)
        worst_split = max(worst_split, abs(val - float(exact)) / mx)
        worst_fp64 = max(worst_fp64, abs(fp64 - float(exact)) / mx)
    print(f"degree {d} fast={fast}: split {worst_split:.2e}, FP64 Clenshaw {worst_fp64:.2e} (of max |C|), {paths}")
    assert worst_split <= 1e-15
    assert worst_split <= max(worst_fp64, 5e-16)
    if fast:  # the 32-bit paths were taken
        assert paths["basis_q30"] > 0 and paths["rows_q30"] > 0


def test_skipped_products_are_zero():
    """A quickly decaying block: every digit product the kernel skips (a
    coefficient digit before its K step's lead, or a row beyond its level's
    rows) is exactly zero, and the skipping removes most of the work."""
    rng = np.random.default_rng(7)
    d = 64
    C = green_like(rng, d, True)
    e = math.frexp(float(np.max(np.abs(C))))[1]
    first, leads, rows = slicing_marks(C, e)
    issued = skipped = 0
    for a in range(d):
        digits = [coefficient_digits(C[a, b], e) for b in range(d)]
        for b in range(d):
            lead = step_lead(leads, b // 16)
            for t in range(1, 9):
                for tp in ([1] if t == 8 else range(1, 9 - t)):
                    tau = 8 if t == 8 else t + tp
                    if t < lead or a >= rows[tau - 2]:
                        skipped += 1
                        assert digits[b][t - 1] == 0, (a, b, t)
                    else:
                        issued += 1
    assert rows == sorted(rows)  # levels widen with tau
    assert skipped > issued
