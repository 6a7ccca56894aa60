"""The double-float arithmetic of the mixed solver's outer residual
(stzpp_gb300/csrc/residual_df.cu), restated with numpy float32 operations
and checked against exact rational arithmetic: the error bounds the kernel's
design rests on.  The kernel itself is checked on the GPU against the FP64
residual (tests/test_gpu_parity.py::test_double_float_residual_matches_fp64).

  * split_double: x = hi + lo, hi the FP32 truncation of x, lo the rounded
    remainder, from the bits of x: |hi + lo - x| <= 2^-48 |x|;
  * a row b - sum a_t x_t with exact products (Dekker) and a two-sum high
    part (Knuth): error <= 2^-42 of sum |a_t x_t|, so residuals ten digits
    below the terms keep their leading digits;
  * the paired form of a symmetric row (opposite neighbours summed as a
    double-float pair, one product per pair): the same bound."""
from fractions import Fraction

import numpy as np

F32 = np.float32


def split(x):
    """split_double of residual_df.cu on an array of float64."""
    x = np.asarray(x, dtype=np.float64)
    u = x.view(np.uint64)
    uh = (u >> np.uint64(32)).astype(np.uint32)
    ul = (u & np.uint64(0xFFFFFFFF)).astype(np.uint32)
    sign = uh & np.uint32(0x80000000)
    e = ((uh >> np.uint32(20)) & np.uint32(0x7FF)).astype(np.int64) - 1023
    ok = (e >= -126) & (e <= 127)
    ec = np.clip(e, -126, 127)
    hb = sign | ((ec + 127).astype(np.uint32) << np.uint32(23)) | ((uh & np.uint32(0xFFFFF)) << np.uint32(3)) | (ul >> np.uint32(29))
    hi = hb.view(np.float32)
    m = (ul & np.uint32(0x1FFFFFFF)).astype(np.float32)   # rounded to 24 bits
    s = ec - 52
    s1 = np.trunc(s / 2).astype(np.int64)   # C integer division truncates toward zero
    s2 = s - s1
    p1 = ((s1 + 127).astype(np.uint32) << np.uint32(23)).view(np.float32)
    p2 = ((s2 + 127).astype(np.uint32) << np.uint32(23)).view(np.float32)
    lo = (m * p1) * p2
    lo = np.where(sign != 0, -lo, lo)
    assert ok.all(), "test values stay inside FP32's normal range"
    return hi, lo.astype(np.float32)


def sub_prod(sh, sl, ah, al, xh, xl):
    """df_sub_prod: (sh, sl) -= (ah + al)(xh + xl), float32 throughout; the
    exact product error fma(ah, xh, -p) is ah*xh - p evaluated in float64,
    where both are exact."""
    p = F32(ah * xh)
    ep = F32(np.float64(ah) * np.float64(xh) - np.float64(p))
    s = F32(sh - p)
    bv = F32(s - sh)
    err = F32(F32(sh - F32(s - bv)) - F32(p + bv))
    cross = F32(np.float64(ah) * np.float64(xl) + np.float64(F32(al * xh)))
    sl = F32(F32(sl + F32(err - ep)) - cross)
    return s, sl


def test_split_error_bound():
    rng = np.random.default_rng(0)
    x = rng.standard_normal(200000) * np.exp2(rng.integers(-70, 100, 200000))
    x[::5] = x[::5].astype(np.float32)   # values exact in FP32: lo must be 0
    hi, lo = split(x)
    rec = hi.astype(np.float64) + lo.astype(np.float64)
    assert np.all(np.abs(rec - x) <= np.exp2(-48) * np.abs(x))
    assert np.all(np.abs(hi.astype(np.float64)) <= np.abs(x)) and np.all(np.sign(hi) == np.sign(x))
    assert np.all(lo[::5] == 0)


def test_row_error_bound_with_cancellation():
    rng = np.random.default_rng(1)
    worst = 0.0
    for _ in range(300):
        nt = 45
        a = rng.standard_normal(nt) * 65536.0
        x = rng.standard_normal(nt) * 1e-3
        exact_sum = sum(Fraction(float(ai)) * Fraction(float(xi)) for ai, xi in zip(a, x))
        mag = sum(abs(Fraction(float(ai)) * Fraction(float(xi))) for ai, xi in zip(a, x))
        # b - sum a x about 1e-12 of the terms: the residual at convergence
        b = float(exact_sum + Fraction(float(rng.standard_normal() * 1e-12)) * mag)
        r_exact = Fraction(b) - exact_sum
        sh, sl = split([b])
        sh, sl = sh[0], sl[0]
        ah, al = split(a)
        xh, xl = split(x)
        for t in range(nt):
            sh, sl = sub_prod(sh, sl, ah[t], al[t], xh[t], xl[t])
        r = F32(sh + sl)
        err = abs(Fraction(float(r)) - r_exact) / mag
        worst = max(worst, float(err))
        # the leading digits of a residual 1e-12 below the terms survive
        if abs(r_exact) > Fraction(1, 10**12) * mag / 4:
            assert abs(Fraction(float(r)) - r_exact) <= abs(r_exact) / 4
    assert worst <= 2.0 ** -42, worst


def add_pair(xh1, xl1, xh2, xl2):
    """df_add: (xh1 + xl1) + (xh2 + xl2) with the high parts' sum exact
    (Knuth's two-sum) and every rounding error in the float low part."""
    s = F32(xh1 + xh2)
    bv = F32(s - xh1)
    err = F32(F32(xh1 - F32(s - bv)) + F32(xh2 - bv))
    return s, F32(F32(xl1 + xl2) + err)


def test_paired_row_error_bound_with_cancellation():
    """The paired form of a symmetric row: the two opposite neighbours of
    each coefficient summed as a double-float pair first, then one product
    per pair.  Its error stays within 2^-42 of the row's sum |a x| (over the
    unpaired terms), as the unpaired form's does, so residuals ten digits
    below the terms keep their leading digits."""
    rng = np.random.default_rng(2)
    worst = 0.0
    for _ in range(300):
        npair = 21
        a = rng.standard_normal(npair) * 65536.0
        x1 = rng.standard_normal(npair) * 1e-3
        x2 = rng.standard_normal(npair) * 1e-3
        exact_sum = sum(Fraction(float(ai)) * (Fraction(float(u)) + Fraction(float(v)))
                        for ai, u, v in zip(a, x1, x2))
        mag = sum(abs(Fraction(float(ai)) * Fraction(float(u))) + abs(Fraction(float(ai)) * Fraction(float(v)))
                  for ai, u, v in zip(a, x1, x2))
        b = float(exact_sum + Fraction(float(rng.standard_normal() * 1e-12)) * mag)
        r_exact = Fraction(b) - exact_sum
        sh, sl = split([b])
        sh, sl = sh[0], sl[0]
        ah, al = split(a)
        h1, l1 = split(x1)
        h2, l2 = split(x2)
        for t in range(npair):
            ph, pl = add_pair(h1[t], l1[t], h2[t], l2[t])
            sh, sl = sub_prod(sh, sl, ah[t], al[t], ph, pl)
        r = F32(sh + sl)
        err = abs(Fraction(float(r)) - r_exact) / mag
        worst = max(worst, float(err))
        if abs(r_exact) > Fraction(1, 10**12) * mag / 4:
            assert abs(Fraction(float(r)) - r_exact) <= abs(r_exact) / 4
    assert worst <= 2.0 ** -42, worst
