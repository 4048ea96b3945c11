"""The arithmetic of the Ozaki slicing used by the tensor-core ROM kernels, restated on the
CPU (IEEE FP32 through numpy, Python integers for the 54-bit form) and checked against
the bounds the kernels rely on.  Method: Ozaki, Ogita, Oishi, Rump, "Error-free
transformations of matrix multiplication by using fast routines of matrix
multiplication and its applications", Numer. Algorithms 59 (2012).

* 6 slices (double-float state): digits 0-2 from the hi word, the lo word folded in at
  weight 2^18, digits 3-5 from that sum; each digit is the nearest integer of 64 h,
  taken by adding and subtracting 1.5 * 2^23.  Digit 0 lies in [-64, 64], the others in
  [-32, 32], and the expansion is within 2^-37 + 2^-43 of h + l.
* 9 slices (FP64 state): the value as a 54-bit fixed-point integer, cut into balanced
  base-64 digits (digit 0 in [-64, 64], digits 1-7 in [-32, 32], the last in [-32, 32))
  that sum back to it exactly.
* The FP32 accumulators hold every diagonal sum exactly for K <= 1024.
"""
from fractions import Fraction

import numpy as np

F32 = np.float32
MAGIC = F32(1.5 * 2.0 ** 23)


def round_int(x):
    """Nearest integer of |x| < 2^22, ties to even, in FP32 (two additions)."""
    return F32(F32(x + MAGIC) - MAGIC)


def six_digits(h, l):
    h, l = F32(h), F32(l)
    out = []
    for s in range(6):
        if s == 3:
            h = F32(h + F32(l * F32(2.0 ** 18)))  # l * 2^18 is exact: a fused multiply-add rounds the same
        th = F32(h * F32(64.0))
        a = round_int(th)
        h = F32(th - a)
        out.append(a)
    return out


def double_float_samples(rng, n):
    """Pairs (h, l): h FP32 with |h| < 1 over many binades, |l| <= ulp(h) / 2."""
    e = rng.integers(-40, 0, n)
    h = (rng.uniform(-1, 1, n) * 2.0 ** (e + 1)).astype(np.float32)
    h = np.clip(h, np.nextafter(F32(-1), F32(0)), np.nextafter(F32(1), F32(0)))
    ulp = np.spacing(np.abs(h)).astype(np.float64)
    l = (rng.uniform(-0.5, 0.5, n) * ulp).astype(np.float32)
    edge = np.array([np.nextafter(F32(1), F32(0)), -np.nextafter(F32(1), F32(0)), F32(0.5), F32(-0.5),
                     F32(1.0 / 128), F32(0.0), F32(2.0 ** -30)], np.float32)
    return np.concatenate([h, edge]), np.concatenate([l, np.zeros(len(edge), np.float32)])


def test_round_int_matches_rint():
    rng = np.random.default_rng(1)
    x = np.concatenate([rng.uniform(-70, 70, 20000), np.arange(-66, 67) + 0.5, np.arange(-66, 67)]).astype(np.float32)
    got = np.array([round_int(v) for v in x], np.float32)
    assert np.array_equal(got, np.rint(x))  # equal as values (a -0 from rint compares equal to +0)


def test_six_digit_slices_ranges_and_error():
    rng = np.random.default_rng(2)
    h, l = double_float_samples(rng, 4000)
    for hv, lv in zip(h, l):
        a = six_digits(hv, lv)
        assert all(float(d).is_integer() for d in a)
        assert abs(a[0]) <= 64 and all(abs(d) <= 32 for d in a[1:])
        # the upper half of the FP32 bits is the BF16 of the digit (low 16 bits zero)
        assert all((np.float32(d).view(np.uint32) & 0xFFFF) == 0 for d in a)
        v = Fraction(float(hv)) + Fraction(float(lv))
        approx = sum(Fraction(int(d)) / Fraction(64) ** (s + 1) for s, d in enumerate(a))
        # the remainder after six digits (<= 2^-37) plus the rounding of the fold (<= 2^-43)
        assert abs(v - approx) <= Fraction(1, 2 ** 37) + Fraction(1, 2 ** 43), (hv, lv)


def fixed54(x, beta):
    """round(x * 2^(54 - beta)) for |x| < 2^beta, ties away from zero on the magnitude."""
    m, e = np.frexp(x)  # x = m * 2^e, 0.5 <= |m| < 1
    mant = int(abs(m) * 2 ** 53)  # exact: 53 bits
    sh = int(e) - 53 + 54 - beta
    v = mant << sh if sh >= 0 else (mant + (1 << (-sh - 1))) >> (-sh)
    return -v if x < 0 else v


def nine_digits(v):
    out = []
    for s in range(9):
        if s == 8:
            out.append(v)
            break
        b = 6 * (8 - s)
        a = (v + (1 << (b - 1))) >> b
        v -= a << b
        out.append(a)
    return out


def test_nine_digit_slices_ranges_and_exactness():
    rng = np.random.default_rng(3)
    for _ in range(4000):
        beta = int(rng.integers(-60, 60))
        x = float(rng.uniform(-1, 1)) * 2.0 ** beta * float(rng.choice([1.0, 0.5, 2.0 ** -20]))
        v = fixed54(x, beta)
        assert abs(v) <= 2 ** 54
        a = nine_digits(v)
        assert abs(a[0]) <= 64 and all(-32 <= d <= 32 for d in a[1:8]) and -32 <= a[8] < 32, a
        assert sum(d * 64 ** (8 - s) for s, d in enumerate(a)) == v
        # 54 bits: the fixed-point value is within half a unit of x * 2^(54 - beta)
        assert abs(Fraction(x) * Fraction(2) ** (54 - beta) - v) <= Fraction(1, 2)


def test_diagonal_sums_exact_in_fp32():
    """Diagonal d holds d + 1 slice pairs; first slices in [-64, 64], the others in
    [-32, 32]: every partial sum stays below 2^24 for K <= 1024, in both forms."""
    K = 1024
    for S in (6, 9):
        for d in range(S):
            pairs = [(s, d - s) for s in range(d + 1)]
            bound = sum((64 if s == 0 else 32) * (64 if t == 0 else 32) for s, t in pairs) * K
            assert bound < 2 ** 24, (S, d, bound)
    assert 2 * 64 * 32 * K + 7 * 32 * 32 * K == 11 * 2 ** 20
    # 9-slice combination in 64-bit integers: H = D0 2^12 + D1 2^6 + D2 (exact as an FP64),
    # L = sum_{d>=3} D_d 2^(6(8-d)) (one rounding to FP64), Y = H 2^36 + L
    bound = [sum((64 if s == 0 else 32) * (64 if d - s == 0 else 32) for s in range(d + 1)) * K for d in range(9)]
    H = bound[0] * 2 ** 12 + bound[1] * 2 ** 6 + bound[2]
    L = sum(bound[d] * 2 ** (6 * (8 - d)) for d in range(3, 9))
    assert H < 2 ** 36 and L < 2 ** 54  # each fits an int64; H is exact in FP64


def two_sum(a, b):
    s = F32(a + b)
    z = F32(s - a)
    return s, F32(F32(a - F32(s - z)) + F32(b - z))


def test_six_diagonal_combine_accuracy():
    """The 6-slice epilogue's combination of the diagonal sums D_d (integers below 2^24 held
    in FP32): the terms D_d 2^(6(5-d)) are exact in FP32 and are added smallest first with
    TwoSum, the errors collected in one FP32 word; hi + lo matches the exact integer sum
    to 2^-47 of the sum of the terms' magnitudes (2^-48 relative when nothing cancels)."""
    rng = np.random.default_rng(5)
    worst = Fraction(0)
    for trial in range(20000):
        mag = 2 ** int(rng.integers(0, 24))
        D = [int(x) for x in rng.integers(-mag, mag, 6)]
        if trial % 7 == 0:
            D[0] = 0
        if trial % 11 == 0:
            D[:3] = [0, 0, 0]
        if trial % 13 == 0:  # cancellation between the leading terms
            D[1] = -64 * D[0] + int(rng.integers(-3, 4))
            if abs(D[1]) >= 2 ** 24:
                D[1] = 0
        s, e = F32(D[5]), F32(0)
        for d in range(4, -1, -1):
            s, err = two_sum(s, F32(F32(D[d]) * F32(2.0 ** (6 * (5 - d)))))
            e = F32(e + err)
        h = F32(s + e)
        l = F32(e - F32(h - s))
        terms = [D[d] * 2 ** (6 * (5 - d)) for d in range(6)]
        err = abs(Fraction(float(h)) + Fraction(float(l)) - sum(terms))
        scale = sum(abs(t) for t in terms)
        assert err <= Fraction(scale, 2 ** 47), (D, float(h), float(l))
        if scale and abs(sum(terms)) * 2 >= scale:
            worst = max(worst, err / abs(sum(terms)))
    assert worst <= Fraction(1, 2 ** 48) * Fraction(11, 10)
