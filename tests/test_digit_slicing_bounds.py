"""The integer arithmetic behind the tensor-core FP64 emulation (no GPU): a numpy / Python-integer
restatement of the digit slicing and recombination of fem_2d_gb300/csrc/ozaki.cu, checking the bounds
its kernels rely on. The kernels themselves are checked against FP64 products on the GPU
(test_gpu_ozaki.py); this file checks that the scheme they implement is exact where it claims to be.

- digits8: A = (mant << 3) >> (E - ex) holds 56 bits, split into eight 7-bit digits d_s with
  A = sum_s d_s 2^(49 - 7 s); a value is sum_s d_s 2^(E - 1029 - 7 s) up to less than 2^(E - 1078);
- every FP32 digit-sum accumulator of an MMA chain stays an exact integer below 2^24 (K = 128 terms
  for the Gram chunk and the block-update chunk, K = 64 for an operator-product item);
- the int64 halves T_hi (groups 0..3) and T_lo (groups 4..7) and the fused integer
  T_hi 2^SH + round(T_lo 2^(SH - 28)) stay below 2^63 for each kernel's SH, and the fused integer is
  within 2^-(SH + 1) of T_hi + T_lo 2^-28;
- one emulated dot product lands within the stated truncation of the exact one.
"""
from fractions import Fraction

import numpy as np

K_DIGITS = 8
SH = {"gram": 20, "gemm": 19, "spmm": 20}   # kFuseGram, kFuseGemm, kFuseSpmm
K_TERMS = {"gram": 128, "gemm": 2 * 128, "spmm": 64}   # terms summed into one T_hi / T_lo pair


def biased_exp(v):
    return (np.float64(v).view(np.uint64) >> np.uint64(52)).astype(np.int64) & 0x7FF


def digits8(v, E):
    """The eight signed digits of v relative to the biased exponent E (ozaki.cu digits8)."""
    bits = int(np.float64(v).view(np.uint64))
    ex = (bits >> 52) & 0x7FF
    shift = E - ex
    mant = (bits & ((1 << 52) - 1)) | (1 << 52)
    A = 0 if (ex == 0 or shift > 55) else ((mant << 3) >> shift)
    sign = -1 if bits >> 63 else 1
    return [sign * ((A >> (49 - 7 * s)) & 0x7F) for s in range(K_DIGITS)], A


def fuse(th, tl, sh):
    """ozaki.cu fuse_digit_sums: arithmetic shifts on int64 (Python ints floor like them)."""
    return (th << sh) + ((tl + (1 << (27 - sh))) >> (28 - sh))


def npairs(g):
    return min(g, 7) - max(0, g - 7) + 1


def test_digits_reconstruct_the_value():
    rng = np.random.default_rng(0)
    for scale in (1e-300, 1e-8, 1.0, 3.7e5, 1e300):
        x = rng.standard_normal(64) * scale
        E = int(max(biased_exp(v) for v in x))
        for v in x:
            d, A = digits8(v, E)
            assert all(abs(q) <= 127 for q in d)
            assert A == sum(abs(q) << (49 - 7 * s) for s, q in enumerate(d))
            approx = sum(Fraction(q) * Fraction(2) ** (E - 1029 - 7 * s) for s, q in enumerate(d))
            assert abs(Fraction(float(v)) - approx) < Fraction(2) ** (E - 1078)


def test_accumulators_are_exact_in_fp32():
    for k in (64, 128):
        for g in range(K_DIGITS):
            assert npairs(g) * k * 127 * 127 < 2 ** 24


def test_fused_integers_fit_int64():
    for name, k in K_TERMS.items():
        chunks = max(1, k // 128)
        per = min(k, 128)
        th = chunks * sum(npairs(g) * per * 127 ** 2 << (7 * (3 - g)) for g in range(4))
        tl = chunks * sum(npairs(g) * per * 127 ** 2 << (7 * (7 - g)) for g in range(4, 8))
        assert th < 2 ** 44 and tl < 2 ** 47, name
        assert abs(fuse(th, tl, SH[name])) < 2 ** 63 and abs(fuse(-th, -tl, SH[name])) < 2 ** 63, name


def test_fused_rounding_error():
    rng = np.random.default_rng(1)
    for sh in set(SH.values()):
        for _ in range(2000):
            th = int(rng.integers(-(2 ** 43), 2 ** 43))
            tl = int(rng.integers(-(2 ** 46), 2 ** 46))
            exact = Fraction(th) + Fraction(tl, 2 ** 28)
            err = abs(Fraction(fuse(th, tl, sh), 2 ** sh) - exact)
            assert err <= Fraction(1, 2 ** (sh + 1))


def test_emulated_dot_product():
    """x . y through digits, exact digit-sum groups (s + t <= 7 kept), T_hi / T_lo, the fused integer
    and one FP64 conversion, against the exact rational dot product: within the dropped pairs
    (s + t >= 8) and the final rounding."""
    rng = np.random.default_rng(2)
    k = 128
    for trial in range(20):
        x = rng.standard_normal(k) * 10.0 ** rng.integers(-3, 4)
        y = rng.standard_normal(k) * 10.0 ** rng.integers(-3, 4)
        Ex = int(max(biased_exp(v) for v in x))
        Ey = int(max(biased_exp(v) for v in y))
        dx = [digits8(v, Ex)[0] for v in x]
        dy = [digits8(v, Ey)[0] for v in y]
        acc = [0] * K_DIGITS
        for a, b in zip(dx, dy):
            for s in range(K_DIGITS):
                for t in range(K_DIGITS - s):
                    acc[s + t] += a[s] * b[t]
        assert all(abs(v) < 2 ** 24 for v in acc)
        th = sum(acc[g] << (7 * (3 - g)) for g in range(4))
        tl = sum(acc[g] << (7 * (7 - g)) for g in range(4, 8))
        got = float(fuse(th, tl, SH["gram"])) * 2.0 ** (Ex + Ey - 2079 - SH["gram"])
        exact = sum(Fraction(float(a)) * Fraction(float(b)) for a, b in zip(x, y))
        scale = Fraction(2) ** (Ex - 1023) * Fraction(2) ** (Ey - 1023)   # >= max|x| max|y| / 4
        # dropped pairs: at most k terms of 9 pairs below 2^-49 of the scale each; plus the roundings
        assert abs(Fraction(got) - exact) <= k * 2 * Fraction(2) ** -49 * scale + abs(exact) * Fraction(2) ** -52, trial
