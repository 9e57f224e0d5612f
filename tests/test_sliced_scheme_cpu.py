"""The arithmetic of the FP64-accurate sliced products, restated on the host
in exact integer arithmetic (the splitting scheme of Ozaki, Ogita, Oishi &
Rump, Numer. Algorithms 59, 2012, as the tensor-core kernels use it):

* a value v with |v| < 2^e is truncated to the 55-bit integer
  trunc(v 2^(55-e)) and cut into eight balanced base-128 digits d_1..d_8,
  |d_s| <= 64 (BF16 holds them exactly), error below 2^(e-55);
* for each level g = s + t (2..9) the digit products summed over K <= 512
  terms stay below 2^24 in magnitude, so FP32 accumulation of a level is
  exact;
* sum_g L_g 2^-7g times the two scales equals the product of the truncated
  operands up to the dropped levels g >= 10: the truncation (below
  2^-54 K 2^(ea+ex)) and the dropped levels (below 2^-53 K 2^(ea+ex)) keep
  the result within 2^-50 K 2^(ea+ex) of the exact product, 2^ea and 2^ex
  bounding the operands' magnitudes (a normwise FP64-accurate product).
No GPU is involved: these are the properties the kernels' comments state."""
import math
from fractions import Fraction

import numpy as np

S = 8
BIAS = 64 * (((1 << 49) - 1) // 127)  # 64 at each of the seven low base-128 positions


def exponent_of(vmax: float) -> int:
    """Smallest e with |v| < 2^e for the largest |v| (0 for zero)."""
    if vmax <= 0.0:
        return 0
    return math.frexp(vmax)[1]


def digits(v: float, e: int) -> list[int]:
    fixed = int(math.ldexp(v, 55 - e))  # exact: a power-of-two scaling, then truncation toward zero
    y = fixed + BIAS
    d = [((y >> (7 * (S - 1 - s))) & 127) - 64 for s in range(1, S)]
    return [y >> 49] + d


def value_of(d: list[int], e: int) -> int:
    """The 55-bit integer the digits stand for."""
    return sum(ds * 128 ** (S - 1 - s) for s, ds in enumerate(d))


def test_digits_are_balanced_and_reconstruct_the_truncated_value():
    rng = np.random.default_rng(5)
    vals = np.concatenate([rng.standard_normal(2000) * 10.0 ** rng.integers(-8, 8, 2000),
                           [0.0, -0.0, 1.0, -1.0, 0.5, 2.0 ** -40, -(2.0 ** 30)]])
    e = exponent_of(float(np.abs(vals).max()))
    for v in vals:
        d = digits(float(v), e)
        assert all(abs(x) <= 64 for x in d), (v, d)
        fixed = value_of(d, e)
        assert fixed == int(math.ldexp(float(v), 55 - e))
        # truncation error below 2^(e - 55)
        assert abs(float(v) - math.ldexp(fixed, e - 55)) < math.ldexp(1.0, e - 55)


def levels(a: np.ndarray, x: np.ndarray, ea: int, ex: int) -> np.ndarray:
    """L_g (g = 2..9) of sum_k a_k x_k from the digits, as exact integers."""
    ad = np.array([digits(float(v), ea) for v in a], dtype=np.int64).T  # [slice][k]
    xd = np.array([digits(float(v), ex) for v in x], dtype=np.int64).T
    out = np.zeros(8, dtype=np.int64)
    for s in range(1, S + 1):
        for t in range(1, S + 1):
            g = s + t
            if g <= 9:
                out[g - 2] += int(np.dot(ad[s - 1], xd[t - 1]))
    return out


def test_level_sums_are_exact_in_fp32_up_to_512_terms():
    rng = np.random.default_rng(6)
    for K in (216, 512):
        a = rng.standard_normal(K)
        x = rng.standard_normal(K)
        L = levels(a, x, exponent_of(float(np.abs(a).max())), exponent_of(float(np.abs(x).max())))
        assert np.abs(L).max() < 2 ** 24  # every partial sum is an integer FP32 holds exactly
        # worst case: every digit at its bound
        worst = levels(np.full(K, -0.999999999), np.full(K, 0.999999999), 0, 0)
        assert np.abs(worst).max() <= 8 * K * 64 * 64 <= 2 ** 24


def test_sliced_product_is_fp64_accurate_normwise():
    rng = np.random.default_rng(7)
    for K in (27, 216, 512):
        for scale_a, scale_x in ((1.0, 1.0), (1e-6, 3e4), (1e8, 1e-9)):
            a = rng.standard_normal(K) * scale_a
            x = rng.standard_normal(K) * scale_x
            ea, ex = exponent_of(float(np.abs(a).max())), exponent_of(float(np.abs(x).max()))
            L = levels(a, x, ea, ex)
            # sum_g L_g 2^-7g, then the scales 2^(ea + 1) 2^(ex + 1)
            acc = sum(math.ldexp(float(L[g - 2]), -7 * g) for g in range(9, 1, -1))
            got = math.ldexp(acc, ea + ex + 2)
            exact = sum(Fraction(float(ai)) * Fraction(float(xi)) for ai, xi in zip(a, x))
            bound = Fraction(K) * Fraction(2) ** (ea + ex - 50)
            assert abs(Fraction(got) - exact) <= bound, (K, scale_a, scale_x, got, float(exact))
            # and, for these random operands, within 2^-48 of sum_k |a_k x_k|
            norm = sum(abs(Fraction(float(ai)) * Fraction(float(xi))) for ai, xi in zip(a, x))
            assert abs(Fraction(got) - exact) <= Fraction(2) ** -48 * norm
