"""The arithmetic of the split-BF16 cell product, restated on the host: each
FP32 operand value x is split into x_hi = bf16(x) and x_lo = bf16(x - x_hi)
(round to nearest even), and a product a x is formed as
a_hi x_hi + a_hi x_lo + a_lo x_hi with FP32 accumulation (the lo.lo term is
dropped).  Per product the error is about 2^-16 of |a x| (hi and lo carry 8
significant bits each, and the dropped term is 2^-16 of the product); over a
K-term cell product with FP32 accumulation the result stays within 1e-4 of
the FP64 product relative to the max-norm of the output block (the tolerance
the GPU parity tests use); 5e-6 for the random operands here.  No GPU is
involved."""
import numpy as np


def bf16(x: np.ndarray) -> np.ndarray:
    """Round float32 values to bfloat16 (nearest, ties to even), returned as float32."""
    u = np.asarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    rounded = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return rounded.astype(np.uint32).view(np.float32)


def split(x: np.ndarray):
    hi = bf16(x)
    lo = bf16(np.asarray(x, dtype=np.float32) - hi)
    return hi, lo


def test_bf16_rounding_known_values():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 2 ** -7, 1.0 + 3 * 2 ** -8, -2.5, 0.0], dtype=np.float32)
    # 1 + 2^-8 is a tie: to even (1.0); 1 + 3 * 2^-8 is a tie: to even (1 + 2^-6)
    np.testing.assert_array_equal(bf16(x), np.array([1.0, 1.0, 1.0 + 2 ** -7, 1.0 + 2 ** -6, -2.5, 0.0],
                                                    dtype=np.float32))


def test_split_represents_fp32_values_to_16_bits():
    rng = np.random.default_rng(8)
    x = (rng.standard_normal(100000) * 10.0 ** rng.integers(-5, 5, 100000)).astype(np.float32)
    hi, lo = split(x)
    rel = np.abs((hi.astype(np.float64) + lo.astype(np.float64)) - x.astype(np.float64)) / np.abs(x)
    assert rel.max() <= 2.0 ** -16


def test_split_bf16_cell_product_within_the_parity_tolerance():
    rng = np.random.default_rng(9)
    for nd, m in ((125, 64), (216, 128)):
        A = rng.standard_normal((nd, nd))          # one cell matrix (FP64 at upload)
        X = rng.standard_normal((nd, m)).astype(np.float32)
        ah, al = split(A.astype(np.float32))
        xh, xl = split(X)
        # three products, FP32 accumulation over K in order
        Y = np.zeros((nd, m), dtype=np.float32)
        for k in range(nd):
            Y = Y + (np.outer(ah[:, k], xh[k]) + np.outer(ah[:, k], xl[k]) + np.outer(al[:, k], xh[k])).astype(
                np.float32)
        ref = A @ X.astype(np.float64)
        err = np.abs(Y.astype(np.float64) - ref).max() / np.abs(ref).max()
        assert err <= 1e-4
        assert err >= 1e-7  # not FP32-exact: the split's 16 bits show
