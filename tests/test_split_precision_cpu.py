"""The split-precision arithmetic of the tensor-core GEMM modes, emulated in numpy (no GPU).

TF32X3 splits an FP32 value x into hi = tf32(x) (round to nearest, ties away: cvt.rna) and
lo = tf32(x - hi), and keeps hi*hi + hi*lo + lo*hi.  BF16X3 splits it into hi = bf16(x),
mid = bf16(x - hi), lo = bf16(x - hi - mid) (round to nearest even: cvt.rn) and keeps the six
products of order <= 2.  These tests pin the claims the kernels rely on: the terms carry the
FP32 value (exactly for BF16X3), and the kept products reach FP32-level accuracy."""
import numpy as np


def _tf32(x):
    """Round float32 to TF32 (10 explicit mantissa bits), ties away from zero."""
    b = np.asarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    b = (b + 0x1000) & 0xFFFFE000
    return b.astype(np.uint32).view(np.float32)


def _bf16(x):
    """Round float32 to bfloat16 (7 explicit mantissa bits), ties to even."""
    b = np.asarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    b = (b + 0x7FFF + ((b >> 16) & 1)) & 0xFFFF0000
    return b.astype(np.uint32).view(np.float32)


def _operands(rng, n):
    # magnitudes in [1, 2) after the kernels' power-of-two scaling, both signs
    return (rng.uniform(1.0, 2.0, n) * rng.choice([-1.0, 1.0], n)).astype(np.float32)


def test_bf16_three_terms_carry_the_fp32_value_exactly():
    rng = np.random.default_rng(0)
    x = _operands(rng, 200000)
    hi = _bf16(x)
    mid = _bf16(x - hi)
    lo = _bf16(x - hi - mid)
    assert np.array_equal(hi.astype(np.float64) + mid + lo, x.astype(np.float64))


def test_tf32_two_terms_carry_22_bits():
    rng = np.random.default_rng(1)
    x = _operands(rng, 200000)
    hi = _tf32(x)
    lo = _tf32(x - hi)
    err = np.abs(hi.astype(np.float64) + lo - x) / np.abs(x)
    assert err.max() <= 2.0 ** -21


def test_kept_products_reach_fp32_accuracy():
    """Per element product, relative to |x y|: TF32X3 drops lo*lo (~2^-22), BF16X3 drops
    the order-3 and order-4 terms (~2^-24); both under the FP32 accumulation level of a
    long dot product."""
    rng = np.random.default_rng(2)
    x = _operands(rng, 100000)
    y = _operands(rng, 100000)
    exact = x.astype(np.float64) * y
    xh, yh = _tf32(x), _tf32(y)
    xl, yl = _tf32(x - xh), _tf32(y - yh)
    t3 = xh.astype(np.float64) * yh + xh.astype(np.float64) * yl + xl.astype(np.float64) * yh
    assert (np.abs(t3 - exact) / np.abs(exact)).max() <= 2.0 ** -20
    xs = [_bf16(x)]
    xs.append(_bf16(x - xs[0]))
    xs.append(_bf16(x - xs[0] - xs[1]))
    ys = [_bf16(y)]
    ys.append(_bf16(y - ys[0]))
    ys.append(_bf16(y - ys[0] - ys[1]))
    b6 = sum(xs[i].astype(np.float64) * ys[j] for i in range(3) for j in range(3) if i + j <= 2)
    assert (np.abs(b6 - exact) / np.abs(exact)).max() <= 2.0 ** -22


def test_split_dot_products_match_fp64_to_fp32_level():
    """A K = 512 dot product accumulated in FP32 from the kept split products agrees with
    the FP64 dot product to the tolerance the GPU tests use (2e-6 of the operands' scale)."""
    rng = np.random.default_rng(3)
    K = 512
    a = rng.standard_normal((64, K)).astype(np.float32)
    b = rng.standard_normal((K, 64)).astype(np.float32)
    exact = a.astype(np.float64) @ b.astype(np.float64)
    ah, bh = _tf32(a), _tf32(b)
    al, bl = _tf32(a - ah), _tf32(b - bh)
    acc = (ah @ bl + al @ bh + ah @ bh).astype(np.float32)  # FP32 accumulation
    scale = np.abs(exact).max()
    assert np.abs(acc - exact).max() <= 2e-6 * scale
