"""The BF16 hi + lo operand splits of the surrogate network's tensor-core
kernels (conv_tc, conv_weight_tc), restated in numpy on the CPU: how much of
an FP32 value the split keeps, that products of the parts are exact in
FP32, and the accuracy of a weight gradient formed from hi.hi + hi.lo +
lo.hi (the three MMAs conv_weight_tc issues) against exact sums. The GPU
kernels themselves are checked against the numpy restatement in
tests/test_gpu_surrogate.py."""
import numpy as np

from oracle import cnn_oracle as co


def split2(a):
    """hi = bf16(a), lo = bf16(a - hi), in FP32 (round to nearest even)."""
    a = np.asarray(a, dtype=np.float32)
    hi = co.bf16_round(a)
    lo = co.bf16_round((a - hi).astype(np.float32))
    return hi, lo


def test_split_keeps_sixteen_significant_bits():
    rng = np.random.default_rng(0)
    a = (rng.standard_normal(100000) * 10.0 ** rng.uniform(-6, 6, 100000)).astype(np.float32)
    hi, lo = split2(a)
    rel = np.abs((hi.astype(np.float64) + lo) - a) / np.abs(a)
    assert rel.max() <= 2.0 ** -16
    # The parts are BF16 values: their low 16 bits are zero.
    assert not (hi.view(np.uint32) & 0xFFFF).any() and not (lo.view(np.uint32) & 0xFFFF).any()


def test_products_of_parts_are_exact_in_fp32():
    rng = np.random.default_rng(1)
    x = rng.standard_normal(50000).astype(np.float32)
    w = co.bf16_round(rng.standard_normal(50000).astype(np.float32))
    hi, lo = split2(x)
    for part in (hi, lo):
        p32 = (part * w).astype(np.float32)
        assert np.array_equal(p32.astype(np.float64), part.astype(np.float64) * w)


def test_three_product_weight_gradient_accuracy():
    # dW[o][c] = sum_n dy[n][o] x[n][c] over 20000 positions with heavy
    # cancellation (random signs), as conv_weight_tc forms it from the
    # split operands (hi.hi + hi.lo + lo.hi; exact products, exact sums
    # here), against the exact FP64 sum of the FP32 inputs.
    rng = np.random.default_rng(2)
    n, o, c = 20000, 16, 45
    dy = (rng.standard_normal((n, o)) * 1e-3).astype(np.float32)
    x = rng.standard_normal((n, c)).astype(np.float32)
    exact = dy.astype(np.float64).T @ x.astype(np.float64)
    dh, dl = split2(dy)
    xh, xl = split2(x)
    d = lambda a: a.astype(np.float64)
    approx = d(dh).T @ d(xh) + d(dh).T @ d(xl) + d(dl).T @ d(xh)
    rel = np.linalg.norm(approx - exact) / np.linalg.norm(exact)
    assert rel <= 1e-5, rel
