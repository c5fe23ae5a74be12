"""The CPU restatement of the surrogate network (oracle/cnn_oracle.py): its
hand-written backward pass against central finite differences of its own
forward pass, and the coarse map's transpose against its forward map."""
import numpy as np

from oracle import cnn_oracle as co


def test_parameter_count_matches_architecture():
    assert co.num_params() == (5 * 32 * 9 + 32) + (32 * 64 * 9 + 64) + (64 * 64 * 9 + 64) + \
        (64 * 4 * 9 + 4)


def test_bf16_rounding_ties_to_even():
    vals = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, 1.0 + 2 ** -9, -2.5, 0.0],
                    dtype=np.float32)
    out = co.bf16_round(vals)
    assert out[0] == 1.0
    assert out[1] == 1.0                    # tie -> even (1.0)
    assert out[2] == np.float32(1.0 + 4 * 2 ** -8)  # tie -> even (upper)
    assert out[3] == 1.0
    assert out[4] == -2.5 and out[5] == 0.0


def test_backward_matches_finite_differences():
    rng = np.random.default_rng(0)
    # Parameters exactly representable in BF16, so that the rounding does not
    # move under the small finite-difference steps of the biases only; the
    # weight entries are probed through the chain rule of the biases' layers.
    params = co.bf16_round(co.init_params(1)).astype(np.float64)
    offs, n = co.offsets()
    x = rng.standard_normal((3, 5, co.H, co.W))
    m_true = rng.standard_normal(3)
    g_true = rng.standard_normal((3, 3, co.H, co.W))
    loss, grad = co.loss_grad(params, x, m_true, g_true, 0.7, 1.3)
    assert grad.shape == (n,)
    # Biases (FP32, not rounded): central differences.
    for l in range(4):
        b0 = offs[l] + co.COUT[l] * co.CIN[l] * 9
        for k in rng.choice(co.COUT[l], size=min(4, co.COUT[l]), replace=False):
            i = b0 + k
            h = 1e-5  # small enough that no ReLU unit changes side
            p = params.copy(); p[i] += h
            lp, _ = co.loss_grad(p, x, m_true, g_true, 0.7, 1.3)
            p[i] -= 2 * h
            lm, _ = co.loss_grad(p, x, m_true, g_true, 0.7, 1.3)
            fd = (lp - lm) / (2 * h)
            assert abs(fd - grad[i]) <= 1e-4 * max(1.0, abs(fd)), (l, k, fd, grad[i])


def test_weight_gradient_matches_finite_differences_without_rounding(monkeypatch):
    # With the BF16 rounding switched off, every weight is differentiable.
    monkeypatch.setattr(co, "bf16_round", lambda a: np.asarray(a, dtype=np.float64))
    rng = np.random.default_rng(1)
    params = co.init_params(2).astype(np.float64)
    offs, n = co.offsets()
    x = rng.standard_normal((2, 5, co.H, co.W))
    m_true = rng.standard_normal(2)
    g_true = rng.standard_normal((2, 3, co.H, co.W))
    _, grad = co.loss_grad(params, x, m_true, g_true, 1.0, 1.0)
    for l in range(4):
        for k in rng.choice(co.COUT[l] * co.CIN[l] * 9, size=4, replace=False):
            i = offs[l] + k
            h = 1e-5
            p = params.copy(); p[i] += h
            lp, _ = co.loss_grad(p, x, m_true, g_true, 1.0, 1.0)
            p[i] -= 2 * h
            lm, _ = co.loss_grad(p, x, m_true, g_true, 1.0, 1.0)
            fd = (lp - lm) / (2 * h)
            assert abs(fd - grad[i]) <= 1e-6 * max(1.0, abs(fd)), (l, k, fd, grad[i])


def test_coarse_map_transpose_is_adjoint():
    rng = np.random.default_rng(3)
    nx, nz, npb, ncx, ncz = 60, 40, 5, 5, 3
    mean = rng.uniform(1, 2, (3, ncx, ncz))
    sigma = rng.uniform(0.1, 0.2, (3, ncx, ncz))
    z = rng.standard_normal((2, 3, ncx, ncz))
    f0 = co.coarse_to_fields(np.zeros_like(z), mean, sigma, nx, nz, npb)
    f = co.coarse_to_fields(z, mean, sigma, nx, nz, npb) - f0  # linear part
    g = rng.standard_normal(f.shape)
    gz = co.coarse_gradient(g, sigma, npb, ncx, ncz)
    assert np.isclose(np.sum(f * g), np.sum(z * gz), rtol=1e-12)
    # Partition of unity: a constant medium maps to the same constant.
    flat = co.coarse_to_fields(np.zeros((1, 3, ncx, ncz)), np.ones((3, ncx, ncz)) * 7.0,
                               sigma, nx, nz, npb)
    assert np.allclose(flat, 7.0)
