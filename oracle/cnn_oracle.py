"""CPU restatement (numpy, float64 arithmetic) of the surrogate network and
the coarse-to-grid parameter map of psvwave_gb300's Monte Carlo workload
(psvwave_gb300/csrc/psv_cnn.cu, psv_cnn.hpp). The reference has no learned
part, so this restates the project's own kernels. It is test infrastructure:
only tests/ may import it. Its own backward pass is checked against central
finite differences (tests/test_cnn_oracle.py), and the GPU kernels are
checked against it (tests/test_gpu_surrogate.py).

Network: four 3x3 convolutions over [5][20][10] inputs (3 parameter and 2
coordinate channels), channels 5-32-64-64-4, dilations 1, 2, 4, 1, zero
padding, ReLU after layers 1-3.
Weights are used rounded to BF16 (round to nearest even), as the GPU stores
them; biases stay FP32. Outputs: gradient map = channels 0..2, misfit = the
grid sum of channel 3. Loss = w_m mean_b (m - m*)^2 + w_g mean (g - g*)^2.
"""
import numpy as np

H, W = 20, 10
P = H * W
CIN = (5, 32, 64, 64)
COUT = (32, 64, 64, 4)
DIL = (1, 2, 4, 1)


def layer_size(l):
    return COUT[l] * CIN[l] * 9 + COUT[l]


def offsets():
    off, out = 0, []
    for l in range(4):
        out.append(off)
        off += layer_size(l)
    return out, off


def num_params():
    return offsets()[1]


def bf16_round(a):
    """Round float32 values to the nearest BF16 (ties to even), as float32."""
    a = np.ascontiguousarray(a, dtype=np.float32)
    bits = a.view(np.uint32).astype(np.uint64)
    rounded = ((bits + 0x7FFF + ((bits >> 16) & 1)) >> 16) << 16
    return (rounded & 0xFFFFFFFF).astype(np.uint32).view(np.float32)


def unpack(params):
    """[(w [cout][cin][3][3] as BF16 values, b [cout])] per layer, float64.
    The GPU keeps float32 parameters; pass them as float32 to match it."""
    params = np.asarray(params)
    offs, _ = offsets()
    layers = []
    for l in range(4):
        o = offs[l]
        nw = COUT[l] * CIN[l] * 9
        w = bf16_round(params[o:o + nw]).astype(np.float64).reshape(COUT[l], CIN[l], 3, 3)
        b = params[o + nw:o + nw + COUT[l]].astype(np.float64)
        layers.append((w, b))
    return layers


def init_params(seed=0):
    """He-style initial parameters (float32), biases zero."""
    rng = np.random.default_rng(seed)
    out = []
    for l in range(4):
        fan_in = CIN[l] * 9
        out.append((rng.standard_normal(COUT[l] * CIN[l] * 9) * np.sqrt(2.0 / fan_in)))
        out.append(np.zeros(COUT[l]))
    return np.concatenate(out).astype(np.float32)


def _pad(x, d):
    return np.pad(x, ((0, 0), (0, 0), (d, d), (d, d)))


def conv(x, w, b, d):
    """y[b,o,h,w] = b[o] + sum_{c,ky,kx} w[o,c,ky,kx] x[b,c,h+(ky-1)d,w+(kx-1)d]."""
    xp = _pad(x, d)
    y = np.broadcast_to(b[None, :, None, None], (x.shape[0], w.shape[0], H, W)).copy()
    for ky in range(3):
        for kx in range(3):
            y += np.einsum("oc,bchw->bohw", w[:, :, ky, kx],
                           xp[:, :, ky * d:ky * d + H, kx * d:kx * d + W])
    return y


def forward(params, x):
    """x [B][5][20][10] -> activations of the four layers (layers 1-3 after
    ReLU), misfit [B], gradient map [B][3][20][10]."""
    layers = unpack(params)
    acts = []
    a = np.asarray(x, dtype=np.float64).reshape(-1, CIN[0], H, W)
    for l, (w, b) in enumerate(layers):
        a = conv(a, w, b, DIL[l])
        if l < 3:
            a = np.maximum(a, 0.0)
        acts.append(a)
    y4 = acts[-1]
    return acts, y4[:, 3].sum(axis=(1, 2)), y4[:, :3]


def loss_grad(params, x, m_true, g_true, w_m, w_g):
    """Loss and its gradient with respect to the parameter vector (float64)."""
    x = np.asarray(x, dtype=np.float64).reshape(-1, CIN[0], H, W)
    B = x.shape[0]
    layers = unpack(params)
    acts, m, g = forward(params, x)
    dm = m - np.asarray(m_true, dtype=np.float64)
    dg = g - np.asarray(g_true, dtype=np.float64).reshape(B, 3, H, W)
    ng = B * 3 * P
    loss = w_m * np.sum(dm * dm) / B + w_g * np.sum(dg * dg) / ng
    dy = np.zeros((B, 4, H, W))
    dy[:, :3] = 2.0 * w_g * dg / ng
    dy[:, 3] = (2.0 * w_m * dm / B)[:, None, None]
    grads = [None] * 4
    for l in range(3, -1, -1):
        w, _ = layers[l]
        d = DIL[l]
        xin = x if l == 0 else acts[l - 1]
        xp = _pad(xin, d)
        dw = np.zeros_like(w)
        for ky in range(3):
            for kx in range(3):
                dw[:, :, ky, kx] = np.einsum("bohw,bchw->oc", dy,
                                             xp[:, :, ky * d:ky * d + H, kx * d:kx * d + W])
        grads[l] = np.concatenate([dw.reshape(-1), dy.sum(axis=(0, 2, 3))])
        if l > 0:
            dxp = np.zeros_like(xp)
            for ky in range(3):
                for kx in range(3):
                    dxp[:, :, ky * d:ky * d + H, kx * d:kx * d + W] += np.einsum(
                        "oc,bohw->bchw", w[:, :, ky, kx], dy)
            dx = dxp[:, :, d:d + H, d:d + W]
            dy = dx * (acts[l - 1] > 0.0)
    return loss, np.concatenate(grads)


def adam(params, grads, m, v, step, lr, beta1=0.9, beta2=0.999, eps=1e-8):
    """One Adam step (float64); returns new (params, m, v)."""
    m = beta1 * m + (1 - beta1) * grads
    v = beta2 * v + (1 - beta2) * grads * grads
    p = params - lr * (m / (1 - beta1 ** step)) / (np.sqrt(v / (1 - beta2 ** step)) + eps)
    return p, m, v


# ---- coarse-to-grid map ------------------------------------------------------

def axis_matrix(n, np_b, nc):
    """U [n][nc]: fine point x takes (1-w) of node i0 and w of node i1,
    node i at inner position (i + 0.5) f - 0.5, clamped; boundary frames
    copy the nearest inner point."""
    inner = n - 2 * np_b
    f = inner / nc
    U = np.zeros((n, nc))
    for x in range(n):
        xi = min(max(x - np_b, 0), inner - 1)
        u = min(max((xi + 0.5) / f - 0.5, 0.0), nc - 1.0)
        a = min(int(np.floor(u)), nc - 1)
        a1 = min(a + 1, nc - 1)
        w = u - a
        U[x, a] += 1.0 - w
        U[x, a1] += w
    return U


def coarse_to_fields(z, mean, sigma, nx, nz, np_b):
    """z [B][3][ncx][ncz] -> fields [B][3][nx][nz]."""
    z = np.asarray(z, dtype=np.float64)
    ncx, ncz = z.shape[-2:]
    Ux, Uz = axis_matrix(nx, np_b, ncx), axis_matrix(nz, np_b, ncz)
    theta = mean[None] + sigma[None] * z
    return np.einsum("xi,bcij,zj->bcxz", Ux, theta, Uz)


def coarse_gradient(gfields, sigma, np_b, ncx, ncz, scale=1.0):
    gfields = np.asarray(gfields, dtype=np.float64)
    nx, nz = gfields.shape[-2:]
    Ux, Uz = axis_matrix(nx, np_b, ncx), axis_matrix(nz, np_b, ncz)
    return scale * sigma[None] * np.einsum("xi,bcxz,zj->bcij", Ux, gfields, Uz)
