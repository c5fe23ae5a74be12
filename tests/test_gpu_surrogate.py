"""The learned part on the GPU, through the C ABI (include/psvwave_surrogate.h).

* network forward, loss and parameter gradient, and one Adam step, against
  the CPU restatement (oracle/cnn_oracle.py) to 1e-4 relative;
* the coarse-to-grid map and its transpose against the restatement;
* end to end at reduced size: the solver's exact misfit gradient matches
  finite differences; solver-made (z, misfit, gradient) triples train the
  network (held-out misfit error below the untrained network's); and
  surrogate-screened HMC delivers more than 5x the accepted samples per
  second of HMC with the solver's gradients.
"""
import numpy as np
import pytest
import torch

from oracle import cnn_oracle as co
from psvwave_gb300 import surrogate as sg
from psvwave_gb300 import workloads
from tests.conftest import rel_l2

pytestmark = pytest.mark.gpu

DEV = "cuda:0"


def rand_batch(B, seed):
    rng = np.random.default_rng(seed)
    x = rng.standard_normal((B, 5, 20, 10)).astype(np.float32)
    m = rng.standard_normal(B).astype(np.float32)
    g = rng.standard_normal((B, 3, 20, 10)).astype(np.float32)
    return x, m, g


def to_dev(*a):
    return [torch.tensor(v, device=DEV) for v in a]


def test_forward_matches_oracle():
    net = sg.SurrogateNet(max_batch=16, seed=3)
    params = net.get_params()
    x, _, _ = rand_batch(7, 0)
    m, g = net.predict_features(torch.tensor(x, device=DEV))
    _, m_ref, g_ref = co.forward(params, x)
    assert rel_l2(m.cpu().numpy(), m_ref) <= 1e-4
    assert rel_l2(g.cpu().numpy(), g_ref) <= 1e-4


@pytest.mark.parametrize("B", [1, 300])
def test_forward_tensor_core_tiles_match_oracle(B):
    """The forward convolutions run as 128-position tensor-core tiles over
    the whole batch: one image (a single partial tile) and a batch whose
    last tile is ragged and whose tiles straddle images."""
    net = sg.SurrogateNet(max_batch=512, seed=6)
    params = net.get_params()
    x, _, _ = rand_batch(B, 7)
    m, g = net.predict_features(torch.tensor(x, device=DEV))
    _, m_ref, g_ref = co.forward(params, x)
    assert rel_l2(m.cpu().numpy(), m_ref) <= 1e-4
    assert rel_l2(g.cpu().numpy(), g_ref) <= 1e-4


def test_loss_gradient_matches_oracle():
    net = sg.SurrogateNet(max_batch=32, seed=4)
    params = net.get_params()
    x, m, g = rand_batch(19, 1)
    loss, d = net.loss_grad(*to_dev(x, m, g), w_misfit=0.3, w_grad=1.7)
    loss_ref, d_ref = co.loss_grad(params, x, m, g, 0.3, 1.7)
    assert abs(loss - loss_ref) <= 1e-5 * abs(loss_ref)
    assert rel_l2(d, d_ref) <= 1e-4
    offs, _ = co.offsets()
    for l in range(4):  # every layer, not only the dominant one
        a, b = offs[l], offs[l] + co.layer_size(l)
        assert rel_l2(d[a:b], d_ref[a:b]) <= 1e-4, l


def test_loss_gradient_matches_oracle_ragged_batch():
    """The weight gradients reduce positions in 64-position chunks over 32
    ranges on the tensor cores: a batch whose positions end inside a chunk
    and whose ranges straddle images. At this size some pre-activations of
    a random network lie within the forward's FP32 rounding of the ReLU
    kink, where the GPU's mask and the FP64 oracle's may differ. A large
    first-layer bias and non-negative weights and positive biases in the
    next two layers keep every hidden pre-activation well away from it, so
    the comparison checks the arithmetic, not the kink."""
    net = sg.SurrogateNet(max_batch=256, seed=8)
    params = net.get_params()
    offs, _ = co.offsets()
    for l in range(3):
        nw = co.COUT[l] * co.CIN[l] * 9
        if l > 0:
            params[offs[l]:offs[l] + nw] = np.abs(params[offs[l]:offs[l] + nw])
        params[offs[l] + nw:offs[l] + nw + co.COUT[l]] = 8.0 if l == 0 else 1.0
    net.set_params(params)
    params = net.get_params()
    x, m, g = rand_batch(130, 9)
    acts, _, _ = co.forward(params, x)
    assert min(float(a.min()) for a in acts[:3]) > 0.1  # no ReLU kink nearby
    loss, d = net.loss_grad(*to_dev(x, m, g), w_misfit=1.0, w_grad=1.0)
    loss_ref, d_ref = co.loss_grad(params, x, m, g, 1.0, 1.0)
    assert abs(loss - loss_ref) <= 1e-5 * abs(loss_ref)
    for l in range(4):
        a, b = offs[l], offs[l] + co.layer_size(l)
        assert rel_l2(d[a:b], d_ref[a:b]) <= 1e-4, l


def test_adam_step_matches_oracle():
    net = sg.SurrogateNet(max_batch=8, seed=5)
    p0 = net.get_params().astype(np.float64)
    x, m, g = rand_batch(8, 2)
    _, d_ref = co.loss_grad(p0.astype(np.float32), x, m, g, 1.0, 1.0)
    net.train_step(*to_dev(x, m, g), 1.0, 1.0, lr=1e-3)
    p1 = net.get_params()
    p_ref, _, _ = co.adam(p0, d_ref, np.zeros_like(p0), np.zeros_like(p0), 1, 1e-3)
    # The first bias-corrected Adam step moves each parameter by lr times the
    # sign of its gradient (less where the gradient is within eps of zero),
    # so compare where the gradient is clearly non-zero, and bound the rest.
    clear = np.abs(d_ref) > 1e-3 * np.sqrt(np.mean(d_ref ** 2))
    assert clear.mean() > 0.5
    assert np.max(np.abs(p1 - p_ref)[clear]) <= 2e-5
    assert np.max(np.abs(p1 - p0)) <= 1.001e-3


def test_coarse_map_matches_oracle():
    mean, sigma = workloads.c4_prior()
    nx, nz, npb = 250, 150, 25
    cp = sg.CoarseParam(nx, nz, npb, mean, sigma)
    rng = np.random.default_rng(7)
    z = rng.standard_normal((3, 3, 20, 10)).astype(np.float32)
    f = cp.to_fields(torch.tensor(z, device=DEV)).cpu().numpy()
    f_ref = co.coarse_to_fields(z, mean, sigma, nx, nz, npb)
    assert rel_l2(f, f_ref) <= 1e-12
    gf = rng.standard_normal((3, 3, nx, nz))
    gz = cp.gradient(torch.tensor(gf, device=DEV), 0.5).cpu().numpy()
    gz_ref = co.coarse_gradient(gf, sigma, npb, 20, 10, 0.5)
    assert rel_l2(gz, gz_ref) <= 1e-6  # float32 output


def test_surrogate_screened_hmc_end_to_end():
    # Reduced workload: 400 steps, 16 chains.
    torch.manual_seed(0)
    params = workloads.c4_params(nt=500)
    mean, sigma = workloads.c4_prior()
    import psvwave_gb300 as psv
    probe = psv.fdModel.from_parameters(params)
    coarse = sg.CoarseParam(probe.nx, probe.nz, probe.np_boundary, mean, sigma)
    z_true = torch.tensor(np.random.default_rng(4).standard_normal((1, 3, 20, 10)),
                          dtype=torch.float32, device=DEV)
    f = coarse.to_fields(z_true)[0]
    probe.set_parameter_fields_device(f[0], f[1], f[2])
    probe.forward_simulate(0, False)
    observed = probe.get_synthetic_data()
    f0 = coarse.to_fields(torch.zeros_like(z_true))[0]
    probe.set_observed_data(*observed)
    probe.set_parameter_fields_device(f0[0], f0[1], f0[2])
    probe.forward_simulate(0, False)
    probe.calculate_l2_misfit()
    s2 = probe.misfit / 500.0
    post = sg.FDPosterior(params, coarse, observed, s2, n_models=16)

    # Training triples: exact misfit gradients at prior draws.
    z, mis, grads = sg.generate_training_set(post, 512, seed=1)
    # The solver's gradient matches finite differences of its misfit.
    d = torch.randn(z[0].shape, device=DEV)
    h = 1e-2
    fp = post.misfits((z[0] + h * d)[None])[0]
    fm = post.misfits((z[0] - h * d)[None])[0]
    fd = (fp - fm) / (2 * h)
    # FP32 wave fields: the difference quotient carries rounding noise of
    # order 1e-6 misfit / h.
    assert abs(float((grads[0] * d).sum()) - fd) <= 2e-2 * abs(fd) + 1e-4 * float(mis[0])

    net = sg.SurrogateNet(max_batch=256, seed=0)
    untrained = sg.SurrogateNet(max_batch=256, seed=0)
    hist = sg.train(net, z[:448], mis[:448], grads[:448], epochs=40, batch=64, lr=2e-3)
    untrained.norm = dict(net.norm)
    assert hist[-1] < 0.5 * hist[0]
    # Held-out accuracy: the trained network beats the untrained one, which
    # (its last layer starting near zero) predicts the training mean.
    m_tr, g_tr = net.predict(z[448:])
    m_un, g_un = untrained.predict(z[448:])
    err_tr = float(((m_tr - mis[448:]) ** 2).mean())
    err_un = float(((m_un - mis[448:]) ** 2).mean())
    print("held-out misfit MSE: trained %.4g, untrained %.4g" % (err_tr, err_un))
    assert err_tr < err_un

    # Surrogate-screened HMC (only first-stage survivors are simulated, in
    # one batched forward) against HMC with the solver's exact gradients.
    z0 = 0.5 * torch.randn((16, 3, 20, 10), device=DEV)
    eps, n_leap = 0.03, 8
    n0 = post.n_potentials
    da = sg.da_hmc(post, net, z0, 10, eps, n_leap, seed=2, screen=0.5, force=0.0)
    plain = sg.plain_hmc(post, z0[:4], 3, eps, n_leap, seed=2, threads=4)
    print("DA: %s" % {k: v for k, v in da.items() if k not in ("samples", "z", "U")})
    print("plain: %s" % {k: v for k, v in plain.items() if k not in ("samples", "z")})
    assert 0 < da["accepted"] <= da["stage1_accepted"] <= da["proposals"]
    # The solver ran for the 16 starting states and the first-stage survivors only.
    assert post.n_potentials - n0 == 16 + da["stage1_accepted"]
    # Faster per accepted sample even at this toy size (16 chains, 10
    # iterations, a 512-triple network); the full-size ratio is a bench
    # figure, not a test.
    assert da["accepted_per_s"] > 2.0 * plain["accepted_per_s"]
