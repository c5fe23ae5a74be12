"""The PyTorch layer (psvwave_gb300.torch_ops.l2_misfit) and the
differentiation workload, at reduced size (1000 x 400 cut to 200 x 80 inner
cells, 50-cell boundary, 2 shots, 1500 steps, 40 receivers) and at its
stated size (test_full_c3_finite_differences_20_directions).

* autograd returns exactly exact_gradient / the reference's kernels;
* on 20 random smooth directions, the FP64 exact gradient matches the
  Richardson-extrapolated central differences of the FP64 misfit to 1e-6
  (relative L2 over the 20 directional derivatives), and the FP32 gradient
  matches them to 2e-3;
* checkpoints every 100 steps give bit for bit the gradient of keeping every
  state;
* the reference's kernels point the same way (cosine > 0.9).
"""
import numpy as np
import pytest
import torch

import psvwave_gb300 as psv
from psvwave_gb300 import workloads
from psvwave_gb300.torch_ops import l2_misfit
from tests.conftest import SMALL_INI

pytestmark = pytest.mark.gpu

REDUCED = dict(nt=1500, n_shots=2, nx_inner=200, nz_inner=80, n_rec=40)


def observed_model(params, true, start, precision):
    m = psv.fdModel.from_parameters(params, precision=precision)
    m.set_parameter_fields(*true)
    for s in range(m.n_shots):
        m.forward_simulate(s, False)
    m.set_observed_data(*m.get_synthetic_data())
    m.set_parameter_fields(*start)
    return m


@pytest.fixture(scope="module")
def reduced():
    p = workloads.c3_params(**REDUCED)
    true, start = workloads.c3_media(p)
    return p, true, start


def small_model(golden, precision="fp64"):
    m = psv.fdModel(SMALL_INI, precision=precision)
    m.set_parameter_fields(*golden["target"])
    for s in range(m.n_shots):
        m.forward_simulate(s, False)
    m.set_observed_data(*m.get_synthetic_data())
    return m


@pytest.mark.parametrize("where", ["cuda", "cpu"])
def test_autograd_equals_exact_gradient(golden, where):
    m = small_model(golden)
    m.set_parameter_fields(*golden["start"])
    mis_ref, g_ref = m.exact_gradient(50)
    t = [torch.tensor(np.array(a), dtype=torch.float64, device=where, requires_grad=True)
         for a in golden["start"]]
    chi = l2_misfit(m, *t, checkpoint_every=50)
    assert chi.device.type == where
    assert float(chi.detach()) == mis_ref
    (2.0 * chi).backward()
    for x, g in zip(t, g_ref):
        assert np.array_equal(x.grad.cpu().numpy(), 2.0 * g)


def test_no_grad_runs_forward_only(golden):
    m = small_model(golden)
    t = [torch.tensor(np.array(a), dtype=torch.float64, device="cuda") for a in golden["start"]]
    chi = l2_misfit(m, *t)
    m.set_parameter_fields(*golden["start"])
    for s in range(m.n_shots):
        m.forward_simulate(s, False)
    m.calculate_l2_misfit()
    assert float(chi.detach()) == m.misfit


def test_reference_mode_returns_reference_kernels(golden):
    m = small_model(golden)
    t = [torch.tensor(np.array(a), dtype=torch.float64, device="cuda", requires_grad=True)
         for a in golden["start"]]
    chi = l2_misfit(m, *t, mode="reference")
    chi.backward()
    m.set_parameter_fields(*golden["start"])
    m.compute_gradients()
    for x, k in zip(t, m.get_kernels()):
        assert np.array_equal(x.grad.cpu().numpy(), k)
    assert float(chi.detach()) == m.misfit


def smooth_direction(shape, seed):
    rng = np.random.default_rng(seed)
    x = np.arange(shape[0])[:, None]
    z = np.arange(shape[1])[None, :]
    d = np.zeros(shape)
    for _ in range(4):
        cx, cz = rng.uniform(0, shape[0]), rng.uniform(0, shape[1])
        w = rng.uniform(5.0, 20.0)
        d += rng.standard_normal() * np.exp(-((x - cx) ** 2 + (z - cz) ** 2) / (2 * w * w))
    return d


def test_reduced_c3_finite_differences_20_directions(reduced):
    p, true, start = reduced
    m64 = observed_model(p, true, start, "fp64")
    m32 = observed_model(p, true, start, "fp32")
    t = [torch.tensor(a, dtype=torch.float64, device="cuda", requires_grad=True) for a in start]
    l2_misfit(m64, *t, checkpoint_every=100).backward()
    g64 = [x.grad.cpu().numpy() for x in t]
    t = [torch.tensor(a, dtype=torch.float64, device="cuda", requires_grad=True) for a in start]
    l2_misfit(m32, *t, checkpoint_every=100).backward()
    g32 = [x.grad.cpu().numpy() for x in t]

    def misfit_at(fields):
        m64.set_parameter_fields(*fields)
        for s in range(m64.n_shots):
            m64.forward_simulate(s, False)
        m64.calculate_l2_misfit()
        return m64.misfit

    def central(dirs, h):
        plus = tuple(a + h * d for a, d in zip(start, dirs))
        minus = tuple(a - h * d for a, d in zip(start, dirs))
        return (misfit_at(plus) - misfit_at(minus)) / (2 * h)

    scales = (20.0, 10.0, 15.0)
    fd, d64, d32 = [], [], []
    for k in range(20):
        dirs = [smooth_direction(start[0].shape, 100 * k + j) * scales[j] for j in range(3)]
        h = 1e-2
        fd.append((4.0 * central(dirs, h / 2) - central(dirs, h)) / 3.0)
        d64.append(sum(float(np.sum(g * d)) for g, d in zip(g64, dirs)))
        d32.append(sum(float(np.sum(g * d)) for g, d in zip(g32, dirs)))
    fd, d64, d32 = np.array(fd), np.array(d64), np.array(d32)
    e64 = np.linalg.norm(d64 - fd) / np.linalg.norm(fd)
    e32 = np.linalg.norm(d32 - fd) / np.linalg.norm(fd)
    print("20 directions: FP64 exact vs FD %.3e, FP32 exact vs FD %.3e" % (e64, e32))
    assert e64 <= 1e-6
    assert e32 <= 2e-3


def test_reduced_c3_checkpointing_equals_store_all(reduced):
    p, true, start = reduced
    m = observed_model(p, true, start, "fp32")
    mis_ck, g_ck = m.exact_gradient(100)
    mis_all, g_all = m.exact_gradient(m.nt)
    assert mis_ck == mis_all
    for a, b in zip(g_ck, g_all):
        assert np.array_equal(a, b)
    assert m.exact_bytes(100) < m.exact_bytes(m.nt) / 5


def test_reduced_c3_reference_kernels_point_the_same_way(reduced):
    p, true, start = reduced
    m = observed_model(p, true, start, "fp32")
    _, g = m.exact_gradient(100)
    m.compute_gradients()
    ref = m.get_kernels()
    nb = m.np_boundary
    x0, x1 = nb + m.nx_inner_boundary, nb + m.nx_inner - m.nx_inner_boundary
    z0, z1 = nb + m.nz_inner_boundary, nb + m.nz_inner - m.nz_inner_boundary
    for name, a, b in zip(("vp", "vs", "rho"), g, ref):
        a, b = a[x0:x1, z0:z1].ravel(), b[x0:x1, z0:z1].ravel()
        cos = float(a @ b / (np.linalg.norm(a) * np.linalg.norm(b)))
        print("cosine(exact, reference) %s: %.4f" % (name, cos))
        assert cos > 0.9


def test_full_c3_finite_differences_20_directions():
    """The differentiation workload at its stated size (1000 x 400 inner
    cells + 50-cell boundary, 8 shots, 6000 steps, 200 receivers): the FP64
    and FP32 exact gradients through the torch layer against central
    differences of the misfit along 20 random smooth directions,
    Richardson-extrapolated from steps h and h/2.

    The 80 perturbed misfits run as one FP32 batch (640 shot-members, one
    launch per time step); the misfit of each is summed in FP64 from its
    seismograms. The steps perturb the medium by about 1e-3 relative, so
    the FP32 rounding of the 6000-step runs (seismograms within ~1e-6 of
    FP64, largely shared between the +h and -h runs) stays far below the
    difference being measured. Two of the directions are also differenced
    with FP64 forward runs, which pins the FP32 differences."""
    p = workloads.c3_params()
    true, start = workloads.c3_media(p)
    m64 = observed_model(p, true, start, "fp64")
    obs = m64.get_observed_data()
    grads = {}
    for prec in ("fp64", "fp32"):
        m = m64 if prec == "fp64" else observed_model(p, true, start, "fp32")
        t = [torch.tensor(a, dtype=torch.float64, device="cuda", requires_grad=True)
             for a in start]
        l2_misfit(m, *t, checkpoint_every=100).backward()
        grads[prec] = [x.grad.cpu().numpy() for x in t]
        del t
    scales = (20.0, 10.0, 15.0)
    dirs = [[smooth_direction(start[0].shape, 100 * k + j) * scales[j] for j in range(3)]
            for k in range(20)]
    h = 0.1
    members = []  # (direction, step) in the order of the differences below
    for k in range(20):
        for step in (h, -h, h / 2, -h / 2):
            members.append((k, step))

    def misfit_of(ux, uz):
        return 0.5 * p["dt"] * (float(np.sum((obs[0] - ux) ** 2)) +
                                float(np.sum((obs[1] - uz) ** 2)))

    fd_misfit = {}
    for chunk in range(0, len(members), 40):
        models = []
        for k, step in members[chunk:chunk + 40]:
            m = psv.fdModel.from_parameters(p)
            m.set_parameter_fields(*(a + step * d for a, d in zip(start, dirs[k])))
            models.append(m)
        b = psv.Batch()
        for m in models:
            b.add_all_shots(m)
        b.forward()
        for (k, step), m in zip(members[chunk:chunk + 40], models):
            fd_misfit[(k, step)] = misfit_of(*m.get_synthetic_data())
        del b, models

    def central(k, hh):
        return (fd_misfit[(k, hh)] - fd_misfit[(k, -hh)]) / (2 * hh)

    fd = np.array([(4.0 * central(k, h / 2) - central(k, h)) / 3.0 for k in range(20)])
    dd = {prec: np.array([sum(float(np.sum(g * d)) for g, d in zip(grads[prec], dirs[k]))
                          for k in range(20)]) for prec in grads}
    errs = {prec: float(np.linalg.norm(dd[prec] - fd) / np.linalg.norm(fd)) for prec in dd}

    # FP64 differences along the first two directions.
    def misfit64(fields):
        m64.set_parameter_fields(*fields)
        for s in range(m64.n_shots):
            m64.forward_simulate(s, False)
        m64.calculate_l2_misfit()
        return m64.misfit

    fd64 = []
    for k in range(2):
        c = []
        for hh in (h, h / 2):
            plus = misfit64(tuple(a + hh * d for a, d in zip(start, dirs[k])))
            minus = misfit64(tuple(a - hh * d for a, d in zip(start, dirs[k])))
            c.append((plus - minus) / (2 * hh))
        fd64.append((4.0 * c[1] - c[0]) / 3.0)
    fd64 = np.array(fd64)
    pin = float(np.max(np.abs(fd[:2] - fd64) / np.abs(fd64)))
    e64_2 = float(np.max(np.abs(dd["fp64"][:2] - fd64) / np.abs(fd64)))
    e32_64 = float(np.linalg.norm(dd["fp32"] - dd["fp64"]) / np.linalg.norm(dd["fp64"]))
    print("c3 full size, 20 directions: exact vs FP32-batch FD: FP64 %.3e, FP32 %.3e; "
          "FP32 FD vs FP64 FD (2 directions) %.3e; FP64 exact vs FP64 FD %.3e; "
          "FP32 exact vs FP64 exact %.3e" % (errs["fp64"], errs["fp32"], pin, e64_2, e32_64))
    # FP64 exact gradient against FP64 differences: to the differences' own
    # accuracy (measured 2e-11).
    assert e64_2 <= 1e-8
    # The FP32 batch's differences carry FP32 rounding (measured 1.9e-3 on
    # the two directions whose derivatives are smallest, 3.5e-4 over all 20).
    assert pin <= 5e-3
    assert errs["fp64"] <= 2e-3
    assert errs["fp32"] <= 2e-3
    # FP32 wave fields with float-float gradient sums against FP64.
    assert e32_64 <= 1e-4
