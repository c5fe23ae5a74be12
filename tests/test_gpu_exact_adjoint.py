"""The exact discrete adjoint (psv_exact_gradient): the transpose of the
time stepping gives the gradient of the discrete L2 misfit.

* FP64: the directional derivative g . d agrees with central finite
  differences of the misfit along random smooth directions; the
  differences converge at second order in the step and their Richardson
  extrapolation matches g . d to 1e-7 relative.
* The result does not depend on the checkpoint interval (bit for bit):
  recomputing forward segments from checkpoints reproduces every state.
* FP32 wave fields give the FP64 gradient to 1e-3 relative L2.
* The reference's adjoint kernels point the same way (cosine > 0.9) but are
  not the gradient of the discrete misfit.
"""
import numpy as np
import pytest

import psvwave_gb300 as psv
from tests.conftest import SMALL_INI, rel_l2

pytestmark = pytest.mark.gpu


def setup(golden, precision):
    m = psv.fdModel(SMALL_INI, precision=precision)
    m.set_parameter_fields(*golden["target"])
    for s in range(m.n_shots):
        m.forward_simulate(s, False)
    m.set_observed_data(*m.get_synthetic_data())
    m.set_parameter_fields(*golden["start"])
    return m


def misfit_at(m, fields):
    m.set_parameter_fields(*fields)
    for s in range(m.n_shots):
        m.forward_simulate(s, False)
    m.calculate_l2_misfit()
    return m.misfit


def smooth_direction(shape, seed):
    rng = np.random.default_rng(seed)
    x = np.arange(shape[0])[:, None]
    z = np.arange(shape[1])[None, :]
    d = np.zeros(shape)
    for _ in range(4):
        cx, cz = rng.uniform(0, shape[0]), rng.uniform(0, shape[1])
        w = rng.uniform(3.0, 8.0)
        d += rng.standard_normal() * np.exp(-((x - cx) ** 2 + (z - cz) ** 2) / (2 * w * w))
    return d


def test_exact_gradient_matches_finite_differences(golden):
    m = setup(golden, "fp64")
    mis, g = m.exact_gradient(100)
    start = tuple(np.array(a) for a in golden["start"])
    scales = (20.0, 8.0, 15.0)  # perturbation size per parameter (m/s, m/s, kg/m^3)

    def central(dirs, h):
        plus = tuple(a + h * d for a, d in zip(start, dirs))
        minus = tuple(a - h * d for a, d in zip(start, dirs))
        return (misfit_at(m, plus) - misfit_at(m, minus)) / (2 * h)

    for seed in range(4):
        dirs = [smooth_direction(start[0].shape, 10 * seed + k) * scales[k] for k in range(3)]
        gd = sum(float(np.sum(gk * dk)) for gk, dk in zip(g, dirs))
        # Cauchy-Schwarz bound on |g . d|: the scale of the derivative.
        bound = sum(float(np.linalg.norm(gk) * np.linalg.norm(dk)) for gk, dk in zip(g, dirs))
        h = 1e-2
        fd_h, fd_h2 = central(dirs, h), central(dirs, h / 2)
        richardson = (4.0 * fd_h2 - fd_h) / 3.0  # cancels the O(h^2) truncation term
        print("direction %d: adjoint %.12e  fd(h) %.12e  fd(h/2) %.12e  extrapolated %.12e  bound %.4e"
              % (seed, gd, fd_h, fd_h2, richardson, bound))
        # Second-order convergence: the step-h/2 difference is about 4x closer.
        assert abs(gd - fd_h2) <= 0.3 * abs(gd - fd_h) + 1e-9 * bound
        assert abs(gd - richardson) <= 1e-7 * (abs(richardson) + 0.01 * bound)


def test_exact_gradient_independent_of_checkpoint_interval(golden):
    m = setup(golden, "fp64")
    mis_all, g_all = m.exact_gradient(m.nt)   # every state kept
    mis_ck, g_ck = m.exact_gradient(37)       # segments of 37 steps, last one partial
    assert mis_all == mis_ck
    for a, b in zip(g_all, g_ck):
        assert np.array_equal(a, b)
    assert m.exact_bytes(37) < m.exact_bytes(m.nt)


def test_exact_gradient_fp32_vs_fp64(golden):
    _, g64 = setup(golden, "fp64").exact_gradient(100)
    _, g32 = setup(golden, "fp32").exact_gradient(100)
    for a, b in zip(g32, g64):
        assert rel_l2(a, b) <= 1e-3


def test_reference_kernels_point_the_same_way(golden):
    m = setup(golden, "fp64")
    _, g = m.exact_gradient(100)
    for s in range(m.n_shots):
        m.forward_simulate(s, True)
    m.calculate_l2_misfit()
    m.calculate_l2_adjoint_sources()
    m.reset_kernels()
    for s in range(m.n_shots):
        m.adjoint_simulate(s)
    m.map_kernels_to_velocity()
    ref = m.get_kernels()
    # The reference correlates over the free region only.
    x0, x1 = m.np_boundary + m.nx_inner_boundary, m.np_boundary + m.nx_inner - m.nx_inner_boundary
    z0, z1 = m.np_boundary + m.nz_inner_boundary, m.np_boundary + m.nz_inner - m.nz_inner_boundary
    for name, a, b in zip(("vp", "vs", "rho"), g, ref):
        a, b = a[x0:x1, z0:z1].ravel(), b[x0:x1, z0:z1].ravel()
        cos = float(a @ b / (np.linalg.norm(a) * np.linalg.norm(b)))
        print("cosine(exact, reference) %s: %.4f" % (name, cos))
        assert cos > 0.9


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_exact_gradient_graph_replay_is_bitwise(golden, precision):
    # First call eager, second captured into per-shot CUDA graphs, third
    # replayed: all three give the same misfit and gradient bit for bit.
    m = setup(golden, precision)
    runs = [m.exact_gradient(40) for _ in range(3)]
    for mis, g in runs[1:]:
        assert mis == runs[0][0]
        for a, b in zip(g, runs[0][1]):
            assert np.array_equal(a, b)


def test_exact_gradient_of_shot_subsets_adds_up(golden):
    # The per-rank part of a shot-sharded gradient: shot subsets add up to
    # the all-shot gradient and misfit.
    m = setup(golden, "fp64")
    mis, g = m.exact_gradient(40)
    parts = [m.exact_gradient(40, shots=[s]) for s in range(m.n_shots)]
    assert abs(sum(p[0] for p in parts) - mis) <= 1e-12 * abs(mis)
    for k in range(3):
        assert rel_l2(sum(p[1][k] for p in parts), g[k]) <= 1e-12
    with pytest.raises(ValueError):
        m.exact_gradient(40, shots=[0, 0])
