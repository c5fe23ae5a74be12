"""Tiny grids against the oracle port, element by element: grids of 16 x 14,
28 x 18 and 18 x 14 points (np_boundary 3-4), smaller than one tile of every
TMA shape, with two sources at one cell, sources and receivers next to the
absorbing frame, coinciding receivers, two shots, and no receivers at all.

* FP64: seismograms, snapshots, Lame and velocity kernels are
  bit-identical to the oracle, the misfit (a parallel reduction) equal to
  1e-12.
* FP32, every step scheme and tile shape: within 1e-4 relative L2 of FP64
  (the cluster scheme runs slabs of 2-4 rows per CTA here, whose edge rows
  go to both neighbours).
"""
import numpy as np
import pytest

import psvwave_gb300 as psv
from tests.conftest import rel_l2

pytestmark = pytest.mark.gpu


def tiny_params(nxi, nzi, npb, sources, receivers, shots, nt=120):
    return dict(nt=nt, nx_inner=nxi, nz_inner=nzi, nx_inner_boundary=1, nz_inner_boundary=1,
                dx=1.0, dz=1.0, dt=1e-4, np_boundary=npb, np_factor=0.05, scalar_rho=1500.0,
                scalar_vp=2000.0, scalar_vs=800.0, npx=1, npz=1, peak_frequency=200.0,
                source_timeshift=0.002, delay_cycles_per_shot=1, n_sources=len(sources),
                ix_sources=[s[0] for s in sources], iz_sources=[s[1] for s in sources],
                moment_angles=[s[2] for s in sources], which_source_to_fire_in_which_shot=shots,
                nr=len(receivers), ix_receivers=[r[0] for r in receivers],
                iz_receivers=[r[1] for r in receivers], snapshot_interval=10)


CASES = {
    "16x14": tiny_params(8, 6, 4, [(3, 2, 30.0), (3, 2, 75.0), (6, 4, 120.0)],
                         [(1, 1), (5, 3), (5, 3)], [[0, 1, 2]]),
    "28x18": tiny_params(20, 10, 4, [(2, 2, 45.0), (17, 7, 10.0)],
                         [(4, 1), (10, 8), (15, 5), (19, 9)], [[0], [1]]),
    "18x14_no_receivers": tiny_params(12, 8, 3, [(5, 4, 60.0)], [], [[0]]),
}


def media(nx, nz, seed):
    """Target and start media: the homogeneous background with a seeded
    smooth +-8% perturbation in the target."""
    rng = np.random.default_rng(seed)
    x = np.arange(nx)[:, None] / nx
    z = np.arange(nz)[None, :] / nz
    bump = np.sin(2 * np.pi * (x * rng.uniform(0.5, 1.5) + rng.uniform())) * \
        np.cos(2 * np.pi * (z * rng.uniform(0.5, 1.5) + rng.uniform()))
    base = (np.full((nx, nz), 2000.0), np.full((nx, nz), 800.0), np.full((nx, nz), 1500.0))
    target = tuple(b * (1.0 + 0.08 * bump) for b in base)
    return target, base


def gradient_run(m, target, start):
    """Observed data from `target`, then the reference's gradient sequence at
    `start`; returns every output the comparison looks at."""
    m.set_parameter_fields(*target)
    for s in range(m.n_shots):
        m.forward_simulate(s, False)
    m.set_observed_data(*m.get_synthetic_data())
    m.set_parameter_fields(*start)
    for s in range(m.n_shots):
        m.forward_simulate(s, True)
    m.calculate_l2_misfit()
    m.calculate_l2_adjoint_sources()
    m.reset_kernels()
    for s in range(m.n_shots):
        m.adjoint_simulate(s)
    m.map_kernels_to_velocity()
    out = {"ux": m.get_synthetic_data()[0], "uz": m.get_synthetic_data()[1]}
    for name, a in zip(("vx", "vz", "txx", "tzz", "txz"), m.get_snapshots()):
        out["snap_" + name] = np.asarray(a)
    for name, a in zip(("lambda", "mu", "rho_l"), m.get_lame_kernels()):
        out["k_" + name] = np.asarray(a)
    for name, a in zip(("vp", "vs", "rho"), m.get_kernels()):
        out["k_" + name] = np.asarray(a)
    return float(m.misfit), out


@pytest.mark.parametrize("case", sorted(CASES))
def test_tiny_grid_fp64_matches_the_oracle_bitwise(case):
    from oracle.portbind import OracleModel

    p = CASES[case]
    m = psv.fdModel.from_parameters(p, precision="fp64")
    target, start = media(m.nx, m.nz, seed=len(case))
    mis, out = gradient_run(m, target, start)
    o = OracleModel(params=p)
    o.set_parameter_fields(*target)
    for s in range(o.n_shots):
        o.forward_simulate(s, False)
    o.set_observed_data(*o.get_synthetic_data())
    o.set_parameter_fields(*start)
    o.run_model(True)
    ref = {"ux": o.get_synthetic_data()[0], "uz": o.get_synthetic_data()[1]}
    for name in ("vx", "vz", "txx", "tzz", "txz"):
        ref["snap_" + name] = o.array("accu_" + name)
    for name, a in zip(("lambda", "mu", "rho_l"), o.get_lame_kernels()):
        ref["k_" + name] = np.asarray(a)
    for name, a in zip(("vp", "vs", "rho"), o.get_kernels()):
        ref["k_" + name] = np.asarray(a)
    # The misfit is a parallel FP64 reduction on the GPU, a serial sum in
    # the reference: equal to rounding; everything else bit for bit.
    assert abs(mis - o.misfit) <= 1e-12 * abs(o.misfit)
    for k in ref:
        assert np.array_equal(out[k], ref[k]), k
    if m.nr == 0:
        assert mis == 0.0 and not out["k_vp"].any()
    else:
        assert mis > 0 and np.abs(out["k_vp"]).max() > 0


FP32_RUNS = [("fused_cluster", None), ("fused_tma", "32x60"), ("fused_tma", "16x28"),
             ("fused_tma", "20x28"), ("fused_tma_persistent", "16x28"), ("fused", None),
             ("two_kernel", None)]


@pytest.mark.parametrize("case", sorted(CASES))
@pytest.mark.parametrize("variant,shape", FP32_RUNS)
def test_tiny_grid_fp32_schemes_within_tolerance(case, variant, shape):
    p = CASES[case]
    m64 = psv.fdModel.from_parameters(p, precision="fp64")
    target, start = media(m64.nx, m64.nz, seed=len(case))
    mis64, ref = gradient_run(m64, target, start)
    m = psv.fdModel.from_parameters(p)
    m.kernel_variant = variant
    if shape:
        m.tile_shape = shape
    mis, out = gradient_run(m, target, start)
    assert abs(mis - mis64) <= 1e-4 * abs(mis64) + 1e-30
    for k in ref:
        assert out[k].shape == ref[k].shape, k
        if ref[k].any():
            assert rel_l2(out[k], ref[k]) <= 1e-4, k
        else:
            assert not out[k].any(), k


def test_cluster_models_of_different_sizes_coexist(golden):
    """The cluster kernel's shared-memory limit is a property of the kernel,
    shared by every model: a 250 x 150 model built first still runs after a
    16 x 14 model (a few KB per CTA) is built, and agrees with its first
    run bit for bit."""
    from psvwave_gb300 import workloads

    big = psv.fdModel.from_parameters(workloads.c0_params())
    big.set_parameter_fields(*workloads.c0_media()[0])
    assert big.kernel_variant == "fused_cluster"
    big.forward_simulate(0, False)
    first = big.get_synthetic_data()[0].copy()
    small = psv.fdModel.from_parameters(CASES["16x14"])
    assert small.kernel_variant == "fused_cluster"
    small.forward_simulate(0, False)
    big.forward_simulate(0, False)
    assert np.array_equal(big.get_synthetic_data()[0], first)
