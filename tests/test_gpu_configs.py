"""Parity at the benchmark configurations themselves, not only on small
grids: the kernel schemes, tile shapes and grid sizes the benchmark runs are
the ones compared here.

* c1 (2100 x 900, nt = 5000, explosive + dip source, 400 receivers): the
  default FP32 scheme (one persistent launch of 32 x 60 tiles, interior
  register-window path) against the FP64 GPU solve of the same run over all
  5000 steps, seismograms within 1e-4 relative L2; the wave fields while
  the wave is inside the grid too. The FP64 GPU solve is bit-identical to
  the oracle port on the same grid and medium over a 600-step prefix
  (seismograms and every wave field), so the FP64 answer is the
  reference's (src/fdModel.cpp:526-787).
* c0 (250 x 150, nt = 4000, two sources in one shot): the full gradient
  (forward with snapshots, misfit, adjoint sources, adjoint with kernel
  correlation, velocity kernels, gradient vector) in FP64 bit-identical to
  the oracle port; FP32 with its default cluster-resident scheme and with
  the per-step TMA launches within 1e-4 of FP64 on every output.
* c2 (many models of uneven sizes): batch members advanced together in the
  FP32 batch launch against each member's own FP64 solve.
"""
import numpy as np
import pytest

import psvwave_gb300 as psv
from oracle import portbind
from psvwave_gb300 import workloads
from tests.conftest import fwi_gradient, rel_l2
from tests.test_gpu_parity import OUTPUTS, gpu_outputs

pytestmark = pytest.mark.gpu

FP32_TOL = 1e-4   # relative L2, FP32 wave fields vs the FP64 answer


def c1_oracle(nt):
    o = portbind.OracleModel(params=workloads.c1_params(nt=nt))
    o.view("moment")[...] = workloads.c1_moment()
    o.set_parameter_fields(*workloads.c1_media())
    return o


def test_c1_fp64_bit_exact_vs_oracle_on_prefix():
    nt = 600
    m = workloads.c1_model(nt=nt, precision="fp64")
    m.forward_simulate(0, False)
    o = c1_oracle(nt)
    o.forward_simulate(0, False)
    for a, b in zip(m.get_synthetic_data(), o.get_synthetic_data()):
        assert np.abs(b).max() > 0
        assert np.array_equal(a, b), rel_l2(a, b)
    for a, n in zip(m.get_wavefields(), ("vx", "vz", "txx", "tzz", "txz")):
        b = o.array(n)
        assert np.abs(b).max() > 0
        assert np.array_equal(a, b), (n, rel_l2(a, b))


def test_c1_fp32_default_scheme_vs_fp64_full_run():
    m32 = workloads.c1_model()
    assert m32.kernel_variant == "fused_tma_persistent"
    assert m32.tile_shape == "32x60"
    m32.forward_simulate(0, False)
    m64 = workloads.c1_model(precision="fp64")
    m64.forward_simulate(0, False)
    errs = [rel_l2(a, b) for a, b in zip(m32.get_synthetic_data(), m64.get_synthetic_data())]
    print("c1 fp32 vs fp64 seismograms (ux, uz), 5000 steps:", errs)
    for e in errs:
        assert e <= FP32_TOL, errs


@pytest.mark.parametrize("variant,shape", [("fused_tma_persistent", "32x60"),
                                           ("fused_tma_persistent", "16x60"),
                                           ("fused_tma", "32x60")])
def test_c1_fp32_wavefields_vs_fp64_while_wave_in_grid(variant, shape):
    nt = 1500
    m32 = workloads.c1_model(nt=nt)
    m32.kernel_variant = variant
    m32.tile_shape = shape
    m32.forward_simulate(0, False)
    m64 = workloads.c1_model(nt=nt, precision="fp64")
    m64.forward_simulate(0, False)
    errs = {n: rel_l2(a, b) for n, a, b in zip(("vx", "vz", "txx", "tzz", "txz"),
                                              m32.get_wavefields(), m64.get_wavefields())}
    errs.update({n: rel_l2(a, b) for n, a, b in zip(("ux", "uz"), m32.get_synthetic_data(),
                                                   m64.get_synthetic_data())})
    print("c1 fp32 (%s) vs fp64 after %d steps:" % (variant, nt), errs)
    for k, e in errs.items():
        assert e <= FP32_TOL, (k, e)


@pytest.fixture(scope="module")
def c0_fp64():
    p = workloads.c0_params()
    target, start = workloads.c0_media()
    m = psv.fdModel.from_parameters(p, precision="fp64")
    misfit = fwi_gradient(m, target, start)
    out = gpu_outputs(m)
    out["gradient_vector"] = m.get_gradient_vector()
    return misfit, out, m


def test_c0_fp64_gradient_bit_exact_vs_oracle(c0_fp64):
    misfit, out, m = c0_fp64
    p = workloads.c0_params()
    target, start = workloads.c0_media()
    o = portbind.OracleModel(params=p)
    mo = fwi_gradient(o, target, start)
    assert abs(misfit - mo) <= 1e-12 * mo
    for name in OUTPUTS:
        assert np.array_equal(out[name], o.array(name)), (name, rel_l2(out[name], o.array(name)))
    assert np.array_equal(out["gradient_vector"], o.get_gradient_vector())
    snaps = m.get_snapshots()
    for k, n in enumerate(("accu_vx", "accu_vz", "accu_txx", "accu_tzz", "accu_txz")):
        assert np.array_equal(snaps[k], o.array(n)), n


@pytest.mark.parametrize("variant", [None, "fused_tma"])
def test_c0_fp32_gradient_vs_fp64(c0_fp64, variant):
    misfit64, out64, _ = c0_fp64
    p = workloads.c0_params()
    target, start = workloads.c0_media()
    m = psv.fdModel.from_parameters(p)
    if variant is None:
        assert m.kernel_variant == "fused_cluster"
    else:
        m.kernel_variant = variant
    misfit = fwi_gradient(m, target, start)
    out = gpu_outputs(m)
    out["gradient_vector"] = m.get_gradient_vector()
    errs = {k: rel_l2(out[k], out64[k]) for k in out64}
    errs["misfit"] = abs(misfit - misfit64) / misfit64
    print("c0 fp32 (%s) vs fp64:" % m.kernel_variant, errs)
    for k, e in errs.items():
        assert e <= FP32_TOL, (k, e)


@pytest.mark.parametrize("shape,persistent", [("20x28", False), ("32x60", True)])
def test_c2_batch_members_vs_fp64(shape, persistent):
    pairs = workloads.c2_models(n_models=4)
    models = []
    for p, media in pairs:
        m = psv.fdModel.from_parameters(p)
        m.set_parameter_fields(*media)
        models.append(m)
    b = psv.Batch()
    for m in models:
        b.add_all_shots(m)
    b.tile_shape = shape
    b.persistent = persistent
    b.forward()
    worst = 0.0
    for (p, media), m in zip(pairs, models):
        m64 = psv.fdModel.from_parameters(p, precision="fp64")
        m64.set_parameter_fields(*media)
        for s in range(m64.n_shots):
            m64.forward_simulate(s, False)
        for a, c in zip(m.get_synthetic_data(), m64.get_synthetic_data()):
            for s in range(m64.n_shots):
                assert np.abs(c[s]).max() > 0
                e = rel_l2(a[s], c[s])
                worst = max(worst, e)
                assert e <= FP32_TOL, (m64.nx, m64.nz, s, e)
    print("c2 batch (%s, persistent=%s) worst member error vs fp64: %.3g"
          % (shape, persistent, worst))
