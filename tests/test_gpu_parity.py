"""Parity of the GPU solver with the reference.

FP64 wave fields reproduce the reference bit for bit (golden fixtures made by
the reference, tests/golden/make_golden.py, and the oracle port on the same
machine); only the misfit, a parallel FP64 reduction, differs in the last
bits (tolerance 1e-12 relative).

FP32 wave fields are held to the tolerance of the production path: relative
L2 error <= 1e-4 against the FP64 answer for seismograms, misfit, adjoint
sources, kernels and the gradient vector.
"""
import numpy as np
import pytest

import psvwave_gb300 as psv
from oracle import portbind
from tests.conftest import (NB2_GRAD_INF, NB2_INI, NB2_MISFIT, SMALL_INI, fwi_gradient,
                            nb2_media, rel_l2)

pytestmark = pytest.mark.gpu

FP32_TOL = 1e-4       # relative L2, FP32 wave fields vs the FP64 answer
MISFIT_FP64_TOL = 1e-12

OUTPUTS = ("rtf_ux", "rtf_uz", "a_stf_ux", "a_stf_uz", "lambda_kernel", "mu_kernel",
           "density_l_kernel", "vp_kernel", "vs_kernel", "density_v_kernel")


def gpu_outputs(m):
    ux, uz = m.get_synthetic_data()
    au, az = m.get_adjoint_sources()
    lk, mk, rk = m.get_lame_kernels()
    vk, sk, dk = m.get_kernels()
    return dict(zip(OUTPUTS, (ux, uz, au, az, lk, mk, rk, vk, sk, dk)))


def test_setup_tables_bit_exact(golden):
    m = psv.fdModel(SMALL_INI, precision="fp64")
    assert np.array_equal(m.get_taper(), golden["taper"])
    assert np.array_equal(m.get_stf(), golden["stf"])
    assert np.array_equal(m.get_moment(), golden["moment"])


def test_fp64_gradient_bit_exact_vs_reference(golden):
    m = psv.fdModel(SMALL_INI, precision="fp64")
    misfit = fwi_gradient(m, tuple(golden["target"]), tuple(golden["start"]))
    assert abs(misfit - golden["misfit"]) <= MISFIT_FP64_TOL * golden["misfit"]
    out = gpu_outputs(m)
    for name in OUTPUTS:
        assert np.array_equal(out[name], golden[name]), (name, rel_l2(out[name], golden[name]))
    assert np.array_equal(m.get_observed_data()[0], golden["obs_ux"])
    assert np.array_equal(m.get_model_vector(), golden["model_vector"])
    assert np.array_equal(m.get_gradient_vector(), golden["gradient_vector"])
    snaps = m.get_snapshots()
    assert np.array_equal(np.stack([s[1, 25] for s in snaps]), golden["snap_shot1_25"])
    assert np.array_equal(np.stack(m.get_wavefields()), golden["adjoint_fields"])


def test_fp64_matches_oracle_port_on_seeded_case():
    """A different medium on the same machine's oracle port: bit-exact."""
    o = portbind.OracleModel(SMALL_INI)
    m = psv.fdModel(SMALL_INI, precision="fp64")
    rng = np.random.default_rng(11)
    shape = (m.nx, m.nz)
    tgt = (2100 * (1 + 0.02 * rng.standard_normal(shape)),
           850 * (1 + 0.02 * rng.standard_normal(shape)),
           1600 * (1 + 0.02 * rng.standard_normal(shape)))
    start = (np.full(shape, 2100.0), np.full(shape, 850.0), np.full(shape, 1600.0))
    mo = fwi_gradient(o, tgt, start)
    mg = fwi_gradient(m, tgt, start)
    assert abs(mg - mo) <= MISFIT_FP64_TOL * mo
    out = gpu_outputs(m)
    for name in OUTPUTS:
        assert np.array_equal(out[name], o.array(name)), name
    assert np.array_equal(m.get_gradient_vector(), o.get_gradient_vector())


def test_fp32_within_tolerance(golden):
    m = psv.fdModel(SMALL_INI, precision="fp32")
    misfit = fwi_gradient(m, tuple(golden["target"]), tuple(golden["start"]))
    assert abs(misfit - golden["misfit"]) <= FP32_TOL * golden["misfit"]
    out = gpu_outputs(m)
    errs = {name: rel_l2(out[name], golden[name]) for name in OUTPUTS}
    errs["gradient_vector"] = rel_l2(m.get_gradient_vector(), golden["gradient_vector"])
    print("fp32 relative L2 errors:", errs)
    for name, e in errs.items():
        assert e <= FP32_TOL, (name, e)


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("fp32", FP32_TOL)])
def test_notebook2_known_answers(precision, tol):
    m = psv.fdModel(NB2_INI, precision=precision)
    target, start = nb2_media(m.nx, m.nz, m.np_boundary, m.dx, m.dz)
    misfit = fwi_gradient(m, target, start)
    g = m.get_gradient_vector()
    assert g.size == 32400
    if precision == "fp64":
        assert round(misfit, 2) == NB2_MISFIT
        assert round(float(np.abs(g).max()), 4) == NB2_GRAD_INF
    else:
        assert abs(misfit - NB2_MISFIT) <= tol * NB2_MISFIT + 0.005
        assert abs(np.abs(g).max() - NB2_GRAD_INF) <= tol * NB2_GRAD_INF + 5e-5


def test_fp32_vs_fp64_gpu_nb2_full_outputs():
    """FP32 against the FP64 GPU solve on the 8000-step Notebook 2 case."""
    res = {}
    for prec in ("fp64", "fp32"):
        m = psv.fdModel(NB2_INI, precision=prec)
        target, start = nb2_media(m.nx, m.nz, m.np_boundary, m.dx, m.dz)
        fwi_gradient(m, target, start)
        res[prec] = gpu_outputs(m)
        res[prec]["g"] = m.get_gradient_vector()
    errs = {k: rel_l2(res["fp32"][k], res["fp64"][k]) for k in res["fp64"]}
    print("NB2 fp32 vs fp64:", errs)
    for k, e in errs.items():
        assert e <= FP32_TOL, (k, e)
