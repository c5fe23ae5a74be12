"""Parity of the GPU solver with the reference.

FP64 wave fields reproduce the reference bit for bit (golden fixtures made by
the reference, tests/golden/make_golden.py, and the oracle port on the same
machine); only the misfit, a parallel FP64 reduction, differs in the last
bits (tolerance 1e-12 relative).

FP32 wave fields are held to the tolerance of the production path: relative
L2 error <= 1e-4 against the FP64 answer for seismograms, misfit, adjoint
sources, kernels and the gradient vector.
"""
import platform

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


# The golden fixtures were made on x86-64. Where the GPU host is another
# architecture, its libm may round exp/sin/cos of the setup tables (Ricker
# wavelet, moment tensor, taper) differently in the last bit, so there the
# comparison with the fixtures is held to 1e-10 relative L2, and bit-exactness
# is asserted against the oracle port built on the same machine instead.
SAME_ARCH_AS_GOLDEN = platform.machine() in ("x86_64", "AMD64")


def assert_golden(a, b, name):
    if SAME_ARCH_AS_GOLDEN:
        assert np.array_equal(a, b), (name, rel_l2(a, b))
    else:
        assert rel_l2(a, b) <= 1e-10, (name, rel_l2(a, b))


def test_setup_tables_bit_exact(golden):
    m = psv.fdModel(SMALL_INI, precision="fp64")
    o = portbind.OracleModel(SMALL_INI)
    assert np.array_equal(m.get_taper(), o.array("taper"))
    assert np.array_equal(m.get_stf(), o.array("stf"))
    assert np.array_equal(m.get_moment(), o.array("moment"))
    for name in ("taper", "stf", "moment"):
        assert_golden(getattr(m, "get_" + name)(), golden[name], name)


def test_fp64_gradient_vs_reference_golden(golden):
    m = psv.fdModel(SMALL_INI, precision="fp64")
    misfit = fwi_gradient(m, tuple(golden["target"]), tuple(golden["start"]))
    assert abs(misfit - golden["misfit"]) <= MISFIT_FP64_TOL * golden["misfit"]
    out = gpu_outputs(m)
    for name in OUTPUTS:
        assert_golden(out[name], golden[name], name)
    assert_golden(m.get_observed_data()[0], golden["obs_ux"], "obs")
    assert np.array_equal(m.get_model_vector(), golden["model_vector"])
    assert_golden(m.get_gradient_vector(), golden["gradient_vector"], "gradient")
    snaps = m.get_snapshots()
    assert_golden(np.stack([s[1, 25] for s in snaps]), golden["snap_shot1_25"], "snapshot")
    assert_golden(np.stack(m.get_wavefields()), golden["adjoint_fields"], "adjoint fields")


def test_fp64_gradient_bit_exact_vs_oracle_same_machine(golden):
    o = portbind.OracleModel(SMALL_INI)
    m = psv.fdModel(SMALL_INI, precision="fp64")
    mo = fwi_gradient(o, tuple(golden["target"]), tuple(golden["start"]))
    mg = fwi_gradient(m, tuple(golden["target"]), tuple(golden["start"]))
    assert abs(mg - mo) <= MISFIT_FP64_TOL * mo
    out = gpu_outputs(m)
    for name in OUTPUTS:
        assert np.array_equal(out[name], o.array(name)), (name, rel_l2(out[name], o.array(name)))
    assert np.array_equal(m.get_gradient_vector(), o.get_gradient_vector())
    snaps = m.get_snapshots()
    for k, n in enumerate(("accu_vx", "accu_vz", "accu_txx", "accu_tzz", "accu_txz")):
        assert np.array_equal(snaps[k], o.array(n)), n
    fields = m.get_wavefields()
    for k, n in enumerate(("vx", "vz", "txx", "tzz", "txz")):
        assert np.array_equal(fields[k], o.array(n)), n


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


def test_default_variants():
    """Small FP32 grids run cluster-resident, whatever nz is (nz = 56 and
    nz = 150, padded to 152); the TMA step is available on them too; FP64
    models use the two-kernel step."""
    for ini in (SMALL_INI, NB2_INI):
        m = psv.fdModel(ini)
        assert m.kernel_variant == "fused_cluster"
        m.kernel_variant = "fused_tma"
        assert m.kernel_variant == "fused_tma"
    assert psv.fdModel(SMALL_INI, precision="fp64").kernel_variant == "two_kernel"
    with pytest.raises(ValueError):
        psv.fdModel(SMALL_INI, precision="fp64").kernel_variant = "fused_tma"
    with pytest.raises(ValueError):
        psv.fdModel(SMALL_INI, precision="fp64").kernel_variant = "fused_cluster"


@pytest.mark.parametrize("variant", ["fused_cluster", "fused_tma", "fused_tma_persistent", "fused",
                                     "two_kernel"])
def test_fp32_variants_within_tolerance(golden, variant):
    m = psv.fdModel(SMALL_INI, precision="fp32")
    m.kernel_variant = variant
    assert m.kernel_variant == variant
    fwi_gradient(m, tuple(golden["target"]), tuple(golden["start"]))
    out = gpu_outputs(m)
    for name in OUTPUTS:
        assert rel_l2(out[name], golden[name]) <= FP32_TOL, name


def test_fp32_fused_vs_two_kernel_agree():
    """The two FP32 kernel variants agree to FP32 rounding on the 8000-step
    Notebook 2 run: seismograms within 1e-5, and the stored wave fields at
    four instants while the wave is in the grid within 1e-4."""
    res = []
    for variant in ("fused", "two_kernel"):
        m = psv.fdModel(NB2_INI, precision="fp32")
        m.kernel_variant = variant
        target, _ = nb2_media(m.nx, m.nz, m.np_boundary, m.dx, m.dz)
        m.set_parameter_fields(*target)
        m.forward_simulate(0, True)
        snaps = m.get_snapshots()
        res.append((m.get_synthetic_data(), [s[0, [100, 200, 400, 600]] for s in snaps]))
    for a, b in zip(res[0][0], res[1][0]):
        assert rel_l2(a, b) <= 1e-5
    for a, b in zip(res[0][1], res[1][1]):
        assert rel_l2(a, b) <= 1e-4


def test_fp64_rejects_fused_variant():
    m = psv.fdModel(SMALL_INI, precision="fp64")
    with pytest.raises(ValueError):
        m.kernel_variant = "fused"


def test_fp32_tma_vs_two_kernel_agree(golden):
    """The TMA variant against the two-kernel variant on the small grid:
    seismograms and every stored snapshot agree to FP32 rounding."""
    res = []
    for variant in ("fused_tma", "two_kernel"):
        m = psv.fdModel(SMALL_INI, precision="fp32")
        m.kernel_variant = variant
        m.set_parameter_fields(*golden["target"])
        for s in range(m.n_shots):
            m.forward_simulate(s, True)
        res.append((m.get_synthetic_data(), m.get_snapshots()))
    for a, b in zip(res[0][0], res[1][0]):
        assert rel_l2(a, b) <= 1e-5
    for a, b in zip(res[0][1], res[1][1]):
        assert rel_l2(a, b) <= 1e-5


def test_tile_shapes_agree_and_autotune(golden):
    """Both tile shapes of the TMA step give the same seismograms to FP32
    rounding and stay within tolerance of the reference; the autotuner picks
    one of them."""
    res = {}
    for shape in ("32x60", "16x28", "20x28", "16x60"):
        m = psv.fdModel(SMALL_INI, precision="fp32")
        m.tile_shape = shape
        assert m.tile_shape == shape
        fwi_gradient(m, tuple(golden["target"]), tuple(golden["start"]))
        out = gpu_outputs(m)
        for name in OUTPUTS:
            assert rel_l2(out[name], golden[name]) <= FP32_TOL, (shape, name)
        res[shape] = out
    for name in ("rtf_ux", "rtf_uz"):
        assert rel_l2(res["32x60"][name], res["16x28"][name]) <= 1e-5
        assert rel_l2(res["32x60"][name], res["20x28"][name]) <= 1e-5
        assert rel_l2(res["32x60"][name], res["16x60"][name]) <= 1e-5
    m = psv.fdModel(SMALL_INI, precision="fp32")
    assert m.autotune(20) in ("32x60", "16x28", "20x28", "16x60")


@pytest.mark.parametrize("shape", ["32x60", "16x28", "20x28", "16x60"])
@pytest.mark.parametrize("ini", [SMALL_INI, NB2_INI])
def test_persistent_step_matches_per_step_launches_bitwise(golden, shape, ini):
    """The persistent variant runs the per-step variant's arithmetic tile by
    tile, only scheduled differently (a tile starts a step once its
    neighbours have finished the previous one): forward seismograms and
    snapshots, and the adjoint's kernels, are identical bit for bit."""
    res = []
    for variant in ("fused_tma", "fused_tma_persistent"):
        m = psv.fdModel(ini, precision="fp32")
        m.kernel_variant = variant
        m.tile_shape = shape
        if ini == SMALL_INI:
            target, start = tuple(golden["target"]), tuple(golden["start"])
        else:
            target, start = nb2_media(m.nx, m.nz, m.np_boundary, m.dx, m.dz)
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
        res.append((m.get_synthetic_data(), m.get_snapshots(), m.get_lame_kernels(), m.misfit))
    (d0, s0, k0, m0), (d1, s1, k1, m1) = res
    assert m0 == m1
    for a, b in zip(d0 + s0 + k0, d1 + s1 + k1):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("ini", [SMALL_INI, NB2_INI])
def test_cluster_matches_per_step_launches(golden, ini):
    """The cluster-resident variant keeps the grid in the shared memory of
    one thread-block cluster and runs the TMA step's point arithmetic (the
    same expressions; the compiler contracts a few products into fused
    multiply-adds differently): forward seismograms and snapshots, the
    adjoint's kernels and the misfit agree to FP32 rounding."""
    res = []
    for variant in ("fused_tma", "fused_cluster"):
        m = psv.fdModel(ini, precision="fp32")
        m.kernel_variant = variant
        if ini == SMALL_INI:
            target, start = tuple(golden["target"]), tuple(golden["start"])
        else:
            target, start = nb2_media(m.nx, m.nz, m.np_boundary, m.dx, m.dz)
        m.set_parameter_fields(*target)
        for s in range(m.n_shots):
            m.forward_simulate(s, False)
        m.set_observed_data(*m.get_synthetic_data())
        m.set_parameter_fields(*start)
        for s in range(m.n_shots):
            m.forward_simulate(s, True)
        fwd = m.get_wavefields()
        m.calculate_l2_misfit()
        m.calculate_l2_adjoint_sources()
        m.reset_kernels()
        for s in range(m.n_shots):
            m.adjoint_simulate(s)
        res.append((m.get_synthetic_data(), m.get_snapshots(), m.get_lame_kernels(), fwd,
                    m.get_wavefields(), m.misfit))
    # (The final wave fields are what the absorbing frame leaves after the
    # wave has gone, rounding-level residue; the snapshots compare the
    # fields while the wave is in the grid.)
    (d0, s0, k0, _, _, m0), (d1, s1, k1, _, _, m1) = res
    assert abs(m0 - m1) <= 1e-6 * abs(m0)
    for a, b in zip(d0 + s0 + k0, d1 + s1 + k1):
        assert rel_l2(a, b) <= 1e-5
