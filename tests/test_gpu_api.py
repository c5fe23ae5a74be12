"""The fdModel API on the GPU: the reference's own tests (determinism,
constructor equivalence, copy, descent) and the getters, setters and text
I/O of src/psvWave.cpp and src/fdModel.cpp."""
import os

import numpy as np
import pytest

import psvwave_gb300 as psv
from oracle import portbind
from tests.conftest import NB2_INI, SMALL_INI, fwi_gradient, nb2_media, rel_l2

pytestmark = pytest.mark.gpu


def small_params():
    return dict(nt=400, nx_inner=48, nz_inner=36, nx_inner_boundary=4, nz_inner_boundary=6,
                dx=1.249, dz=1.249, dt=0.00025, np_boundary=10, np_factor=0.05,
                scalar_rho=1500.0, scalar_vp=2000.0, scalar_vs=800.0, npx=2, npz=2,
                peak_frequency=50.0, source_timeshift=0.005, delay_cycles_per_shot=3,
                n_sources=3, ix_sources=[10, 30, 38], iz_sources=[8, 8, 27],
                moment_angles=[90, 45, 180], which_source_to_fire_in_which_shot=[[0, 1], [2]],
                nr=7, ix_receivers=[6, 12, 18, 24, 30, 36, 42],
                iz_receivers=[30, 30, 30, 30, 30, 30, 4], snapshot_interval=10)


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_forward_is_deterministic(precision):
    """tests/test_file_constructor.cpp: repeated forward runs give identical
    seismograms."""
    m = psv.fdModel(NB2_INI, precision=precision)
    sums = []
    for _ in range(2):
        for s in range(m.n_shots):
            m.forward_simulate(s, False)
        sums.append(m.get_synthetic_data()[0].sum())
    assert sums[0] == sums[1]


def test_explicit_constructor_matches_ini():
    """tests/test_constructor_comparison.cpp."""
    a = psv.fdModel(SMALL_INI, precision="fp64")
    b = psv.fdModel.from_parameters(small_params(), precision="fp64")
    for m in (a, b):
        for s in range(m.n_shots):
            m.forward_simulate(s, False)
    assert np.array_equal(a.get_synthetic_data()[0], b.get_synthetic_data()[0])
    assert np.array_equal(a.get_synthetic_data()[1], b.get_synthetic_data()[1])


def test_copy_gives_same_seismograms_and_is_independent():
    """tests/test_copy_constructor.cpp and tests/python/test_copy.py."""
    a = psv.fdModel(SMALL_INI)
    b = a.copy()
    for m in (a, b):
        m.forward_simulate(0, False)
    assert np.array_equal(a.get_synthetic_data()[0], b.get_synthetic_data()[0])
    a.set_model_vector(a.get_model_vector() + 1)
    b.set_model_vector(b.get_model_vector() - 1)
    assert np.any(a.get_model_vector() != b.get_model_vector())


def test_attributes_match_oracle():
    m = psv.fdModel(SMALL_INI)
    o = portbind.OracleModel(SMALL_INI)
    for k in ("nt", "nx", "nz", "nx_inner", "nz_inner", "nx_inner_boundary",
              "nz_inner_boundary", "np_boundary", "n_shots", "n_sources", "nr",
              "snapshot_interval", "snapshots", "nx_free_parameters", "nz_free_parameters",
              "free_parameters"):
        assert getattr(m, k) == o.info[k], k
    assert m.which_source_to_fire_in_which_shot == [[0, 1], [2]]
    assert (m.dt, m.dx, m.dz) == (0.00025, 1.249, 1.249)


def test_geometry_getters():
    m = psv.fdModel(SMALL_INI)
    np_, dx = m.np_boundary, m.dx
    x, z = m.get_sources()
    assert np.allclose(x, np.array([10, 30, 38]) * dx) and np.allclose(z, np.array([8, 8, 27]) * dx)
    x, z = m.get_sources(False, True)
    assert np.array_equal(x, np.array([10, 30, 38]) + np_)
    x, z = m.get_receivers(False, False)
    assert np.array_equal(x, [6, 12, 18, 24, 30, 36, 42]) and z[-1] == 4
    IX, IZ = m.get_coordinates(True)
    assert IX.shape == (m.nx, m.nz) and IX[0, 0] == -np_ * dx and IZ[0, 1] == (1 - np_) * dx
    IX, IZ = m.get_coordinates(False)
    assert IX[3, 0] == 3 and IZ[0, 5] == 5
    assert m.get_extent(True) == (-np_, dx * (48 + np_), -np_, dx * (36 + np_))
    assert m.get_extent(False) == (0, dx * 48, 0, dx * 36)


def test_setters_validate_shapes():
    m = psv.fdModel(SMALL_INI)
    vp, vs, rho = m.get_parameter_fields()
    with pytest.raises(ValueError, match="_vp"):
        m.set_parameter_fields(vp[:-1], vs, rho)
    ux, uz = m.get_synthetic_data()
    with pytest.raises(ValueError):
        m.set_observed_data(ux[:, :-1], uz)
    with pytest.raises(ValueError):
        m.forward_simulate(5)


def test_parameter_and_model_vector_roundtrip(golden):
    m = psv.fdModel(SMALL_INI, precision="fp64")
    m.set_parameter_fields(*golden["target"])
    vp, vs, rho = m.get_parameter_fields()
    assert np.array_equal(vp, golden["target"][0])
    o = portbind.OracleModel(SMALL_INI)
    o.set_parameter_fields(*golden["target"])
    assert np.array_equal(m.get_model_vector(), o.get_model_vector())
    v = m.get_model_vector() * 1.01
    m.set_model_vector(v)
    o.set_model_vector(v)
    assert np.array_equal(np.stack(m.get_parameter_fields()), np.stack(o.get_parameter_fields()))


def test_run_model_equals_manual_sequence(golden):
    a = psv.fdModel(SMALL_INI, precision="fp64")
    b = psv.fdModel(SMALL_INI, precision="fp64")
    fwi_gradient(a, tuple(golden["target"]), tuple(golden["start"]))
    b.set_parameter_fields(*golden["target"])
    for s in range(b.n_shots):
        b.forward_simulate(s)
    b.set_observed_data(*b.get_synthetic_data())
    b.set_parameter_fields(*golden["start"])
    b.run_model(False, True)
    assert a.misfit == b.misfit
    assert np.array_equal(a.get_gradient_vector(), b.get_gradient_vector())
    mis, g = b.compute_gradients()
    assert mis == a.misfit and np.array_equal(g, a.get_gradient_vector())


def test_text_io_roundtrips(tmp_path, golden):
    m = psv.fdModel(SMALL_INI, precision="fp64")
    cwd = os.getcwd()
    os.chdir(tmp_path)
    try:
        m.set_parameter_fields(*golden["target"])
        for s in range(m.n_shots):
            m.forward_simulate(s, False)
        m.write_receivers()
        m.write_sources()
        assert os.path.exists("rtf_ux1.txt") and os.path.exists("sources_shot_1.txt")
        m.load_receivers()
        assert np.array_equal(m.get_observed_data()[0], m.get_synthetic_data()[0])
        # load_model: ix-major whitespace text, exact round trip.
        names = []
        for name, arr in zip(("de", "vp", "vs"), (golden["start"][2], golden["start"][0],
                                                 golden["start"][1])):
            np.savetxt(name + ".txt", arr.reshape(-1), fmt="%.17g")
            names.append(name + ".txt")
        m.load_model(*names)
        vp, vs, rho = m.get_parameter_fields()
        assert np.array_equal(vp, golden["start"][0]) and np.array_equal(rho, golden["start"][2])
        with open("short.txt", "w") as f:
            f.write("1 2 3\n")
        with pytest.raises(ValueError, match="domain"):
            m.load_model("short.txt", names[1], names[2])
        with pytest.raises(ValueError):
            m.load_model("missing.txt", names[1], names[2])
        np.savetxt("vec.txt", np.arange(3 * m.nx_free_parameters * m.nz_free_parameters))
        v = m.load_vector("vec.txt")
        assert v.size == 3 * m.nx_free_parameters * m.nz_free_parameters and v[5] == 5
        m.reset_kernels()
        m.map_kernels_to_velocity()
        m.write_kernels()
        assert os.path.exists("kernel_vp.txt")
        os.makedirs("snapshots", exist_ok=True)
        m.forward_simulate(0, False, False, True)
        vx = np.loadtxt("snapshots/vx00010.txt")
        assert vx.shape == (m.nx, m.nz)
    finally:
        os.chdir(cwd)


def test_output_wavefields_does_not_change_results():
    a = psv.fdModel(SMALL_INI, precision="fp64")
    b = psv.fdModel(SMALL_INI, precision="fp64")
    a.forward_simulate(0, True)
    cwd = os.getcwd()
    import tempfile
    with tempfile.TemporaryDirectory() as d:
        os.chdir(d)
        os.makedirs("snapshots")
        try:
            b.forward_simulate(0, True, False, True)
        finally:
            os.chdir(cwd)
    assert np.array_equal(a.get_synthetic_data()[0], b.get_synthetic_data()[0])
    assert np.array_equal(a.get_snapshots()[2], b.get_snapshots()[2])


def test_descent_decreases_misfit():
    """tests/python/test_descent.py: three steps m -= 0.25 g on the
    Notebook 2 configuration lower the misfit."""
    m = psv.fdModel(NB2_INI)
    target, start = nb2_media(m.nx, m.nz, m.np_boundary, m.dx, m.dz)
    fwi_gradient(m, target, start)
    v = m.get_model_vector()
    misfits = []
    for _ in range(3):
        v = v - 0.25 * m.get_gradient_vector()
        m.set_model_vector(v)
        m.run_model(False, True)
        misfits.append(m.misfit)
    assert misfits[0] > misfits[-1]


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_graph_replay_matches_eager(golden, precision):
    """Repeated forward/adjoint loops replayed as CUDA graphs give the same
    bits as kernel-by-kernel launches."""
    res = []
    for graphs in (False, True):
        m = psv.fdModel(SMALL_INI, precision=precision)
        m.set_graph_capture(graphs)
        m.set_parameter_fields(*golden["target"])
        for _ in range(3):  # eager, capture, replay
            for s in range(m.n_shots):
                m.forward_simulate(s, True)
        m.set_observed_data(*m.get_synthetic_data())
        m.set_parameter_fields(*golden["start"])
        for _ in range(3):
            for s in range(m.n_shots):
                m.forward_simulate(s, True)
            m.calculate_l2_adjoint_sources()
            m.reset_kernels()
            for s in range(m.n_shots):
                m.adjoint_simulate(s)
        m.map_kernels_to_velocity()
        res.append((m.get_synthetic_data()[0], m.get_kernels()[1], m.get_wavefields()[0]))
    for a, b in zip(res[0], res[1]):
        assert np.array_equal(a, b)


def test_large_grid_defaults_to_persistent_launch():
    # 2100 x 900 points: 990 tiles of 32 x 60 per step, at least a full wave
    # of resident CTAs, so every time step runs in one persistent launch.
    from psvwave_gb300 import workloads

    m = psv.fdModel.from_parameters(workloads.c1_params(nt=10))
    assert m.tile_shape == "32x60"
    assert m.kernel_variant == "fused_tma_persistent"
    small = psv.fdModel(SMALL_INI)
    assert small.kernel_variant == "fused_cluster"


def test_mid_grid_defaults_to_small_tiles():
    # 1100 x 500 points: 315 tiles of 32 x 60 are less than a wave of
    # resident CTAs, so each step is one launch of 16 x 28 tiles.
    from psvwave_gb300 import workloads

    m = psv.fdModel.from_parameters(workloads.c3_params(nt=10, n_shots=1))
    assert m.kernel_variant == "fused_tma"
    assert m.tile_shape == "16x28"


def test_returned_arrays_are_independent_copies():
    """Getters return fresh arrays (src/psvWave.cpp:33-63) even though large
    ones are backed by pooled page-locked blocks: an array still held keeps
    its block, so later calls never write into it; a freed array's block is
    reused."""
    p = small_params()
    p.update(nt=10000)  # 2 shots x 7 receivers x 10000 steps x 8 B = 1.1 MB per component
    m = psv.fdModel.from_parameters(p, precision="fp64")
    big = m.get_lame_kernels()  # kernels: small grids stay plain numpy arrays
    m.forward_simulate(0, False)
    first = m.get_synthetic_data()
    keep = [a.copy() for a in first]
    m.set_parameter_fields(*(a * 1.01 for a in m.get_parameter_fields()))
    m.forward_simulate(0, False)
    second = m.get_synthetic_data()
    for a, k in zip(first, keep):
        assert np.array_equal(a, k)
    assert not np.array_equal(first[0], second[0])
    assert big[0].shape == (m.nx, m.nz)


def test_pinned_pool_reuses_freed_blocks():
    from psvwave_gb300 import model as model_module

    pool = model_module._PINNED
    shape = (256, 1024)  # 2 MB: taken from the pool
    a = pool.array(shape)
    a[...] = 1.0
    b = pool.array(shape)
    assert a.ctypes.data != b.ctypes.data
    addr = a.ctypes.data
    del a
    import gc

    gc.collect()
    c = pool.array(shape)
    assert c.ctypes.data == addr
    assert b.ctypes.data != c.ctypes.data


@pytest.mark.parametrize("variant", ["fused_tma", "fused_tma_persistent"])
def test_fp32_run_model_lanes_equal_serial_calls(golden, variant):
    """FP32 run_model runs its shots in concurrent lanes (per-shot kernel sums
    added in shot order); the serial forward_simulate / adjoint_simulate
    calls give the same seismograms, misfit and final wave fields bit for
    bit, and the same kernels up to the order of their FP64 sums."""
    a = psv.fdModel(SMALL_INI, precision="fp32")
    b = psv.fdModel(SMALL_INI, precision="fp32")
    for m in (a, b):
        m.kernel_variant = variant
    fwi_gradient(a, tuple(golden["target"]), tuple(golden["start"]))
    b.set_parameter_fields(*golden["target"])
    for s in range(b.n_shots):
        # Store snapshots as fwi_gradient does: at snapshot steps every tile
        # takes the general path, whose FMA contractions may differ from the
        # register-window paths' in the last bit.
        b.forward_simulate(s, True)
    b.set_observed_data(*b.get_synthetic_data())
    b.set_parameter_fields(*golden["start"])
    for _ in range(3):  # eager, graph capture, graph replay
        b.run_model(False, True)
        assert a.misfit == b.misfit
        for x, y in zip(a.get_synthetic_data(), b.get_synthetic_data()):
            assert np.array_equal(x, y)
        for x, y in zip(a.get_wavefields(), b.get_wavefields()):
            assert np.array_equal(x, y)
        for x, y in zip(a.get_lame_kernels(), b.get_lame_kernels()):
            assert rel_l2(y, x) <= 1e-12
        assert rel_l2(b.get_gradient_vector(), a.get_gradient_vector()) <= 1e-12
