import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")
SMALL_INI = os.path.join(GOLDEN, "small.ini")
NB2_INI = os.path.join(GOLDEN, "nb2.ini")

# Known answers of the reference's Notebook 2 ("Full-waveform inversion using
# psvWave", cells 10 and 17): the starting L2 misfit and the max-norm of the
# first gradient (L-BFGS-B's |proj g| at iterate 0, N = 32400).
NB2_MISFIT = 1920401.82
NB2_GRAD_INF = 77.1590


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def gpu_count():
    try:
        import ctypes

        from psvwave_gb300 import _capi

        n = ctypes.c_int(0)
        _capi.load().psv_device_count(ctypes.byref(n))
        return n.value
    except Exception:
        return 0


@pytest.fixture(scope="session")
def golden():
    return dict(np.load(os.path.join(GOLDEN, "small_golden.npz")))


def rel_l2(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    den = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (den if den > 0 else 1.0))


def nb2_media(nx, nz, np_boundary, dx, dz):
    from tests.golden.make_golden import nb2_media as f

    return f(nx, nz, np_boundary, dx, dz)


def fwi_gradient(m, target, start):
    """Observed data from `target`, one gradient at `start`, through the
    reference's documented call order (src/psvWave.cpp:518-545)."""
    m.set_parameter_fields(*target)
    for s in range(m.n_shots):
        m.forward_simulate(s, True)
    m.set_observed_data(*m.get_synthetic_data())
    m.set_parameter_fields(*start)
    for s in range(m.n_shots):
        m.forward_simulate(s, True)
    m.calculate_l2_misfit()
    misfit = m.misfit
    m.calculate_l2_adjoint_sources()
    m.reset_kernels()
    for s in range(m.n_shots):
        m.adjoint_simulate(s)
    m.map_kernels_to_velocity()
    return misfit
