"""psv_l2_misfit_noalloc: the L2 misfit for callers that cannot allocate
device memory (code running inside another framework's execution step, such
as a TensorRT plugin's enqueue or an XLA custom call, or inside a CUDA graph
capture). It takes the caller's device arrays and keeps its partial sums in a
fixed device array instead of allocated scratch.

Checked through the C ABI against the misfit of the existing entry point
(psv_calculate_l2_misfit on a model holding the same data), on two calls in
a row, to the FP64 reduction tolerance of the other misfit tests (1e-12
relative). This file is named to be collected last.
"""
import ctypes

import numpy as np
import pytest

import psvwave_gb300 as psv
from psvwave_gb300 import _capi
from tests.conftest import SMALL_INI

pytestmark = pytest.mark.gpu

MISFIT_TOL = 1e-12
MAX_SAMPLES = 8192 * 2048


def test_noalloc_misfit_matches_model_misfit_twice():
    torch = pytest.importorskip("torch")
    lib = _capi.load()
    m = psv.fdModel(SMALL_INI, precision="fp64")
    shape = (m.n_shots, m.nr, m.nt)
    n = int(np.prod(shape))
    rng = np.random.default_rng(2024)
    torch.cuda.set_device(0)
    stream = torch.cuda.current_stream()
    for call in range(2):
        obs = [rng.standard_normal(shape) * (call + 1) for _ in range(2)]
        syn = [rng.standard_normal(shape) for _ in range(2)]
        m.set_observed_data(*obs)
        m.set_synthetic_data(*syn)
        m.calculate_l2_misfit()
        expected = m.misfit
        dev = [torch.from_numpy(a).to("cuda:0") for a in (obs[0], syn[0], obs[1], syn[1])]
        out = torch.full((1,), float("nan"), dtype=torch.float64, device="cuda:0")
        torch.cuda.synchronize()
        rc = lib.psv_l2_misfit_noalloc(*[ctypes.c_void_p(t.data_ptr()) for t in dev], n, m.dt,
                                       ctypes.c_void_p(out.data_ptr()),
                                       ctypes.c_void_p(stream.cuda_stream))
        assert rc == _capi.PSV_OK, lib.psv_last_error()
        torch.cuda.synchronize()
        got = float(out.item())
        assert abs(got - expected) <= MISFIT_TOL * abs(expected), (call, got, expected)


def test_noalloc_misfit_rejects_oversize_input():
    torch = pytest.importorskip("torch")
    lib = _capi.load()
    buf = torch.zeros(4, dtype=torch.float64, device="cuda:0")
    out = torch.zeros(1, dtype=torch.float64, device="cuda:0")
    p = ctypes.c_void_p(buf.data_ptr())
    rc = lib.psv_l2_misfit_noalloc(p, p, p, p, MAX_SAMPLES + 1, 1.0,
                                   ctypes.c_void_p(out.data_ptr()), None)
    assert rc == _capi.PSV_ERR_INVALID_ARGUMENT
    assert b"maximum of 16777216" in lib.psv_last_error()


def test_noalloc_misfit_accepts_the_maximum_size():
    """n at the stated maximum (every one of the 8192 partial sums in use)
    is accepted and sums like a plain FP64 reduction of the same samples."""
    torch = pytest.importorskip("torch")
    lib = _capi.load()
    g = torch.Generator(device="cuda:0")
    g.manual_seed(7)
    obs_ux, syn_ux, obs_uz, syn_uz = (
        torch.randn(MAX_SAMPLES, dtype=torch.float64, device="cuda:0", generator=g)
        for _ in range(4))
    dt = 2.5e-4
    expected = float(0.5 * dt * (((obs_ux - syn_ux) ** 2).sum() + ((obs_uz - syn_uz) ** 2).sum()))
    out = torch.full((1,), float("nan"), dtype=torch.float64, device="cuda:0")
    torch.cuda.synchronize()
    rc = lib.psv_l2_misfit_noalloc(*[ctypes.c_void_p(t.data_ptr())
                                     for t in (obs_ux, syn_ux, obs_uz, syn_uz)],
                                   MAX_SAMPLES, dt, ctypes.c_void_p(out.data_ptr()), None)
    assert rc == _capi.PSV_OK, lib.psv_last_error()
    torch.cuda.synchronize()
    got = float(out.item())
    assert abs(got - expected) <= MISFIT_TOL * abs(expected), (got, expected)
