"""Source generalisation (fdModel.set_stf / set_moment, psv_set_stf /
psv_set_moment): custom wavelets and full, non-symmetric 2 x 2 moment
tensors go through the same injection terms as the reference's Ricker
dip sources (src/fdModel.cpp:681-751).

* FP64: seismograms are bit-identical to the oracle port run with the same
  wavelets and tensors written into its arrays.
* FP32: within 1e-4 relative L2 of FP64.
* Putting back the defaults restores the default seismograms bit for bit,
  and doubling the wavelets doubles the seismograms (the scheme is linear
  in the source; scaling by 2 is exact in floating point except where
  intermediates are subnormal).
"""
import numpy as np
import pytest

import psvwave_gb300 as psv
from tests.conftest import SMALL_INI, rel_l2

pytestmark = pytest.mark.gpu


def custom_sources(n_sources, nt, dt):
    """Seeded wavelets (Gaussian-windowed sine bursts of differing
    frequency and delay) and non-symmetric tensors."""
    rng = np.random.default_rng(11)
    t = np.arange(nt) * dt
    stf = np.empty((n_sources, nt))
    for s in range(n_sources):
        f = rng.uniform(30.0, 60.0)
        t0 = rng.uniform(0.01, 0.03)
        stf[s] = np.sin(2 * np.pi * f * (t - t0)) * np.exp(-((t - t0) * f * 1.5) ** 2)
    moment = rng.standard_normal((n_sources, 2, 2)) * 1e15
    return stf, moment


def run(m, fields):
    m.set_parameter_fields(*fields)
    for s in range(m.n_shots):
        m.forward_simulate(s, False)
    return m.get_synthetic_data()


def test_custom_sources_match_the_oracle_bitwise(golden):
    from oracle.portbind import OracleModel

    m = psv.fdModel(SMALL_INI, precision="fp64")
    stf, moment = custom_sources(m.n_sources, m.nt, m.dt)
    m.set_stf(stf)
    m.set_moment(moment)
    assert np.array_equal(m.get_stf(), stf) and np.array_equal(m.get_moment(), moment)
    ux, uz = run(m, golden["target"])

    o = OracleModel(SMALL_INI)
    o.view("stf")[...] = stf
    o.view("moment")[...] = moment
    o.set_parameter_fields(*golden["target"])
    for s in range(o.n_shots):
        o.forward_simulate(s, False)
    ox, oz = o.get_synthetic_data()
    assert np.abs(ox).max() > 0
    assert np.array_equal(ux, ox) and np.array_equal(uz, oz)

    m32 = psv.fdModel(SMALL_INI)
    m32.set_stf(stf)
    m32.set_moment(moment)
    fx, fz = run(m32, golden["target"])
    assert rel_l2(fx, ox) <= 1e-4 and rel_l2(fz, oz) <= 1e-4


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_defaults_restore_and_wavelets_scale_exactly(golden, precision):
    m = psv.fdModel(SMALL_INI, precision=precision)
    base = run(m, golden["target"])
    stf0, mom0 = m.get_stf(), m.get_moment()
    stf, moment = custom_sources(m.n_sources, m.nt, m.dt)
    m.set_stf(stf)
    m.set_moment(moment)
    custom = run(m, golden["target"])
    assert not np.array_equal(custom[0], base[0])
    m.set_stf(2.0 * stf)
    doubled = run(m, golden["target"])
    # Exact up to subnormal intermediates near the leading wave front, whose
    # rounding does not scale.
    tol = 1e-12 if precision == "fp64" else 1e-6
    for a, b in zip(doubled, custom):
        print("exactly doubled:", np.array_equal(a, 2.0 * b))
        assert rel_l2(a, 2.0 * b) <= tol
    m.set_stf(stf0)
    m.set_moment(mom0)
    for a, b in zip(run(m, golden["target"]), base):
        assert np.array_equal(a, b)


def test_bad_source_arrays_are_rejected():
    m = psv.fdModel(SMALL_INI)
    with pytest.raises(ValueError):
        m.set_stf(np.zeros((m.n_sources, m.nt + 1)))
    bad = m.get_moment()
    bad[0, 0, 0] = np.nan
    with pytest.raises(Exception):
        m.set_moment(bad)
