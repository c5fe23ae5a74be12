"""The oracle port (oracle/psv_oracle.c) pinned against the reference's own
solver: bit-exact against the golden fixtures that the reference produced
(tests/golden/make_golden.py), against Notebook 2's known answers, and, where
the reference build is present, against the reference on further cases."""
import numpy as np
import pytest

from oracle import portbind, refbind
from tests.conftest import (NB2_GRAD_INF, NB2_INI, NB2_MISFIT, SMALL_INI, fwi_gradient,
                            nb2_media)


def test_port_config_matches_reference(golden):
    m = portbind.OracleModel(SMALL_INI)
    assert [m.info[k] for k in portbind.INFO_FIELDS] == list(golden["info"])
    assert np.array_equal(m.array("taper"), golden["taper"])
    assert np.array_equal(m.array("stf"), golden["stf"])
    assert np.array_equal(m.array("moment"), golden["moment"])


def test_port_fwi_gradient_bit_exact(golden):
    m = portbind.OracleModel(SMALL_INI)
    misfit = fwi_gradient(m, tuple(golden["target"]), tuple(golden["start"]))
    assert misfit == golden["misfit"]
    for name in ("rtf_ux", "rtf_uz", "a_stf_ux", "a_stf_uz", "lambda_kernel", "mu_kernel",
                 "density_l_kernel", "vp_kernel", "vs_kernel", "density_v_kernel"):
        assert np.array_equal(m.array(name), golden[name]), name
    assert np.array_equal(m.array("rtf_ux_true"), golden["obs_ux"])
    assert np.array_equal(m.get_model_vector(), golden["model_vector"])
    assert np.array_equal(m.get_gradient_vector(), golden["gradient_vector"])
    snap = np.stack([m.array(n)[1, 25] for n in
                     ("accu_vx", "accu_vz", "accu_txx", "accu_tzz", "accu_txz")])
    assert np.array_equal(snap, golden["snap_shot1_25"])
    fields = np.stack([m.array(n) for n in ("vx", "vz", "txx", "tzz", "txz")])
    assert np.array_equal(fields, golden["adjoint_fields"])


def test_port_notebook2_known_answers():
    m = portbind.OracleModel(NB2_INI)
    s = m.scalars()
    target, start = nb2_media(m.nx, m.nz, m.np_boundary, s["dx"], s["dz"])
    misfit = fwi_gradient(m, target, start)
    g = m.get_gradient_vector()
    assert g.size == 32400
    assert round(misfit, 2) == NB2_MISFIT
    assert round(float(np.abs(g).max()), 4) == NB2_GRAD_INF


def test_port_copy_is_independent(golden):
    a = portbind.OracleModel(SMALL_INI)
    a.set_parameter_fields(*golden["target"])
    b = a.copy()
    assert np.array_equal(b.array("lm"), a.array("lm"))
    a.set_model_vector(a.get_model_vector() + 1)
    b.set_model_vector(b.get_model_vector() - 1)
    assert np.any(a.get_model_vector() != b.get_model_vector())


@pytest.mark.parametrize("edit,msg", [
    ({"n_sources": 2}, "n_sources"),
    ({"nr": 5}, "nr"),
    ({"snapshot_interval": 7}, "Snapshot interval"),
])
def test_port_rejects_inconsistent_configs(tmp_path, edit, msg):
    text = open(SMALL_INI).read()
    for k, v in edit.items():
        lines = []
        for line in text.splitlines():
            if line.split("=")[0].strip() == k:
                line = "%s = %s" % (k, v)
            lines.append(line)
        text = "\n".join(lines)
    p = tmp_path / "bad.ini"
    p.write_text(text)
    with pytest.raises(ValueError, match=msg):
        portbind.OracleModel(str(p))


@pytest.mark.skipif(not refbind.available(), reason="reference build not present")
def test_port_matches_reference_on_seeded_case(tmp_path):
    """A second configuration: 3 shots, np_factor 0.03, receivers on two
    depths, seeded random medium; every output bit-exact."""
    text = open(SMALL_INI).read()
    text = text.replace("np_factor = 0.05", "np_factor = 0.03")
    text = text.replace("nt = 400;", "nt = 300;")
    text = text.replace("n_sources = 3;", "n_sources = 3;")
    text = text.replace("n_shots = 2;", "n_shots = 3;")
    text = text.replace("{{0, 1}, {2}}", "{{0}, {1}, {2}}")
    text = text.replace("moment_angles = {90, 45, 180}", "moment_angles = {30, 60, 120}")
    p = tmp_path / "case.ini"
    p.write_text(text)
    r, o = refbind.RefModel(str(p)), portbind.OracleModel(str(p))
    rng = np.random.default_rng(3)
    tgt = (2000 * (1 + 0.03 * rng.standard_normal((r.nx, r.nz))),
           800 * (1 + 0.03 * rng.standard_normal((r.nx, r.nz))),
           1500 * (1 + 0.03 * rng.standard_normal((r.nx, r.nz))))
    start = tuple(np.full((r.nx, r.nz), v) for v in (2000.0, 800.0, 1500.0))
    mr = fwi_gradient(r, tgt, start)
    mo = fwi_gradient(o, tgt, start)
    assert mr == mo
    for name in ("rtf_ux", "rtf_uz", "lambda_kernel", "mu_kernel", "density_l_kernel",
                 "vp_kernel", "vs_kernel", "density_v_kernel", "vx", "txz"):
        assert np.array_equal(r.array(name), o.array(name)), name
    assert np.array_equal(r.get_gradient_vector(), o.get_gradient_vector())


def _tiny_ini(nxi, nzi, npb, sources, receivers, shots, nt=120):
    """A tiny configuration in the reference's INI dialect (sources as
    (ix, iz, angle), receivers as (ix, iz), inner-grid indices)."""
    lst = lambda v: "{" + ", ".join(str(x) for x in v) + "}"
    return "\n".join([
        "[domain]", "nt = %d" % nt, "nx_inner = %d" % nxi, "nz_inner = %d" % nzi,
        "nx_inner_boundary = 1", "nz_inner_boundary = 1", "dx = 1.0", "dz = 1.0",
        "dt = 0.0001",
        "[boundary]", "np_boundary = %d" % npb, "np_factor = 0.05",
        "[medium]", "scalar_rho = 1500.0", "scalar_vp = 2000.0", "scalar_vs = 800.0",
        "[sources]", "peak_frequency = 200.0", "n_sources = %d" % len(sources),
        "n_shots = %d" % len(shots), "source_timeshift = 0.002", "delay_cycles_per_shot = 1",
        "moment_angles = " + lst([s[2] for s in sources]),
        "ix_sources = " + lst([s[0] for s in sources]),
        "iz_sources = " + lst([s[1] for s in sources]),
        "which_source_to_fire_in_which_shot = {" + ", ".join(lst(s) for s in shots) + "}",
        "[receivers]", "nr = %d" % len(receivers),
        "ix_receivers = " + lst([r[0] for r in receivers]),
        "iz_receivers = " + lst([r[1] for r in receivers]),
        "[inversion]", "snapshot_interval = 10",
        "[basis]", "npx = 1", "npz = 1",
        "[output]", "observed_data_folder = .", "stf_folder = .", ""])


@pytest.mark.skipif(not refbind.available(), reason="reference build not present")
@pytest.mark.parametrize("case", [
    # 16 x 14 points: two sources at one cell, coinciding receivers
    (8, 6, 4, [(3, 2, 30.0), (3, 2, 75.0), (6, 4, 120.0)], [(1, 1), (5, 3), (5, 3)],
     [[0, 1, 2]]),
    # 28 x 18 points: two shots, sources and receivers next to the frame
    (20, 10, 4, [(2, 2, 45.0), (17, 7, 10.0)], [(4, 1), (10, 8), (15, 5), (19, 9)],
     [[0], [1]]),
])
def test_port_matches_reference_on_tiny_grids(tmp_path, case):
    """Grids smaller than a GPU tile, with coinciding sources and receivers:
    every output bit-exact between the port and the reference."""
    p = tmp_path / "tiny.ini"
    p.write_text(_tiny_ini(*case))
    r, o = refbind.RefModel(str(p)), portbind.OracleModel(str(p))
    rng = np.random.default_rng(1)
    tgt = tuple(v * (1 + 0.05 * rng.standard_normal((r.nx, r.nz)))
                for v in (2000.0, 800.0, 1500.0))
    start = tuple(np.full((r.nx, r.nz), v) for v in (2000.0, 800.0, 1500.0))
    assert fwi_gradient(r, tgt, start) == fwi_gradient(o, tgt, start)
    for name in ("rtf_ux", "rtf_uz", "lambda_kernel", "mu_kernel", "density_l_kernel",
                 "vp_kernel", "vs_kernel", "density_v_kernel", "vx", "vz", "txx", "tzz", "txz"):
        assert np.array_equal(r.array(name), o.array(name)), name
    assert np.array_equal(r.get_gradient_vector(), o.get_gradient_vector())
