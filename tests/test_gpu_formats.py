"""Text files cross between this library and the psvWave reference.

tests/golden/ref_written.npz holds files the reference's own solver wrote
for the small golden run (tests/golden/make_formats.py): receivers
(src/fdModel.cpp:971-1006), sources (:1008-1032), kernels (:1326-1356),
wave-field dumps (:753-776) and a model-vector file its load_vector read
(:1517-1572).

* The FP64 GPU model, run the same way, writes the same files: byte for
  byte where the host matches the fixtures' (x86-64); elsewhere the same
  lines and numbers, within the last-bit libm differences of the setup
  tables (1e-10 for the 25-digit files, the sixth digit for the
  default-precision ones).
* It loads the reference-written receivers (load_receivers,
  src/fdModel.cpp:1053-1126) and vector file exactly.
"""
import os
import platform

import numpy as np
import pytest

import psvwave_gb300 as psv
from tests.conftest import GOLDEN, SMALL_INI, fwi_gradient

pytestmark = pytest.mark.gpu

SAME_ARCH_AS_FIXTURES = platform.machine() in ("x86_64", "AMD64")
FULL_PRECISION = ("rtf_", "sources_shot_")


@pytest.fixture(scope="module")
def ref_files():
    d = np.load(os.path.join(GOLDEN, "ref_written.npz"))
    return {k[5:]: d[k].tobytes() for k in d.files if k.startswith("file:")}, d["loaded_vector"]


def numbers(b):
    return np.array([float(x) for x in b.split()])


def write_ours(m, golden):
    os.makedirs("snapshots", exist_ok=True)
    fwi_gradient(m, tuple(golden["target"]), tuple(golden["start"]))
    m.write_receivers()
    m.write_sources()
    m.write_kernels()
    m.forward_simulate(0, False, output_wavefields=True)


def test_written_files_match_the_reference(golden, ref_files, tmp_path, monkeypatch):
    files, _ = ref_files
    monkeypatch.chdir(tmp_path)
    write_ours(psv.fdModel(SMALL_INI, precision="fp64"), golden)
    for name, ref in files.items():
        if name == "model_vector.txt":
            continue
        with open(name, "rb") as f:
            ours = f.read()
        if SAME_ARCH_AS_FIXTURES:
            assert ours == ref, name
            continue
        assert ours.count(b"\n") == ref.count(b"\n"), name
        a, b = numbers(ours), numbers(ref)
        assert a.shape == b.shape, name
        tol = 1e-10 if name.startswith(FULL_PRECISION) else 2e-5
        assert np.max(np.abs(a - b)) <= tol * np.max(np.abs(b)), name


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_loads_reference_written_receivers(ref_files, tmp_path, monkeypatch, precision):
    files, _ = ref_files
    monkeypatch.chdir(tmp_path)
    for name, data in files.items():
        if name.startswith("rtf_"):
            with open(name, "wb") as f:
                f.write(data)
    m = psv.fdModel(SMALL_INI, precision=precision)
    m.load_receivers()
    ux, uz = m.get_observed_data()
    for s in range(m.n_shots):
        assert np.array_equal(ux[s].reshape(-1), numbers(files["rtf_ux%d.txt" % s]))
        assert np.array_equal(uz[s].reshape(-1), numbers(files["rtf_uz%d.txt" % s]))


def test_load_vector_reads_the_reference_file(ref_files, tmp_path, monkeypatch):
    files, loaded = ref_files
    monkeypatch.chdir(tmp_path)
    with open("model_vector.txt", "wb") as f:
        f.write(files["model_vector.txt"])
    v = psv.fdModel(SMALL_INI).load_vector("model_vector.txt")
    assert np.array_equal(v, loaded)


def test_written_receivers_and_sources_load_back(golden, tmp_path, monkeypatch):
    """What this library writes, it reads back exactly (25 significant
    digits round-trip every double)."""
    monkeypatch.chdir(tmp_path)
    m = psv.fdModel(SMALL_INI, precision="fp64")
    write_ours(m, golden)
    m.load_receivers()
    for a, b in zip(m.get_observed_data(), m.get_synthetic_data()):
        assert np.array_equal(a, b)
