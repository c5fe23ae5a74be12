"""Files this library writes load in the psvWave reference's own build.

tests/golden/repo_written.npz holds the receiver and source files that the
FP64 GPU model wrote for the small golden run
(tests/golden/make_repo_written.py, on a GPU host), with the seismograms it
held. Here, where the reference's build (oracle/_ref) exists, the reference's
load_receivers (src/fdModel.cpp:1053-1126) reads them exactly, and they
carry the seismograms the reference itself computes for the same run (to
1e-10: the fixture was made on an aarch64 host whose libm may round the
setup tables' last bit differently). The reference-written fixtures
(tests/golden/ref_written.npz) parse to the golden seismograms bit for bit.
"""
import os

import numpy as np
import pytest

from oracle import refbind
from tests.conftest import GOLDEN, SMALL_INI, fwi_gradient, rel_l2


def numbers(b):
    return np.array([float(x) for x in b.split()])


def files(name):
    d = np.load(os.path.join(GOLDEN, name))
    return {k[5:]: d[k].tobytes() for k in d.files if k.startswith("file:")}, d


def test_reference_written_fixture_parses_to_golden_seismograms(golden):
    f, _ = files("ref_written.npz")
    for s in range(2):
        assert np.array_equal(numbers(f["rtf_ux%d.txt" % s]), golden["rtf_ux"][s].reshape(-1))
        assert np.array_equal(numbers(f["rtf_uz%d.txt" % s]), golden["rtf_uz"][s].reshape(-1))


@pytest.mark.skipif(not refbind.available(), reason="the reference's build is not on this host")
def test_reference_loads_repo_written_receivers(golden, tmp_path, monkeypatch):
    f, d = files("repo_written.npz")
    monkeypatch.chdir(tmp_path)
    for name, data in f.items():
        with open(name, "wb") as fh:
            fh.write(data)
    r = refbind.RefModel(SMALL_INI)
    r.load_receivers()
    ox, oz = r.get_observed_data()
    assert np.array_equal(ox, d["rtf_ux"]) and np.array_equal(oz, d["rtf_uz"])
    for s in range(2):
        assert np.array_equal(ox[s].reshape(-1), numbers(f["rtf_ux%d.txt" % s]))
    ref = refbind.RefModel(SMALL_INI)
    fwi_gradient(ref, tuple(golden["target"]), tuple(golden["start"]))
    for a, b in zip((ox, oz), ref.get_synthetic_data()):
        assert rel_l2(a, b) <= 1e-10
    for s in range(2):
        a = numbers(f["sources_shot_%d.txt" % s])
        src = [k for k in range(3) if k in ([0, 1], [2])[s]]
        b = np.concatenate([ref.array("stf")[k] for k in src])
        assert rel_l2(a, b) <= 1e-10
