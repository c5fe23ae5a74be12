"""The C-ABI library without a GPU: it loads, exports every function that
include/psvwave.h declares, parses and validates configurations like the
reference, and reports errors through status codes and psv_last_error()."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

import psvwave_gb300
from oracle import portbind
from psvwave_gb300 import _capi
from tests.conftest import NB2_INI, ROOT, SMALL_INI


def declared_functions():
    names = set()
    for header in ("psvwave.h", "psvwave_surrogate.h"):
        text = open(os.path.join(ROOT, "include", header)).read()
        names |= set(re.findall(r"^\s*(?:int|const char \*)\s*(psv_\w+)\s*\(", text, re.M))
    return sorted(names)


def test_library_exports_every_declared_function():
    lib_path = _capi.load() and _capi.library_path()
    out = subprocess.run(["nm", "-D", "--defined-only", lib_path], capture_output=True,
                         text=True, check=True).stdout
    exported = set(re.findall(r"\bT (psv_\w+)", out))
    declared = declared_functions()
    assert len(declared) >= 50
    missing = [f for f in declared if f not in exported]
    assert not missing, missing
    lib = _capi.load()
    for f in declared:
        assert hasattr(lib, f)
    assert set(declared) <= set(_capi._SIGNATURES), set(declared) - set(_capi._SIGNATURES)


def test_abi_version_and_errors():
    lib = _capi.load()
    assert lib.psv_abi_version() == 1
    info = _capi.PsvInfo()
    assert lib.psv_config_info(b"/nonexistent/config.ini", ctypes.byref(info)) == \
        _capi.PSV_ERR_INVALID_ARGUMENT
    assert lib.psv_last_error() == b"Can't load .ini file."
    assert lib.psv_config_info(None, ctypes.byref(info)) == _capi.PSV_ERR_INVALID_ARGUMENT
    assert lib.psv_destroy(None) == _capi.PSV_OK
    assert lib.psv_forward_simulate(None, 0, 1, 0, 0) == _capi.PSV_ERR_INVALID_ARGUMENT


def config_info(path):
    info = _capi.PsvInfo()
    _capi.check(_capi.load().psv_config_info(str(path).encode(), ctypes.byref(info)))
    return info


@pytest.mark.parametrize("ini", [SMALL_INI, NB2_INI])
def test_config_parse_matches_oracle(ini):
    info = config_info(ini)
    o = portbind.OracleModel(ini)
    for k in portbind.INFO_FIELDS:
        key = {"npx": "basis_gridpoints_x", "npz": "basis_gridpoints_z"}.get(k, k)
        assert getattr(info, key) == o.info[k], k
    s = o.scalars()
    for k in ("dt", "dx", "dz", "np_factor", "peak_frequency", "alpha", "delay_cycles_per_shot"):
        assert getattr(info, k) == s[k], k


def write_ini(tmp_path, text, name="c.ini"):
    p = tmp_path / name
    p.write_text(text)
    return str(p)


@pytest.mark.parametrize("edit,code,msg", [
    (("n_sources = 3;", "n_sources = 2;"), 1, "n_sources"),
    (("n_shots = 2;", "n_shots = 3;"), 1, "n_shots"),
    (("nr = 7;", "nr = 6;"), 1, "nr"),
    (("snapshot_interval = 10;", "snapshot_interval = 7;"), 2, "Snapshot interval"),
    (("npx = 2", "npx = 3"), 1, "basis"),
    (("ix_sources = {10, 30, 38}", "ix_sources = {10, 30, 80}"), 1, "outside the grid"),
    (("iz_receivers = {30, 30, 30, 30, 30, 30, 4}", "iz_receivers = {30, 30, 30, 30, 30, 30, 99}"),
     1, "outside the grid"),
    (("{{0, 1}, {2}}", "{{0, 1}, {5}}"), 1, "unknown source"),
])
def test_config_validation(tmp_path, edit, code, msg):
    text = open(SMALL_INI).read()
    assert edit[0] in text
    p = write_ini(tmp_path, text.replace(edit[0], edit[1]))
    info = _capi.PsvInfo()
    assert _capi.load().psv_config_info(p.encode(), ctypes.byref(info)) == code
    assert msg in _capi.load().psv_last_error().decode()
    with pytest.raises(ValueError, match=msg):
        config_info(p)


def test_ini_dialect(tmp_path):
    """inih rules the reference relies on: numeric prefixes before ';',
    inline comments after whitespace, case-insensitive names, nested lists
    with or without the trailing "};"."""
    text = open(SMALL_INI).read()
    text = text.replace("nt = 400;                 int", "NT = 400;int ; comment")
    text = text.replace("{{0, 1}, {2}};", "{{0,1},{2}} ; trailing")
    info = config_info(write_ini(tmp_path, text))
    assert info.nt == 400 and info.n_shots == 2 and info.n_sources == 3


def test_dictionary_roundtrip(tmp_path):
    d = psvwave_gb300.get_dictionary()
    d["domain"]["nx_inner"] = 60
    d["domain"]["nz_inner"] = 40
    d["domain"]["nt"] = 100
    d["sources"]["ix_sources"] = [20, 40]
    d["sources"]["iz_sources"] = [10, 10]
    d["receivers"]["ix_receivers"] = [5, 15, 25, 35]
    d["receivers"]["iz_receivers"] = [30, 30, 30, 30]
    p = str(tmp_path / "d.ini")
    psvwave_gb300.write_dictionary(p, d)
    info = config_info(p)
    assert (info.nx, info.nz, info.nt, info.n_sources, info.nr) == (110, 90, 100, 2, 4)
    o = portbind.OracleModel(p)
    assert o.nx == 110 and o.nz == 90


def test_fdmodel_without_gpu_fails_loudly():
    if _capi.load() and __import__("tests.conftest", fromlist=["gpu_count"]).gpu_count() > 0:
        pytest.skip("a GPU is present")
    with pytest.raises(_capi.PsvError, match="CUDA"):
        psvwave_gb300.fdModel(SMALL_INI)


def test_empty_receiver_list_rejected_like_the_reference(tmp_path):
    """An INI with nr = 0 and empty receiver lists is refused, with the
    reference's message (its parser does the same)."""
    from oracle import refbind
    from tests.test_oracle import _tiny_ini

    p = tmp_path / "no_receivers.ini"
    p.write_text(_tiny_ini(12, 8, 3, [(5, 4, 60.0)], [], [[0]]))
    info = _capi.PsvInfo()
    assert _capi.load().psv_config_info(str(p).encode(), ctypes.byref(info)) == 1
    msg = _capi.load().psv_last_error().decode()
    assert "Mismatch between nr and receivers" in msg
    if refbind.available():
        with pytest.raises(Exception, match="Mismatch between nr and receivers"):
            refbind.RefModel(str(p))
