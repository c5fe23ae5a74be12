"""ctypes binding of the oracle port (oracle/psv_oracle.c, built into
oracle/_build/libpsv_oracle.so by oracle/build.py).

Test infrastructure only: used by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py as the checker; never by the product.
"""
import ctypes
import os

import numpy as np

from . import build as _build

INFO_FIELDS = ("nt", "nx", "nz", "nx_inner", "nz_inner", "nx_inner_boundary",
               "nz_inner_boundary", "np_boundary", "n_shots", "n_sources", "nr",
               "snapshot_interval", "snapshots", "nx_free_parameters",
               "nz_free_parameters", "free_parameters", "npx", "npz")
SCALAR_FIELDS = ("dt", "dx", "dz", "np_factor", "peak_frequency", "alpha",
                 "delay_cycles_per_shot", "misfit")

_lib = None


class _Params(ctypes.Structure):
    _fields_ = [
        ("nt", ctypes.c_int), ("nx_inner", ctypes.c_int), ("nz_inner", ctypes.c_int),
        ("nx_inner_boundary", ctypes.c_int), ("nz_inner_boundary", ctypes.c_int),
        ("dx", ctypes.c_double), ("dz", ctypes.c_double), ("dt", ctypes.c_double),
        ("np_boundary", ctypes.c_int), ("np_factor", ctypes.c_double),
        ("scalar_rho", ctypes.c_double), ("scalar_vp", ctypes.c_double),
        ("scalar_vs", ctypes.c_double), ("npx", ctypes.c_int), ("npz", ctypes.c_int),
        ("peak_frequency", ctypes.c_double), ("source_timeshift", ctypes.c_double),
        ("delay_cycles_per_shot", ctypes.c_double), ("n_sources", ctypes.c_int),
        ("n_shots", ctypes.c_int), ("ix_sources", ctypes.POINTER(ctypes.c_int)),
        ("iz_sources", ctypes.POINTER(ctypes.c_int)),
        ("moment_angles", ctypes.POINTER(ctypes.c_double)),
        ("shot_offsets", ctypes.POINTER(ctypes.c_int)),
        ("shot_sources", ctypes.POINTER(ctypes.c_int)), ("nr", ctypes.c_int),
        ("ix_receivers", ctypes.POINTER(ctypes.c_int)),
        ("iz_receivers", ctypes.POINTER(ctypes.c_int)),
        ("snapshot_interval", ctypes.c_int),
    ]


def lib_path():
    return _build.PORT_LIB


def _load():
    global _lib
    if _lib is None:
        path = _build.build_port()
        lib = ctypes.CDLL(path)
        vp = ctypes.c_void_p
        dp = ctypes.POINTER(ctypes.c_double)
        lib.po_create.restype = vp
        lib.po_create.argtypes = [ctypes.POINTER(_Params), ctypes.c_char_p, ctypes.c_int]
        lib.po_create_from_ini.restype = vp
        lib.po_create_from_ini.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int]
        lib.po_copy.restype = vp
        lib.po_copy.argtypes = [vp]
        lib.po_destroy.argtypes = [vp]
        lib.po_info.argtypes = [vp, ctypes.POINTER(ctypes.c_int)]
        lib.po_scalars.argtypes = [vp, dp]
        lib.po_array.restype = dp
        lib.po_array.argtypes = [vp, ctypes.c_char_p]
        lib.po_int_array.restype = ctypes.POINTER(ctypes.c_int)
        lib.po_int_array.argtypes = [vp, ctypes.c_char_p]
        for name in ("po_update_from_velocity", "po_adjoint_sources", "po_reset_kernels",
                     "po_map_kernels"):
            getattr(lib, name).argtypes = [vp]
        lib.po_forward.argtypes = [vp, ctypes.c_int, ctypes.c_int]
        lib.po_forward_steps.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        lib.po_adjoint.argtypes = [vp, ctypes.c_int]
        lib.po_misfit.restype = ctypes.c_double
        lib.po_misfit.argtypes = [vp]
        lib.po_run_model.argtypes = [vp, ctypes.c_int]
        lib.po_get_model_vector.argtypes = [vp, dp]
        lib.po_set_model_vector.argtypes = [vp, dp]
        lib.po_get_gradient_vector.argtypes = [vp, dp]
        _lib = lib
    return _lib


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _ip(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))


class OracleModel:
    """CPU oracle model with the reference fdModel's method names."""

    def __init__(self, ini_path=None, params=None, _handle=None):
        lib = _load()
        err = ctypes.create_string_buffer(512)
        if _handle is None:
            if params is not None:
                _handle = self._create_from_params(lib, params, err)
            else:
                _handle = lib.po_create_from_ini(str(ini_path).encode(), err, 512)
            if not _handle:
                raise ValueError(err.value.decode())
        self._h = _handle
        info = (ctypes.c_int * len(INFO_FIELDS))()
        lib.po_info(self._h, info)
        self.info = dict(zip(INFO_FIELDS, list(info)))
        for k, v in self.info.items():
            setattr(self, k, v)

    @staticmethod
    def _create_from_params(lib, d, err):
        keep = {}
        shots = d["which_source_to_fire_in_which_shot"]
        offs = np.zeros(len(shots) + 1, np.int32)
        offs[1:] = np.cumsum([len(s) for s in shots])
        keep["shot_offsets"] = offs
        keep["shot_sources"] = np.array([i for s in shots for i in s] or [0], np.int32)
        for k in ("ix_sources", "iz_sources", "ix_receivers", "iz_receivers"):
            keep[k] = np.ascontiguousarray(np.asarray(d[k], np.int32).reshape(-1))
        keep["moment_angles"] = np.ascontiguousarray(np.asarray(d["moment_angles"], np.float64))
        p = _Params()
        for name, ctype in _Params._fields_:
            if name in keep:
                arr = keep[name]
                setattr(p, name, _dp(arr) if arr.dtype == np.float64 else _ip(arr))
            elif name == "n_shots":
                p.n_shots = len(shots)
            else:
                setattr(p, name, ctype(d[name]).value)
        h = lib.po_create(ctypes.byref(p), err, 512)
        return h

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.po_destroy(self._h)
            self._h = None

    def copy(self):
        return OracleModel(_handle=_load().po_copy(self._h))

    def scalars(self):
        out = (ctypes.c_double * len(SCALAR_FIELDS))()
        _load().po_scalars(self._h, out)
        return dict(zip(SCALAR_FIELDS, list(out)))

    @property
    def misfit(self):
        return self.scalars()["misfit"]

    def _shape(self, name):
        if name == "stf":
            return (self.n_sources, self.nt)
        if name == "moment":
            return (self.n_sources, 2, 2)
        if name.startswith("rtf") or name.startswith("a_stf"):
            return (self.n_shots, self.nr, self.nt)
        if name.startswith("accu"):
            return (self.n_shots, self.snapshots, self.nx, self.nz)
        return (self.nx, self.nz)

    def view(self, name):
        """Writable numpy view of one of the oracle's arrays."""
        p = _load().po_array(self._h, name.encode())
        if not p:
            raise KeyError(name)
        return np.ctypeslib.as_array(p, shape=self._shape(name))

    def array(self, name):
        return self.view(name).copy()

    def int_array(self, name):
        n = self.n_sources if "sources" in name else self.nr
        p = _load().po_int_array(self._h, name.encode())
        return np.ctypeslib.as_array(p, shape=(n,)).copy()

    def set_parameter_fields(self, vp, vs, rho):
        self.view("vp")[...] = vp
        self.view("vs")[...] = vs
        self.view("rho")[...] = rho
        _load().po_update_from_velocity(self._h)

    def get_parameter_fields(self):
        return self.array("vp"), self.array("vs"), self.array("rho")

    def set_observed_data(self, ux, uz):
        self.view("rtf_ux_true")[...] = ux
        self.view("rtf_uz_true")[...] = uz

    def set_synthetic_data(self, ux, uz):
        self.view("rtf_ux")[...] = ux
        self.view("rtf_uz")[...] = uz

    def get_synthetic_data(self):
        return self.array("rtf_ux"), self.array("rtf_uz")

    def get_observed_data(self):
        return self.array("rtf_ux_true"), self.array("rtf_uz_true")

    def forward_simulate(self, shot, store_fields=True, n_steps=None):
        if n_steps is None:
            _load().po_forward(self._h, shot, int(store_fields))
        else:
            _load().po_forward_steps(self._h, shot, int(store_fields), int(n_steps))

    def adjoint_simulate(self, shot):
        _load().po_adjoint(self._h, shot)

    def calculate_l2_misfit(self):
        return _load().po_misfit(self._h)

    def calculate_l2_adjoint_sources(self):
        _load().po_adjoint_sources(self._h)

    def reset_kernels(self):
        _load().po_reset_kernels(self._h)

    def map_kernels_to_velocity(self):
        _load().po_map_kernels(self._h)

    def run_model(self, simulate_adjoint=True):
        _load().po_run_model(self._h, int(simulate_adjoint))

    def get_model_vector(self):
        out = np.empty(self.free_parameters)
        _load().po_get_model_vector(self._h, _dp(out))
        return out

    def set_model_vector(self, m):
        m = np.ascontiguousarray(m, dtype=np.float64)
        _load().po_set_model_vector(self._h, _dp(m))

    def get_gradient_vector(self):
        out = np.empty(self.free_parameters)
        _load().po_get_gradient_vector(self._h, _dp(out))
        return out

    def get_kernels(self):
        return tuple(self.array(n) for n in ("vp_kernel", "vs_kernel", "density_v_kernel"))

    def get_lame_kernels(self):
        return tuple(self.array(n) for n in ("lambda_kernel", "mu_kernel", "density_l_kernel"))
