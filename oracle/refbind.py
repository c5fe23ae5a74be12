"""ctypes binding of oracle/_ref/libpsv_ref.so: the psvWave reference's own
solver core (src/fdModel.cpp), built unmodified by oracle/build_ref.sh.

Test infrastructure only. It exists only where the reference sources were
present at build time; callers must skip when `available()` is False.
"""
import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_ref", "libpsv_ref.so")
_lib = None

INFO_FIELDS = ("nt", "nx", "nz", "nx_inner", "nz_inner", "nx_inner_boundary",
               "nz_inner_boundary", "np_boundary", "n_shots", "n_sources", "nr",
               "snapshot_interval", "snapshots", "nx_free_parameters",
               "nz_free_parameters", "free_parameters", "npx", "npz")
SCALAR_FIELDS = ("dt", "dx", "dz", "np_factor", "peak_frequency", "alpha",
                 "delay_cycles_per_shot", "misfit")


def available():
    return os.path.exists(_LIB_PATH)


def _load():
    global _lib
    if _lib is None:
        lib = ctypes.CDLL(_LIB_PATH)
        vp = ctypes.c_void_p
        dp = ctypes.POINTER(ctypes.c_double)
        lib.ref_create.restype = vp
        lib.ref_create.argtypes = [ctypes.c_char_p]
        lib.ref_copy.restype = vp
        lib.ref_copy.argtypes = [vp]
        lib.ref_destroy.argtypes = [vp]
        lib.ref_last_error.restype = ctypes.c_char_p
        lib.ref_info.argtypes = [vp, ctypes.POINTER(ctypes.c_int)]
        lib.ref_scalars.argtypes = [vp, dp]
        lib.ref_array.restype = dp
        lib.ref_array.argtypes = [vp, ctypes.c_char_p]
        lib.ref_int_array.restype = ctypes.POINTER(ctypes.c_int)
        lib.ref_int_array.argtypes = [vp, ctypes.c_char_p]
        lib.ref_set_parameter_fields.argtypes = [vp, dp, dp, dp]
        lib.ref_set_data.argtypes = [vp, ctypes.c_int, dp, dp]
        lib.ref_forward.argtypes = [vp, ctypes.c_int, ctypes.c_int]
        lib.ref_forward_output.argtypes = [vp, ctypes.c_int, ctypes.c_int]
        lib.ref_adjoint.argtypes = [vp, ctypes.c_int]
        lib.ref_misfit.restype = ctypes.c_double
        lib.ref_misfit.argtypes = [vp]
        for name in ("ref_adjoint_sources", "ref_reset_kernels", "ref_map_kernels",
                     "ref_write_receivers", "ref_write_sources", "ref_write_kernels"):
            getattr(lib, name).argtypes = [vp]
        lib.ref_load_receivers.argtypes = [vp]
        lib.ref_load_receivers.restype = ctypes.c_int
        lib.ref_run_model.argtypes = [vp, ctypes.c_int]
        lib.ref_get_model_vector.argtypes = [vp, dp]
        lib.ref_set_model_vector.argtypes = [vp, dp]
        lib.ref_get_gradient_vector.argtypes = [vp, dp]
        lib.ref_load_vector.argtypes = [vp, ctypes.c_char_p, dp]
        lib.ref_load_vector.restype = ctypes.c_int
        lib.ref_load_model.argtypes = [vp, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p]
        lib.ref_load_model.restype = ctypes.c_int
        _lib = lib
    return _lib


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


class RefModel:
    """Thin handle on a reference fdModel built from an INI file."""

    def __init__(self, ini_path=None, _handle=None):
        lib = _load()
        if _handle is None:
            _handle = lib.ref_create(str(ini_path).encode())
            if not _handle:
                raise ValueError(lib.ref_last_error().decode())
        self._h = _handle
        info = (ctypes.c_int * len(INFO_FIELDS))()
        lib.ref_info(self._h, info)
        self.info = dict(zip(INFO_FIELDS, list(info)))
        for k, v in self.info.items():
            setattr(self, k, v)

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.ref_destroy(self._h)
            self._h = None

    def copy(self):
        return RefModel(_handle=_load().ref_copy(self._h))

    def scalars(self):
        out = (ctypes.c_double * len(SCALAR_FIELDS))()
        _load().ref_scalars(self._h, out)
        return dict(zip(SCALAR_FIELDS, list(out)))

    @property
    def misfit(self):
        return self.scalars()["misfit"]

    def array(self, name):
        shapes = {
            "grid": (self.nx, self.nz),
            "stf": (self.n_sources, self.nt),
            "moment": (self.n_sources, 2, 2),
            "rec": (self.n_shots, self.nr, self.nt),
            "accu": (self.n_shots, self.snapshots, self.nx, self.nz),
        }
        if name == "stf":
            shape = shapes["stf"]
        elif name == "moment":
            shape = shapes["moment"]
        elif name.startswith("rtf") or name.startswith("a_stf"):
            shape = shapes["rec"]
        elif name.startswith("accu"):
            shape = shapes["accu"]
        else:
            shape = shapes["grid"]
        p = _load().ref_array(self._h, name.encode())
        if not p:
            raise KeyError(name)
        return np.ctypeslib.as_array(p, shape=shape).copy()

    def int_array(self, name):
        n = self.n_sources if "sources" in name else self.nr
        p = _load().ref_int_array(self._h, name.encode())
        return np.ctypeslib.as_array(p, shape=(n,)).copy()

    def set_parameter_fields(self, vp, vs, rho):
        a = [np.ascontiguousarray(x, dtype=np.float64) for x in (vp, vs, rho)]
        _load().ref_set_parameter_fields(self._h, *[_dp(x) for x in a])

    def set_observed_data(self, ux, uz):
        a = [np.ascontiguousarray(x, dtype=np.float64) for x in (ux, uz)]
        _load().ref_set_data(self._h, 1, _dp(a[0]), _dp(a[1]))

    def set_synthetic_data(self, ux, uz):
        a = [np.ascontiguousarray(x, dtype=np.float64) for x in (ux, uz)]
        _load().ref_set_data(self._h, 0, _dp(a[0]), _dp(a[1]))

    def forward_simulate(self, shot, store_fields=True):
        _load().ref_forward(self._h, shot, int(store_fields))

    def adjoint_simulate(self, shot):
        _load().ref_adjoint(self._h, shot)

    def calculate_l2_misfit(self):
        return _load().ref_misfit(self._h)

    def calculate_l2_adjoint_sources(self):
        _load().ref_adjoint_sources(self._h)

    def reset_kernels(self):
        _load().ref_reset_kernels(self._h)

    def map_kernels_to_velocity(self):
        _load().ref_map_kernels(self._h)

    def run_model(self, simulate_adjoint=True):
        _load().ref_run_model(self._h, int(simulate_adjoint))

    def get_model_vector(self):
        out = np.empty(self.free_parameters)
        _load().ref_get_model_vector(self._h, _dp(out))
        return out

    def set_model_vector(self, m):
        m = np.ascontiguousarray(m, dtype=np.float64)
        _load().ref_set_model_vector(self._h, _dp(m))

    def get_gradient_vector(self):
        out = np.empty(self.free_parameters)
        _load().ref_get_gradient_vector(self._h, _dp(out))
        return out

    def get_kernels(self):
        return tuple(self.array(n) for n in ("vp_kernel", "vs_kernel", "density_v_kernel"))

    def get_synthetic_data(self):
        return self.array("rtf_ux"), self.array("rtf_uz")

    def get_observed_data(self):
        return self.array("rtf_ux_true"), self.array("rtf_uz_true")

    def forward_simulate_output(self, shot, store_fields=True):
        """forward_simulate with the reference's wave-field dumps into
        snapshots/ under the working directory."""
        _load().ref_forward_output(self._h, shot, int(store_fields))

    def write_receivers(self):
        _load().ref_write_receivers(self._h)

    def write_sources(self):
        _load().ref_write_sources(self._h)

    def write_kernels(self):
        _load().ref_write_kernels(self._h)

    def load_receivers(self):
        """The reference's load_receivers (observed data from
        observed_data_folder/rtf_u{x,z}{shot}.txt); raises on its errors."""
        if _load().ref_load_receivers(self._h) != 0:
            raise ValueError(_load().ref_last_error().decode())

    def load_vector(self, path):
        """The reference's load_vector: 3 nx_free nz_free values, one per
        free cell and parameter (not per basis block)."""
        out = np.empty(3 * self.info["nx_free_parameters"] * self.info["nz_free_parameters"])
        if _load().ref_load_vector(self._h, str(path).encode(), _dp(out)) != 0:
            raise ValueError(_load().ref_last_error().decode())
        return out
