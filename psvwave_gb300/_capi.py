"""ctypes declarations of the psvwave_gb300 C ABI (include/psvwave.h).

The library is the only compute path: if it cannot be loaded, importing the
package raises. There is no CPU fallback.
"""
import ctypes
import os

from . import build as _build

PSV_OK = 0
PSV_ERR_INVALID_ARGUMENT = 1
PSV_ERR_LENGTH = 2
PSV_ERR_IO = 3
PSV_ERR_CUDA = 4
PSV_ERR_NUMERIC = 5
PSV_ERR_INTERNAL = 6
PSV_FP32 = 0
PSV_FP64 = 1

_c_int = ctypes.c_int
_c_double = ctypes.c_double
_vp = ctypes.c_void_p
_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)


class PsvInfo(ctypes.Structure):
    _fields_ = [(n, _c_int) for n in (
        "nt", "nx", "nz", "nx_inner", "nz_inner", "nx_inner_boundary", "nz_inner_boundary",
        "np_boundary", "n_shots", "n_sources", "nr", "snapshot_interval", "snapshots",
        "nx_free_parameters", "nz_free_parameters", "free_parameters",
        "basis_gridpoints_x", "basis_gridpoints_z", "precision", "device")] + [
        (n, _c_double) for n in (
            "dt", "dx", "dz", "np_factor", "peak_frequency", "alpha", "delay_cycles_per_shot",
            "source_timeshift", "scalar_rho", "scalar_vp", "scalar_vs", "misfit")]


class PsvParams(ctypes.Structure):
    _fields_ = [
        ("nt", _c_int), ("nx_inner", _c_int), ("nz_inner", _c_int),
        ("nx_inner_boundary", _c_int), ("nz_inner_boundary", _c_int),
        ("dx", _c_double), ("dz", _c_double), ("dt", _c_double),
        ("np_boundary", _c_int), ("np_factor", _c_double), ("scalar_rho", _c_double),
        ("scalar_vp", _c_double), ("scalar_vs", _c_double), ("npx", _c_int), ("npz", _c_int),
        ("peak_frequency", _c_double), ("source_timeshift", _c_double),
        ("delay_cycles_per_shot", _c_double), ("n_sources", _c_int), ("n_shots", _c_int),
        ("ix_sources", _ip), ("iz_sources", _ip), ("moment_angles", _dp),
        ("shot_offsets", _ip), ("shot_sources", _ip), ("nr", _c_int),
        ("ix_receivers", _ip), ("iz_receivers", _ip), ("snapshot_interval", _c_int),
        ("observed_data_folder", ctypes.c_char_p), ("stf_folder", ctypes.c_char_p),
    ]


# name -> argument types (all return int status unless listed in _RESTYPES)
_SIGNATURES = {
    "psv_abi_version": [],
    "psv_last_error": [],
    "psv_device_count": [_ip],
    "psv_host_alloc": [ctypes.c_size_t, ctypes.POINTER(ctypes.c_void_p)],
    "psv_host_free": [_vp],
    "psv_config_info": [ctypes.c_char_p, ctypes.POINTER(PsvInfo)],
    "psv_create_from_ini": [ctypes.c_char_p, _c_int, _c_int, ctypes.POINTER(_vp)],
    "psv_create": [ctypes.POINTER(PsvParams), _c_int, _c_int, ctypes.POINTER(_vp)],
    "psv_clone": [_vp, ctypes.POINTER(_vp)],
    "psv_destroy": [_vp],
    "psv_get_info": [_vp, ctypes.POINTER(PsvInfo)],
    "psv_get_shot_sources": [_vp, _ip, _ip],
    "psv_get_folders": [_vp, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_size_t],
    "psv_forward_simulate": [_vp, _c_int, _c_int, _c_int, _c_int],
    "psv_adjoint_simulate": [_vp, _c_int, _c_int],
    "psv_calculate_l2_misfit": [_vp, _dp],
    "psv_calculate_l2_adjoint_sources": [_vp],
    "psv_reset_kernels": [_vp],
    "psv_map_kernels_to_velocity": [_vp],
    "psv_run_model": [_vp, _c_int, _c_int],
    "psv_update_from_velocity": [_vp],
    "psv_get_parameter_fields": [_vp, _dp, _dp, _dp],
    "psv_set_parameter_fields": [_vp, _dp, _dp, _dp],
    "psv_load_model": [_vp, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p, _c_int],
    "psv_get_kernels": [_vp, _dp, _dp, _dp],
    "psv_get_lame_kernels": [_vp, _dp, _dp, _dp],
    "psv_get_synthetic_data": [_vp, _dp, _dp],
    "psv_set_synthetic_data": [_vp, _dp, _dp],
    "psv_get_observed_data": [_vp, _dp, _dp],
    "psv_set_observed_data": [_vp, _dp, _dp],
    "psv_get_adjoint_sources": [_vp, _dp, _dp],
    "psv_get_snapshots": [_vp, _dp, _dp, _dp, _dp, _dp],
    "psv_get_wavefields": [_vp, _dp, _dp, _dp, _dp, _dp],
    "psv_get_stf": [_vp, _dp],
    "psv_get_moment": [_vp, _dp],
    "psv_set_stf": [_vp, _dp],
    "psv_set_moment": [_vp, _dp],
    "psv_get_taper": [_vp, _dp],
    "psv_get_model_vector": [_vp, _dp],
    "psv_set_model_vector": [_vp, _dp],
    "psv_get_gradient_vector": [_vp, _dp],
    "psv_load_vector": [_vp, ctypes.c_char_p, _c_int, _dp],
    "psv_get_sources": [_vp, _c_int, _c_int, _dp, _dp],
    "psv_get_receivers": [_vp, _c_int, _c_int, _dp, _dp],
    "psv_get_coordinates": [_vp, _c_int, _dp, _dp],
    "psv_get_extent": [_vp, _c_int, _dp],
    "psv_write_receivers": [_vp, ctypes.c_char_p],
    "psv_load_receivers": [_vp, _c_int],
    "psv_write_sources": [_vp],
    "psv_write_kernels": [_vp],
    "psv_set_stream": [_vp, _vp],
    "psv_set_async": [_vp, _c_int],
    "psv_set_graph_capture": [_vp, _c_int],
    "psv_synchronize": [_vp],
    "psv_set_parameter_fields_device": [_vp, _vp, _vp, _vp],
    "psv_set_observed_data_device": [_vp, _vp, _vp],
    "psv_get_synthetic_data_device": [_vp, _vp, _vp],
    "psv_get_kernels_device": [_vp, _vp, _vp, _vp],
    "psv_device_bytes": [_vp, ctypes.POINTER(ctypes.c_size_t)],
    "psv_profile_forward": [_vp, _c_int, _c_int, _dp, _dp, _c_int, _ip],
    "psv_step_kernel_name": [_vp, _c_int],
    "psv_set_kernel_variant": [_vp, _c_int],
    "psv_get_kernel_variant": [_vp, _ip],
    "psv_set_tile_shape": [_vp, _c_int],
    "psv_get_tile_shape": [_vp, _ip],
    "psv_autotune": [_vp, _c_int, _ip],
    "psv_exact_gradient": [_vp, _c_int, _dp],
    "psv_exact_gradient_shots": [_vp, _c_int, _ip, _c_int, _dp],
    "psv_get_exact_gradient": [_vp, _dp, _dp, _dp],
    "psv_get_exact_gradient_device": [_vp, _vp, _vp, _vp],
    "psv_exact_bytes": [_vp, _c_int, ctypes.POINTER(ctypes.c_size_t)],
    "psv_batch_create": [_c_int, ctypes.POINTER(_vp)],
    "psv_batch_destroy": [_vp],
    "psv_batch_add": [_vp, _vp, _c_int],
    "psv_batch_forward": [_vp, _c_int, _c_int],
    "psv_batch_set_tile_shape": [_vp, _c_int],
    "psv_batch_autotune": [_vp, _c_int, _ip],
    "psv_batch_info": [_vp, _ip, _ip, _dp],
    "psv_batch_set_active": [_vp, _ip, _c_int],
    "psv_batch_misfits": [_vp, _dp, _c_int],
    "psv_batch_set_parameter_fields_device": [_vp, _vp, ctypes.c_longlong, _ip],
    "psv_batch_set_cluster": [_vp, _c_int],
    "psv_batch_get_cluster": [_vp, _ip],
    "psv_batch_cluster_fits": [_vp, _ip],
    "psv_batch_get_persistent": [_vp, ctypes.POINTER(ctypes.c_int)],
    "psv_batch_set_persistent": [_vp, _c_int],
    "psv_l2_misfit_noalloc": [_vp, _vp, _vp, _vp, ctypes.c_size_t, _c_double, _vp, _vp],
    # include/psvwave_surrogate.h
    "psv_coarse_create": [_c_int, _c_int, _c_int, _c_int, _c_int, _c_int, _dp, _dp,
                          ctypes.POINTER(_vp)],
    "psv_coarse_destroy": [_vp],
    "psv_coarse_to_fields": [_vp, _c_int, _vp, _vp, _vp],
    "psv_coarse_gradient": [_vp, _c_int, _vp, _vp, _c_double, _vp],
    "psv_cnn_create": [_c_int, _c_int, ctypes.POINTER(_vp)],
    "psv_cnn_destroy": [_vp],
    "psv_cnn_num_params": [ctypes.POINTER(ctypes.c_size_t)],
    "psv_cnn_set_params": [_vp, _vp],
    "psv_cnn_get_params": [_vp, _vp],
    "psv_cnn_predict": [_vp, _c_int, _vp, _vp, _vp],
    "psv_cnn_loss_grad": [_vp, _c_int, _vp, _vp, _vp, ctypes.c_float, ctypes.c_float, _dp, _vp],
    "psv_cnn_train_step": [_vp, _c_int, _vp, _vp, _vp, ctypes.c_float, ctypes.c_float,
                           ctypes.c_float, ctypes.c_float, ctypes.c_float, ctypes.c_float, _dp],
}
_RESTYPES = {"psv_last_error": ctypes.c_char_p, "psv_step_kernel_name": ctypes.c_char_p}

_lib = None


def library_path():
    return _build.LIB_PATH


def load():
    """Load (building first if needed) and declare the C-ABI library."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.build()
    if not os.path.exists(path):
        raise RuntimeError("psvwave_gb300: CUDA library %s is missing" % path)
    lib = ctypes.CDLL(path)
    for name, args in _SIGNATURES.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = _RESTYPES.get(name, _c_int)
    if lib.psv_abi_version() != 1:
        raise RuntimeError("psvwave_gb300: unexpected C ABI version")
    _lib = lib
    return lib


class PsvError(RuntimeError):
    """A failure reported by the C library that is not an argument error."""


def check(status):
    if status == PSV_OK:
        return
    msg = load().psv_last_error().decode(errors="replace")
    if status in (PSV_ERR_INVALID_ARGUMENT, PSV_ERR_LENGTH, PSV_ERR_IO):
        raise ValueError(msg)
    raise PsvError(msg)
