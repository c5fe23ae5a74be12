"""`fdModel`: the reference's Python class (src/psvWave.cpp:465-655,
psvWave/__init__.py:6), backed by the GB300 C library.

Method names, argument names, defaults, return shapes and error types follow
the reference binding. Arrays are returned as fresh float64 numpy copies, as
the reference's getters do (src/psvWave.cpp:33-63). The extra keyword
`precision` picks the wave-field precision ("fp32" production, "fp64" the
reference's own precision, bit-identical to it); `device` picks the GPU.
"""
import ctypes
import threading
import weakref

import numpy as np

from . import _capi

_DP = ctypes.POINTER(ctypes.c_double)


def _ptr(a):
    return a.ctypes.data_as(_DP)


class _PinnedPool:
    """Page-locked host blocks (psv_host_alloc) behind the large arrays the
    getters return. A device-to-host copy into page-locked memory runs at
    the host link's rate; into a fresh pageable array it goes through the
    driver's staging and first-touch page faults. A block returns to the
    pool when the last array viewing it is freed, so a loop that reads
    seismograms every iteration reuses the same blocks. Arrays below
    MIN_BYTES, and any array once the pool holds MAX_BYTES, are plain numpy
    arrays."""

    MIN_BYTES = 1 << 20
    MAX_BYTES = 4 << 30

    def __init__(self):
        self._free = {}
        self._held = 0
        self._lock = threading.Lock()
        self._off = False  # set when the first allocation fails (no device)

    def array(self, shape):
        n = int(np.prod(shape)) * 8
        if n < self.MIN_BYTES or self._off:
            return np.empty(shape, dtype=np.float64)
        ptr = None
        with self._lock:
            blocks = self._free.get(n)
            if blocks:
                ptr = blocks.pop()
            elif self._held + n <= self.MAX_BYTES:
                p = ctypes.c_void_p()
                if _capi.load().psv_host_alloc(n, ctypes.byref(p)) == _capi.PSV_OK and p.value:
                    ptr = p.value
                    self._held += n
                else:
                    self._off = True
        if ptr is None:
            return np.empty(shape, dtype=np.float64)
        buf = (ctypes.c_double * (n // 8)).from_address(ptr)
        weakref.finalize(buf, self._release, n, ptr)
        return np.frombuffer(buf, dtype=np.float64).reshape(shape)

    def _release(self, n, ptr):
        with self._lock:
            self._free.setdefault(n, []).append(ptr)


_PINNED = _PinnedPool()


def _out(shape):
    """A fresh float64 array for a getter to fill (page-locked when large)."""
    return _PINNED.array(shape)


def _in(a, shape, name):
    a = np.asarray(a)
    if a.shape != tuple(shape):
        raise ValueError("The input ndarray %s does not have the right shape." % name)
    return np.ascontiguousarray(a, dtype=np.float64)


class fdModel:
    """fdModel(configuration_file_path: str)

    Class to simulate P-SV wave physics and its adjoint state on a GB300 GPU.

    :param configuration_file_path: Path to the desired configuration.
    :param precision: "fp32" (default) or "fp64".
    :param device: CUDA device index.
    """

    units = [r"$m/s$", r"$m/s$", r"$kg/m^3$"]
    parameters = [r"$v_p$", r"$v_s$", r"$\rho$"]

    def __init__(self, configuration_file_path=None, precision="fp32", device=0, _handle=None):
        self._lib = _capi.load()
        self._h = None
        if _handle is None:
            prec = self._precision_code(precision)
            h = ctypes.c_void_p()
            _capi.check(self._lib.psv_create_from_ini(
                str(configuration_file_path).encode(), prec, int(device), ctypes.byref(h)))
            _handle = h
        self._h = _handle
        self._refresh_info()

    @staticmethod
    def _precision_code(precision):
        p = str(precision).lower()
        if p in ("fp32", "float32", "single", "float"):
            return _capi.PSV_FP32
        if p in ("fp64", "float64", "double"):
            return _capi.PSV_FP64
        raise ValueError("precision must be 'fp32' or 'fp64'")

    @classmethod
    def from_parameters(cls, params, precision="fp32", device=0):
        """Build from explicit parameters (the reference's second constructor,
        src/fdModel.cpp:29-62). `params` is a dict with the keys of that
        constructor; `which_source_to_fire_in_which_shot` is a list of lists."""
        lib = _capi.load()
        shots = params["which_source_to_fire_in_which_shot"]
        keep = {
            "shot_offsets": np.concatenate([[0], np.cumsum([len(s) for s in shots])]).astype(np.int32),
            "shot_sources": np.array([i for s in shots for i in s] or [0], dtype=np.int32),
        }
        for k in ("ix_sources", "iz_sources", "ix_receivers", "iz_receivers"):
            keep[k] = np.ascontiguousarray(np.asarray(params[k], dtype=np.int32).reshape(-1))
        keep["moment_angles"] = np.ascontiguousarray(
            np.asarray(params["moment_angles"], dtype=np.float64).reshape(-1))
        p = _capi.PsvParams()
        for name, ctype in _capi.PsvParams._fields_:
            if name in keep:
                arr = keep[name]
                ptype = _DP if arr.dtype == np.float64 else ctypes.POINTER(ctypes.c_int)
                setattr(p, name, arr.ctypes.data_as(ptype))
            elif name == "n_shots":
                p.n_shots = len(shots)
            elif name in ("observed_data_folder", "stf_folder"):
                setattr(p, name, str(params.get(name, ".")).encode())
            elif name in ("npx", "npz"):
                setattr(p, name, int(params.get(name, 1)))
            elif name == "source_timeshift":
                p.source_timeshift = float(params.get(name, 0.0))
            else:
                setattr(p, name, ctype(params[name]).value)
        h = ctypes.c_void_p()
        _capi.check(lib.psv_create(ctypes.byref(p), cls._precision_code(precision), int(device),
                                   ctypes.byref(h)))
        return cls(_handle=h)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            try:
                self._lib.psv_destroy(h)
            except Exception:
                pass
            self._h = None

    def _refresh_info(self):
        info = _capi.PsvInfo()
        _capi.check(self._lib.psv_get_info(self._h, ctypes.byref(info)))
        self._info = info

    # ---- read-only attributes (src/psvWave.cpp:499-588) ------------------
    def _i(name):
        return property(lambda self: getattr(self._info, name))

    dt = _i("dt")
    dx = _i("dx")
    dz = _i("dz")
    nt = _i("nt")
    nx = _i("nx")
    nz = _i("nz")
    nx_inner = _i("nx_inner")
    nz_inner = _i("nz_inner")
    nx_inner_boundary = _i("nx_inner_boundary")
    nz_inner_boundary = _i("nz_inner_boundary")
    np_boundary = _i("np_boundary")
    nx_free_parameters = _i("nx_free_parameters")
    nz_free_parameters = _i("nz_free_parameters")
    free_parameters = _i("free_parameters")
    # basis block size (points per model-vector cell in x and z)
    npx = _i("basis_gridpoints_x")
    npz = _i("basis_gridpoints_z")
    snapshot_interval = _i("snapshot_interval")
    snapshots = _i("snapshots")
    n_shots = _i("n_shots")
    n_sources = _i("n_sources")
    nr = _i("nr")
    np_factor = _i("np_factor")
    peak_frequency = _i("peak_frequency")
    basis_gridpoints_x = _i("basis_gridpoints_x")
    basis_gridpoints_z = _i("basis_gridpoints_z")
    del _i

    @property
    def precision(self):
        return "fp64" if self._info.precision == _capi.PSV_FP64 else "fp32"

    @property
    def device(self):
        return self._info.device

    @property
    def misfit(self):
        """Current misfit; updated by calculate_l2_misfit()."""
        self._refresh_info()
        return self._info.misfit

    @property
    def which_source_to_fire_in_which_shot(self):
        offs = np.zeros(self.n_shots + 1, dtype=np.int32)
        src = np.zeros(max(self.n_sources, 1), dtype=np.int32)
        _capi.check(self._lib.psv_get_shot_sources(
            self._h, offs.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
            src.ctypes.data_as(ctypes.POINTER(ctypes.c_int))))
        return [list(map(int, src[offs[s]:offs[s + 1]])) for s in range(self.n_shots)]

    @property
    def observed_data_folder(self):
        return self._folders()[0]

    @property
    def stf_folder(self):
        return self._folders()[1]

    def _folders(self):
        a, b = ctypes.create_string_buffer(4096), ctypes.create_string_buffer(4096)
        _capi.check(self._lib.psv_get_folders(self._h, a, b, 4096))
        return a.value.decode(), b.value.decode()

    @property
    def handle(self):
        """Opaque psv_model* for the C ABI."""
        return self._h

    # ---- construction ---------------------------------------------------
    def copy(self):
        """copy() -> fdModel: a deep copy of every member (src/psvWave.cpp:421-425)."""
        h = ctypes.c_void_p()
        _capi.check(self._lib.psv_clone(self._h, ctypes.byref(h)))
        return type(self)(_handle=h)

    # ---- simulation -----------------------------------------------------
    def forward_simulate(self, i_shot, store_fields=True, verbose=False, output_wavefields=False,
                         omp_threads_override=0):
        """Run forward simulations for a given 'shot' (src/psvWave.cpp:476-498).

        `omp_threads_override` is accepted for compatibility; the GPU ignores it.
        """
        _capi.check(self._lib.psv_forward_simulate(self._h, int(i_shot), int(bool(store_fields)),
                                                   int(bool(verbose)),
                                                   int(bool(output_wavefields))))

    def adjoint_simulate(self, i_shot, verbose=False, omp_threads_override=0):
        """Adjoint simulate the wavefield for a given shot, accumulating the
        kernels (src/psvWave.cpp:634-650)."""
        _capi.check(self._lib.psv_adjoint_simulate(self._h, int(i_shot), int(bool(verbose))))

    def calculate_l2_misfit(self):
        """Calculate L2 misfit for simulated waveforms w.r.t. observed data."""
        out = ctypes.c_double()
        _capi.check(self._lib.psv_calculate_l2_misfit(self._h, ctypes.byref(out)))
        self._info.misfit = out.value

    def calculate_l2_adjoint_sources(self):
        _capi.check(self._lib.psv_calculate_l2_adjoint_sources(self._h))

    def reset_kernels(self):
        _capi.check(self._lib.psv_reset_kernels(self._h))

    def map_kernels_to_velocity(self):
        _capi.check(self._lib.psv_map_kernels_to_velocity(self._h))

    def run_model(self, verbose=False, simulate_adjoint=True):
        """All shots forward, misfit and, if simulate_adjoint, the full
        adjoint and kernel mapping (src/fdModel.cpp:1291-1308)."""
        _capi.check(self._lib.psv_run_model(self._h, int(bool(verbose)),
                                            int(bool(simulate_adjoint))))

    def compute_gradients(self, verbose=False):
        """One FWI gradient: run_model with the adjoint; returns (misfit, g)."""
        self.run_model(verbose=verbose, simulate_adjoint=True)
        return self.misfit, self.get_gradient_vector()

    def exact_gradient(self, checkpoint_every=100, on_device=False, shots=None):
        """Misfit and its gradient with respect to (vp, vs, rho) over all
        shots (or the listed `shots`) by the exact discrete adjoint (the
        transpose of the time stepping), with forward states rebuilt from
        checkpoints every `checkpoint_every` steps. Returns (misfit,
        (g_vp, g_vs, g_rho)), numpy arrays, or CUDA tensors with
        on_device=True."""
        mis = ctypes.c_double()
        if shots is None:
            _capi.check(self._lib.psv_exact_gradient(self._h, int(checkpoint_every),
                                                     ctypes.byref(mis)))
        else:
            s = np.ascontiguousarray(np.asarray(shots, dtype=np.int32).reshape(-1))
            _capi.check(self._lib.psv_exact_gradient_shots(
                self._h, int(checkpoint_every), s.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                int(s.size), ctypes.byref(mis)))
        if on_device:
            self._info.misfit = mis.value
            return mis.value, self.get_exact_gradient_device()
        g = [_out((self.nx, self.nz)) for _ in range(3)]
        _capi.check(self._lib.psv_get_exact_gradient(self._h, *[_ptr(a) for a in g]))
        self._info.misfit = mis.value
        return mis.value, tuple(g)

    def exact_bytes(self, checkpoint_every=100):
        n = ctypes.c_size_t()
        _capi.check(self._lib.psv_exact_bytes(self._h, int(checkpoint_every), ctypes.byref(n)))
        return n.value

    def update_from_velocity(self):
        _capi.check(self._lib.psv_update_from_velocity(self._h))

    # ---- medium ---------------------------------------------------------
    def get_parameter_fields(self):
        vp, vs, rho = _out((self.nx, self.nz)), _out((self.nx, self.nz)), _out((self.nx, self.nz))
        _capi.check(self._lib.psv_get_parameter_fields(self._h, _ptr(vp), _ptr(vs), _ptr(rho)))
        return vp, vs, rho

    def set_parameter_fields(self, _vp, _vs, _rho):
        shape = (self.nx, self.nz)
        vp, vs, rho = _in(_vp, shape, "_vp"), _in(_vs, shape, "_vs"), _in(_rho, shape, "_rho")
        _capi.check(self._lib.psv_set_parameter_fields(self._h, _ptr(vp), _ptr(vs), _ptr(rho)))

    def load_model(self, de_path, vp_path, vs_path, verbose=False):
        """Load density, P- and S-velocity from text files (src/fdModel.cpp:1185-1289)."""
        _capi.check(self._lib.psv_load_model(self._h, str(de_path).encode(), str(vp_path).encode(),
                                             str(vs_path).encode(), int(bool(verbose))))

    # ---- kernels and data -----------------------------------------------
    def get_kernels(self):
        k = [_out((self.nx, self.nz)) for _ in range(3)]
        _capi.check(self._lib.psv_get_kernels(self._h, *[_ptr(a) for a in k]))
        return tuple(k)

    def get_lame_kernels(self):
        k = [_out((self.nx, self.nz)) for _ in range(3)]
        _capi.check(self._lib.psv_get_lame_kernels(self._h, *[_ptr(a) for a in k]))
        return tuple(k)

    def _data_shape(self):
        return (self.n_shots, self.nr, self.nt)

    def get_synthetic_data(self):
        ux, uz = _out(self._data_shape()), _out(self._data_shape())
        _capi.check(self._lib.psv_get_synthetic_data(self._h, _ptr(ux), _ptr(uz)))
        return ux, uz

    def set_synthetic_data(self, ux, uz):
        a, b = _in(ux, self._data_shape(), "ux"), _in(uz, self._data_shape(), "uz")
        _capi.check(self._lib.psv_set_synthetic_data(self._h, _ptr(a), _ptr(b)))

    def get_observed_data(self):
        ux, uz = _out(self._data_shape()), _out(self._data_shape())
        _capi.check(self._lib.psv_get_observed_data(self._h, _ptr(ux), _ptr(uz)))
        return ux, uz

    def set_observed_data(self, ux, uz):
        a, b = _in(ux, self._data_shape(), "ux"), _in(uz, self._data_shape(), "ux")
        _capi.check(self._lib.psv_set_observed_data(self._h, _ptr(a), _ptr(b)))

    def get_adjoint_sources(self):
        ux, uz = _out(self._data_shape()), _out(self._data_shape())
        _capi.check(self._lib.psv_get_adjoint_sources(self._h, _ptr(ux), _ptr(uz)))
        return ux, uz

    def get_snapshots(self):
        """The stored forward fields (vx, vz, txx, tzz, txz), each
        [n_shots, snapshots, nx, nz] (src/psvWave.cpp:90-97)."""
        shape = (self.n_shots, self.snapshots, self.nx, self.nz)
        out = [_out(shape) for _ in range(5)]
        _capi.check(self._lib.psv_get_snapshots(self._h, *[_ptr(a) for a in out]))
        return tuple(out)

    def get_wavefields(self):
        out = [_out((self.nx, self.nz)) for _ in range(5)]
        _capi.check(self._lib.psv_get_wavefields(self._h, *[_ptr(a) for a in out]))
        return tuple(out)

    def get_stf(self):
        out = _out((self.n_sources, self.nt))
        _capi.check(self._lib.psv_get_stf(self._h, _ptr(out)))
        return out

    def get_moment(self):
        out = _out((self.n_sources, 2, 2))
        _capi.check(self._lib.psv_get_moment(self._h, _ptr(out)))
        return out

    def set_stf(self, stf):
        """Custom source time functions [n_sources][nt] in place of the
        Ricker wavelets, for every later simulation (no reference
        counterpart: source generalisation)."""
        a = np.ascontiguousarray(np.asarray(stf, dtype=np.float64))
        if a.shape != (self.n_sources, self.nt):
            raise ValueError("stf must have shape (n_sources, nt)")
        _capi.check(self._lib.psv_set_stf(self._h, _ptr(a)))

    def set_moment(self, moment):
        """Full 2 x 2 moment tensors [n_sources][2][2] (M01 drives the (x,z)
        couple, M10 the (z,x) couple) in place of the dip-angle tensors, for
        every later simulation (no reference counterpart: source
        generalisation)."""
        a = np.ascontiguousarray(np.asarray(moment, dtype=np.float64))
        if a.shape != (self.n_sources, 2, 2):
            raise ValueError("moment must have shape (n_sources, 2, 2)")
        _capi.check(self._lib.psv_set_moment(self._h, _ptr(a)))

    def get_taper(self):
        out = _out((self.nx, self.nz))
        _capi.check(self._lib.psv_get_taper(self._h, _ptr(out)))
        return out

    # ---- model / gradient vectors ---------------------------------------
    def get_model_vector(self):
        out = _out((self.free_parameters,))
        _capi.check(self._lib.psv_get_model_vector(self._h, _ptr(out)))
        return out

    def set_model_vector(self, m):
        m = np.ascontiguousarray(np.asarray(m, dtype=np.float64).reshape(-1))
        if m.size != self.free_parameters:
            raise ValueError("model vector must have free_parameters entries")
        _capi.check(self._lib.psv_set_model_vector(self._h, _ptr(m)))

    def get_gradient_vector(self):
        out = _out((self.free_parameters,))
        _capi.check(self._lib.psv_get_gradient_vector(self._h, _ptr(out)))
        return out

    def load_vector(self, relative_path, verbose=False):
        out = _out((3 * self.nx_free_parameters * self.nz_free_parameters,))
        _capi.check(self._lib.psv_load_vector(self._h, str(relative_path).encode(),
                                              int(bool(verbose)), _ptr(out)))
        return out

    # ---- geometry -------------------------------------------------------
    def get_sources(self, in_units=True, include_absorbing_boundary_as_index=True):
        x, z = _out((self.n_sources,)), _out((self.n_sources,))
        _capi.check(self._lib.psv_get_sources(self._h, int(bool(in_units)),
                                              int(bool(include_absorbing_boundary_as_index)),
                                              _ptr(x), _ptr(z)))
        return x, z

    def get_receivers(self, in_units=True, include_absorbing_boundary_as_index=True):
        x, z = _out((self.nr,)), _out((self.nr,))
        _capi.check(self._lib.psv_get_receivers(self._h, int(bool(in_units)),
                                                int(bool(include_absorbing_boundary_as_index)),
                                                _ptr(x), _ptr(z)))
        return x, z

    def get_coordinates(self, in_units=True):
        ix, iz = _out((self.nx, self.nz)), _out((self.nx, self.nz))
        _capi.check(self._lib.psv_get_coordinates(self._h, int(bool(in_units)), _ptr(ix), _ptr(iz)))
        return ix, iz

    def get_extent(self, include_absorbing_boundary=True):
        out = _out((4,))
        _capi.check(self._lib.psv_get_extent(self._h, int(bool(include_absorbing_boundary)),
                                             _ptr(out)))
        # The reference returns the integer entries as Python ints
        # (src/psvWave.cpp:99-110).
        return (int(out[0]), float(out[1]), int(out[2]), float(out[3]))

    # ---- text I/O -------------------------------------------------------
    def write_receivers(self, prefix=""):
        _capi.check(self._lib.psv_write_receivers(self._h, str(prefix).encode()))

    def load_receivers(self, verbose=False):
        _capi.check(self._lib.psv_load_receivers(self._h, int(bool(verbose))))

    def write_sources(self):
        _capi.check(self._lib.psv_write_sources(self._h))

    def write_kernels(self):
        _capi.check(self._lib.psv_write_kernels(self._h))

    # ---- device-side interface ------------------------------------------
    def set_stream(self, stream_handle):
        """Order this model's GPU work on a CUDA stream handle (int), e.g.
        torch.cuda.current_stream().cuda_stream; 0 restores its own stream."""
        _capi.check(self._lib.psv_set_stream(self._h, ctypes.c_void_p(int(stream_handle))))

    def set_async(self, async_calls=True):
        _capi.check(self._lib.psv_set_async(self._h, int(bool(async_calls))))

    def set_graph_capture(self, enable=True):
        """Replay repeated time loops as CUDA graphs (default on)."""
        _capi.check(self._lib.psv_set_graph_capture(self._h, int(bool(enable))))

    def synchronize(self):
        _capi.check(self._lib.psv_synchronize(self._h))

    def device_bytes(self):
        n = ctypes.c_size_t()
        _capi.check(self._lib.psv_device_bytes(self._h, ctypes.byref(n)))
        return n.value

    # Device buffers (torch CUDA tensors, float64, contiguous). Inputs are read
    # on this model's stream after the caller's current stream has finished
    # with them; outputs are complete when the call returns.
    def _device_tensor(self, t, shape, name, sync=True):
        import torch

        if tuple(t.shape) != tuple(shape):
            raise ValueError("The input tensor %s does not have the right shape." % name)
        if not t.is_cuda or t.device.index != self.device:
            raise ValueError("tensor %s must live on cuda:%d" % (name, self.device))
        t = t.detach().to(torch.float64).contiguous()
        if sync:
            torch.cuda.current_stream(t.device).synchronize()
        return t

    def _device_out(self, shape):
        import torch

        return torch.empty(shape, dtype=torch.float64, device="cuda:%d" % self.device)

    def set_parameter_fields_device(self, vp, vs, rho, sync=True):
        """set_parameter_fields from CUDA tensors [nx, nz]. sync=False skips
        the wait for torch's current stream: the caller has already waited
        for the tensors (float64, contiguous) and keeps them alive until the
        model's stream has copied them (with set_async(True) the copies and
        the medium update are only queued on the model's stream)."""
        shape = (self.nx, self.nz)
        t = [self._device_tensor(a, shape, n, sync)
             for a, n in zip((vp, vs, rho), ("_vp", "_vs", "_rho"))]
        _capi.check(self._lib.psv_set_parameter_fields_device(
            self._h, *[ctypes.cast(x.data_ptr(), _DP) for x in t]))

    def set_observed_data_device(self, ux, uz):
        t = [self._device_tensor(a, self._data_shape(), n) for a, n in ((ux, "ux"), (uz, "uz"))]
        _capi.check(self._lib.psv_set_observed_data_device(
            self._h, *[ctypes.cast(x.data_ptr(), _DP) for x in t]))

    def get_synthetic_data_device(self):
        out = [self._device_out(self._data_shape()) for _ in range(2)]
        _capi.check(self._lib.psv_get_synthetic_data_device(
            self._h, *[ctypes.cast(x.data_ptr(), _DP) for x in out]))
        return tuple(out)

    def get_kernels_device(self):
        out = [self._device_out((self.nx, self.nz)) for _ in range(3)]
        _capi.check(self._lib.psv_get_kernels_device(
            self._h, *[ctypes.cast(x.data_ptr(), _DP) for x in out]))
        return tuple(out)

    def get_exact_gradient_device(self):
        """The last exact_gradient as CUDA tensors (g_vp, g_vs, g_rho)."""
        out = [self._device_out((self.nx, self.nz)) for _ in range(3)]
        _capi.check(self._lib.psv_get_exact_gradient_device(
            self._h, *[ctypes.cast(x.data_ptr(), _DP) for x in out]))
        return tuple(out)

    def profile_forward(self, i_shot=0, n_steps=100):
        """Average device time (ms) per forward time step and per launch of
        each step kernel, from CUDA events on this model's stream."""
        per_step = ctypes.c_double()
        ks = (ctypes.c_double * 8)()
        n = ctypes.c_int()
        _capi.check(self._lib.psv_profile_forward(self._h, int(i_shot), int(n_steps),
                                                  ctypes.byref(per_step), ks, 8, ctypes.byref(n)))
        names = [self._lib.psv_step_kernel_name(self._h, k).decode() for k in range(n.value)]
        return per_step.value, dict(zip(names, list(ks)[:n.value]))

    VARIANTS = {"fused": 0, "two_kernel": 1, "fused_tma": 2, "fused_tma_persistent": 3,
                "fused_cluster": 4}

    @property
    def kernel_variant(self):
        """'fused_tma' (one launch per step with TMA tile loads),
        'fused_tma_persistent' (the same step, all time steps in one
        persistent launch; the default on large grids), 'fused_cluster'
        (all time steps in one launch of one thread-block cluster holding
        the grid in shared memory; the default on small grids), 'fused' (one
        launch per step, FP32) or 'two_kernel' (stress and velocity
        launches; the FP64 variant)."""
        v = ctypes.c_int()
        _capi.check(self._lib.psv_get_kernel_variant(self._h, ctypes.byref(v)))
        return {k: n for n, k in self.VARIANTS.items()}[v.value]

    @kernel_variant.setter
    def kernel_variant(self, name):
        _capi.check(self._lib.psv_set_kernel_variant(self._h, self.VARIANTS[name]))

    TILE_SHAPES = {"32x60": 0, "16x28": 1, "20x28": 2, "16x60": 3}

    @property
    def tile_shape(self):
        """Tile shape (x rows by z columns) of the FP32 TMA step."""
        v = ctypes.c_int()
        _capi.check(self._lib.psv_get_tile_shape(self._h, ctypes.byref(v)))
        return {k: n for n, k in self.TILE_SHAPES.items()}[v.value]

    @tile_shape.setter
    def tile_shape(self, name):
        _capi.check(self._lib.psv_set_tile_shape(self._h, self.TILE_SHAPES[name]))

    def autotune(self, n_steps=50):
        """Time every tile shape with both TMA launch schemes (one launch per
        step, one persistent launch) on n_steps forward steps; keep the
        fastest pair and return its tile shape."""
        v = ctypes.c_int()
        _capi.check(self._lib.psv_autotune(self._h, int(n_steps), ctypes.byref(v)))
        return {k: n for n, k in self.TILE_SHAPES.items()}[v.value]
