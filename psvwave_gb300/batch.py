"""Batched forward simulation: shots of many fdModels, of uneven grid sizes,
advanced together (C ABI psv_batch_*): one TMA-step launch per time step
with the whole time loop replayed as one CUDA graph (the default), every
step in one persistent launch, or every member in its own cluster-resident
launch; the autotuner picks. Media updates and misfits of many members go
through one call each."""
import ctypes

from . import _capi


class Batch:
    """Batch(device=0); add(model, i_shot) members, then forward().

    Members are FP32 fdModels sharing nt. Seismograms (and, with
    store_fields, snapshots) land in each model as forward_simulate would
    leave them. The models must stay alive while the batch exists.
    """

    def __init__(self, device=0):
        self._lib = _capi.load()
        h = ctypes.c_void_p()
        _capi.check(self._lib.psv_batch_create(int(device), ctypes.byref(h)))
        self._h = h
        self._models = []

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            try:
                self._lib.psv_batch_destroy(h)
            except Exception:
                pass
            self._h = None

    def add(self, model, i_shot=0):
        _capi.check(self._lib.psv_batch_add(self._h, model.handle, int(i_shot)))
        self._models.append(model)

    def add_all_shots(self, model):
        for s in range(model.n_shots):
            self.add(model, s)

    @property
    def persistent(self):
        v = ctypes.c_int()
        _capi.check(self._lib.psv_batch_get_persistent(self._h, ctypes.byref(v)))
        return bool(v.value)

    @persistent.setter
    def persistent(self, on):
        """Launch scheme: one launch per time step, captured as one graph
        (False, the default), or every step in one persistent launch (True).
        Results are identical."""
        _capi.check(self._lib.psv_batch_set_persistent(self._h, int(bool(on))))

    @property
    def cluster(self):
        v = ctypes.c_int()
        _capi.check(self._lib.psv_batch_get_cluster(self._h, ctypes.byref(v)))
        return bool(v.value)

    @cluster.setter
    def cluster(self, on):
        """Cluster-resident scheme (True): every member in its own
        thread-block cluster holding its whole grid in shared memory for
        every step, all members in one launch; results equal each model's
        own `fused_cluster` run bit for bit. ValueError when a member does
        not fit (`cluster_fits`). Setting `persistent` switches it off."""
        _capi.check(self._lib.psv_batch_set_cluster(self._h, int(bool(on))))

    @property
    def cluster_fits(self):
        v = ctypes.c_int()
        _capi.check(self._lib.psv_batch_cluster_fits(self._h, ctypes.byref(v)))
        return bool(v.value)

    def set_active(self, mask=None):
        """Members the next forward() advances (a boolean per member, in the
        order added); None = all."""
        if mask is None:
            _capi.check(self._lib.psv_batch_set_active(self._h, None, len(self._models)))
            return
        import numpy as np
        flags = np.ascontiguousarray(np.asarray(mask, dtype=bool).astype(np.int32))
        _capi.check(self._lib.psv_batch_set_active(
            self._h, flags.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), flags.size))

    def forward(self, store_fields=False, n_steps=0):
        _capi.check(self._lib.psv_batch_forward(self._h, int(bool(store_fields)), int(n_steps)))

    def set_parameter_fields_device(self, fields, mask=None):
        """set_parameter_fields for many members at once: `fields` is a CUDA
        float64 tensor whose row k holds member k's (vp, vs, rho), each
        [nx][nz] (rows past the last flagged member are not read); `mask`
        selects the members (all by default). One wait for torch's stream,
        then each model queues its copies and medium update on its own
        stream; forward() waits for them. Keep `fields` alive until then."""
        import numpy as np
        import torch
        if not fields.is_cuda or fields.dtype != torch.float64 or not fields.is_contiguous():
            raise ValueError("fields must be a contiguous float64 CUDA tensor")
        n = len(self._models)
        if mask is None:
            flags = np.ones(n, dtype=np.int32)
        else:
            m = np.asarray(mask, dtype=bool)
            flags = np.zeros(n, dtype=np.int32)
            flags[:m.size] = m
        rows = fields.shape[0]
        if flags[rows:].any():
            raise ValueError("a selected member has no row in fields")
        stride = fields[0].numel() if rows else 0
        for k in np.flatnonzero(flags):
            mdl = self._models[k]
            if 3 * mdl.nx * mdl.nz > stride:
                raise ValueError("fields rows are too short for member %d" % k)
        torch.cuda.current_stream(fields.device).synchronize()
        _capi.check(self._lib.psv_batch_set_parameter_fields_device(
            self._h, ctypes.c_void_p(fields.data_ptr()), stride,
            flags.ctypes.data_as(ctypes.POINTER(ctypes.c_int))))

    def misfits(self):
        """L2 misfit of each member's model after forward() (float64, one per
        member in the order added; NaN for inactive members), equal bit for
        bit to each model's calculate_l2_misfit(), which it also updates:
        one reduction per member and one copy back."""
        import numpy as np
        out = np.empty(len(self._models), dtype=np.float64)
        _capi.check(self._lib.psv_batch_misfits(
            self._h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), out.size))
        return out

    @property
    def tile_shape(self):
        return self._tile_shape if hasattr(self, "_tile_shape") else "16x28"

    @tile_shape.setter
    def tile_shape(self, name):
        _capi.check(self._lib.psv_batch_set_tile_shape(self._h, {"32x60": 0, "16x28": 1, "20x28": 2, "16x60": 3}[name]))
        self._tile_shape = name

    def autotune(self, n_steps=50):
        """Times every tile shape with both tile launch schemes, and the
        cluster-resident scheme when the members fit, on n_steps steps of
        the active members and keeps the fastest; returns the tile shape
        (the scheme is `cluster`, else `persistent`)."""
        v = ctypes.c_int()
        _capi.check(self._lib.psv_batch_autotune(self._h, int(n_steps), ctypes.byref(v)))
        self._tile_shape = {0: "32x60", 1: "16x28", 2: "20x28", 3: "16x60"}[v.value]
        return self._tile_shape

    def info(self):
        m, t, c = ctypes.c_int(), ctypes.c_int(), ctypes.c_double()
        _capi.check(self._lib.psv_batch_info(self._h, ctypes.byref(m), ctypes.byref(t),
                                             ctypes.byref(c)))
        return {"members": m.value, "tiles": t.value, "cells": c.value}
