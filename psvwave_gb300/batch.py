"""Batched forward simulation: shots of many fdModels, of uneven grid sizes,
advanced together in one TMA-step launch per time step with the whole time
loop replayed as one CUDA graph (C ABI psv_batch_*)."""
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

    @property
    def tile_shape(self):
        return self._tile_shape if hasattr(self, "_tile_shape") else "16x28"

    @tile_shape.setter
    def tile_shape(self, name):
        _capi.check(self._lib.psv_batch_set_tile_shape(self._h, {"32x60": 0, "16x28": 1, "20x28": 2, "16x60": 3}[name]))
        self._tile_shape = name

    def autotune(self, n_steps=50):
        """Times every tile shape with both launch schemes on n_steps steps
        of the active members and keeps the fastest pair; returns the shape
        (the scheme is `persistent`)."""
        v = ctypes.c_int()
        _capi.check(self._lib.psv_batch_autotune(self._h, int(n_steps), ctypes.byref(v)))
        self._tile_shape = {0: "32x60", 1: "16x28", 2: "20x28", 3: "16x60"}[v.value]
        return self._tile_shape

    def info(self):
        m, t, c = ctypes.c_int(), ctypes.c_int(), ctypes.c_double()
        _capi.check(self._lib.psv_batch_info(self._h, ctypes.byref(m), ctypes.byref(t),
                                             ctypes.byref(c)))
        return {"members": m.value, "tiles": t.value, "cells": c.value}
