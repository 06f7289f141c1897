"""GPU runtime objects over the C ABI: a context per device, device ray
buffers and uploaded scenes.  Thin ctypes wrappers; all work happens in
``librp_gb300.so``."""
from __future__ import annotations

import ctypes
import threading

import numpy as np

from . import _native

_default = {}
_lock = threading.Lock()


class Context:
    """One CUDA device, one stream, one device-memory budget (rp_ctx)."""

    def __init__(self, device: int = 0, hbm_budget: int = 0):
        self.lib = _native.load()
        self.device = device
        h = ctypes.c_void_p()
        _native.check(self.lib.rp_ctx_create(device, hbm_budget, ctypes.byref(h)), "rp_ctx_create")
        self.handle = h

    def synchronize(self):
        _native.check(self.lib.rp_ctx_synchronize(self.handle), "rp_ctx_synchronize")

    def memory_in_use(self) -> int:
        v = ctypes.c_uint64()
        _native.check(self.lib.rp_ctx_memory(self.handle, ctypes.byref(v)), "rp_ctx_memory")
        return v.value

    def close(self):
        if getattr(self, "handle", None):
            self.lib.rp_ctx_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def get_context(device: int = 0) -> Context:
    """The process-wide default context for `device` (created on first use)."""
    with _lock:
        ctx = _default.get(device)
        if ctx is None:
            ctx = Context(device)
            _default[device] = ctx
        return ctx


class DeviceGausslets:
    """A device Gausslet buffer (rp_gausslets): base rays plus six parabasal rays."""

    def __init__(self, ctx: Context, capacity: int):
        self.ctx = ctx
        self.lib = ctx.lib
        h = ctypes.c_void_p()
        _native.check(self.lib.rp_gausslets_alloc(ctx.handle, int(capacity), ctypes.byref(h)), "rp_gausslets_alloc")
        self.handle = h

    def count(self) -> int:
        v = ctypes.c_uint64()
        _native.check(self.lib.rp_gausslets_count(self.handle, ctypes.byref(v)), "rp_gausslets_count")
        return v.value

    def upload(self, records: np.ndarray):
        records = np.ascontiguousarray(records)
        _native.check(self.lib.rp_gausslets_upload(self.handle, records.ctypes.data, records.shape[0]),
                      "rp_gausslets_upload")

    def download(self, out: np.ndarray, n: int):
        assert out.flags.c_contiguous and out.shape[0] >= n
        _native.check(self.lib.rp_gausslets_download(self.handle, out.ctypes.data, n), "rp_gausslets_download")

    def free(self):
        if getattr(self, "handle", None):
            self.lib.rp_gausslets_free(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class DeviceRays:
    """A device structure-of-arrays ray buffer (rp_rays)."""

    def __init__(self, ctx: Context, capacity: int, handle=None):
        self.ctx = ctx
        self.lib = ctx.lib
        if handle is None:
            h = ctypes.c_void_p()
            _native.check(self.lib.rp_rays_alloc(ctx.handle, int(capacity), ctypes.byref(h)), "rp_rays_alloc")
            handle = h
        self.handle = handle

    def count(self) -> int:
        v = ctypes.c_uint64()
        _native.check(self.lib.rp_rays_count(self.handle, ctypes.byref(v)), "rp_rays_count")
        return v.value

    def capacity(self) -> int:
        v = ctypes.c_uint64()
        _native.check(self.lib.rp_rays_capacity(self.handle, ctypes.byref(v)), "rp_rays_capacity")
        return v.value

    def upload(self, records: np.ndarray):
        records = np.ascontiguousarray(records)
        _native.check(self.lib.rp_rays_upload_aos(self.handle, records.ctypes.data, records.shape[0]),
                      "rp_rays_upload_aos")

    def download(self, out: np.ndarray, n: int):
        assert out.flags.c_contiguous and out.shape[0] >= n
        _native.check(self.lib.rp_rays_download_aos(self.handle, out.ctypes.data, n), "rp_rays_download_aos")

    def field_ptr(self, name: str) -> int:
        p = ctypes.c_void_p()
        _native.check(self.lib.rp_rays_field(self.handle, name.encode(), ctypes.byref(p)), "rp_rays_field")
        return p.value

    def free(self):
        if getattr(self, "handle", None):
            self.lib.rp_rays_free(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class DeviceScene:
    """Scene tables uploaded to one context (rp_scene)."""

    def __init__(self, ctx: Context, tables, wavelengths):
        self.ctx = ctx
        self.lib = ctx.lib
        self.tables = tables
        wl = np.ascontiguousarray(wavelengths, dtype=np.double)
        self._wl = wl
        desc = tables.desc()
        h = ctypes.c_void_p()
        _native.check(self.lib.rp_scene_create(ctx.handle, ctypes.byref(desc), wl.ctypes.data if wl.size else None,
                                               wl.shape[0], ctypes.byref(h)), "rp_scene_create")
        self.handle = h

    def face_counts(self, reset: bool = True) -> np.ndarray:
        n = self.tables.n_faces
        out = np.zeros(n, dtype=np.uint32)
        if n:
            _native.check(self.lib.rp_scene_face_counts(self.handle, out.ctypes.data, n, int(reset)),
                          "rp_scene_face_counts")
        return out

    def free(self):
        if getattr(self, "handle", None):
            self.lib.rp_scene_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass
