"""GPU runtime objects over the C ABI: a context per device, device ray
buffers and uploaded scenes.  Thin ctypes wrappers; all work happens in
``librp_gb300.so``."""
from __future__ import annotations

import ctypes
import hashlib
import threading
from collections import OrderedDict

import numpy as np

from . import _native

_default = {}
_lock = threading.Lock()


class Context:
    """One CUDA device, one stream, one device-memory budget (rp_ctx).

    Buffers, scenes, fields and lenses made on a context hold it (``attach``)
    until they are freed (``detach``).  The native context is destroyed only
    once none is left: at interpreter exit, objects reachable only from a
    reference cycle (a script's globals) are finalised in no fixed order, so
    the context's own finaliser may run before theirs."""

    def __init__(self, device: int = 0, hbm_budget: int = 0):
        self.lib = _native.load()
        self.device = device
        self._live = 0
        self._close_pending = False
        h = ctypes.c_void_p()
        _native.check(self.lib.rp_ctx_create(device, hbm_budget, ctypes.byref(h)), "rp_ctx_create")
        self.handle = h

    def attach(self):
        self._live += 1

    def detach(self):
        self._live -= 1
        if self._live <= 0 and self._close_pending:
            self.close()

    def synchronize(self):
        _native.check(self.lib.rp_ctx_synchronize(self.handle), "rp_ctx_synchronize")

    def memory_in_use(self) -> int:
        v = ctypes.c_uint64()
        _native.check(self.lib.rp_ctx_memory(self.handle, ctypes.byref(v)), "rp_ctx_memory")
        return v.value

    def close(self):
        """Destroys the native context, at once if nothing made on it is
        alive, else when the last such object is freed."""
        if getattr(self, "handle", None):
            for scene in self.__dict__.pop("_scenes", {}).values():
                scene.free()
            if self._live > 0:
                self._close_pending = True
                return
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
        ctx.attach()

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
            self.ctx.detach()

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
        ctx.attach()

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
            self.ctx.detach()

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
        self.counts_pending = False
        ctx.attach()

    def face_counts(self, reset: bool = True) -> np.ndarray:
        n = self.tables.n_faces
        out = np.zeros(n, dtype=np.uint32)
        if n:
            _native.check(self.lib.rp_scene_face_counts(self.handle, out.ctypes.data, n, int(reset)),
                          "rp_scene_face_counts")
        if reset:
            self.counts_pending = False
        return out

    def free(self):
        if getattr(self, "handle", None):
            self.lib.rp_scene_destroy(self.handle)
            self.handle = None
            self.ctx.detach()

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


SCENE_CACHE_SIZE = 8


def _scene_key(tables, wavelengths) -> bytes:
    """Digest of everything rp_scene_create reads: every packed table and the
    wavelengths.  Two face-list states that pack to the same bytes give the
    same device scene."""
    h = hashlib.blake2b(digest_size=20)
    h.update(np.array([tables.n_faces], dtype=np.int64).tobytes())
    for a in (tables.lists, tables.faces, tables.materials, tables.shape_ops, tables.distortions,
              tables.dispersions, tables.aux, np.ascontiguousarray(wavelengths, dtype=np.double)):
        h.update(np.array([a.shape[0]], dtype=np.int64).tobytes())
        h.update(np.ascontiguousarray(a).tobytes())
    return h.digest()


def cached_scene(ctx: Context, tables, wavelengths) -> DeviceScene:
    """The uploaded scene for `tables` on `ctx`, created once per distinct
    content and kept in a small per-context LRU.  A caller driving the
    generation loop itself (trace_segment once per generation) therefore
    uploads the scene once; changing a face's parameters changes the packed
    tables and uploads a new scene.  The per-face hit counts of a reused scene
    are cleared if its previous user did not read them back."""
    key = _scene_key(tables, wavelengths)
    with _lock:
        cache = ctx.__dict__.setdefault("_scenes", OrderedDict())
        scene = cache.get(key)
        if scene is not None:
            cache.move_to_end(key)
        else:
            scene = DeviceScene(ctx, tables, wavelengths)
            ctx.scene_uploads = getattr(ctx, "scene_uploads", 0) + 1
            cache[key] = scene
            while len(cache) > SCENE_CACHE_SIZE:
                cache.popitem(last=False)[1].free()
    if scene.counts_pending:
        scene.face_counts(reset=True)
    scene.counts_pending = True
    return scene
