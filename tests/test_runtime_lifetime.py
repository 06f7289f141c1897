"""Context lifetime on CPU with a fake library: the native context is
destroyed after every buffer and scene made on it, whatever order Python
finalises them in (objects reachable only from a reference cycle, such as a
script's globals at exit, are finalised in no fixed order)."""
import ctypes
import gc

import numpy as np

from raypier_optics_gb300 import runtime


class FakeLib:
    def __init__(self):
        self.log = []
        self.next = 100

    def _new(self, out):
        self.next += 1
        ctypes.cast(out, ctypes.POINTER(ctypes.c_void_p))[0] = self.next
        return 0

    def rp_ctx_create(self, device, budget, out):
        return self._new(out)

    def rp_rays_alloc(self, ctx, cap, out):
        return self._new(out)

    def rp_scene_create(self, ctx, desc, wl, n_wl, out):
        return self._new(out)

    def rp_rays_free(self, h):
        self.log.append(("rays", h.value))
        return 0

    def rp_scene_destroy(self, h):
        self.log.append(("scene", h.value))
        return 0

    def rp_ctx_destroy(self, h):
        self.log.append(("ctx", h.value))
        return 0


class FakeTables:
    n_faces = 0

    def desc(self):
        return runtime._native.SceneDesc()


def make(monkeypatch):
    lib = FakeLib()
    monkeypatch.setattr(runtime._native, "load", lambda *a, **k: lib)
    ctx = runtime.Context(0)
    return lib, ctx


def test_close_waits_for_live_objects(monkeypatch):
    lib, ctx = make(monkeypatch)
    rays = runtime.DeviceRays(ctx, 16)
    sc = runtime.DeviceScene(ctx, FakeTables(), np.zeros(0))
    ctx.close()
    assert lib.log == []  # deferred: two objects still use the context
    rays.free()
    assert [k for k, _ in lib.log] == ["rays"]
    sc.free()
    assert [k for k, _ in lib.log] == ["rays", "scene", "ctx"]
    ctx.close()
    sc.free()
    assert len(lib.log) == 3  # nothing is destroyed twice


def test_close_without_objects_is_immediate(monkeypatch):
    lib, ctx = make(monkeypatch)
    rays = runtime.DeviceRays(ctx, 16)
    rays.free()
    ctx.close()
    assert [k for k, _ in lib.log] == ["rays", "ctx"]


def test_cycle_collection_destroys_context_last(monkeypatch):
    lib, ctx = make(monkeypatch)
    holder = {}
    holder["self"] = holder  # a cycle, like a module's globals and its functions
    holder["ctx"] = ctx
    holder["rays"] = runtime.DeviceRays(ctx, 16)
    holder["scene"] = runtime.DeviceScene(ctx, FakeTables(), np.zeros(0))
    del ctx, holder
    gc.collect()
    kinds = [k for k, _ in lib.log]
    assert sorted(kinds) == ["ctx", "rays", "scene"] and kinds[-1] == "ctx"
