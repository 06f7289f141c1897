"""The host-buffer entry point rp_trace_rays_host against the device-resident
trace: with pageable buffers (staged copies) and with page-locked buffers
(layout kernels reading and writing host memory directly, each generation
downloaded while the next is traced), including an output record offset that
is not 16-byte aligned, for both arithmetic paths."""
import ctypes

import numpy as np
import pytest

from helpers import build
from raypier_optics_gb300 import _native, ctracer, runtime, scene, tracer
from raypier_optics_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _host_trace(ctx, dscene, rays, P, flags, pinned, out_cap):
    lib = ctx.lib
    n = len(rays)
    max_gens = P["recursion_limit"] + 1
    offs = (ctypes.c_uint64 * (max_gens + 1))()
    ng = ctypes.c_int32(0)
    st = _native.Stats()
    if pinned:
        pin_in, pin_out = ctypes.c_void_p(), ctypes.c_void_p()
        _native.check(lib.rp_host_alloc(n * 188, ctypes.byref(pin_in)), "rp_host_alloc")
        _native.check(lib.rp_host_alloc(out_cap * 188, ctypes.byref(pin_out)), "rp_host_alloc")
        ctypes.memmove(pin_in, np.ascontiguousarray(rays).ctypes.data, n * 188)
        src, dst = pin_in, pin_out
    else:
        host_in = np.ascontiguousarray(rays).copy()
        host_out = np.zeros(out_cap, dtype=ctracer.ray_dtype)
        src, dst = ctypes.c_void_p(host_in.ctypes.data), ctypes.c_void_p(host_out.ctypes.data)
    _native.check(lib.rp_trace_rays_host(ctx.handle, dscene.handle, src, n, P["recursion_limit"],
                                         ctypes.c_float(P["max_length"]), flags, float(P["e2_terminate"]), dst,
                                         out_cap, offs, max_gens, ctypes.byref(ng), ctypes.byref(st)),
                  "rp_trace_rays_host")
    total = offs[ng.value]
    out = np.zeros(total, dtype=ctracer.ray_dtype)
    ctypes.memmove(out.ctypes.data, dst, total * 188)
    if pinned:
        lib.rp_host_free(pin_in)
        lib.rp_host_free(pin_out)
    return [out[offs[g]:offs[g + 1]] for g in range(ng.value)]


@pytest.mark.parametrize("flags", [tracer.RP_TRACE_PLAIN_FP64, tracer.RP_TRACE_MIXED])
def test_host_api_matches_device_trace(flags):
    rays, wl = W.config1_rays(ctracer.ray_dtype)
    rays = rays[:1001]  # odd sizes: unaligned generation offsets in the output
    P = W.CONFIG1
    lists, _ = build(W.config1_spec())
    ctx = runtime.get_context()
    tables = scene.compile_scene(lists)
    dscene = runtime.DeviceScene(ctx, tables, wl)
    rc = ctracer.RayCollection.from_array(rays.copy())
    rc.wavelengths = wl
    traced, _ = tracer.trace_rays(rc, build(W.config1_spec())[0], recursion_limit=P["recursion_limit"],
                                  max_length=P["max_length"], flags=flags, e2_terminate=P["e2_terminate"])
    ref = [t.copy_as_array() for t in traced]
    cap = sum(len(g) for g in ref) + 7
    for pinned in (False, True):
        gens = _host_trace(ctx, dscene, rays, P, flags, pinned, cap)
        assert [len(g) for g in gens] == [len(g) for g in ref]
        for a, b in zip(gens, ref):
            assert np.array_equal(a.view(np.uint8), b.view(np.uint8))
