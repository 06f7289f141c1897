"""Generation drivers, mirroring ``raypier.core.tracer`` (core/tracer.py).

``trace_rays`` keeps the reference's signature and return value
``(traced_rays, all_faces)``; the generation loop itself runs in the C ABI
(``rp_trace_rays``): generations stay on the device, linked by ``parent``,
and are copied to the host only when a RayCollection property is read.
"""
from __future__ import annotations

import ctypes
from itertools import chain

import numpy

from . import _native, runtime
from .ctracer import RayCollection
from .scene import check_face_indices, compile_scene

RP_TRACE_PLAIN_FP64 = 0
RP_TRACE_MIXED = 1

# The |E|^2 termination threshold applied between generations (0 = off).
# The reference has no such rule; it is applied as a stable filter on the
# children of each generation.
DEFAULT_E2_TERMINATE = 0.0


def _prepare(input_rays, face_lists, max_length):
    all_faces = list(chain(*(fs.faces for fs in face_lists)))
    wavelengths = numpy.asarray(input_rays.wavelengths)
    for i, f in enumerate(all_faces):   # core/tracer.py:28-34
        f.idx = i
        f.count = 0
        f.update()
        f.material.wavelengths = wavelengths
        f.max_length = max_length
    return all_faces, wavelengths


def _apply_counts(scene, tables):
    counts = scene.face_counts(reset=True)
    for rec, c in enumerate(counts):
        if c:
            tables.face_objects[rec].count += int(c)


def trace_rays(input_rays, face_lists, recursion_limit=100, max_length=100.0, flags=RP_TRACE_PLAIN_FP64,
               e2_terminate=DEFAULT_E2_TERMINATE, ctx=None):
    """Non-sequential trace of `input_rays` through `face_lists`
    (core/tracer.py:9-47).  Returns (traced_rays, all_faces)."""
    from .ctracer import GaussletCollection
    if isinstance(input_rays, GaussletCollection):
        return _trace_gausslets(input_rays, face_lists, recursion_limit, max_length, ctx=ctx)
    if not isinstance(input_rays, RayCollection):
        raise TypeError("input_rays must be a RayCollection or a GaussletCollection")
    ctx = ctx or runtime.get_context()
    input_rays.reset_length(max_length)   # core/tracer.py:22
    all_faces, wavelengths = _prepare(input_rays, face_lists, max_length)
    face_sets = list(face_lists)
    for fs in face_sets:
        fs.sync_transforms()
    tables = compile_scene(face_sets)
    scene = runtime.cached_scene(ctx, tables, wavelengths)
    dev0 = input_rays._device(ctx)
    max_gens = max(int(recursion_limit), 1) + 1
    gens = (ctypes.c_void_p * max_gens)()
    gens[0] = dev0.handle
    n_gens = ctypes.c_int32(0)
    stats = _native.Stats()
    lib = ctx.lib
    _native.check(lib.rp_trace_rays(ctx.handle, scene.handle, gens, max_gens, int(recursion_limit),
                                    ctypes.c_float(max_length), flags, float(e2_terminate),
                                    ctypes.byref(n_gens), ctypes.byref(stats)), "rp_trace_rays")
    traced = []
    if n_gens.value > 0:
        input_rays._mark_device_written()   # lengths / end_face_idx were updated on the device
        traced.append(input_rays)
    prev = input_rays
    for g in range(1, n_gens.value):
        rc = RayCollection._from_device(runtime.DeviceRays(ctx, 0, handle=ctypes.c_void_p(gens[g])), parent=prev)
        traced.append(rc)
        prev = rc
    # free generations the library allocated but the reference would not return
    # (gens[0] is the caller's input buffer and stays with input_rays)
    for g in range(max(n_gens.value, 1), max_gens):
        if gens[g]:
            lib.rp_rays_free(ctypes.c_void_p(gens[g]))
    _apply_counts(scene, tables)
    trace_rays.last_stats = stats
    return traced, all_faces


trace_rays.last_stats = None


def _trace_generation(rays, face_sets, all_faces, max_length, one_face=None, flags=RP_TRACE_PLAIN_FP64,
                      e2_terminate=DEFAULT_E2_TERMINATE, ctx=None):
    """One generation (trace_segment_c / trace_one_face_segment_c)."""
    ctx = ctx or runtime.get_context()
    check_face_indices(face_sets, all_faces)
    tables = compile_scene(face_sets)
    scene = runtime.cached_scene(ctx, tables, rays.wavelengths)
    dev_in = rays._device(ctx)
    out = runtime.DeviceRays(ctx, 2 * max(rays.n_rays, 1))
    stats = _native.Stats()
    lib = ctx.lib
    if one_face is None:
        st = lib.rp_trace_segment(ctx.handle, scene.handle, dev_in.handle, out.handle, ctypes.c_float(max_length),
                                  flags, float(e2_terminate), ctypes.byref(stats))
        _native.check(st, "rp_trace_segment")
    else:
        li, fi = one_face
        st = lib.rp_trace_one_face_segment(ctx.handle, scene.handle, dev_in.handle, out.handle, li, fi,
                                           ctypes.c_float(max_length), flags, float(e2_terminate),
                                           ctypes.byref(stats))
        _native.check(st, "rp_trace_one_face_segment")
    rays._mark_device_written()
    _apply_counts(scene, tables)
    return RayCollection._from_device(out, parent=rays)


def _trace_gausslet_generation(gc, face_sets, all_faces, max_length, one_face=None, decomp_faces=(), ctx=None):
    """One Gausslet generation (trace_gausslet_c / trace_one_face_gausslet_c,
    ctracer.pyx:2214-2350).  The device traces the gausslets; the
    decomposition materials' captures and eval_func run here, on the host, as
    in the reference (cmaterials.pyx:1806-1830)."""
    from .ctracer import GaussletCollection
    ctx = ctx or runtime.get_context()
    check_face_indices(face_sets, all_faces)
    tables = compile_scene(face_sets)
    scene = runtime.cached_scene(ctx, tables, gc.wavelengths)
    n = gc.n_rays
    capture = len(decomp_faces) > 0
    before = gc.copy_as_array() if capture else None
    dev_in = gc._device(ctx)
    out = runtime.DeviceGausslets(ctx, 2 * max(n, 1))
    captured = numpy.zeros(max(n, 1), dtype=numpy.int32) if capture else None
    stats = _native.Stats()
    li, fi = one_face if one_face is not None else (-1, -1)
    _native.check(ctx.lib.rp_trace_gausslet_segment(ctx.handle, scene.handle, dev_in.handle, out.handle, li, fi,
                                                     ctypes.c_double(max_length),
                                                     captured.ctypes.data if capture else None,
                                                     ctypes.byref(stats)), "rp_trace_gausslet_segment")
    gc._mark_device_written()
    _apply_counts(scene, tables)
    new = GaussletCollection._from_device(out, parent=gc)
    if capture:
        mutated = gc.copy_as_array()
        for i in numpy.flatnonzero(captured[:n]):
            mat = tables.material_objects[int(captured[i]) - 1]
            rec = mutated[i].copy()
            rec['para_rays'] = before[i]['para_rays']  # captured before its parabasal rays were traced
            mat.captured_rays.add_gausslet(_gausslet_of(rec))
            mat.capture_count += 1
        for face in decomp_faces:  # ctracer.pyx:2274-2278
            if face.count:
                face.material.eval_decomposed_rays(new)
                face.count = 0
        new.reset_length(max_length)
    _trace_gausslet_generation.last_stats = stats
    return new


_trace_gausslet_generation.last_stats = None


def _gausslet_of(rec):
    from .ctracer import Gausslet
    g = Gausslet()
    g.gausslet[()] = rec
    return g


def _trace_gausslets(input_rays, face_lists, recursion_limit, max_length, ctx=None):
    """trace_rays for a GaussletCollection (core/tracer.py:9-47 with
    trace_func = trace_gausslet)."""
    input_rays.reset_length(max_length)
    all_faces, _ = _prepare(input_rays, face_lists, max_length)
    face_sets = list(face_lists)
    for fs in face_sets:
        fs.sync_transforms()
    decomp_faces = [f for f in all_faces if f.material.is_decomp_material()]
    traced = []
    rays = input_rays
    count = 0
    while rays.n_rays > 0 and count < recursion_limit:
        traced.append(rays)
        rays = _trace_gausslet_generation(rays, face_sets, all_faces, max_length, decomp_faces=decomp_faces,
                                          ctx=ctx)
        count += 1
    return traced, all_faces


def trace_ray_sequence(input_rays, face_sequence, recursion_limit=100, max_length=100.0, ctx=None):
    """Sequential trace through (FaceList, face_idx) pairs (core/tracer.py:50-99)."""
    from .ctracer import GaussletCollection, trace_one_face_gausslet, trace_one_face_segment
    input_rays.reset_length(max_length)
    traced_rays = [input_rays]
    face_lists = [fl for fl, fidx in face_sequence]
    face_idx_list = [fidx for fl, fidx in face_sequence]
    count = 0
    all_faces, wavelengths = _prepare(input_rays, face_lists, max_length)
    trace_func = trace_one_face_segment if isinstance(input_rays, RayCollection) else trace_one_face_gausslet
    decomp_faces = [f for f in all_faces if f.material.is_decomp_material()]
    rays = input_rays
    for next_face_list, next_face_idx in zip(face_lists, face_idx_list):
        rays = trace_func(rays, next_face_list, next_face_idx, all_faces, max_length=max_length,
                          decomp_faces=decomp_faces)
        if (count > recursion_limit) or (rays.n_rays == 0):
            break
        traced_rays.append(rays)
        count += 1
    return traced_rays, all_faces
