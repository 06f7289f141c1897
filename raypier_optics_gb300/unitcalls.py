"""Single-plugin GPU calls behind the reference's Python-visible unit methods
(Face.intersect / compute_normal, Shape.point_inside, Distortion.z_offset*,
InterfaceMaterial.eval_child_ray, Convert_to_SP, BaseDispersionCurve.evaluate_n).

Each call builds a one-list scene around the object, uploads it and runs the
same device functions the generation kernel uses (rp_unit.cu)."""
from __future__ import annotations

import ctypes

import numpy as np

from . import _native, runtime
from .ctracer import FaceList, Ray, ray_dtype
from .scene import SceneTables


def _scene_for(ctx, build, wavelengths=()):
    t = SceneTables()
    build(t)
    t.finish()
    return runtime.DeviceScene(ctx, t, np.asarray(wavelengths, dtype=np.double)), t


def _pts(a):
    return np.ascontiguousarray(np.asarray(a, dtype=np.double).reshape(-1, 3))


def face_intersect(face, p1, p2, is_base_ray, ctx=None):
    ctx = ctx or runtime.get_context()
    fl = FaceList()
    fl.faces = [face]
    scene, _ = _scene_for(ctx, lambda t: t.add_list(fl))
    a, b = _pts(p1), _pts(p2)
    out = np.zeros(a.shape[0])
    _native.check(ctx.lib.rp_face_intersect(scene.handle, 0, a.ctypes.data, b.ctypes.data, a.shape[0],
                                            int(is_base_ray), out.ctypes.data), "rp_face_intersect")
    return out


def face_normal(face, p, ctx=None):
    ctx = ctx or runtime.get_context()
    fl = FaceList()
    fl.faces = [face]
    scene, _ = _scene_for(ctx, lambda t: t.add_list(fl))
    a = _pts(p)
    out = np.zeros_like(a)
    _native.check(ctx.lib.rp_face_normal(scene.handle, 0, a.ctypes.data, a.shape[0], out.ctypes.data),
                  "rp_face_normal")
    return out


def shape_inside(shape, xy, ctx=None):
    ctx = ctx or runtime.get_context()
    holder = {}
    scene, _ = _scene_for(ctx, lambda t: holder.__setitem__("prog", t.add_shape(shape)))
    a = np.ascontiguousarray(np.asarray(xy, dtype=np.double).reshape(-1, 2))
    out = np.zeros(a.shape[0], dtype=np.int32)
    _native.check(ctx.lib.rp_shape_inside(scene.handle, holder["prog"], a.ctypes.data, a.shape[0],
                                          out.ctypes.data), "rp_shape_inside")
    return out.astype(bool)


def distortion_eval(dist, x, y, ctx=None):
    ctx = ctx or runtime.get_context()
    x = np.asarray(x, dtype=np.double).reshape(-1)
    y = np.asarray(y, dtype=np.double).reshape(-1)
    if len(x) != len(y):
        raise ValueError("Both x and y must have the same length")
    holder = {}
    scene, _ = _scene_for(ctx, lambda t: holder.__setitem__("d", t.add_distortion(dist)))
    xy = np.ascontiguousarray(np.stack([x, y], axis=1))
    out = np.zeros((len(x), 4))
    _native.check(ctx.lib.rp_distortion_eval(scene.handle, holder["d"], xy.ctypes.data, len(x), out.ctypes.data),
                  "rp_distortion_eval")
    return out


def _records(rays):
    rec = np.zeros(len(rays), dtype=ray_dtype)
    for i, r in enumerate(rays):
        rec[i] = r.ray
    return rec


def eval_child_rays(material, rays, ray_idx, points, normals, tangents, ctx=None):
    """Children of each (ray, point, orientation) as lists of Ray objects."""
    ctx = ctx or runtime.get_context()
    rec = _records(rays)
    n = len(rays)
    idx = np.broadcast_to(np.asarray(ray_idx, dtype=np.uint32), (n,)).copy()
    holder = {}
    wl = getattr(material, "wavelengths", np.zeros(0))
    scene, _ = _scene_for(ctx, lambda t: holder.__setitem__("m", t.add_material(material)), wl)
    p, nn, tt = _pts(points), _pts(normals), _pts(tangents)
    children = np.zeros(2 * n, dtype=ray_dtype)
    nc = np.zeros(n, dtype=np.int32)
    _native.check(ctx.lib.rp_material_eval(scene.handle, holder["m"], rec.ctypes.data, idx.ctypes.data,
                                           p.ctypes.data, nn.ctypes.data, tt.ctypes.data, n,
                                           children.ctypes.data, nc.ctypes.data), "rp_material_eval")
    out = []
    for i in range(n):
        lst = []
        for k in range(nc[i]):
            r = Ray()
            r.ray[()] = children[2 * i + k]
            lst.append(r)
        out.append(lst)
    return out


def convert_to_sp(rays, normals, ctx=None):
    ctx = ctx or runtime.get_context()
    rec = _records(rays)
    nn = _pts(normals)
    out = np.zeros_like(rec)
    _native.check(ctx.lib.rp_convert_to_sp(ctx.handle, rec.ctypes.data, nn.ctypes.data, len(rays),
                                           out.ctypes.data), "rp_convert_to_sp")
    res = []
    for i in range(len(rays)):
        r = Ray()
        r.ray[()] = out[i]
        res.append(r)
    return res


def dispersion_n(curve, wavelengths, ctx=None):
    ctx = ctx or runtime.get_context()
    holder = {}
    scene, _ = _scene_for(ctx, lambda t: holder.__setitem__("c", t.add_dispersion(curve)))
    wl = np.ascontiguousarray(wavelengths, dtype=np.double)
    out = np.zeros(2 * len(wl))
    _native.check(ctx.lib.rp_dispersion_eval(scene.handle, holder["c"], wl.ctypes.data, len(wl), out.ctypes.data),
                  "rp_dispersion_eval")
    return out[0::2] + 1j * out[1::2]
