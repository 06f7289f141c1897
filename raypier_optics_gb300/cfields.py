"""Mirror of ``raypier.core.cfields``: Gaussian-mode fitting and E-field
summation over traced rays / gausslets, on the GPU.

``evaluate_modes`` and ``sum_gaussian_modes`` keep the reference's names,
arguments and results (cfields.pyx:49-234); the work runs in the sm_103a
library (include/rp_gb300.h, rp_field_*).  ``calc_mode_curvature`` and
``apply_mode_curvature`` are small per-ray host routines, restated here with
numpy.  There is no CPU fallback for the GPU entry points.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _native, runtime
from .ctracer import cross, norm, ray_dtype


def evaluate_modes(x, y, dx, dy, blending=1.0):
    """Least-squares Gaussian-mode coefficients (A, B, C) of each row of
    parabasal offsets x, y and slopes dx, dy (cfields.pyx:150-234).  Returns an
    (n, 3) complex array; raises ZeroDivisionError for a degenerate row, as the
    reference does."""
    ctx = runtime.get_context()
    a = [np.ascontiguousarray(v, dtype=np.double) for v in (x, y, dx, dy)]
    if a[0].ndim != 2 or any(v.shape != a[0].shape for v in a):
        raise ValueError("x, y, dx and dy must be 2-d arrays of one shape")
    n, size = a[0].shape
    out = np.zeros((n, 3), dtype=np.complex128)
    st = ctx.lib.rp_field_evaluate_modes(ctx.handle, a[0].ctypes.data, a[1].ctypes.data, a[2].ctypes.data,
                                         a[3].ctypes.data, n, size, float(blending), out.ctypes.data)
    if st == -1:
        raise ZeroDivisionError("float division")
    _native.check(st, "rp_field_evaluate_modes")
    return out


class GaussianModes:
    """A set of modes held on the device (rp_field) for repeated evaluation."""

    def __init__(self, rays, modes, wavelengths):
        self.ctx = runtime.get_context()
        recs = rays.copy_as_array() if hasattr(rays, "copy_as_array") else np.ascontiguousarray(rays)
        recs = np.ascontiguousarray(recs)
        assert recs.dtype == ray_dtype
        m = np.ascontiguousarray(modes, dtype=np.complex128).reshape(-1, 3)
        if m.shape[0] != recs.shape[0]:
            raise ValueError("one row of modes is needed per ray")
        wl = np.ascontiguousarray(wavelengths, dtype=np.double)
        h = ctypes.c_void_p()
        _native.check(self.ctx.lib.rp_field_create(self.ctx.handle, recs.ctypes.data, recs.shape[0], m.ctypes.data,
                                                   wl.ctypes.data if wl.size else None, wl.shape[0],
                                                   ctypes.byref(h)), "rp_field_create")
        self.handle = h

    def evaluate(self, points, time_ps=0.0):
        p = np.ascontiguousarray(points, dtype=np.double).reshape(-1, 3)
        out = np.zeros((p.shape[0], 3), dtype=np.complex128)
        _native.check(self.ctx.lib.rp_field_evaluate(self.handle, p.ctypes.data, p.shape[0], float(time_ps),
                                                     out.ctypes.data), "rp_field_evaluate")
        return out

    def close(self):
        if getattr(self, "handle", None):
            self.ctx.lib.rp_field_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def sum_gaussian_modes(rays, modes, wavelengths, points, time_ps):
    """The E-field (n_points, 3) complex at `points` from the Gaussian modes of
    `rays` (a RayCollection or ray_dtype array) with coefficients `modes`
    (cfields.pyx:49-117), on the GPU."""
    g = GaussianModes(rays, modes, wavelengths)
    try:
        return g.evaluate(points, time_ps)
    finally:
        g.close()


def calc_mode_curvature(rx, ry, dx, dy, dx2, dy2, dxdy):
    """Mode curvature A, B, C and local bases at each point (cfields.pyx:237-290)."""
    N = len(rx)
    A, B, C = np.empty(N), np.empty(N), np.empty(N)
    X, Y, Z = np.empty((N, 3)), np.empty((N, 3)), np.empty((N, 3))
    for i in range(N):
        c = norm((-float(dx[i]), -float(dy[i]), 1.0))
        a = norm(cross((0.0, 0.0, 1.0), c))
        b = cross(c, a)
        X[i], Y[i], Z[i] = a, b, c
        Fz = c[0] * dx[i] + c[1] * dy[i] + c[2]
        A[i] = -(a[0] * a[0] * dx2[i] + 2 * a[0] * a[1] * dxdy[i] + a[1] * a[1] * dy2[i]) / Fz
        B[i] = -(a[0] * b[0] * dx2[i] + (a[0] * b[1] + b[0] * a[1]) * dxdy[i] + a[1] * b[1] * dy2[i]) / Fz
        C[i] = -(b[0] * b[0] * dx2[i] + 2 * b[0] * b[1] * dxdy[i] + b[1] * b[1] * dy2[i]) / Fz
    return (A, B, C, X, Y, Z)


def apply_mode_curvature(gc, A, B, C):
    """Tilts each gausslet's parabasal rays by the given wavefront curvature
    (cfields.pyx:397-426)."""
    arr = gc.copy_as_array()
    for i in range(len(arr)):
        ray = arr[i]['base_ray']
        z = tuple(float(v) for v in ray['direction'])
        x = tuple(float(v) for v in ray['E_vector'])
        y = cross(x, z)
        for j in range(6):
            para = arr[i]['para_rays'][j]
            r = tuple(float(para['origin'][k] - ray['origin'][k]) for k in range(3))
            px = r[0] * x[0] + r[1] * x[1] + r[2] * x[2]
            py = r[0] * y[0] + r[1] * y[1] + r[2] * y[2]
            sx = (-A[i] * px - B[i] * py)
            sy = (-C[i] * py - B[i] * px)
            shift = tuple(x[k] * sx + y[k] * sy for k in range(3))
            d = tuple(shift[k] + float(para['direction'][k]) for k in range(3))
            arr[i]['para_rays'][j]['direction'] = norm(d)
    new = type(gc).from_array(arr)
    gc._host, gc._n = new._host, new._n
    gc._mark_host_written()
