"""Mirror of ``raypier.core.cfields``: Gaussian-mode fitting and E-field
summation over traced rays / gausslets, on the GPU.

Every function keeps the reference's name, arguments and results
(cfields.pyx:49-426); the work runs in the sm_103a library
(include/rp_gb300.h, rp_field_*).  There is no CPU fallback.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _native, runtime
from .ctracer import ray_dtype


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


def _field_check(status, where):
    """A degenerate mode fit is the reference's ZeroDivisionError."""
    if status == -1:
        lib = _native.load(build_if_needed=False)
        if (lib.rp_last_error() or b"") == b"float division":
            raise ZeroDivisionError("float division")
    _native.check(status, where)


class GaussianModes:
    """A set of modes held on the device (rp_field) for repeated evaluation:
    from host rays and coefficients, or fitted on the device from a gausslet
    collection (``from_gausslets``) or a ray lattice (``from_rays``)."""

    def __init__(self, rays, modes, wavelengths, _handle=None, _ctx=None):
        self.ctx = _ctx or runtime.get_context()
        if _handle is not None:
            self.handle = _handle
            self.ctx.attach()
            return
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
        self.ctx.attach()

    @classmethod
    def from_gausslets(cls, dev_gausslets, wavelengths, blending=1.0):
        """Modes fitted on the device to the parabasal rays of a device gausslet
        collection (runtime.DeviceGausslets)."""
        ctx = dev_gausslets.ctx
        wl = np.ascontiguousarray(wavelengths, dtype=np.double)
        h = ctypes.c_void_p()
        _field_check(ctx.lib.rp_field_create_from_gausslets(dev_gausslets.handle, wl.ctypes.data if wl.size else None,
                                                            wl.shape[0], float(blending), ctypes.byref(h)),
                     "rp_field_create_from_gausslets")
        return cls(None, None, None, _handle=h, _ctx=ctx)

    @classmethod
    def from_rays(cls, dev_rays, neighbours, wavelengths, blending=1.0, centre=(0.0, 0.0, 0.0), radius=0.0):
        """Modes fitted on the device to a ray lattice (runtime.DeviceRays) and
        its (n, 6) neighbour table, after projection to the sphere of `radius`
        about `centre` when radius is non-zero."""
        ctx = dev_rays.ctx
        n = dev_rays.count()
        nb = np.ascontiguousarray(neighbours, dtype=np.int32).reshape(-1, 6)
        if nb.shape[0] != n:
            raise IndexError(f"boolean index did not match: {nb.shape[0]} neighbour rows for {n} rays")
        wl = np.ascontiguousarray(wavelengths, dtype=np.double)
        c = np.ascontiguousarray(centre, dtype=np.double).reshape(3)
        h = ctypes.c_void_p()
        st = ctx.lib.rp_field_create_from_rays(dev_rays.handle, nb.ctypes.data, c.ctypes.data, float(radius),
                                               float(blending), wl.ctypes.data if wl.size else None, wl.shape[0],
                                               ctypes.byref(h))
        if st == -1 and b"outside the collection" in (ctx.lib.rp_last_error() or b""):
            raise IndexError(ctx.lib.rp_last_error().decode())
        if st == -1 and b"miss the projection sphere" in (ctx.lib.rp_last_error() or b""):
            raise IndexError(ctx.lib.rp_last_error().decode())
        _field_check(st, "rp_field_create_from_rays")
        return cls(None, None, None, _handle=h, _ctx=ctx)

    def download(self, records=True, modes=True):
        """(base-ray records or None, n x 3 complex modes or None)."""
        n = ctypes.c_uint64()
        _native.check(self.ctx.lib.rp_field_download(self.handle, ctypes.byref(n), None, None), "rp_field_download")
        recs = np.zeros(n.value, dtype=ray_dtype) if records else None
        m = np.zeros((n.value, 3), dtype=np.complex128) if modes else None
        _native.check(self.ctx.lib.rp_field_download(self.handle, ctypes.byref(n),
                                                     recs.ctypes.data if recs is not None and n.value else None,
                                                     m.ctypes.data if m is not None and n.value else None),
                      "rp_field_download")
        return recs, m

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
            self.ctx.detach()

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
    """Wavefront curvature A, B, C and the local bases x', y', z' at each
    point (cfields.pyx:232-290), on the GPU.  Returns (A, B, C, x, y, z), the
    last three (N, 3)."""
    n = len(rx)
    a = [np.ascontiguousarray(v, dtype=np.double).reshape(-1) for v in (dx, dy, dx2, dy2, dxdy)]
    if any(v.shape[0] < n for v in a):
        raise IndexError("Out of bounds on buffer access (axis 0)")
    ctx = runtime.get_context()
    out = [np.empty(n) for _ in range(3)] + [np.empty((n, 3)) for _ in range(3)]
    _native.check(ctx.lib.rp_field_mode_curvature(ctx.handle, *[v.ctypes.data for v in a], n,
                                                  *[o.ctypes.data for o in out]), "rp_field_mode_curvature")
    return tuple(out)


def build_interaction_matrix(rx, ry, tx, ty, A, B, C, x, y, z, wavelength, spacing, max_spacing, blending,
                             test_spacing):
    """The sparse matrix of the field of mode i at test point j for every pair
    within max_spacing (cfields.pyx:295-395), on the GPU, as the tuple
    (data, (i, j)) that scipy.sparse.coo_matrix takes, ordered by i then j.
    The reference sizes its output by an estimate from test_spacing and
    writes past it when the estimate is short; here the exact count is used."""
    n, L = len(rx), len(tx)
    v = [np.ascontiguousarray(a, dtype=np.double).reshape(-1) for a in (rx, ry, A, B, C)]
    t = [np.ascontiguousarray(a, dtype=np.double).reshape(-1) for a in (tx, ty)]
    b = [np.ascontiguousarray(a, dtype=np.double).reshape(-1, 3) for a in (x, y, z)]
    if any(a.shape[0] < n for a in v + b) or t[1].shape[0] < L:
        raise IndexError("Out of bounds on buffer access (axis 0)")
    ctx = runtime.get_context()
    cap = n * (1 + int((7 * max_spacing * max_spacing) / (test_spacing * test_spacing)))
    count = ctypes.c_uint64()
    for _ in range(2):
        data = np.zeros(cap, np.complex128)
        xi = np.zeros(cap, np.uint)
        xj = np.zeros(cap, np.uint)
        st = ctx.lib.rp_field_interaction_matrix(
            ctx.handle, v[0].ctypes.data, v[1].ctypes.data, n, t[0].ctypes.data, t[1].ctypes.data, L,
            v[2].ctypes.data, v[3].ctypes.data, v[4].ctypes.data, b[0].ctypes.data, b[1].ctypes.data, b[2].ctypes.data,
            float(wavelength), float(spacing), float(max_spacing), float(blending), cap, ctypes.byref(count),
            data.ctypes.data, xi.ctypes.data, xj.ctypes.data)
        if st == _native.RP_ERR_CAPACITY:
            cap = count.value  # the estimate was short: once more at the exact size
            continue
        _native.check(st, "rp_field_interaction_matrix")
        ct = count.value
        return (data[:ct], (xi[:ct], xj[:ct]))
    _native.check(st, "rp_field_interaction_matrix")


def apply_mode_curvature(gc, A, B, C):
    """Tilts each gausslet's parabasal rays by the given wavefront curvature
    (cfields.pyx:397-426), on the GPU, in place."""
    n = gc.n_rays
    a = [np.ascontiguousarray(v, dtype=np.double).reshape(-1) for v in (A, B, C)]
    if any(v.shape[0] < n for v in a):
        raise IndexError("Out of bounds on buffer access (axis 0)")
    if n == 0:
        return
    ctx = runtime.get_context()
    dev = gc._device(ctx)
    _native.check(ctx.lib.rp_field_apply_mode_curvature(dev.handle, *[v.ctypes.data for v in a]),
                  "rp_field_apply_mode_curvature")
    gc._mark_device_written()
