"""E-field evaluation from traced rays and gausslets by summation of general
astigmatic Gaussian beams, with the public surface of raypier's
``core.fields`` (core/fields.py:1-277).

Every step runs on the device: the wavefront samples each mode is fitted to
(a gausslet's parabasal rays, or a ray's lattice neighbours carried to its
normal plane), the closed-form least-squares fit of the mode, the optional
projection of a ray lattice to an exit-pupil sphere, and the summation of
all modes at the evaluation points (``cfields``, include/rp_gb300.h
``rp_field_*``).  A traced collection that is already on the device is
fitted where it lies; host arrays are uploaded once.
"""
from __future__ import annotations

import ctypes
import math

import numpy

from . import _native, runtime
from .cfields import GaussianModes, evaluate_modes as evaluate_modes_c, sum_gaussian_modes  # noqa: F401
from .ctracer import GaussletCollection, RayCollection, gausslet_dtype, ray_dtype


def find_ray_gen(probe_centre, traced_rays):
    """The index of the traced generation whose segments pass the probe
    (core/fields.py:15-47), or -1 beyond the last one.

    Each generation is summarised by the mean of its origins, and the last
    one also by the mean of its end points, giving a chain of waypoints.
    The probe belongs to the segment leaving the waypoint nearest to it when
    it lies beyond the plane through that waypoint whose normal bisects the
    chain's incoming and outgoing directions there, else to the segment
    arriving at it."""
    probe = numpy.asarray(probe_centre, dtype=numpy.double).reshape(3)
    pts = [numpy.asarray(r.origin, dtype=numpy.double).mean(axis=0) for r in traced_rays]
    pts.append(numpy.asarray(traced_rays[-1].termination, dtype=numpy.double).mean(axis=0))
    k = int(numpy.argmin([float(numpy.sum((p - probe) ** 2)) for p in pts]))
    last = len(pts) - 1
    if k == last:
        return -1
    if k == 0:
        return 0

    def unit(v):
        return v / math.sqrt(float(numpy.sum(v * v)))

    bisector = unit(unit(pts[k] - pts[k - 1]) + unit(pts[k + 1] - pts[k]))
    gen = k if float(numpy.dot(probe - pts[k], bisector)) > 0 else k - 1
    return -1 if gen > last - 1 else gen


def _device_rays(records, ctx):
    recs = numpy.ascontiguousarray(records)
    if recs.dtype != ray_dtype:
        raise ValueError("an array of ray_dtype records is required")
    dev = runtime.DeviceRays(ctx, max(recs.shape[0], 1))
    dev.upload(recs)
    return dev, recs


def _device_gausslets(gausslets, ctx):
    if isinstance(gausslets, GaussletCollection):
        return gausslets._device(ctx), None
    arr = numpy.ascontiguousarray(gausslets)
    if arr.dtype != gausslet_dtype:
        raise ValueError("a GaussletCollection or an array of gausslet_dtype records is required")
    dev = runtime.DeviceGausslets(ctx, max(arr.shape[0], 1))
    dev.upload(arr)
    return dev, arr


def project_to_sphere(rays, centre=(0, 0, 0), radius=10.0):
    """The rays (ray_dtype array) that meet the sphere of `radius` about
    `centre`, each moved along its direction to the nearer-behind intercept,
    its optical path changed by that distance times the real refractive
    index (core/fields.py:51-77).  Computed on the device."""
    ctx = runtime.get_context()
    dev, recs = _device_rays(rays, ctx)
    n = recs.shape[0]
    hit = numpy.zeros(n, dtype=numpy.uint8)
    c = numpy.ascontiguousarray(centre, dtype=numpy.double).reshape(3)
    _native.check(ctx.lib.rp_rays_project_to_sphere(dev.handle, c.ctypes.data, float(radius),
                                                    hit.ctypes.data if n else None), "rp_rays_project_to_sphere")
    out = numpy.zeros(n, dtype=ray_dtype)
    dev.download(out, n)
    dev.free()
    return out[hit.astype(bool)]


def _samples(n):
    return [numpy.zeros((n, 6)) for _ in range(4)]


def evaluate_neighbours(rays, neighbours_idx):
    """(rays, x, y, dx, dy) for each ray of a lattice (ray_dtype array) with
    all six neighbours of ``neighbours_idx`` (n, 6): the neighbours' offsets
    in the ray's (E, E x d) frame after carrying them to its normal plane,
    and their slopes (core/fields.py:80-111).  Rays with a missing neighbour
    are dropped.  Computed on the device."""
    ctx = runtime.get_context()
    dev, recs = _device_rays(rays, ctx)
    n = recs.shape[0]
    nb = numpy.ascontiguousarray(neighbours_idx, dtype=numpy.int32).reshape(-1, 6)
    if nb.shape[0] != n:
        raise IndexError(f"boolean index did not match: {nb.shape[0]} neighbour rows for {n} rays")
    x, y, dx, dy = _samples(n)
    kept = numpy.zeros(n, dtype=numpy.uint64)
    nk = ctypes.c_uint64()
    st = ctx.lib.rp_field_ray_samples(dev.handle, nb.ctypes.data if n else None, x.ctypes.data, y.ctypes.data,
                                      dx.ctypes.data, dy.ctypes.data, kept.ctypes.data, ctypes.byref(nk))
    dev.free()
    if st == -1 and b"outside the collection" in (ctx.lib.rp_last_error() or b""):
        raise IndexError(ctx.lib.rp_last_error().decode())
    _native.check(st, "rp_field_ray_samples")
    k = nk.value
    return recs[kept[:k].astype(numpy.int64)], x[:k], y[:k], dx[:k], dy[:k]


def evaluate_neighbours_gc(gausslets):
    """(base rays, x, y, dx, dy): the offsets of each gausslet's six parabasal
    rays in its base ray's (E, E x d) frame and their slopes
    (core/fields.py:114-136), for a GaussletCollection or a gausslet_dtype
    array.  Computed on the device."""
    ctx = runtime.get_context()
    dev, arr = _device_gausslets(gausslets, ctx)
    n = dev.count()
    x, y, dx, dy = _samples(n)
    _native.check(ctx.lib.rp_field_gausslet_samples(dev.handle, x.ctypes.data, y.ctypes.data, dx.ctypes.data,
                                                    dy.ctypes.data), "rp_field_gausslet_samples")
    if arr is None:
        base = gausslets.copy_as_array()['base_ray']
    else:
        base = arr['base_ray']
        dev.free()
    return base, x, y, dx, dy


def evaluate_modes(neighbour_x, neighbour_y, dx, dy, blending=1.0):
    """The (n, 3) complex Gaussian-mode coefficients of each row of samples
    (core/fields.py:139-175).  The reference solves the two least-squares
    problems with scipy's iterative ``lsqr``; here they are solved exactly by
    their 3 x 3 normal equations on the device (``cfields.evaluate_modes``),
    the solution lsqr converges to."""
    return evaluate_modes_c(neighbour_x, neighbour_y, dx, dy, blending=blending)


def Gamma(z, A, B, C):
    """The mode parameters (A, B, C) after propagating a distance z
    (core/fields.py:178-185).  With G the 2 x 2 symmetric matrix [[A, B], [B, C]],
    propagation gives G (1 + z G)^-1, whose determinant-based inverse yields
    the three entries below."""
    det = (A * C) - (B * B)
    scale = 1.0 / (1.0 + z * (A + C) + (z * z) * det)
    return (A + z * det) * scale, B * scale, (C + z * det) * scale


def ExtractGamma(gausslet_collection, blending=1.0):
    """The mode coefficients of every gausslet, fitted on the device
    (core/fields.py:188-193)."""
    ctx = runtime.get_context()
    dev, arr = _device_gausslets(gausslet_collection, ctx)
    g = GaussianModes.from_gausslets(dev, numpy.zeros(0), blending)
    _, modes = g.download(records=False)
    g.close()
    if arr is not None:
        dev.free()
    return modes


def eval_Efield_from_rays(ray_collection, points, wavelengths, blending=1.0, time_ps=0.0, exit_pupil_offset=0.0,
                          exit_pupil_centre=(0.0, 0.0, 0.0)):
    """The complex E-field vector at each point from a ray lattice with
    neighbour indices (core/fields.py:195-224): optional projection to the
    exit-pupil sphere of radius ``exit_pupil_offset``, mode fit and
    summation, all on the device."""
    ctx = runtime.get_context()
    nb = ray_collection.neighbours
    dev = ray_collection._device(ctx)
    g = GaussianModes.from_rays(dev, nb, wavelengths, blending=blending, centre=exit_pupil_centre,
                                radius=float(exit_pupil_offset or 0.0))
    try:
        return g.evaluate(points, time_ps)
    finally:
        g.close()


class EFieldSummation:
    """The modes of a GaussletCollection fitted once on the device and kept
    there, for evaluation at any number of point sets
    (core/fields.py:227-266).  ``modes`` and ``base_rays`` are read back from
    the device when first used."""

    def __init__(self, gausslet_collection, wavelengths=None, blending=1.0):
        if wavelengths is None:
            wavelengths = numpy.asarray(gausslet_collection.wavelengths)
        if wavelengths is None:
            raise ValueError("No wavelengths supplied")
        self.wavelengths = wavelengths
        self._src = gausslet_collection
        ctx = runtime.get_context()
        dev, arr = _device_gausslets(gausslet_collection, ctx)
        self._dev = GaussianModes.from_gausslets(dev, wavelengths, blending)
        if arr is not None:
            dev.free()
        self._modes = None
        self._base = None

    @property
    def gc(self):
        src = self._src
        return src.copy_as_array() if isinstance(src, GaussletCollection) else numpy.asarray(src)

    def _read_back(self):
        recs, modes = self._dev.download()
        self._modes = modes
        self._base = RayCollection.from_array(recs)

    @property
    def modes(self):
        if self._modes is None:
            self._read_back()
        return self._modes

    @property
    def base_rays(self):
        if self._base is None:
            self._read_back()
        return self._base

    def evaluate(self, points, time_ps=0.0):
        points = numpy.ascontiguousarray(points)
        shape = points.shape
        E = self._dev.evaluate(points.reshape(-1, 3), time_ps)
        return E.reshape(shape)


def eval_Efield_from_gausslets(gausslet_collection, points, wavelengths=None, blending=1.0, time_ps=0.0, **kwds):
    """The complex E-field vector at each point from a GaussletCollection
    (core/fields.py:269-277): mode fit and summation on the device."""
    if wavelengths is None:
        wavelengths = numpy.asarray(gausslet_collection.wavelengths)
    ctx = runtime.get_context()
    dev, arr = _device_gausslets(gausslet_collection, ctx)
    g = GaussianModes.from_gausslets(dev, wavelengths, blending)
    if arr is not None:
        dev.free()
    try:
        return g.evaluate(points, time_ps)
    finally:
        g.close()
