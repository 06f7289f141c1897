"""Mirror of ``raypier.core.fields``: E-field evaluation from traced rays and
gausslets by summation of general astigmatic Gaussian beams
(core/fields.py:1-277).

The geometric set-up (neighbour offsets, projections) is numpy on the host as
in the reference; the mode fit and the points x modes summation run on the
GPU (``cfields``).
"""
from __future__ import annotations

import numpy

from .cfields import GaussianModes, evaluate_modes as evaluate_modes_c, sum_gaussian_modes
from .ctracer import RayCollection

scipy = None


def _normalise(a):
    a = numpy.asarray(a)
    mag = numpy.sqrt((a ** 2).sum(axis=-1))[..., numpy.newaxis]
    return a / mag


def _dot(a, b):
    return (a * b).sum(axis=-1)[..., numpy.newaxis]


def find_ray_gen(probe_centre, traced_rays):
    """Index of the traced generation passing nearest to a probe (core/fields.py:15-47)."""
    probe = numpy.asarray(probe_centre)
    waypoints = [rays.origin.mean(axis=0) for rays in traced_rays]
    waypoints.append(traced_rays[-1].termination.mean(axis=0))
    dist = [((wpt - probe) ** 2).sum() for wpt in waypoints]
    imin = numpy.argmin(dist)
    if imin + 1 >= len(waypoints):
        return -1
    closest = waypoints[imin]
    dir1 = _normalise(closest - waypoints[imin - 1])
    dir2 = _normalise(waypoints[imin + 1] - closest)
    normal = _normalise(dir1 + dir2)
    if _dot(probe - closest, normal) > 0:
        idx = imin
    else:
        idx = imin - 1
    if idx < 0:
        idx = 0
    if idx > len(waypoints) - 2:
        idx = -1
    return idx


def project_to_sphere(rays, centre=(0, 0, 0), radius=10.0):
    """Move rays back to their intercept with a sphere (core/fields.py:53-80)."""
    centre = numpy.asarray(centre).reshape(1, 3)
    origin = rays['origin'] - centre
    direction = rays['direction']
    c = (origin ** 2).sum(axis=1) - (radius ** 2)
    b = 2 * (direction * origin).sum(axis=1)
    d = b ** 2 - 4 * c
    selector = (d >= 0.0)
    d = numpy.sqrt(d[selector])
    b = b[selector]
    root1 = (-b + d) / 2
    root2 = (-b - d) / 2
    alpha = numpy.column_stack((root1, root2)).min(axis=1)
    rays = rays[selector]
    rays['origin'] += alpha[:, None] * direction[selector]
    rays['accumulated_path'] += alpha * rays['refractive_index'].real
    return rays


def evaluate_neighbours(rays, neighbours_idx):
    """Offsets and slopes of each ray's six neighbours in the plane normal to
    it (core/fields.py:83-119); rays without six neighbours are dropped."""
    mask = (neighbours_idx >= 0).all(axis=1)
    nb = neighbours_idx[mask, :]
    n_origin = rays['origin'][nb, :]
    n_direction = rays['direction'][nb, :]
    origin = rays['origin'][mask, None, :]
    direction = rays['direction'][mask, None, :]
    E = rays['E_vector'][mask, None, :]
    H = numpy.cross(E, direction)
    offsets = n_origin - origin
    alpha = -(offsets * direction).sum(axis=-1) / (n_direction * direction).sum(axis=-1)
    projected = (offsets + alpha[:, :, None] * n_direction)
    x = (projected * E).sum(axis=-1)
    y = (projected * H).sum(axis=-1)
    dz = (n_direction * direction).sum(axis=-1)
    dx = (n_direction * E).sum(axis=-1) / dz
    dy = (n_direction * H).sum(axis=-1) / dz
    return (rays[mask], x, y, dx, dy)


def evaluate_neighbours_gc(gausslets):
    """Parabasal offsets and slopes of gausslet records in the base ray's frame
    (core/fields.py:122-148)."""
    ga = gausslets
    origin = ga['base_ray']['origin'][:, None, :]
    direction = ga['base_ray']['direction'][:, None, :]
    n_direction = ga['para_rays']['direction']
    E = ga['base_ray']['E_vector'][:, None, :]
    H = numpy.cross(E, direction)
    offsets = ga['para_rays']['origin'] - origin
    x = (offsets * E).sum(axis=-1)
    y = (offsets * H).sum(axis=-1)
    dz = (n_direction * direction).sum(axis=-1)
    dx = (n_direction * E).sum(axis=-1) / dz
    dy = (n_direction * H).sum(axis=-1) / dz
    return (ga['base_ray'], x, y, dx, dy)


def evaluate_modes(neighbour_x, neighbour_y, dx, dy, blending=1.0):
    """The sparse least-squares form of the mode fit (core/fields.py:151-182),
    kept for comparison with the closed form (``cfields.evaluate_modes``)."""
    global scipy
    if scipy is None:
        import scipy as _scipy
        import scipy.sparse  # noqa: F401
        import scipy.sparse.linalg  # noqa: F401
        scipy = _scipy
    from scipy.sparse import block_diag
    from scipy.sparse.linalg import lsqr
    x = neighbour_x
    y = neighbour_y
    M = block_diag(numpy.dstack((x ** 2, 2 * x * y, y ** 2)))
    b = numpy.ones(M.shape[0])
    im_coefs = lsqr(M, b)[0].reshape(x.shape[0], 3)
    O = numpy.zeros_like(x)
    M_ = numpy.dstack((x, y, O, O, x, y)).reshape(-1, 12, 3)
    b = numpy.dstack((dx, dy)).reshape(-1)
    re_coefs = lsqr(block_diag(M_), b)[0].reshape(x.shape[0], 3)
    return ((blending * 1j) * im_coefs) + re_coefs


def Gamma(z, A, B, C):
    """Mode parameters after propagating a distance z (core/fields.py:185-192)."""
    detG0 = (A * C) - (B * B)
    denom = (1 + (z * (A + C)) + (z * z) * detG0)
    return (A + z * detG0) / denom, B / denom, (C + z * detG0) / denom


def ExtractGamma(gausslet_collection, blending=1.0):
    gc = gausslet_collection.copy_as_array()
    rays, x, y, dx, dy = evaluate_neighbours_gc(gc)
    return evaluate_modes_c(x, y, dx, dy, blending=blending)


def eval_Efield_from_rays(ray_collection, points, wavelengths, blending=1.0, time_ps=0.0, exit_pupil_offset=0.0,
                          exit_pupil_centre=(0.0, 0.0, 0.0)):
    """E-field at `points` from a ray field with neighbour indices
    (core/fields.py:205-224)."""
    rays = ray_collection.copy_as_array()
    radius = exit_pupil_offset
    projected = project_to_sphere(rays, exit_pupil_centre, radius) if radius else rays
    rays, x, y, dx, dy = evaluate_neighbours(projected, ray_collection.neighbours)
    modes = evaluate_modes_c(x, y, dx, dy, blending=blending)
    return sum_gaussian_modes(RayCollection.from_array(rays), modes, wavelengths, points, time_ps)


class EFieldSummation:
    """Modes of a GaussletCollection computed once, kept on the GPU and
    evaluated at any set of points (core/fields.py:227-266)."""

    def __init__(self, gausslet_collection, wavelengths=None, blending=1.0):
        if wavelengths is None:
            wavelengths = numpy.asarray(gausslet_collection.wavelengths)
        if wavelengths is None:
            raise ValueError("No wavelengths supplied")
        self.wavelengths = wavelengths
        self.gc = gc = gausslet_collection.copy_as_array()
        rays, x, y, dx, dy = evaluate_neighbours_gc(gc)
        self.modes = evaluate_modes_c(x, y, dx, dy, blending=blending)
        self.base_rays = RayCollection.from_array(numpy.ascontiguousarray(rays))
        self._dev = GaussianModes(self.base_rays, self.modes, self.wavelengths)

    def evaluate(self, points, time_ps=0.0):
        points = numpy.ascontiguousarray(points)
        shape = points.shape
        E = self._dev.evaluate(points.reshape(-1, 3), time_ps)
        return E.reshape(shape)


def eval_Efield_from_gausslets(gausslet_collection, points, wavelengths=None, blending=1.0, time_ps=0.0, **kwds):
    """The complex E-field vector at each point from a GaussletCollection
    (core/fields.py:269-277)."""
    gc = gausslet_collection.copy_as_array()
    if wavelengths is None:
        wavelengths = numpy.asarray(gausslet_collection.wavelengths)
    rays, x, y, dx, dy = evaluate_neighbours_gc(gc)
    modes = evaluate_modes_c(x, y, dx, dy, blending=blending)
    return sum_gaussian_modes(RayCollection.from_array(numpy.ascontiguousarray(rays)), modes, wavelengths, points,
                              time_ps)
