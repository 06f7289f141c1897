"""Face types, mirroring ``raypier.core.cfaces`` (cfaces.pyx).

Each class keeps the reference's constructor keywords, public attributes and
``params`` list, and packs itself into an ``rp_face`` record (``_pack``) whose
layout include/rp_gb300.h documents per type.  Intersection and normal
evaluation run on the GPU; faces the device does not implement are not
listed here (the scene compiler raises ``NotImplementedError`` for them).
"""
from __future__ import annotations

import math

import numpy as np

from .ctracer import Face, Shape, Transform, norm, cross

FACE_NONE, CIRCULAR, RECTANGULAR, SHAPED_PLANAR, SPHERICAL, SHAPED_SPHERICAL, CONIC, ASPHERIC, EXTPOLY, \
    DISTORTION, ORIENTED_POLYGON, POLYGON, ELLIPTICAL_PLANE, OFF_AXIS_PARABOLIC, ELLIPSOIDAL, SADDLE, CYLINDRICAL, \
    AXICON = range(18)


class ShapedFace(Face):
    """cfaces.pyx:47-137"""

    def __init__(self, owner=None, tolerance=0.0001, max_length=100, material=None, **kwds):
        super().__init__(owner, tolerance, max_length, material, **kwds)
        self.shape = kwds.get("shape", Shape())
        self.invert_normals = int(kwds.get('invert_normals', 0))

    def _pack_shape(self, rec, tables):
        rec['shape'] = tables.add_shape(self.shape)


class CircularFace(Face):
    """cfaces.pyx:140-191; p = (diameter, offset, z_plane)."""
    params = ['diameter', 'offset']
    type_code = CIRCULAR

    def __init__(self, owner=None, tolerance=0.0001, max_length=100, material=None, **kwds):
        super().__init__(owner, tolerance, max_length, material, **kwds)
        self.diameter = 0.0
        self.offset = 0.0
        self.z_plane = float(kwds.get('z_plane', 0.0))
        self.invert_normals = int(kwds.get("invert_normals", False))

    def _pack(self, rec, tables):
        rec['p'][:3] = (self.diameter, self.offset, self.z_plane)
        rec['invert_normals'] = int(self.invert_normals)


class ShapedPlanarFace(ShapedFace):
    """cfaces.pyx:194-242; p = (z_height,)."""
    type_code = SHAPED_PLANAR

    def __init__(self, owner=None, tolerance=0.0001, max_length=100, material=None, **kwds):
        super().__init__(owner, tolerance, max_length, material, **kwds)
        self.z_height = float(kwds.get('z_height', 0.0))

    def _pack(self, rec, tables):
        rec['p'][0] = self.z_height
        self._pack_shape(rec, tables)

    def eval_z_c(self, x, y):
        return self.z_height


class ElipticalPlaneFace(Face):
    """cfaces.pyx:313-351; p = (g_x, g_y, diameter)."""
    params = ['diameter']
    type_code = ELLIPTICAL_PLANE

    def __init__(self, owner=None, tolerance=0.0001, max_length=100, material=None, **kwds):
        super().__init__(owner, tolerance, max_length, material, **kwds)
        self.g_x = float(kwds.get('g_x', 0.0))
        self.g_y = float(kwds.get('g_y', 0.0))
        self.diameter = 0.0

    def _pack(self, rec, tables):
        rec['p'][:3] = (self.g_x, self.g_y, self.diameter)


class RectangularFace(Face):
    """cfaces.pyx:354-407; p = (length, width, offset, z_plane)."""
    params = ['length', 'width', 'offset']
    type_code = RECTANGULAR

    def __init__(self, owner=None, tolerance=0.0001, max_length=100, material=None, **kwds):
        super().__init__(owner, tolerance, max_length, material, **kwds)
        self.z_plane = float(kwds.get('z_plane', 0.0))
        self.width = float(kwds.get("width", 2.0))
        self.length = float(kwds.get("length", 5.0))
        self.offset = float(kwds.get("offset", 0.0))

    def _pack(self, rec, tables):
        rec['p'][:4] = (self.length, self.width, self.offset, self.z_plane)


class SphericalFace(Face):
    """cfaces.pyx:410-498; p = (diameter, curvature, z_height)."""
    params = ['diameter']
    type_code = SPHERICAL

    def __init__(self, owner=None, tolerance=0.0001, max_length=100, material=None, **kwds):
        super().__init__(owner, tolerance, max_length, material, **kwds)
        self.diameter = 0.0
        self.z_height = float(kwds.get('z_height', 0.0))
        self.curvature = float(kwds.get('curvature', 25.0))

    def _pack(self, rec, tables):
        rec['p'][:3] = (self.diameter, self.curvature, self.z_height)


class ShapedSphericalFace(ShapedFace):
    """cfaces.pyx:501-608; p = (curvature, z_height)."""
    type_code = SHAPED_SPHERICAL

    def __init__(self, owner=None, tolerance=0.0001, max_length=100, material=None, **kwds):
        super().__init__(owner, tolerance, max_length, material, **kwds)
        self.z_height = float(kwds.get('z_height', 0.0))
        self.curvature = float(kwds.get("curvature", 100.0))

    def _pack(self, rec, tables):
        rec['p'][:2] = (self.curvature, self.z_height)
        self._pack_shape(rec, tables)

    def eval_z_c(self, x, y):
        r2 = x * x + y * y
        c = self.curvature
        if c >= 0:
            return self.z_height + math.sqrt(c * c - r2) - c
        return self.z_height - math.sqrt(c * c - r2) - c


class ConicRevolutionFace(ShapedFace):
    """cfaces.pyx:1751-1837; p = (curvature, z_height, conic_const)."""
    type_code = CONIC

    def __init__(self, owner=None, tolerance=0.0001, max_length=100, material=None, **kwds):
        super().__init__(owner, tolerance, max_length, material, **kwds)
        self.z_height = float(kwds.get('z_height', 0.0))
        self.conic_const = float(kwds.get('conic_const', 0.0))
        self.curvature = float(kwds.get('curvature', 10.0))

    def _pack(self, rec, tables):
        rec['p'][:3] = (self.curvature, self.z_height, self.conic_const)
        self._pack_shape(rec, tables)


class AsphericFace(ShapedFace):
    """cfaces.pyx:1840-2025; p = (curvature, z_height, conic_const, A4..A16,
    atol, highest non-zero power of r^2, (-curvature)**3)."""
    type_code = ASPHERIC

    def __init__(self, owner=None, tolerance=0.0001, max_length=100, material=None, **kwds):
        super().__init__(owner, tolerance, max_length, material, **kwds)
        self.z_height = float(kwds.get('z_height', 0.0))
        self.conic_const = float(kwds.get('conic_const', 0.0))
        self.curvature = float(kwds.get('curvature', 25.0))
        for k in ("A4", "A6", "A8", "A10", "A12", "A14", "A16"):
            setattr(self, k, float(kwds.get(k, 0.0)))
        self.atol = float(kwds.get("atol", 1.0e-8))

    def _pack(self, rec, tables):
        coefs = [self.A4, self.A6, self.A8, self.A10, self.A12, self.A14, self.A16]
        kmax = 2
        for i, a in enumerate(coefs):
            if a != 0.0:
                kmax = i + 2
        R = -self.curvature
        rec['p'][:13] = [self.curvature, self.z_height, self.conic_const] + coefs + \
            [self.atol, float(kmax), math.pow(R, 3.0)]
        self._pack_shape(rec, tables)


class ExtendedPolynomialFace(ShapedFace):
    """cfaces.pyx:2128-2320.  Stores R = -curvature and beta = 1 + conic_const
    as the reference does (2141-2152); p = (R, beta, norm_radius, z_height,
    atol), aux = coefs (Nx x Ny)."""
    type_code = EXTPOLY

    def __init__(self, owner=None, tolerance=0.0001, max_length=100, material=None, **kwds):
        super().__init__(owner, tolerance, max_length, material, **kwds)
        self._R = 0.0
        self._beta = 1.0
        self.z_height = float(kwds.get('z_height', 0.0))
        self.conic_const = float(kwds.get('conic_const', 0.0))
        self.curvature = float(kwds.get('curvature', 0.0))
        self.nterms = float(kwds.get('nterms', 0.0))
        self.norm_radius = float(kwds.get('norm_radius', 100.0))
        self.coefs = kwds.get('coefs', np.array([[0.0]]))
        self.atol = float(kwds.get("atol", 1.0e-8))

    @property
    def curvature(self):
        return -self._R

    @curvature.setter
    def curvature(self, v):
        self._R = -float(v)

    @property
    def conic_const(self):
        return self._beta - 1

    @conic_const.setter
    def conic_const(self, v):
        self._beta = float(v) + 1.0

    @property
    def coefs(self):
        return self._coefs

    @coefs.setter
    def coefs(self, c):
        self._coefs = np.ascontiguousarray(c, dtype=np.double).reshape(np.shape(c))

    def _pack(self, rec, tables):
        c = self._coefs
        if c.ndim != 2 or c.shape[0] > 8 or c.shape[1] > 8:
            raise NotImplementedError("ExtendedPolynomialFace coefficients are limited to 8 x 8 on the device")
        rec['p'][:5] = (self._R, self._beta, self.norm_radius, self.z_height, self.atol)
        rec['aux'] = tables.add_aux(c.reshape(-1))
        rec['n_aux0'], rec['n_aux1'] = c.shape
        self._pack_shape(rec, tables)


class DistortionFace(ShapedFace):
    """cfaces.pyx:2323-2438; p = (accuracy,), base -> sub-face record."""
    type_code = DISTORTION

    def __init__(self, owner=None, tolerance=0.0001, max_length=100, material=None, **kwds):
        super().__init__(owner, tolerance, max_length, material, **kwds)
        face = kwds.get("base_face")
        self.base_face = face
        self.distortion = kwds.get("distortion")
        self.shape = kwds.get('shape', face.shape if face is not None else Shape())
        self.accuracy = float(kwds.get("accuracy", 1e-6))

    def _pack(self, rec, tables):
        if isinstance(self.base_face, DistortionFace):
            raise NotImplementedError("nested DistortionFace is not supported on the device")
        rec['p'][0] = self.accuracy
        rec['distortion'] = tables.add_distortion(self.distortion)
        rec['base'] = tables.add_subface(self.base_face)
        self._pack_shape(rec, tables)


class PolygonFace(Face):
    """cfaces.pyx:1077-1118; p = (z_plane,), aux = xy points."""
    type_code = POLYGON

    def __init__(self, owner=None, tolerance=0.0001, max_length=100, material=None, z_plane=0.0,
                 xy_points=((),), **kwds):
        super().__init__(owner, tolerance, max_length, material, **kwds)
        self.z_plane = float(z_plane)
        self.xy_points = xy_points

    @property
    def xy_points(self):
        return self._xy_points

    @xy_points.setter
    def xy_points(self, pts):
        self._xy_points = np.ascontiguousarray(pts, dtype=np.float64).reshape(-1, 2)

    def _pack(self, rec, tables):
        rec['p'][0] = self.z_plane
        rec['aux'] = tables.add_aux(self._xy_points.reshape(-1))
        rec['n_aux0'] = self._xy_points.shape[0]


class OrientedPolygonFace(Face):
    """cfaces.pyx:1121-1222; p = (origin, normal, x_axis, y_axis), aux = xy points."""
    type_code = ORIENTED_POLYGON

    def __init__(self, owner=None, tolerance=0.0001, max_length=100, material=None, **kwds):
        self._origin = (0.0, 0.0, 0.0)
        self._normal = (0.0, 0.0, 0.0)
        self._x_axis = (0.0, 0.0, 0.0)
        self._y_axis = (0.0, 0.0, 0.0)
        self._xy_points = np.zeros((0, 2))
        super().__init__(owner, tolerance, max_length, material, **kwds)
        for k in kwds:
            setattr(self, k, kwds[k])

    @property
    def origin(self):
        return self._origin

    @origin.setter
    def origin(self, v):
        self._origin = (float(v[0]), float(v[1]), float(v[2]))

    @property
    def normal(self):
        return self._normal

    @normal.setter
    def normal(self, v):
        self._normal = norm((float(v[0]), float(v[1]), float(v[2])))
        self._y_axis = cross(self._normal, self._x_axis)

    @property
    def x_axis(self):
        return self._x_axis

    @x_axis.setter
    def x_axis(self, v):
        self._x_axis = norm((float(v[0]), float(v[1]), float(v[2])))
        self._y_axis = cross(self._normal, self._x_axis)

    @property
    def xy_points(self):
        return np.asarray(self._xy_points).reshape(-1, 2)

    @xy_points.setter
    def xy_points(self, xy):
        a = np.asarray(xy).astype(np.double)
        if a.ndim != 2 or a.shape[1] != 2:
            raise ValueError("XY points must be an array with shape (N,2)")
        self._xy_points = a

    def compute_tangent(self, p):
        return self._x_axis

    def _pack(self, rec, tables):
        rec['p'][:12] = list(self._origin) + list(self._normal) + list(self._x_axis) + list(self._y_axis)
        rec['aux'] = tables.add_aux(np.ascontiguousarray(self._xy_points).reshape(-1))
        rec['n_aux0'] = self._xy_points.shape[0]


class OffAxisParabolicFace(Face):
    """cfaces.pyx:1224-1315: the paraboloid z + EFL/2 = (x^2 + y^2) / (2 EFL)
    cut by a circular aperture of `diameter` centred on x = EFL;
    p = (EFL, diameter, height).  The keywords EFL / diameter / height are
    accepted for convenience (the reference's owner sets the attributes)."""
    type_code = OFF_AXIS_PARABOLIC

    def __init__(self, owner=None, tolerance=0.0001, max_length=100, material=None, **kwds):
        super().__init__(owner, tolerance, max_length, material, **kwds)
        self.EFL = float(kwds.get("EFL", 0.0))
        self.diameter = float(kwds.get("diameter", 0.0))
        self.height = float(kwds.get("height", 0.0))

    def _pack(self, rec, tables):
        rec['p'][:3] = (self.EFL, self.diameter, self.height)


class EllipsoidalFace(Face):
    """cfaces.pyx:1318-1410: an ellipsoid of revolution about the x axis of
    its own frame (semi-axes major, minor), reached from the face-list frame by
    `transform` and back by `inverse_transform`, clipped to the open block
    x1 < x < x2, y1 < y < y2, z1 < z < z2 of the face-list frame.
    p = (major, minor, x1, x2, y1, y2, z1, z2); aux = trans (m, t), inv_trans (m, t)."""
    type_code = ELLIPSOIDAL

    def __init__(self, owner=None, tolerance=0.0001, max_length=100, material=None, **kwds):
        super().__init__(owner, tolerance, max_length, material, **kwds)
        self.major = float(kwds.get("major", 0.0))
        self.minor = float(kwds.get("minor", 0.0))
        for k in ("x1", "x2", "y1", "y2", "z1", "z2"):
            setattr(self, k, float(kwds.get(k, 0.0)))
        self.transform = Transform()
        self.inverse_transform = Transform()

    def update(self):
        """ellipsoids.py owner protocol (cfaces.pyx:1398-1405): ellipse_trans,
        axes and the X/Y/Z bounds are pulled when the owner provides them."""
        super().update()
        owner = self.owner
        if owner is None or not hasattr(owner, "ellipse_trans"):
            return
        self.sync_transform(owner.ellipse_trans)
        self.major, self.minor = owner.axes
        self.x1, self.x2 = owner.X_bounds
        self.y1, self.y2 = owner.Y_bounds
        self.z1, self.z2 = owner.Z_bounds

    def sync_transform(self, vtk_trans):
        """cfaces.pyx:1398-1410: copies a 4x4 affine map (anything with
        ``matrix.get_element(i, j)`` and ``linear_inverse``) into transform and
        inverse_transform."""
        def split(t):
            m = t.matrix
            return ([[m.get_element(i, j) for j in range(3)] for i in range(3)],
                    [m.get_element(i, 3) for i in range(3)])
        rot, dt = split(vtk_trans)
        self.transform = Transform(rotation=rot, translation=dt)
        rot, dt = split(vtk_trans.linear_inverse)
        self.inverse_transform = Transform(rotation=rot, translation=dt)

    def _pack(self, rec, tables):
        rec['p'][:8] = (self.major, self.minor, self.x1, self.x2, self.y1, self.y2, self.z1, self.z2)
        t, ti = self.transform, self.inverse_transform
        rec['aux'] = tables.add_aux(np.concatenate([np.ravel(t.rotation), t.translation,
                                                    np.ravel(ti.rotation), ti.translation]))
        rec['n_aux0'] = 24


class SaddleFace(ShapedFace):
    """cfaces.pyx:1413-1511: z = z_height + sqrt(6) curvature x y;
    p = (z_height, curvature)."""
    type_code = SADDLE
    params = []

    def __init__(self, owner=None, tolerance=0.0001, max_length=100, material=None, **kwds):
        super().__init__(owner, tolerance, max_length, material, **kwds)
        self.z_height = float(kwds.get("z_height", 0.0))
        self.curvature = float(kwds.get("curvature", 0.0))

    def _pack(self, rec, tables):
        rec['p'][:2] = (self.z_height, self.curvature)
        self._pack_shape(rec, tables)

    def eval_z_c(self, x, y):
        return math.sqrt(6) * self.curvature * x * y


class CylindericalFace(ShapedFace):
    """cfaces.pyx:1516-1602: a cylinder of `radius` with its axis along y,
    vertex at z_height; p = (z_height, radius)."""
    type_code = CYLINDRICAL
    params = []

    def __init__(self, owner=None, tolerance=0.0001, max_length=100, material=None, **kwds):
        super().__init__(owner, tolerance, max_length, material, **kwds)
        self.z_height = float(kwds.get("z_height", 0.0))
        self.radius = float(kwds.get("radius", 100.0))

    def _pack(self, rec, tables):
        rec['p'][:2] = (self.z_height, self.radius)
        self._pack_shape(rec, tables)

    def eval_z_c(self, x, y):
        R = self.radius
        if R >= 0:
            return self.z_height + math.sqrt(R * R - x * x) - R
        return self.z_height - math.sqrt(R * R - x * x) - R


class AxiconFace(ShapedFace):
    """cfaces.pyx:1605-1680: the cone z = z_height - gradient r;
    p = (z_height, gradient)."""
    type_code = AXICON

    def __init__(self, owner=None, tolerance=0.0001, max_length=100, material=None, **kwds):
        super().__init__(owner, tolerance, max_length, material, **kwds)
        self.z_height = float(kwds.get("z_height", 0.0))
        self.gradient = float(kwds.get("gradient", 0.0))

    def _pack(self, rec, tables):
        rec['p'][:2] = (self.z_height, self.gradient)
        self._pack_shape(rec, tables)

    def eval_z_c(self, x, y):
        return self.z_height - (self.gradient * math.sqrt(x * x + y * y))


def point_in_polygon(X, Y, point_list):
    """cfaces.pyx:1050-1075 (host predicate)."""
    pts = np.ascontiguousarray(point_list, dtype=np.float64)
    assert pts.shape[1] == 2
    size = pts.shape[0]
    ct = 0
    y1, x1 = pts[size - 1, 1], pts[size - 1, 0]
    for i in range(size):
        y2, x2 = pts[i, 1], pts[i, 0]
        with np.errstate(divide='ignore', invalid='ignore'):
            h = (Y - y1) / (y2 - y1)
        if 0 < h <= 1.0:
            x = x1 + h * (x2 - x1)
            if x > X:
                ct = not ct
        y1, x1 = y2, x2
    return bool(ct)
