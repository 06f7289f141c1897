"""2-D aperture shapes, mirroring ``raypier.core.cshapes`` (cshapes.pyx).

A shape is compiled into a short postfix program of ``rp_shape_op`` records
(include/rp_gb300.h) that the device evaluates; ``point_inside`` on the host
evaluates the same program in Python (it is a predicate on two numbers, used
by callers that build scenes, not on the tracing path).
"""
from __future__ import annotations

import math

import numpy as np

from .ctracer import Shape

OP_END, OP_TRUE, OP_CIRCLE, OP_RECT, OP_POLYGON, OP_AND, OP_OR, OP_XOR, OP_NOT = range(9)


class LogicalOpShape(Shape):
    def __and__(self, other):
        return BooleanAND(self, other)

    def __or__(self, other):
        return BooleanOR(self, other)

    def __xor__(self, other):
        return BooleanXOR(self, other)

    def __invert__(self):
        return InvertShape(self)


class InvertShape(LogicalOpShape):
    """cshapes.pyx:30-36"""

    def __init__(self, shape):
        self.shape = shape

    def point_inside(self, x, y):
        return bool(1 & (~int(self.shape.point_inside(x, y))))

    def _emit(self, ops, aux):
        self.shape._emit(ops, aux)
        ops.append((OP_NOT, 0, 0, 0.0, 0.0, 0.0, 0.0))


class BooleanShape(LogicalOpShape):
    def __init__(self, shape1, shape2):
        self.shape1 = shape1
        self.shape2 = shape2

    _op = None

    def _emit(self, ops, aux):
        self.shape1._emit(ops, aux)
        self.shape2._emit(ops, aux)
        ops.append((self._op, 0, 0, 0.0, 0.0, 0.0, 0.0))


class BooleanAND(BooleanShape):
    """cshapes.pyx:48-50"""
    _op = OP_AND

    def point_inside(self, x, y):
        return bool(int(self.shape1.point_inside(x, y)) & int(self.shape2.point_inside(x, y)))


class BooleanOR(BooleanShape):
    """cshapes.pyx:53-55"""
    _op = OP_OR

    def point_inside(self, x, y):
        return bool(int(self.shape1.point_inside(x, y)) | int(self.shape2.point_inside(x, y)))


class BooleanXOR(BooleanShape):
    """cshapes.pyx:58-60"""
    _op = OP_XOR

    def point_inside(self, x, y):
        return bool(int(self.shape1.point_inside(x, y)) ^ int(self.shape2.point_inside(x, y)))


class BasicShape(LogicalOpShape):
    """cshapes.pyx:63-97"""

    def __init__(self, **kwds):
        if "centre" in kwds:
            self.centre = kwds["centre"]
        else:
            self.centre_x = float(kwds.get("centre_x", 0.0))
            self.centre_y = float(kwds.get("centre_y", 0.0))

    @property
    def centre(self):
        return (self.centre_x, self.centre_y)

    @centre.setter
    def centre(self, v):
        self.centre_x = float(v[0])
        self.centre_y = float(v[1])


class CircleShape(BasicShape):
    """cshapes.pyx:102-116 (strict ``<`` on the squared radius)."""

    def __init__(self, **kwds):
        super().__init__(**kwds)
        self.radius = float(kwds.get("radius", 1.0))

    def point_inside(self, x, y):
        dx = x - self.centre_x
        dy = y - self.centre_y
        return (dx * dx) + (dy * dy) < (self.radius * self.radius)

    def _emit(self, ops, aux):
        ops.append((OP_CIRCLE, 0, 0, self.centre_x, self.centre_y, self.radius, 0.0))


class RectangleShape(BasicShape):
    """cshapes.pyx:119-136"""

    def __init__(self, **kwds):
        super().__init__(**kwds)
        self.width = float(kwds.get("width", 5.0))
        self.height = float(kwds.get("height", 7.0))

    def point_inside(self, x, y):
        dx = x - self.centre_x
        dy = y - self.centre_y
        return (2 * math.fabs(dx) < self.width) and (2 * math.fabs(dy)) < self.height

    def _emit(self, ops, aux):
        ops.append((OP_RECT, 0, 0, self.centre_x, self.centre_y, self.width, self.height))


class PolygonShape(BasicShape):
    """cshapes.pyx:139-168 (crossing test on the polygon's edges)."""

    def __init__(self, **kwds):
        super().__init__(**kwds)
        self._coordinates = None
        if "coordinates" in kwds:
            self.coordinates = kwds["coordinates"]

    @property
    def coordinates(self):
        return self._coordinates

    @coordinates.setter
    def coordinates(self, val):
        self._coordinates = np.ascontiguousarray(val, dtype=np.float64).reshape(-1, 2)

    def point_inside(self, X, Y):
        pts = self._coordinates
        size = pts.shape[0]
        ct = 0
        y1, x1 = pts[size - 1, 1], pts[size - 1, 0]
        for i in range(size):
            y2, x2 = pts[i, 1], pts[i, 0]
            if (y1 <= Y < y2) or (y2 <= Y < y1):
                if (x1 + (Y - y1) * (x2 - x1) / (y2 - y1)) > X:
                    ct = not ct
            y1, x1 = y2, x2
        return bool(ct)

    def _emit(self, ops, aux):
        off = len(aux)
        aux.extend(self._coordinates.reshape(-1).tolist())
        ops.append((OP_POLYGON, off, self._coordinates.shape[0], 0.0, 0.0, 0.0, 0.0))
