"""Drop-in mirror of ``raypier.core.ctracer`` for the GB300 tracing path.

The reference module (raypier/core/ctracer.pyx) holds the ray record, the
RayCollection container, the Face / FaceList / InterfaceMaterial / Shape /
Distortion base classes and the per-generation entry point ``trace_segment``.
Here the same names and signatures are kept; the work of ``trace_segment``
runs in the sm_103a library behind ``include/rp_gb300.h``:

* ``RayCollection`` keeps its rays either as a host ``ray_dtype`` array or as a
  device structure-of-arrays buffer (or both), and copies between them only
  when the other side is asked for.  Generations produced by ``trace_segment``
  / ``trace_rays`` stay on the device until a property is read.
* ``trace_segment`` compiles the face lists into scene tables, traces one
  generation on the GPU and returns the children as a new device-resident
  RayCollection; like the reference it mutates the input's ``length`` and
  ``end_face_idx`` (ctracer.pyx:2086-2087, 1899-1903) and increments
  ``Face.count`` (2108).

There is no CPU fallback: without the CUDA library (or a GPU) the tracing
calls raise.
"""
from __future__ import annotations

import ctypes
import math
import sys
from typing import Optional

import numpy as np

from . import _native, runtime

# ctracer.pyx:45-60
ray_dtype = np.dtype([('origin', np.double, (3,)),
                      ('direction', np.double, (3,)),
                      ('normal', np.double, (3,)),
                      ('E_vector', np.double, (3,)),
                      ('refractive_index', np.complex128),
                      ('E1_amp', np.complex128),
                      ('E2_amp', np.complex128),
                      ('length', np.double),
                      ('phase', np.double),
                      ('accumulated_path', np.double),
                      ('wavelength_idx', np.uint32),
                      ('parent_idx', np.uint32),
                      ('end_face_idx', np.uint32),
                      ('ray_ident', np.uint32),
                      ('ray_type_id', np.uint32)])
assert ray_dtype.itemsize == 188

# ctracer.pyx:66-76
NPARA = 6
para_dtype = np.dtype([('origin', np.double, (3,)),
                       ('direction', np.double, (3,)),
                       ('normal', np.double, (3,)),
                       ('length', np.double)])
gausslet_dtype = np.dtype([('base_ray', ray_dtype),
                           ('para_rays', para_dtype, (NPARA,))])
assert gausslet_dtype.itemsize == 668

REFL_RAY = 1 << 0
GAUSSLET = 1 << 1
PARABASAL = 1 << 2
INF = float("inf")
root2 = math.sqrt(2.0)


def get_ray_size():
    """sizeof(ray_t) (ctracer.pyx:2399-2400)."""
    return ray_dtype.itemsize


# ---- vector helpers (ctracer.pyx:97-262, the Python-visible wrappers) ----------
def py_set_v(O):
    return (float(O[0]), float(O[1]), float(O[2]))


def sep(a, b):
    x, y, z = b[0] - a[0], b[1] - a[1], b[2] - a[2]
    return math.sqrt((x * x) + (y * y) + (z * z))


def invert(v):
    return (-v[0], -v[1], -v[2])


def multvv(a, b):
    return tuple(float(x) * float(y) for x, y in zip(a, b))


def multvs(a, b):
    return tuple(float(x) * b for x in a)


def addvv(a, b):
    return tuple(float(x) + float(y) for x, y in zip(a, b))


def addvs(a, b):
    return tuple(float(x) + b for x in a)


def subvv(a, b):
    return tuple(float(x) - float(y) for x, y in zip(a, b))


def subvs(a, b):
    return tuple(float(x) - b for x in a)


def mag(a):
    return math.sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2])


def mag_sq(a):
    return a[0] * a[0] + a[1] * a[1] + a[2] * a[2]


def dotprod(a, b):
    return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]


def cross(a, b):
    return (a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0])


def norm(a):
    m = math.sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2])
    return (a[0] / m, a[1] / m, a[2] / m)


# ---- Transform (ctracer.pyx:268-296) -----------------------------------------
class Transform:
    def __init__(self, rotation=((1, 0, 0), (0, 1, 0), (0, 0, 1)), translation=(0, 0, 0)):
        self.rotation = rotation
        self.translation = translation

    @property
    def rotation(self):
        return [list(map(float, r)) for r in self._rot]

    @rotation.setter
    def rotation(self, rot):
        self._rot = np.array(rot, dtype=np.float64).reshape(3, 3)

    @property
    def translation(self):
        return tuple(map(float, self._t))

    @translation.setter
    def translation(self, dt):
        self._t = np.array(dt, dtype=np.float64).reshape(3)


# ---- Ray (ctracer.pyx:396-676) -----------------------------------------------
class Ray:
    """A single ray record with the reference's attribute surface."""

    def __init__(self, **kwds):
        self.ray = np.zeros((), dtype=ray_dtype)
        self.max_length = 1000.0
        for k, v in kwds.items():
            setattr(self, k, v)

    def __repr__(self):
        return "Ray(o=%s, d=%s)" % (str(self.origin), str(self.direction))

    def _vec(name):
        def get(self):
            return tuple(float(x) for x in self.ray[name])

        def set_(self, v):
            self.ray[name] = (v[0], v[1], v[2])
        return property(get, set_)

    def _scalar(name, cast):
        def get(self):
            return cast(self.ray[name])

        def set_(self, v):
            self.ray[name] = v
        return property(get, set_)

    origin = _vec('origin')
    direction = _vec('direction')
    normal = _vec('normal')
    E_vector = _vec('E_vector')
    length = _scalar('length', float)
    phase = _scalar('phase', float)
    accumulated_path = _scalar('accumulated_path', float)
    wavelength_idx = _scalar('wavelength_idx', int)
    parent_idx = _scalar('parent_idx', int)
    end_face_idx = _scalar('end_face_idx', int)
    ray_ident = _scalar('ray_ident', int)
    ray_type_id = _scalar('ray_type_id', int)
    refractive_index = _scalar('refractive_index', complex)
    E1_amp = _scalar('E1_amp', complex)
    E2_amp = _scalar('E2_amp', complex)
    del _vec, _scalar

    @property
    def termination(self):
        length = self.max_length if self.length > self.max_length else self.length
        length = float(np.float32(length))
        o, d = self.origin, self.direction
        return tuple(o[i] + d[i] * length for i in range(3))

    @property
    def power(self):
        """ray_power_ (ctracer.pyx:1971-1978)"""
        e1, e2, n = self.E1_amp, self.E2_amp, self.refractive_index
        return (e1.real ** 2 + e1.imag ** 2) * n.real + (e2.real ** 2 + e2.imag ** 2) * n.real

    @property
    def amplitude(self):
        e1, e2 = self.E1_amp, self.E2_amp
        return math.sqrt(e1.real ** 2 + e1.imag ** 2 + e2.real ** 2 + e2.imag ** 2)

    @property
    def jones_vector(self):
        amp = self.amplitude
        return (self.E1_amp / amp, self.E2_amp / amp)

    @property
    def E_left(self):
        return (self.E1_amp + 1.0j * self.E2_amp) / math.sqrt(2)

    @property
    def E_right(self):
        return (self.E1_amp - 1.0j * self.E2_amp) / math.sqrt(2)

    @property
    def ellipticity(self):
        alpha, beta = self.jones_vector
        R = (alpha - 1j * beta) / root2
        L = (alpha + 1j * beta) / root2
        PR = R.real ** 2 + R.imag ** 2
        PL = L.real ** 2 + L.imag ** 2
        return (PR - PL) / (PR + PL)

    @property
    def major_minor_axes(self):
        d, E = self.direction, self.E_vector
        E2v = norm(cross(d, E))
        E1v = norm(cross(E2v, d))
        e1, e2 = self.E1_amp, self.E2_amp
        E1, E2 = abs(e1), abs(e2)
        phi1, phi2 = math.atan2(e1.imag, e1.real), math.atan2(e2.imag, e2.real)
        A = E1 * E1 * math.sin(2 * phi1) + E2 * E2 * math.sin(2 * phi2)
        B = E1 * E1 * math.cos(2 * phi1) + E2 * E2 * math.cos(2 * phi2)
        m = math.sqrt(A * A + B * B)
        t1 = math.atan((B - m) / A)
        t2 = math.atan((B + m) / A)
        ax1 = addvv(multvs(E1v, E1 * math.cos(phi1 + t1)), multvs(E2v, E2 * math.cos(phi2 + t1)))
        ax2 = addvv(multvs(E1v, E1 * math.cos(phi1 + t2)), multvs(E2v, E2 * math.cos(phi2 + t2)))
        return (ax1, ax2)

    def project_E(self, *axis):
        """Rotate the E_vector onto the given axis (ctracer.pyx:646-676)."""
        E1, E2 = self.E1_amp, self.E2_amp
        d = self.direction
        E_vector = norm(cross(cross(d, self.E_vector), d))
        E2bar = norm(cross(d, axis))
        E_vector2 = norm(cross(E2bar, d))
        A = dotprod(E_vector, E_vector2)
        B = dotprod(E_vector, E2bar)
        self.E1_amp = complex(-(E2.real * B - E1.real * A), -(E2.imag * B - E1.imag * A))
        self.E2_amp = complex(E2.real * A + E1.real * B, E2.imag * A + E1.imag * B)
        self.E_vector = E_vector2


# ---- RayCollection (ctracer.pyx:973-1154) ---------------------------------------
class RayCollection:
    """A growable collection of rays, on the host, the device, or both.

    Host side: a ``ray_dtype`` array with spare capacity (``add_ray`` doubles
    it as the reference's ``add_ray_c`` does).  Device side: a structure-of-
    arrays buffer owned by the GPU context.  Whichever side was written last
    is authoritative; the other is refreshed on demand.
    """

    def __init__(self, max_size=0):
        self._host = np.zeros(max(int(max_size), 0), dtype=ray_dtype)
        self._n = 0
        self._dev: Optional[runtime.DeviceRays] = None
        self._host_ok = True
        self._dev_ok = False
        self._parent = None
        self._wavelengths = np.zeros(0, dtype=np.double)
        self._neighbours = None
        self._nb_source = None

    # -- residency ------------------------------------------------------------
    @classmethod
    def _from_device(cls, dev: "runtime.DeviceRays", parent=None):
        rc = cls(0)
        rc._dev = dev
        rc._n = dev.count()
        rc._host_ok = False
        rc._dev_ok = True
        if parent is not None:
            rc.parent = parent
        return rc

    def _sync_host(self):
        if not self._host_ok:
            if self._host.shape[0] < self._n:
                self._host = np.zeros(self._n, dtype=ray_dtype)
            self._dev.download(self._host, self._n)
            self._host_ok = True

    def _device(self, ctx) -> "runtime.DeviceRays":
        """Device buffer holding these rays (uploaded if the host copy is newer)."""
        if self._dev_ok and self._dev is not None and self._dev.ctx is ctx:
            return self._dev
        self._sync_host()
        dev = runtime.DeviceRays(ctx, max(self._n, 1))
        dev.upload(self._host[:self._n])
        self._dev = dev
        self._dev_ok = True
        return dev

    def _mark_host_written(self):
        self._host_ok = True
        self._dev_ok = False

    def _mark_device_written(self):
        self._dev_ok = True
        self._host_ok = False

    # -- container API ----------------------------------------------------------
    @property
    def n_rays(self):
        return self._n

    @property
    def max_size(self):
        return max(self._host.shape[0], self._n)

    def __len__(self):
        return self._n

    def __getitem__(self, idx):
        if idx >= self._n:
            raise IndexError("Requested index %d from a size %d array" % (idx, self._n))
        self._sync_host()
        r = Ray()
        r.ray[()] = self._host[idx]
        return r

    def __setitem__(self, idx, r):
        if idx >= self._n:
            raise IndexError("Attempting to set index %d from a size %d array" % (idx, self._n))
        self._sync_host()
        self._host[idx] = r.ray
        self._mark_host_written()

    def __iter__(self):
        for i in range(self._n):
            yield self[i]

    def get_ray_list(self):
        return [self[i] for i in range(self._n)]

    def _grow(self):
        cap = self._host.shape[0]
        new = np.zeros(1 if cap == 0 else 2 * cap, dtype=ray_dtype)
        new[:cap] = self._host
        self._host = new

    def add_ray(self, r):
        self._sync_host()
        if self._n == self._host.shape[0]:
            self._grow()
        self._host[self._n] = r.ray
        self._n += 1
        self._mark_host_written()

    def add_ray_list(self, rays):
        for i, r in enumerate(rays):
            if not isinstance(r, Ray):
                raise TypeError("ray list contains non-Ray instance at index %d" % i)
        for r in rays:
            self.add_ray(r)

    def clear_ray_list(self):
        self._n = 0
        self._mark_host_written()

    def reset_length(self, max_length=INF):
        self._sync_host()
        self._host['length'][:self._n] = max_length
        self._mark_host_written()

    def copy_as_array(self):
        self._sync_host()
        return self._host[:self._n].copy()

    @classmethod
    def from_array(cls, data):
        data = np.ascontiguousarray(data)
        assert data.dtype == ray_dtype
        rc = cls(data.shape[0])
        rc._host[:] = data
        rc._n = data.shape[0]
        return rc

    @property
    def base_rays(self):
        return self

    @property
    def wavelengths(self):
        return np.asarray(self._wavelengths)

    @wavelengths.setter
    def wavelengths(self, wl_list):
        self._wavelengths = np.ascontiguousarray(wl_list, dtype=np.double)

    @property
    def parent(self):
        return self._parent

    @parent.setter
    def parent(self, rc):
        self._parent = rc
        self._neighbours = None
        self._wavelengths = rc._wavelengths

    @property
    def neighbours(self):
        """Indices of each ray's neighbours (n, k), -1 where there is none.  A
        child generation derives them from its parent's through parent_idx and
        the reflected / transmitted type (ctracer.pyx:1084-1131)."""
        if self._parent is None:
            return None if self._neighbours is None else np.asarray(self._neighbours)
        pnb = self._parent.neighbours
        if pnb is None:
            return None if self._neighbours is None else np.asarray(self._neighbours)
        if self._neighbours is None or self._nb_source is not pnb:
            self._neighbours = self._eval_neighbours(np.asarray(pnb))
            self._nb_source = pnb
        return np.asarray(self._neighbours)

    @neighbours.setter
    def neighbours(self, nb):
        self._neighbours = np.asarray(nb, dtype=np.int32)
        self._nb_source = None

    def _eval_neighbours(self, pnb):
        self._sync_host()
        h = self._host[:self._n]
        rtype = (h['ray_type_id'] & REFL_RAY).astype(np.int64)
        pidx = h['parent_idx'].astype(np.int64)
        rmap = np.full((self._parent.n_rays, 2), -1, dtype=np.int32)
        for i in range(self._n):   # later children of one parent and type win, as in the reference
            rmap[pidx[i], rtype[i]] = i
        cand = pnb[pidx]
        nb = np.where(cand >= 0, rmap[np.maximum(cand, 0), rtype[:, None]], -1).astype(np.int32)
        return nb

    # -- field views (ctracer.pyx:755-969) ----------------------------------------
    def _field(self, name):
        self._sync_host()
        return self._host[name][:self._n].copy()

    origin = property(lambda self: self._field('origin'))
    direction = property(lambda self: self._field('direction'))
    normal = property(lambda self: self._field('normal'))
    E_vector = property(lambda self: self._field('E_vector'))
    refractive_index = property(lambda self: self._field('refractive_index'))
    E1_amp = property(lambda self: self._field('E1_amp'))
    E2_amp = property(lambda self: self._field('E2_amp'))
    length = property(lambda self: self._field('length'))
    phase = property(lambda self: self._field('phase'))
    accumulated_path = property(lambda self: self._field('accumulated_path'))
    wavelength_idx = property(lambda self: self._field('wavelength_idx'))
    parent_idx = property(lambda self: self._field('parent_idx'))
    end_face_idx = property(lambda self: self._field('end_face_idx'))
    ray_ident = property(lambda self: self._field('ray_ident'))
    ray_type_id = property(lambda self: self._field('ray_type_id'))

    @property
    def termination(self):
        self._sync_host()
        h = self._host[:self._n]
        return h['origin'] + h['direction'] * h['length'][:, None]


# ---- Gausslets (ctracer.pyx:315-394, 1157-1570) ------------------------------------
class ParabasalRay:
    """One parabasal ray (ctracer.pyx:332-394)."""

    def __init__(self, **kwds):
        self.ray = np.zeros((), dtype=para_dtype)
        self.max_length = 1000.0
        for k, v in kwds.items():
            setattr(self, k, v)

    def __repr__(self):
        return "Parabasal Ray(o=%s, d=%s)" % (str(self.origin), str(self.direction))

    def _vec(name):
        def get(self):
            return tuple(float(x) for x in self.ray[name])

        def set_(self, v):
            self.ray[name] = (v[0], v[1], v[2])
        return property(get, set_)

    origin = _vec('origin')
    direction = _vec('direction')
    normal = _vec('normal')

    @property
    def length(self):
        return float(self.ray['length'])

    @length.setter
    def length(self, v):
        self.ray['length'] = v

    @property
    def termination(self):
        length = min(self.length, self.max_length)
        length = float(np.float32(length))  # the reference holds it in a C float
        o, d = self.origin, self.direction
        return tuple(o[k] + d[k] * length for k in range(3))


class Gausslet:
    """A base ray with six parabasal rays (ctracer.pyx:700-752)."""

    def __init__(self, **kwds):
        self.gausslet = np.zeros((), dtype=gausslet_dtype)
        for k, v in kwds.items():
            setattr(self, k, v)

    @property
    def base_ray(self):
        r = Ray()
        r.ray[()] = self.gausslet['base_ray']
        return r

    @base_ray.setter
    def base_ray(self, r):
        self.gausslet['base_ray'] = r.ray

    @property
    def parabasal_rays(self):
        out = []
        for j in range(NPARA):
            p = ParabasalRay()
            p.ray[()] = self.gausslet['para_rays'][j]
            out.append(p)
        return tuple(out)

    @parabasal_rays.setter
    def parabasal_rays(self, rays):
        for j, p in enumerate(rays):
            self.gausslet['para_rays'][j] = p.ray


class GaussletCollection:
    """A growable collection of gausslets (ctracer.pyx:1185-1570), resident on
    the host, the device, or both, like RayCollection."""

    def __init__(self, max_size=0):
        self._host = np.zeros(max(int(max_size), 0), dtype=gausslet_dtype)
        self._n = 0
        self._dev = None
        self._host_ok = True
        self._dev_ok = False
        self._parent = None
        self._wavelengths = np.zeros(0, dtype=np.double)

    # -- residency --------------------------------------------------------------
    @classmethod
    def _from_device(cls, dev, parent=None):
        gc = cls(0)
        gc._dev = dev
        gc._n = dev.count()
        gc._host_ok = False
        gc._dev_ok = True
        if parent is not None:
            gc.parent = parent
        return gc

    def _sync_host(self):
        if not self._host_ok:
            if self._host.shape[0] < self._n:
                self._host = np.zeros(self._n, dtype=gausslet_dtype)
            self._dev.download(self._host, self._n)
            self._host_ok = True

    def _device(self, ctx):
        if self._dev_ok and self._dev is not None and self._dev.ctx is ctx:
            return self._dev
        self._sync_host()
        dev = runtime.DeviceGausslets(ctx, max(self._n, 1))
        dev.upload(self._host[:self._n])
        self._dev = dev
        self._dev_ok = True
        return dev

    def _mark_host_written(self):
        self._host_ok = True
        self._dev_ok = False

    def _mark_device_written(self):
        self._dev_ok = True
        self._host_ok = False

    # -- container API ------------------------------------------------------------
    @property
    def n_rays(self):
        return self._n

    @property
    def max_size(self):
        return max(self._host.shape[0], self._n)

    def __len__(self):
        return self._n

    def __getitem__(self, idx):
        if idx >= self._n:
            raise IndexError("Requested index %d from a size %d array" % (idx, self._n))
        self._sync_host()
        g = Gausslet()
        g.gausslet[()] = self._host[idx]
        return g

    def __setitem__(self, idx, g):
        if idx >= self._n:
            raise IndexError("Attempting to set index %d from a size %d array" % (idx, self._n))
        self._sync_host()
        self._host[idx] = g.gausslet
        self._mark_host_written()

    def __iter__(self):
        for i in range(self._n):
            yield self[i]

    def get_gausslet_list(self):
        return [self[i] for i in range(self._n)]

    def add_gausslet(self, g):
        self._sync_host()
        if self._n == self._host.shape[0]:
            cap = self._host.shape[0]
            new = np.zeros(1 if cap == 0 else 2 * cap, dtype=gausslet_dtype)
            new[:cap] = self._host
            self._host = new
        self._host[self._n] = g.gausslet
        self._n += 1
        self._mark_host_written()

    def add_gausslet_list(self, rays):
        for i, r in enumerate(rays):
            if not isinstance(r, Gausslet):
                raise TypeError("ray list contains non-Gausslet instance at index %d" % i)
        for r in rays:
            self.add_gausslet(r)

    def clear_ray_list(self):
        self._n = 0
        self._mark_host_written()

    def reset_length(self, max_length=INF):
        """ctracer.pyx:1224-1235: base and parabasal lengths."""
        self._sync_host()
        self._host['base_ray']['length'][:self._n] = max_length
        self._host['para_rays']['length'][:self._n] = max_length
        self._mark_host_written()

    def copy_as_array(self):
        self._sync_host()
        return self._host[:self._n].copy()

    def extend(self, gc):
        arr = gc.copy_as_array()
        self._sync_host()
        if self._n + arr.shape[0] > self._host.shape[0]:
            new = np.zeros(self._n * 2 + arr.shape[0], dtype=gausslet_dtype)
            new[:self._n] = self._host[:self._n]
            self._host = new
        self._host[self._n:self._n + arr.shape[0]] = arr
        self._n += arr.shape[0]
        self._mark_host_written()

    @classmethod
    def from_array(cls, data):
        data = np.ascontiguousarray(data)
        if data.dtype != gausslet_dtype:
            raise ValueError("Array must have gausslet_dtype dtype")
        gc = cls(data.shape[0])
        gc._host[:] = data
        gc._n = data.shape[0]
        return gc

    @classmethod
    def from_rays(cls, data):
        """ctracer.pyx:1320-1343: every parabasal ray starts as a copy of its base ray."""
        data = np.ascontiguousarray(data)
        if data.dtype != ray_dtype:
            raise ValueError("Array must have gausslet_dtype dtype")
        gc = cls(data.shape[0])
        h = gc._host
        h['base_ray'] = data
        for f in ('origin', 'direction', 'normal'):
            h['para_rays'][f] = data[f][:, None, :]
        h['para_rays']['length'] = data['length'][:, None]
        gc._n = data.shape[0]
        return gc

    @property
    def base_rays(self):
        """The base rays as a RayCollection copy (GaussletBaseRayView.copy_as_array)."""
        return RayCollection.from_array(self.copy_as_array()['base_ray'])

    @property
    def wavelengths(self):
        return np.asarray(self._wavelengths)

    @wavelengths.setter
    def wavelengths(self, wl_list):
        self._wavelengths = np.ascontiguousarray(wl_list, dtype=np.double)

    @property
    def parent(self):
        return self._parent

    @parent.setter
    def parent(self, gc):
        self._parent = gc
        self._wavelengths = gc._wavelengths

    def _para(self, name):
        self._sync_host()
        return self._host['para_rays'][name][:self._n].copy()

    para_origin = property(lambda self: self._para('origin'))
    para_direction = property(lambda self: self._para('direction'))
    para_normal = property(lambda self: self._para('normal'))
    para_length = property(lambda self: self._para('length'))

    @property
    def total_power(self):
        """ctracer.pyx:1482-1496: the sum of (|E1|^2 + |E2|^2) Re(n) over the
        base rays, reduced on the device."""
        if self._n == 0:
            return 0.0
        ctx = runtime.get_context()
        dev = self._device(ctx)
        out = ctypes.c_double()
        _native.check(ctx.lib.rp_gausslets_total_power(dev.handle, ctypes.byref(out)), "rp_gausslets_total_power")
        return out.value

    def scale_amplitude(self, scale):
        self._sync_host()
        self._host['base_ray']['E1_amp'][:self._n] *= scale
        self._host['base_ray']['E2_amp'][:self._n] *= scale
        self._mark_host_written()

    def project_to_plane(self, origin, direction):
        """ctracer.pyx:1397-1420: move every base and parabasal ray to the
        plane through `origin` with normal `direction`."""
        self._sync_host()
        o = np.asarray(origin, dtype=np.double)
        d = np.asarray(norm(tuple(float(x) for x in direction)))
        b = self._host['base_ray'][:self._n]
        a = ((o - b['origin']) @ d) / (b['direction'] @ d)
        b['origin'] = b['origin'] + b['direction'] * a[:, None]
        b['accumulated_path'] = b['accumulated_path'] + b['refractive_index'].real * a
        self._host['base_ray'][:self._n] = b
        p = self._host['para_rays'][:self._n]
        a = ((o - p['origin']) @ d) / (p['direction'] @ d)
        p['origin'] = p['origin'] + p['direction'] * a[..., None]
        self._host['para_rays'][:self._n] = p
        self._mark_host_written()

    def config_parabasal_rays(self, wavelength_list, radius, working_dist):
        """ctracer.pyx:1430-1476: parabasal rays of a circular Gaussian mode of
        1/e^2 waist `radius` (mm) whose waist lies `working_dist` from the base
        ray's origin, set on the device for every gausslet."""
        if self._n == 0:
            return
        wl = np.ascontiguousarray(wavelength_list, dtype=np.double)
        ctx = runtime.get_context()
        dev = self._device(ctx)
        _native.check(ctx.lib.rp_gausslets_config_parabasal(dev.handle, wl.ctypes.data if wl.size else None,
                                                            wl.shape[0], float(radius), float(working_dist)),
                      "rp_gausslets_config_parabasal")
        self._mark_device_written()


# ---- plugin base classes ---------------------------------------------------------
class InterfaceMaterial:
    """Base material (ctracer.pyx:1573-1655): generates no child rays."""

    type_code = 0

    def __init__(self, **kwds):
        self._wavelengths = np.zeros(0, dtype=np.double)

    @property
    def wavelengths(self):
        return self._wavelengths

    @wavelengths.setter
    def wavelengths(self, wl):
        self._wavelengths = np.asarray(wl, dtype=np.double)
        self.on_set_wavelengths()

    def on_set_wavelengths(self):
        pass

    def is_decomp_material(self):
        return False

    def eval_child_ray(self, old_ray, ray_idx, point, normal, tangent, new_rays):
        """Evaluates this material for one ray on the GPU and appends the
        children to ``new_rays`` (ctracer.pyx:1620-1632)."""
        from . import unitcalls
        for child in unitcalls.eval_child_rays(self, [old_ray], ray_idx, [point], [normal], [tangent])[0]:
            new_rays.add_ray(child)


class Shape:
    """Base shape: every point is inside (ctracer.pyx:1653-1658)."""

    def point_inside(self, x, y):
        return True

    def _emit(self, ops, aux):
        ops.append((1, 0, 0, 0.0, 0.0, 0.0, 0.0))


class Distortion:
    """Base distortion: zero sag (ctracer.pyx:1673-1729)."""

    def z_offset_and_gradient(self, x, y):
        x = np.asarray(x, dtype=np.double)
        y = np.asarray(y, dtype=np.double)
        if len(y) != len(x):
            raise ValueError("Both x and y must have the same length")
        return np.zeros((len(x), 3))

    def z_offset(self, x, y):
        x = np.asarray(x, dtype=np.double)
        if len(np.asarray(y)) != len(x):
            raise ValueError("Both x and y must have the same length")
        return np.zeros(len(x))


class Face:
    """Base face (ctracer.pyx:1732-1811).  Subclasses in ``cfaces`` set
    ``type_code`` and pack their parameters; the base face is never hit."""

    params = []
    type_code = 0

    def __init__(self, owner=None, tolerance=0.0001, max_length=100, material=None, **kwds):
        self.name = "base Face class"
        self.tolerance = float(tolerance)
        self.owner = owner
        self.max_length = max_length
        if isinstance(material, InterfaceMaterial):
            self.material = material
        else:
            from .cmaterials import PECMaterial
            self.material = PECMaterial()
        self.invert_normal = int(kwds.get('invert_normal', 0))
        self.idx = 0
        self.count = 0

    def update(self):
        """Pull ``params`` from the owner (ctracer.pyx:1761-1767)."""
        for name in self.params:
            setattr(self, name, getattr(self.owner, name))

    def _pack(self, rec, tables):
        """Fill the type-specific part of an rp_face record."""

    def intersect(self, p1, p2, is_base_ray):
        """Distance to this face along p1->p2 in local coordinates, evaluated on
        the GPU (Face.intersect, ctracer.pyx:1769-1777)."""
        from . import unitcalls
        return float(unitcalls.face_intersect(self, [p1], [p2], is_base_ray)[0])

    def compute_normal(self, p):
        from . import unitcalls
        return tuple(unitcalls.face_normal(self, [p])[0])

    def compute_tangent(self, p):
        return (1.0, 0.0, 0.0)


class FaceList:
    """A group of faces sharing one transform (ctracer.pyx:1814-1964)."""

    def __init__(self, owner=None):
        self.transform = Transform()
        self.inverse_transform = Transform()
        self.owner = owner
        self.faces = []

    def sync_transforms(self):
        """Take the owner's transform (a VTK-style matrix) if it has one;
        otherwise keep the preset transforms, as the reference does
        (ctracer.pyx:1820-1837).  The reference prints "NO OWNER" on every
        call; here the notice goes to stderr once per face list, so that
        stdout stays machine-readable and repeated traces stay quiet."""
        try:
            trans = self.owner.transform
        except AttributeError:
            if not getattr(self, "_no_owner_noted", False):
                print("NO OWNER", self.owner, file=sys.stderr)
                self._no_owner_noted = True
            return
        m = trans.matrix
        rot = [[m.get_element(i, j) for j in range(3)] for i in range(3)]
        dt = [m.get_element(i, 3) for i in range(3)]
        self.transform = Transform(rotation=rot, translation=dt)
        m = trans.linear_inverse.matrix
        rot = [[m.get_element(i, j) for j in range(3)] for i in range(3)]
        dt = [m.get_element(i, 3) for i in range(3)]
        self.inverse_transform = Transform(rotation=rot, translation=dt)

    def __getitem__(self, idx):
        return self.faces[idx]


# ---- entry points -------------------------------------------------------------------
def trace_segment(rays, face_sets, all_faces, max_length=100, decomp_faces=()):
    """Trace one generation on the GPU (ctracer.pyx:2173-2182 -> 2062-2118).

    Returns a new RayCollection of children (device-resident until read); the
    input's ``length`` / ``end_face_idx`` are updated and every hit face's
    ``count`` is incremented.
    """
    for fs in face_sets:
        fs.sync_transforms()
    from .tracer import _trace_generation
    return _trace_generation(rays, list(face_sets), list(all_faces), max_length)


def trace_one_face_segment(rays, face_set, face_idx, all_faces, max_length=100, decomp_faces=()):
    """Sequential variant: only ``face_set.faces[face_idx]`` is tested
    (ctracer.pyx:2184-2191 -> 2121-2170)."""
    face_set.sync_transforms()
    from .tracer import _trace_generation
    return _trace_generation(rays, [face_set], list(all_faces), max_length, one_face=(0, face_idx))


def trace_gausslet(rays, face_sets, all_faces, max_length=100, decomp_faces=()):
    """One Gausslet generation on the GPU (ctracer.pyx:2193-2202 -> 2214-2282)."""
    for fs in face_sets:
        fs.sync_transforms()
    from .tracer import _trace_gausslet_generation
    return _trace_gausslet_generation(rays, list(face_sets), list(all_faces), max_length,
                                      decomp_faces=list(decomp_faces))


def trace_one_face_gausslet(rays, face_set, face_idx, all_faces, max_length=100, decomp_faces=()):
    """Sequential Gausslet variant (ctracer.pyx:2204-2211 -> 2285-2350)."""
    face_set.sync_transforms()
    from .tracer import _trace_gausslet_generation
    return _trace_gausslet_generation(rays, [face_set], list(all_faces), max_length, one_face=(0, face_idx),
                                      decomp_faces=list(decomp_faces))


def _select(face_set, ray_col_list, gausslets):
    from .scene import compile_scene
    ctx = runtime.get_context()
    if hasattr(face_set, "sync_transforms"):
        face_set.sync_transforms()
    tables = compile_scene([face_set])
    scene = runtime.DeviceScene(ctx, tables, np.zeros(0))  # no material is evaluated here
    wl_list, parts, offset = [], [], 0
    dtype = gausslet_dtype if gausslets else ray_dtype
    for rc in ray_col_list:
        wl_list.append(np.asarray(rc.wavelengths, dtype=np.double))
        dev = rc._device(ctx)
        if gausslets:
            out = runtime.DeviceGausslets(ctx, max(rc.n_rays, 1))
            st = ctx.lib.rp_select_gausslet_intersections(ctx.handle, scene.handle, 0, dev.handle, out.handle, offset)
        else:
            out = runtime.DeviceRays(ctx, max(rc.n_rays, 1))
            st = ctx.lib.rp_select_intersections(ctx.handle, scene.handle, 0, dev.handle, out.handle, offset)
        from . import _native
        _native.check(st, "rp_select_intersections")
        n = out.count()
        host = np.zeros(n, dtype=dtype)
        out.download(host, n)
        out.free()
        parts.append(host)
        offset += len(rc.wavelengths)
    recs = np.concatenate(parts) if parts else np.zeros(0, dtype=dtype)
    reduced, inverse = np.unique(np.concatenate(wl_list) if wl_list else np.zeros(0), return_inverse=True)
    base = recs['base_ray'] if gausslets else recs
    base['wavelength_idx'] = inverse.reshape(-1)[base['wavelength_idx']]
    if gausslets:
        recs['base_ray'] = base
    out_col = (GaussletCollection if gausslets else RayCollection).from_array(recs)
    out_col.wavelengths = reduced
    return out_col


def select_ray_intersections(face_set, ray_col_list):
    """The rays of the traced collections that meet a face of `face_set`, with
    their length cut to the nearest such face (ctracer.pyx:1981-2015).  The
    intersections run on the GPU; the wavelength lists of the collections are
    merged onto their unique values, as in the reference."""
    return _select(face_set, list(ray_col_list), gausslets=False)


def select_gausslet_intersections(face_set, ray_col_list):
    """select_ray_intersections for GaussletCollections, by their base rays
    (ctracer.pyx:2018-2058)."""
    return _select(face_set, list(ray_col_list), gausslets=True)
