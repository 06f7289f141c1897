"""Scene compiler: FaceList / Face / material / shape / distortion objects ->
the plain tables of include/rp_gb300.h.

The reference reaches every face, material, shape and distortion through
Cython virtual calls at trace time (ctracer.pyx:1882-1904, 2110-2117).  The
GPU path instead needs them as POD records: this module walks the objects
once per trace call and packs them.  Objects of a type the device does not
implement raise ``NotImplementedError`` here -- there is no CPU fallback.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _native
from .ctracer import Face, InterfaceMaterial, Shape


def _check_type(obj, kind):
    """Type tag of a face / material / distortion object.  A subclass that does
    not declare its own device type (e.g. a user's Cython-level subclass of
    Face or InterfaceMaterial in the reference) has no GPU implementation."""
    t = getattr(type(obj), "type_code", None)
    if not t or not hasattr(obj, "_pack"):
        raise NotImplementedError(f"{kind} type {type(obj).__name__} is not implemented on the GPU path")
    return t


class SceneTables:
    """Packed scene tables plus the objects they came from."""

    def __init__(self):
        self._lists = []
        self._faces = []           # rp_face records (numpy void scalars)
        self.face_objects = []     # record -> Face
        self._materials = []
        self.material_objects = []  # material index -> InterfaceMaterial
        self._mat_index = {}
        self._shape_ops = []
        self._shape_index = {}
        self._dists = []
        self._dist_index = {}
        self._disps = []
        self._disp_index = {}
        self._aux = []
        self._pending_sub = []     # (record index, face) of DistortionFace base faces
        self.n_faces = 0

    # -- adders used by the _pack methods ---------------------------------------
    def add_aux(self, values) -> int:
        off = len(self._aux)
        self._aux.extend(float(v) for v in np.asarray(values, dtype=np.double).reshape(-1))
        return off

    def add_shape(self, shape) -> int:
        if shape is None:
            return -1
        key = id(shape)
        if key in self._shape_index:
            return self._shape_index[key]
        if not hasattr(shape, "_emit"):
            raise NotImplementedError(f"shape type {type(shape).__name__} is not implemented on the GPU path")
        start = len(self._shape_ops)
        ops = []
        shape._emit(ops, self._aux)
        ops.append((0, 0, 0, 0.0, 0.0, 0.0, 0.0))
        self._shape_ops.extend(ops)
        self._shape_index[key] = start
        return start

    def add_material(self, mat) -> int:
        key = id(mat)
        if key in self._mat_index:
            return self._mat_index[key]
        if type(mat) is InterfaceMaterial:
            code = 0
        else:
            code = _check_type(mat, "material")
        rec = np.zeros((), dtype=_native.MATERIAL_DT)
        rec['type'] = code
        if code:
            mat._pack(rec, self)
        self._materials.append(rec)
        self.material_objects.append(mat)
        self._mat_index[key] = len(self._materials) - 1
        return self._mat_index[key]

    def add_distortion(self, dist) -> int:
        key = id(dist)
        if key in self._dist_index:
            return self._dist_index[key]
        _check_type(dist, "distortion")
        rec = np.zeros((), dtype=_native.DISTORTION_DT)
        dist._pack(rec, self)
        self._dists.append(rec)
        self._dist_index[key] = len(self._dists) - 1
        return self._dist_index[key]

    def add_dispersion(self, curve) -> int:
        key = id(curve)
        if key in self._disp_index:
            return self._disp_index[key]
        if curve.formula_id not in (0, 1, 2, 3):
            raise NotImplementedError(f"dispersion formula {curve.formula_id} is not supported "
                                      "(the reference's formula 5 returns no value)")
        rec = np.zeros((), dtype=_native.DISPERSION_DT)
        rec['formula_id'] = curve.formula_id
        rec['n_coefs'] = len(curve.coefs)
        rec['aux'] = self.add_aux(curve.coefs)
        rec['absorption'] = curve.absorption
        rec['wavelength_min'] = curve.wavelength_min
        rec['wavelength_max'] = curve.wavelength_max
        self._disps.append(rec)
        self._disp_index[key] = len(self._disps) - 1
        return self._disp_index[key]

    def add_subface(self, face) -> int:
        """Reserve a record after the traced faces for a DistortionFace's base."""
        idx = len(self._pending_sub)
        self._pending_sub.append(face)
        return -(idx + 2)  # patched to a record index in finish()

    def _face_record(self, face, material_index):
        code = 0 if type(face) is Face else _check_type(face, "face")
        rec = np.zeros((), dtype=_native.FACE_DT)
        rec['type'] = code
        rec['idx'] = int(face.idx)
        rec['material'] = material_index
        rec['invert_normal'] = int(face.invert_normal)
        rec['invert_normals'] = int(getattr(face, "invert_normals", 0))
        rec['shape'] = -1
        rec['base'] = -1
        rec['distortion'] = -1
        rec['tolerance'] = float(face.tolerance)
        if code:
            face._pack(rec, self)
        return rec

    # -- build ----------------------------------------------------------------------
    def add_list(self, fs, faces=None):
        faces = list(fs.faces) if faces is None else faces
        lrec = np.zeros((), dtype=_native.FACELIST_DT)
        t, it = fs.transform, fs.inverse_transform
        lrec['trans']['m'] = np.asarray(t._rot).reshape(-1)
        lrec['trans']['t'] = np.asarray(t._t)
        lrec['inv_trans']['m'] = np.asarray(it._rot).reshape(-1)
        lrec['inv_trans']['t'] = np.asarray(it._t)
        lrec['first_face'] = len(self._faces)
        lrec['n_faces'] = len(faces)
        self._lists.append(lrec)
        for f in faces:
            mi = self.add_material(f.material)
            self._faces.append(self._face_record(f, mi))
            self.face_objects.append(f)

    def finish(self):
        self.n_faces = len(self._faces)
        # DistortionFace base faces become sub-records after the traced faces
        sub_index = {}
        k = 0
        while k < len(self._pending_sub):
            face = self._pending_sub[k]
            rec = self._face_record(face, -1)
            sub_index[k] = len(self._faces)
            self._faces.append(rec)
            k += 1
        for rec in self._faces:
            if rec['base'] <= -2:
                rec['base'] = sub_index[-int(rec['base']) - 2]
        self.lists = np.array(self._lists, dtype=_native.FACELIST_DT).reshape(-1)
        self.faces = np.array(self._faces, dtype=_native.FACE_DT).reshape(-1)
        self.materials = np.array(self._materials, dtype=_native.MATERIAL_DT).reshape(-1)
        ops = np.zeros(len(self._shape_ops), dtype=_native.SHAPE_OP_DT)
        for i, (op, aux, n, a, b, c, d) in enumerate(self._shape_ops):
            ops[i] = (op, aux, n, 0, a, b, c, d)
        self.shape_ops = ops
        self.distortions = np.array(self._dists, dtype=_native.DISTORTION_DT).reshape(-1)
        self.dispersions = np.array(self._disps, dtype=_native.DISPERSION_DT).reshape(-1)
        self.aux = np.array(self._aux, dtype=np.double)
        return self

    def desc(self) -> _native.SceneDesc:
        """ctypes view of the tables (the arrays must outlive the call)."""
        def ptr(a):
            return a.ctypes.data if a.size else None
        d = _native.SceneDesc()
        d.n_lists = self.lists.shape[0]
        d.n_faces = self.n_faces
        d.n_face_records = self.faces.shape[0]
        d.n_materials = self.materials.shape[0]
        d.n_shape_ops = self.shape_ops.shape[0]
        d.n_distortions = self.distortions.shape[0]
        d.n_dispersions = self.dispersions.shape[0]
        d.n_aux = self.aux.shape[0]
        d.lists = ptr(self.lists)
        d.faces = ptr(self.faces)
        d.materials = ptr(self.materials)
        d.shape_ops = ptr(self.shape_ops)
        d.distortions = ptr(self.distortions)
        d.dispersions = ptr(self.dispersions)
        d.aux = ptr(self.aux)
        return d


def compile_scene(face_sets, one_face=None) -> SceneTables:
    """Pack the face lists (in trace order) into tables.  ``one_face`` =
    (list position, face index) restricts the scene to one face for the
    sequential trace."""
    t = SceneTables()
    for li, fs in enumerate(face_sets):
        t.add_list(fs)
    return t.finish()


def check_face_indices(face_sets, all_faces):
    """The reference takes the hit face from all_faces[face.idx]
    (ctracer.pyx:2107); the device uses the intersected face itself, so the
    two must agree."""
    for fs in face_sets:
        for f in fs.faces:
            i = int(f.idx)
            if i < 0 or i >= len(all_faces) or all_faces[i] is not f:
                raise ValueError("face.idx does not index the face in all_faces; "
                                 "assign face.idx as trace_rays does (core/tracer.py:28-30)")
