"""ctypes front end of the C restatement oracle (oracle/rp_oracle.c).

TEST INFRASTRUCTURE ONLY: used by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py to check or time the reference algorithm on the
host.  The product package never imports this module.

Scenes are passed as the table form of include/rp_gb300.h (built by
``raypier_optics_gb300.scene``), rays as the reference's 188-byte records.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
SRC = os.path.join(HERE, "rp_oracle.c")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "librp_oracle.so")

_lib = None
_lock = threading.Lock()


def build(force=False):
    """gcc -O2 -ffp-contract=off: the reference's own optimisation level and no
    FMA contraction, so results match the reference's C bit for bit."""
    os.makedirs(BUILD, exist_ok=True)
    hdr = os.path.join(REPO, "include", "rp_gb300.h")
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= max(os.path.getmtime(SRC),
                                                                           os.path.getmtime(hdr)):
        return LIB
    tmp = LIB + ".tmp"
    subprocess.run(["gcc", "-O2", "-ffp-contract=off", "-fno-strict-aliasing", "-fPIC", "-shared",
                    "-std=gnu11", "-o", tmp, SRC, "-lm"], check=True)
    os.replace(tmp, LIB)
    return LIB


def load():
    global _lib
    with _lock:
        if _lib is None:
            build()
            lib = ctypes.CDLL(LIB)
            P, I, U64, D = ctypes.c_void_p, ctypes.c_int, ctypes.c_uint64, ctypes.c_double
            lib.rp_oracle_trace_rays.argtypes = [P, P, ctypes.c_int64, P, U64, I, ctypes.c_float, D, P, U64, P, I,
                                                 ctypes.POINTER(I), P]
            lib.rp_oracle_trace_segment.argtypes = [P, P, ctypes.c_int64, P, U64, ctypes.c_float, I, I, D, P, U64,
                                                    ctypes.POINTER(U64), P]
            lib.rp_oracle_face_intersect.argtypes = [P, I, P, P, I]
            lib.rp_oracle_face_intersect.restype = D
            lib.rp_oracle_face_normal.argtypes = [P, I, P, P]
            lib.rp_oracle_shape_inside.argtypes = [P, I, D, D]
            lib.rp_oracle_distortion.argtypes = [P, I, D, D, P, P]
            lib.rp_oracle_convert_to_sp.argtypes = [P, P, P]
            lib.rp_oracle_eval_child_ray.argtypes = [P, P, ctypes.c_int64, I, P, ctypes.c_uint32, P, P, P, P]
            lib.rp_oracle_dispersion_n.argtypes = [P, I, P, ctypes.c_int64, P]
            lib.rp_oracle_trace_gausslet_segment.argtypes = [P, P, ctypes.c_int64, P, U64, D, I, I, P, U64,
                                                             ctypes.POINTER(U64), P, P]
            lib.rp_oracle_select_intersections.argtypes = [P, I, P, U64, ctypes.c_uint32, P, ctypes.POINTER(U64)]
            lib.rp_oracle_evaluate_modes.argtypes = [P, P, P, P, ctypes.c_int64, I, D, P]
            lib.rp_oracle_sum_gaussian_modes.argtypes = [P, ctypes.c_int64, P, P, P, ctypes.c_int64, D, P]
            lib.rp_oracle_mode_curvature.argtypes = [P, P, P, P, P, ctypes.c_int64, P, P, P, P, P, P]
            lib.rp_oracle_interaction_matrix.argtypes = [P, P, ctypes.c_int64, P, P, ctypes.c_int64, P, P, P, P, P, P,
                                                         D, D, D, D, ctypes.c_int64, P, P, P]
            lib.rp_oracle_interaction_matrix.restype = ctypes.c_int64
            lib.rp_oracle_apply_mode_curvature.argtypes = [P, ctypes.c_int64, P, P, P]
            lib.rp_oracle_gausslet_samples.argtypes = [P, ctypes.c_int64, P, P, P, P]
            lib.rp_oracle_ray_samples.argtypes = [P, ctypes.c_int64, P, P, P, P, P, P]
            lib.rp_oracle_ray_samples.restype = ctypes.c_int64
            lib.rp_oracle_project_to_sphere.argtypes = [P, ctypes.c_int64, P, D, P]
            lib.rp_oracle_eval_parabasal.argtypes = [P, P, ctypes.c_int64, I, P, P, P, P, P, ctypes.c_uint32, P]
            _lib = lib
        return _lib


def _rays(records):
    from raypier_optics_gb300.ctracer import ray_dtype
    r = np.ascontiguousarray(records)
    assert r.dtype == ray_dtype
    return r


def trace_rays(tables, wavelengths, records, recursion_limit, max_length, e2_terminate=0.0, max_total=None):
    """trace_rays (core/tracer.py:9-47) on the host.  Returns (list of
    generation record arrays, face hit counts per face record)."""
    from raypier_optics_gb300.ctracer import ray_dtype
    lib = load()
    rin = _rays(records).copy()
    n = rin.shape[0]
    cap = max_total if max_total else max(n * (2 ** min(recursion_limit, 24)), 16)
    while True:
        out = np.zeros(cap, dtype=ray_dtype)
        offs = np.zeros(recursion_limit + 2, dtype=np.uint64)
        counts = np.zeros(tables.faces.shape[0], dtype=np.uint32)
        ng = ctypes.c_int(0)
        desc = tables.desc()
        wl = np.ascontiguousarray(wavelengths, dtype=np.double)
        rc = lib.rp_oracle_trace_rays(ctypes.byref(desc), wl.ctypes.data, wl.shape[0], rin.ctypes.data, n,
                                      int(recursion_limit), ctypes.c_float(max_length), float(e2_terminate),
                                      out.ctypes.data, cap, offs.ctypes.data, recursion_limit + 1, ctypes.byref(ng),
                                      counts.ctypes.data)
        if rc == -2 and not max_total:
            cap *= 2
            continue
        if rc != 0:
            raise RuntimeError(f"oracle trace_rays failed with {rc}")
        gens = [out[int(offs[g]):int(offs[g + 1])].copy() for g in range(ng.value)]
        return gens, counts


def trace_segment(tables, wavelengths, records, max_length, e2_terminate=0.0, one_list=-1, one_face=-1):
    """One generation (trace_segment_c).  Returns (mutated input, children, face counts)."""
    from raypier_optics_gb300.ctracer import ray_dtype
    lib = load()
    rin = _rays(records).copy()
    n = rin.shape[0]
    out = np.zeros(max(2 * n, 1), dtype=ray_dtype)
    n_out = ctypes.c_uint64(0)
    counts = np.zeros(tables.faces.shape[0], dtype=np.uint32)
    desc = tables.desc()
    wl = np.ascontiguousarray(wavelengths, dtype=np.double)
    rc = lib.rp_oracle_trace_segment(ctypes.byref(desc), wl.ctypes.data, wl.shape[0], rin.ctypes.data, n,
                                     ctypes.c_float(max_length), one_list, one_face, float(e2_terminate),
                                     out.ctypes.data, out.shape[0], ctypes.byref(n_out), counts.ctypes.data)
    if rc != 0:
        raise RuntimeError(f"oracle trace_segment failed with {rc}")
    return rin, out[:n_out.value].copy(), counts


def face_intersect(tables, rec, p1, p2, is_base_ray):
    lib = load()
    desc = tables.desc()
    p1 = np.ascontiguousarray(p1, dtype=np.double).reshape(-1, 3)
    p2 = np.ascontiguousarray(p2, dtype=np.double).reshape(-1, 3)
    return np.array([lib.rp_oracle_face_intersect(ctypes.byref(desc), rec, p1[i].ctypes.data, p2[i].ctypes.data,
                                                  int(is_base_ray)) for i in range(p1.shape[0])])


def face_normal(tables, rec, p):
    lib = load()
    desc = tables.desc()
    p = np.ascontiguousarray(p, dtype=np.double).reshape(-1, 3)
    out = np.zeros_like(p)
    for i in range(p.shape[0]):
        o = np.zeros(3)
        lib.rp_oracle_face_normal(ctypes.byref(desc), rec, p[i].ctypes.data, o.ctypes.data)
        out[i] = o
    return out


def shape_inside(tables, prog, xy):
    lib = load()
    desc = tables.desc()
    xy = np.asarray(xy, dtype=np.double).reshape(-1, 2)
    return np.array([bool(lib.rp_oracle_shape_inside(ctypes.byref(desc), prog, x, y)) for x, y in xy])


def distortion(tables, d, x, y):
    lib = load()
    desc = tables.desc()
    out = np.zeros((len(x), 4))
    for i in range(len(x)):
        o = np.zeros(3)
        z = ctypes.c_double(0)
        lib.rp_oracle_distortion(ctypes.byref(desc), d, float(x[i]), float(y[i]), o.ctypes.data, ctypes.byref(z))
        out[i, :3] = o
        out[i, 3] = z.value
    return out


def convert_to_sp(records, normals):
    lib = load()
    r = _rays(records)
    nn = np.ascontiguousarray(normals, dtype=np.double).reshape(-1, 3)
    out = np.zeros_like(r)
    for i in range(r.shape[0]):
        lib.rp_oracle_convert_to_sp(r[i:i + 1].ctypes.data, nn[i].ctypes.data, out[i:i + 1].ctypes.data)
    return out


def eval_child_rays(tables, wavelengths, mat, records, idx, points, normals, tangents):
    from raypier_optics_gb300.ctracer import ray_dtype
    lib = load()
    desc = tables.desc()
    wl = np.ascontiguousarray(wavelengths, dtype=np.double)
    r = _rays(records)
    P = np.ascontiguousarray(points, dtype=np.double).reshape(-1, 3)
    N = np.ascontiguousarray(normals, dtype=np.double).reshape(-1, 3)
    T = np.ascontiguousarray(tangents, dtype=np.double).reshape(-1, 3)
    res = []
    for i in range(r.shape[0]):
        out = np.zeros(2, dtype=ray_dtype)
        k = lib.rp_oracle_eval_child_ray(ctypes.byref(desc), wl.ctypes.data, wl.shape[0], mat, r[i:i + 1].ctypes.data,
                                         int(idx[i]), P[i].ctypes.data, N[i].ctypes.data, T[i].ctypes.data,
                                         out.ctypes.data)
        if k < 0:
            raise RuntimeError("oracle material evaluation failed")
        res.append(out[:k].copy())
    return res


def dispersion_n(tables, curve, wavelengths):
    lib = load()
    desc = tables.desc()
    wl = np.ascontiguousarray(wavelengths, dtype=np.double)
    out = np.zeros(2 * wl.shape[0])
    if lib.rp_oracle_dispersion_n(ctypes.byref(desc), curve, wl.ctypes.data, wl.shape[0], out.ctypes.data):
        raise ValueError("wavelength outside the dispersion curve's range")
    return out[0::2] + 1j * out[1::2]


# ---- Gausslets ----------------------------------------------------------------------
def trace_gausslet_segment(tables, wavelengths, records, max_length, one_list=-1, one_face=-1):
    """One Gausslet generation (trace_gausslet_c / trace_one_face_gausslet_c)
    before the decomposition step and the final length reset.  Returns
    (mutated input, children, face counts, captured material + 1 per input)."""
    from raypier_optics_gb300.ctracer import gausslet_dtype
    lib = load()
    gin = np.ascontiguousarray(records).copy()
    assert gin.dtype == gausslet_dtype
    n = gin.shape[0]
    out = np.zeros(max(2 * n, 1), dtype=gausslet_dtype)
    n_out = ctypes.c_uint64(0)
    counts = np.zeros(tables.faces.shape[0], dtype=np.uint32)
    captured = np.zeros(max(n, 1), dtype=np.int32)
    desc = tables.desc()
    wl = np.ascontiguousarray(wavelengths, dtype=np.double)
    rc = lib.rp_oracle_trace_gausslet_segment(ctypes.byref(desc), wl.ctypes.data, wl.shape[0], gin.ctypes.data, n,
                                              float(max_length), one_list, one_face, out.ctypes.data, out.shape[0],
                                              ctypes.byref(n_out), counts.ctypes.data, captured.ctypes.data)
    if rc != 0:
        raise RuntimeError(f"oracle trace_gausslet_segment failed with {rc}")
    return gin, out[:n_out.value].copy(), counts, captured[:n]


def trace_gausslets(tables, wavelengths, records, recursion_limit, max_length, decompose=None, sequence=None):
    """trace_rays / trace_ray_sequence (core/tracer.py:9-99) for gausslets on
    the host.  `decompose` maps a material index to a callable taking the
    captured gausslet records and returning the records to append (the
    ResampleGaussletMaterial eval_func, cmaterials.pyx:1820-1830); `sequence`
    is a list of (list index, face index) steps.  Returns (generations, counts)."""
    from raypier_optics_gb300.ctracer import gausslet_dtype
    g = np.ascontiguousarray(records).copy()
    g['base_ray']['length'] = max_length
    g['para_rays']['length'] = max_length
    counts = np.zeros(tables.faces.shape[0], dtype=np.uint32)

    def generation(before, li, fi):
        mutated, kids, c, captured = trace_gausslet_segment(tables, wavelengths, before, max_length, li, fi)
        counts[:] += c
        if decompose:
            # decomposition faces in face order (core/tracer.py:37, ctracer.pyx:2274-2278);
            # a material's captures go to its first face with hits, later faces
            # sharing it see an empty set.  A captured gausslet is the record as
            # the material saw it: base ray intersected, parabasal rays not yet.
            done = set()
            for rec in range(tables.n_faces):
                m = int(tables.faces[rec]['material'])
                if m in decompose and counts[rec]:
                    sel = captured == m + 1 if m not in done else np.zeros(len(mutated), dtype=bool)
                    done.add(m)
                    counts[rec] = 0
                    cap = mutated[sel].copy()
                    cap['para_rays'] = before[sel]['para_rays']
                    extra = decompose[m](cap)
                    kids = np.concatenate([kids, np.asarray(extra, dtype=gausslet_dtype)])
        kids['base_ray']['length'] = max_length
        kids['para_rays']['length'] = max_length
        return mutated, kids

    gens = []
    if sequence is None:   # core/tracer.py:40-45
        rays, count = g, 0
        while len(rays) > 0 and count < recursion_limit:
            gens.append(rays)
            gens[-1], rays = generation(rays, -1, -1)
            count += 1
    else:                  # core/tracer.py:88-97
        gens.append(g)
        for count, (li, fi) in enumerate(sequence):
            gens[-1], kids = generation(gens[-1], li, fi)
            if count > recursion_limit or len(kids) == 0:
                break
            gens.append(kids)
    return gens, counts


def eval_parabasal(tables, wavelengths, mat, base_ray, direction, point, normal, tangent, ray_type):
    """InterfaceMaterial.eval_parabasal_ray of one material.  Returns a para_dtype record."""
    from raypier_optics_gb300.ctracer import para_dtype
    lib = load()
    desc = tables.desc()
    wl = np.ascontiguousarray(wavelengths, dtype=np.double)
    b = np.ascontiguousarray(base_ray).reshape(1)
    out = np.zeros(1, dtype=para_dtype)
    vs = [np.ascontiguousarray(v, dtype=np.double) for v in (direction, point, normal, tangent)]
    rc = lib.rp_oracle_eval_parabasal(ctypes.byref(desc), wl.ctypes.data, wl.shape[0], mat, b.ctypes.data,
                                      vs[0].ctypes.data, vs[1].ctypes.data, vs[2].ctypes.data, vs[3].ctypes.data,
                                      int(ray_type), out.ctypes.data)
    if rc != 0:
        raise RuntimeError("oracle eval_parabasal failed")
    return out[0]


def select_ray_intersections(tables, list_idx, collections):
    """select_ray_intersections (ctracer.pyx:1981-2015) on the host:
    `collections` is a list of (ray records, wavelengths).  Returns (records,
    merged wavelengths)."""
    from raypier_optics_gb300.ctracer import ray_dtype
    lib = load()
    desc = tables.desc()
    parts, wls, offset = [], [], 0
    for recs, wl in collections:
        r = _rays(recs)
        out = np.zeros(max(len(r), 1), dtype=ray_dtype)
        n = ctypes.c_uint64(0)
        lib.rp_oracle_select_intersections(ctypes.byref(desc), list_idx, r.ctypes.data, len(r), offset,
                                           out.ctypes.data, ctypes.byref(n))
        parts.append(out[:n.value].copy())
        wls.append(np.asarray(wl, dtype=np.double))
        offset += len(wl)
    recs = np.concatenate(parts)
    reduced, inverse = np.unique(np.concatenate(wls), return_inverse=True)
    recs['wavelength_idx'] = inverse.reshape(-1)[recs['wavelength_idx']]
    return recs, reduced


# ---- E-field summation (cfields.pyx) ------------------------------------------------
def evaluate_modes(x, y, dx, dy, blending=1.0):
    """evaluate_modes (cfields.pyx:225-234) on the host: n x 3 complex mode coefficients."""
    lib = load()
    a = [np.ascontiguousarray(v, dtype=np.double) for v in (x, y, dx, dy)]
    n, size = a[0].shape
    out = np.zeros((n, 3), dtype=np.complex128)
    if lib.rp_oracle_evaluate_modes(a[0].ctypes.data, a[1].ctypes.data, a[2].ctypes.data, a[3].ctypes.data, n, size,
                                    float(blending), out.ctypes.data) != 0:
        raise ZeroDivisionError("float division")
    return out


def sum_gaussian_modes(rays, modes, wavelengths, points, time_ps=0.0):
    """sum_gaussian_modes (cfields.pyx:49-117) on the host: n_points x 3 complex."""
    lib = load()
    r = _rays(rays)
    m = np.ascontiguousarray(modes, dtype=np.complex128)
    wl = np.ascontiguousarray(wavelengths, dtype=np.double)
    p = np.ascontiguousarray(points, dtype=np.double).reshape(-1, 3)
    out = np.zeros((p.shape[0], 3), dtype=np.complex128)
    lib.rp_oracle_sum_gaussian_modes(r.ctypes.data, len(r), m.ctypes.data, wl.ctypes.data, p.ctypes.data,
                                     p.shape[0], float(time_ps), out.ctypes.data)
    return out


def calc_mode_curvature(rx, ry, dx, dy, dx2, dy2, dxdy):
    """calc_mode_curvature (cfields.pyx:232-290) on the host: (A, B, C, x, y, z)."""
    lib = load()
    n = len(rx)
    a = [np.ascontiguousarray(v, dtype=np.double).reshape(-1) for v in (dx, dy, dx2, dy2, dxdy)]
    out = [np.empty(n) for _ in range(3)] + [np.empty((n, 3)) for _ in range(3)]
    lib.rp_oracle_mode_curvature(*[v.ctypes.data for v in a], n, *[o.ctypes.data for o in out])
    return tuple(out)


def build_interaction_matrix(rx, ry, tx, ty, A, B, C, x, y, z, wavelength, spacing, max_spacing, blending,
                             test_spacing=None):
    """build_interaction_matrix (cfields.pyx:295-395) on the host:
    (data, (i, j)) in loop order, sized exactly (test_spacing only sizes the
    reference's buffer)."""
    lib = load()
    n, L = len(rx), len(tx)
    v = [np.ascontiguousarray(a, dtype=np.double).reshape(-1) for a in (rx, ry, A, B, C)]
    t = [np.ascontiguousarray(a, dtype=np.double).reshape(-1) for a in (tx, ty)]
    b = [np.ascontiguousarray(a, dtype=np.double).reshape(-1, 3) for a in (x, y, z)]
    args = [v[0].ctypes.data, v[1].ctypes.data, n, t[0].ctypes.data, t[1].ctypes.data, L, v[2].ctypes.data,
            v[3].ctypes.data, v[4].ctypes.data, b[0].ctypes.data, b[1].ctypes.data, b[2].ctypes.data,
            float(wavelength), float(spacing), float(max_spacing), float(blending)]
    ct = lib.rp_oracle_interaction_matrix(*args, 0, None, None, None)
    data = np.zeros(max(ct, 1), np.complex128)
    xi = np.zeros(max(ct, 1), np.uint64)
    xj = np.zeros(max(ct, 1), np.uint64)
    lib.rp_oracle_interaction_matrix(*args, ct, data.ctypes.data, xi.ctypes.data, xj.ctypes.data)
    return (data[:ct], (xi[:ct], xj[:ct]))


def apply_mode_curvature(gausslets, A, B, C):
    """apply_mode_curvature (cfields.pyx:398-426) on the host: a new
    gausslet_dtype array with the parabasal directions tilted."""
    lib = load()
    from raypier_optics_gb300.ctracer import gausslet_dtype
    g = np.array(gausslets, dtype=gausslet_dtype, copy=True)
    a = [np.ascontiguousarray(v, dtype=np.double).reshape(-1) for v in (A, B, C)]
    lib.rp_oracle_apply_mode_curvature(g.ctypes.data, len(g), *[v.ctypes.data for v in a])
    return g


# ---- wavefront samples for the mode fit (core/fields.py:51-148) ---------------------
def gausslet_samples(gausslets):
    """evaluate_neighbours_gc (core/fields.py:114-136) on the host:
    (base rays, x, y, dx, dy), each sample array n x 6."""
    lib = load()
    from raypier_optics_gb300.ctracer import gausslet_dtype
    g = np.ascontiguousarray(gausslets, dtype=gausslet_dtype)
    n = len(g)
    out = [np.zeros((n, 6)) for _ in range(4)]
    lib.rp_oracle_gausslet_samples(g.ctypes.data, n, *[o.ctypes.data for o in out])
    return (g['base_ray'],) + tuple(out)


def ray_samples(rays, neighbours):
    """evaluate_neighbours (core/fields.py:80-111) on the host:
    (kept rays, x, y, dx, dy)."""
    lib = load()
    r = _rays(rays)
    nb = np.ascontiguousarray(neighbours, dtype=np.int32).reshape(-1, 6)
    n = len(r)
    out = [np.zeros((n, 6)) for _ in range(4)]
    kept = np.zeros(n, dtype=np.int64)
    k = lib.rp_oracle_ray_samples(r.ctypes.data, n, nb.ctypes.data, *[o.ctypes.data for o in out], kept.ctypes.data)
    return (r[kept[:k]],) + tuple(o[:k] for o in out)


def project_to_sphere(rays, centre, radius):
    """project_to_sphere (core/fields.py:51-77) on the host: the rays that
    meet the sphere, moved to it."""
    lib = load()
    r = np.array(_rays(rays), copy=True)
    hit = np.zeros(len(r), dtype=np.uint8)
    c = np.ascontiguousarray(centre, dtype=np.double).reshape(3)
    lib.rp_oracle_project_to_sphere(r.ctypes.data, len(r), c.ctypes.data, float(radius), hit.ctypes.data)
    return r[hit.astype(bool)]
