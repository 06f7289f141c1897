"""Seeded synthetic workloads (the benchmark configurations) and a scene
builder that works for any module namespace with the reference's API.

``build_scene(spec, ns)`` takes a JSON-able scene description and a namespace
``ns`` holding ``ctracer, cfaces, cmaterials, cshapes, cdistortions`` modules
-- either this package's or the reference's -- so the identical scene can be
constructed for both sides of a parity check.  No public dataset is involved:
every ray set is generated from a fixed numpy PCG64 seed.

Configurations (sizes as in the benchmark definition):

* ``config1``: 4,096 rays on a hexagonal grid in a 10 mm collimated beam at
  0.55 um, a 5 mm window at z=10, a biconvex R=50 singlet at z=30 and an
  absorbing detector at z=130; every dielectric face splits, 6 generations.
* ``config2``: 1,048,576 rays from a point source at z=-200 in a 0.1 rad cone,
  per-ray wavelength U[0.45, 0.65] um and polarisation angle, through two
  cemented doublets (Sellmeier crown / flint) and two even-asphere singlets
  (k=-0.6, A4=1e-5, A6=-2e-8, A8=5e-11) onto a detector; 8 generations.
* ``config3``: the 64-face clutter scene (seeded positions and orientations
  in a 100 mm cube) of spheres, conic mirrors, Zernike-distorted planes,
  2-D polynomial faces and prism faces; 12 generations.
"""
from __future__ import annotations

import copy
import math
import types

import numpy as np

# The fixed prescription of config 2 (mm): (z of the element's first vertex,
# faces).  Chosen once and frozen; the benchmark text leaves it open.
CROWN = {"formula_id": 2, "coefs": [0.0, 1.04, 0.006, 0.23, 0.020, 1.01, 103.6]}
FLINT = {"formula_id": 2, "coefs": [0.0, 1.34, 0.010, 0.21, 0.047, 0.94, 111.9]}
AIR = {"formula_id": 0, "coefs": [1.0]}


def _rot_translation(rotation, translation):
    R = np.asarray(rotation, dtype=np.double).reshape(3, 3)
    t = np.asarray(translation, dtype=np.double).reshape(3)
    Ri = R.T.copy()
    ti = -(Ri @ t)
    return R, t, Ri, ti


def _make_shape(spec, ns):
    if spec is None:
        return ns.ctracer.Shape()
    kind = spec["type"]
    if kind in ("and", "or", "xor"):
        a, b = _make_shape(spec["a"], ns), _make_shape(spec["b"], ns)
        return {"and": a & b, "or": a | b, "xor": a ^ b}[kind]
    if kind == "not":
        return ~_make_shape(spec["a"], ns)
    cls = getattr(ns.cshapes, kind)
    kw = dict(spec.get("kw", {}))
    obj = cls(**kw)
    if "coordinates" in spec:
        obj.coordinates = np.asarray(spec["coordinates"], dtype=np.double)
    return obj


def _make_curve(spec, ns):
    return ns.cmaterials.BaseDispersionCurve(spec["formula_id"], np.asarray(spec["coefs"], dtype=np.double),
                                              spec.get("absorption", 0.0),
                                              spec.get("wavelength_min", 0.1),
                                              spec.get("wavelength_max", 1000000.0))


def resample_shift(gc):
    """A ResampleGaussletMaterial eval_func for tests and examples: relaunches
    every captured gausslet 1 mm beyond the point where its base ray met the
    face (base and parabasal rays each advanced by that distance along their
    own direction), with the GAUSSLET bit cleared so that it is not captured
    again.  Works on any GaussletCollection class offering copy_as_array /
    from_array."""
    arr = gc.copy_as_array()
    step = arr['base_ray']['length'] + 1.0
    b, p = arr['base_ray'], arr['para_rays']
    arr['base_ray']['origin'] = b['origin'] + b['direction'] * step[:, None]
    arr['para_rays']['origin'] = p['origin'] + p['direction'] * step[:, None, None]
    arr['base_ray']['ray_type_id'] = b['ray_type_id'] & ~np.uint32(2)
    return type(gc).from_array(arr)


EVAL_FUNCS = {"resample_shift": resample_shift}


def _make_material(spec, ns, curves):
    cls = getattr(ns.cmaterials, spec["type"])
    kw = dict(spec.get("kw", {}))
    if isinstance(kw.get("eval_func"), str):
        kw["eval_func"] = EVAL_FUNCS[kw["eval_func"]]
    for k in ("dispersion_inside", "dispersion_outside", "dispersion_coating"):
        if k in kw:
            kw[k] = curves[kw[k]]
    for k in ("n_inside", "n_outside", "n_coating"):
        if k in kw and isinstance(kw[k], (list, tuple)):
            kw[k] = complex(kw[k][0], kw[k][1])
    return cls(**kw)


def _make_distortion(spec, ns):
    if spec["type"] == "ZernikeDistortion":
        return ns.cdistortions.ZernikeDistortion([(int(j), float(v)) for j, v in spec["coefs"]],
                                                 **spec.get("kw", {}))
    return getattr(ns.cdistortions, spec["type"])(**spec.get("kw", {}))


class AffineMatrix:
    """A 4x4 affine map offering the two members EllipsoidalFace reads from
    its owner's VTK transform (ellipsoids.py ellipse_trans):
    ``matrix.get_element(i, j)`` and ``linear_inverse``.  The inverse is
    given, not computed, so that every platform sees the same bits."""

    def __init__(self, matrix, inverse):
        self._m = np.asarray(matrix, dtype=np.float64).reshape(4, 4)
        self._inv = np.asarray(inverse, dtype=np.float64).reshape(4, 4)

    @property
    def matrix(self):
        return self

    def get_element(self, i, j):
        return float(self._m[i, j])

    @property
    def linear_inverse(self):
        return AffineMatrix(self._inv, self._m)


def _make_face(spec, ns, materials, curves):
    cls = getattr(ns.cfaces, spec["type"])
    kw = dict(spec.get("kw", {}))
    owner_kw = dict(spec.get("owner", {}))
    if "ellipse_trans" in owner_kw:
        owner_kw["ellipse_trans"] = AffineMatrix(**owner_kw["ellipse_trans"])
    owner = types.SimpleNamespace(**owner_kw)
    if "shape" in spec:
        kw["shape"] = _make_shape(spec["shape"], ns)
    if "base_face" in spec:
        kw["base_face"] = _make_face(spec["base_face"], ns, materials, curves)
    if "distortion" in spec:
        kw["distortion"] = _make_distortion(spec["distortion"], ns)
    mat = materials[spec["material"]] if spec.get("material") else None
    face = cls(owner=owner, material=mat, **kw)
    for k, v in spec.get("attrs", {}).items():
        if k == "coefs":
            v = np.asarray(v, dtype=np.double)
        setattr(face, k, v)
    return face


def build_scene(spec, ns):
    """Face lists for `spec` built from the classes in namespace `ns`."""
    curves = {name: _make_curve(c, ns) for name, c in spec.get("curves", {}).items()}
    materials = {name: _make_material(m, ns, curves) for name, m in spec["materials"].items()}
    lists = []
    for lspec in spec["lists"]:
        fl = ns.ctracer.FaceList(owner=None)
        R, t, Ri, ti = _rot_translation(lspec.get("rotation", np.eye(3)), lspec.get("translation", (0, 0, 0)))
        fl.transform = ns.ctracer.Transform(rotation=R.tolist(), translation=t.tolist())
        fl.inverse_transform = ns.ctracer.Transform(rotation=Ri.tolist(), translation=ti.tolist())
        fl.faces = [_make_face(f, ns, materials, curves) for f in lspec["faces"]]
        lists.append(fl)
    return lists


# ---- rays ---------------------------------------------------------------------------
def hex_grid(n, radius):
    """The n hexagonal-lattice points nearest the origin, ordered by (r^2,
    angle), scaled so that the outermost lies at `radius`."""
    m = int(math.sqrt(n) * 1.2) + 4
    i, j = np.meshgrid(np.arange(-m, m + 1), np.arange(-m, m + 1))
    i, j = i.reshape(-1), j.reshape(-1)
    r2_int = (2 * i + j) ** 2 + 3 * j ** 2          # 4 * r^2 in lattice units, exact
    x = i + 0.5 * j
    y = (math.sqrt(3.0) / 2.0) * j
    ang = np.arctan2(y, x)
    order = np.lexsort((ang, r2_int))[:n]
    x, y = x[order], y[order]
    scale = radius / math.sqrt(float(np.max(x * x + y * y)))
    return x * scale, y * scale


def _ray_array(n, ns_ray_dtype):
    return np.zeros(n, dtype=ns_ray_dtype)


def fill_rays(rays, origin, direction, E_vector, E1=1.0 + 0j, E2=0j, n_index=1.0 + 0j, wavelength_idx=0):
    rays['origin'] = origin
    rays['direction'] = direction
    rays['E_vector'] = E_vector
    rays['E1_amp'] = E1
    rays['E2_amp'] = E2
    rays['refractive_index'] = n_index
    rays['wavelength_idx'] = wavelength_idx
    rays['ray_ident'] = np.arange(rays.shape[0], dtype=np.uint32)
    rays['normal'] = (0.0, 0.0, 1.0)
    return rays


# ---- configuration 1 -----------------------------------------------------------------
def config1_spec():
    glass = {"type": "FullDielectricMaterial",
             "kw": {"n_inside": 1.5168, "n_outside": 1.0, "reflection_threshold": -1.0,
                    "transmission_threshold": -1.0}}
    owner25 = {"diameter": 25.0, "offset": 0.0}
    return {
        "materials": {"glass": glass, "detector": {"type": "OpaqueMaterial"}},
        "lists": [
            {"translation": [0, 0, 10], "faces": [
                {"type": "CircularFace", "kw": {"z_plane": 0.0}, "owner": owner25, "material": "glass"},
                {"type": "CircularFace", "kw": {"z_plane": 5.0, "invert_normals": 1}, "owner": owner25,
                 "material": "glass"}]},
            {"translation": [0, 0, 30], "faces": [
                {"type": "SphericalFace", "kw": {"curvature": -50.0, "z_height": 0.0, "invert_normal": 1},
                 "owner": {"diameter": 25.0}, "material": "glass"},
                {"type": "SphericalFace", "kw": {"curvature": 50.0, "z_height": 6.0},
                 "owner": {"diameter": 25.0}, "material": "glass"}]},
            {"translation": [0, 0, 130], "faces": [
                {"type": "CircularFace", "kw": {"z_plane": 0.0}, "owner": {"diameter": 100.0, "offset": 0.0},
                 "material": "detector"}]},
        ]}


def config1_rays(ray_dtype, n=4096):
    x, y = hex_grid(n, 5.0)
    rays = np.zeros(n, dtype=ray_dtype)
    origin = np.stack([x, y, np.zeros(n)], axis=1)
    return fill_rays(rays, origin, (0.0, 0.0, 1.0), (1.0, 0.0, 0.0)), np.array([0.55])


CONFIG1 = {"recursion_limit": 6, "max_length": 1000.0, "e2_terminate": 1e-6}


# ---- configuration 2 -----------------------------------------------------------------
def config2_spec():
    def disp(inside, outside):
        return {"type": "FullDielectricDispersiveMaterial",
                "kw": {"dispersion_inside": inside, "dispersion_outside": outside,
                       "reflection_threshold": -1.0, "transmission_threshold": -1.0}}
    mats = {"air_crown": disp("crown", "air"), "crown_flint": disp("crown", "flint"),
            "flint_air": disp("flint", "air"), "detector": {"type": "OpaqueMaterial"}}

    # cemented doublet, 50 mm: biconvex crown (R1 = 100, R2 = -80, 12 mm) and a
    # flint meniscus (R3 = -250, 4 mm); every element has a positive edge thickness
    def doublet(z):
        return {"translation": [0, 0, z], "faces": [
            {"type": "SphericalFace", "kw": {"curvature": -100.0, "z_height": 0.0, "invert_normal": 1},
             "owner": {"diameter": 50.0}, "material": "air_crown"},
            {"type": "SphericalFace", "kw": {"curvature": 80.0, "z_height": 12.0},
             "owner": {"diameter": 50.0}, "material": "crown_flint"},
            {"type": "SphericalFace", "kw": {"curvature": 250.0, "z_height": 16.0},
             "owner": {"diameter": 50.0}, "material": "flint_air"}]}

    # even-asphere singlet, 50 mm: asphere front (sag 10.6 mm at r = 25), plane back 14 mm behind
    def asphere(z):
        circ = {"type": "CircleShape", "kw": {"radius": 25.0}}
        return {"translation": [0, 0, z], "faces": [
            {"type": "AsphericFace", "kw": {"curvature": -80.0, "z_height": 0.0, "conic_const": -0.6,
                                            "A4": 1e-5, "A6": -2e-8, "A8": 5e-11, "invert_normals": 1},
             "shape": circ, "material": "air_crown"},
            {"type": "ShapedPlanarFace", "kw": {"z_height": 14.0}, "shape": circ, "material": "air_crown"}]}

    return {"curves": {"crown": CROWN, "flint": FLINT, "air": AIR}, "materials": mats,
            "lists": [doublet(0.0), doublet(30.0), asphere(60.0), asphere(90.0),
                      {"translation": [0, 0, 160], "faces": [
                          {"type": "CircularFace", "kw": {"z_plane": 0.0},
                           "owner": {"diameter": 200.0, "offset": 0.0}, "material": "detector"}]}]}


def config2_rays(ray_dtype, n=1048576, seed=2):
    rng = np.random.Generator(np.random.PCG64(seed))
    cos_t = rng.uniform(math.cos(0.1), 1.0, n)
    phi = rng.uniform(0.0, 2 * math.pi, n)
    wl = rng.uniform(0.45, 0.65, n)
    psi = rng.uniform(0.0, math.pi, n)
    sin_t = np.sqrt(1.0 - cos_t * cos_t)
    d = np.stack([sin_t * np.cos(phi), sin_t * np.sin(phi), cos_t], axis=1)
    # basis perpendicular to d: e1 = normalise(y x d), e2 = d x e1
    e1 = np.cross(np.array([0.0, 1.0, 0.0]), d)
    e1 /= np.linalg.norm(e1, axis=1)[:, None]
    e2 = np.cross(d, e1)
    E = np.cos(psi)[:, None] * e1 + np.sin(psi)[:, None] * e2
    rays = np.zeros(n, dtype=ray_dtype)
    fill_rays(rays, (0.0, 0.0, -200.0), d, E)
    rays['wavelength_idx'] = np.arange(n, dtype=np.uint32)
    return rays, wl


CONFIG2 = {"recursion_limit": 8, "max_length": 1000.0, "e2_terminate": 1e-6}


# ---- configuration 3 -----------------------------------------------------------------
# Noll index -> ANSI j for the first 15 Zernike terms (the reference indexes
# ZernikeDistortion by ANSI j, cdistortions.pyx:104-136).
# Noll (1976) index -> (n, m) for the first 15 terms.
NOLL_NM = {1: (0, 0), 2: (1, 1), 3: (1, -1), 4: (2, 0), 5: (2, -2), 6: (2, 2), 7: (3, -1), 8: (3, 1),
           9: (3, -3), 10: (3, 3), 11: (4, 0), 12: (4, 2), 13: (4, -2), 14: (4, 4), 15: (4, -4)}


def noll_to_nm(j):
    return NOLL_NM[j]


def ansi_j(n, m):
    return (n * (n + 2) + m) // 2


def _random_rotation(rng):
    q, r = np.linalg.qr(rng.standard_normal((3, 3)))
    q = q * np.sign(np.diag(r))[None, :]
    if np.linalg.det(q) < 0:
        q[:, 0] = -q[:, 0]
    return q


def config3_spec(face_seed=4):
    rng = np.random.Generator(np.random.PCG64(face_seed))
    mats = {"glass": {"type": "FullDielectricMaterial",
                      "kw": {"n_inside": 1.5, "n_outside": 1.0, "reflection_threshold": -1.0,
                             "transmission_threshold": -1.0}},
            "mirror": {"type": "PECMaterial"}}
    circ = {"type": "CircleShape", "kw": {"radius": 12.5}}
    lists = []

    def place(faces):
        lists.append({"rotation": _random_rotation(rng).tolist(),
                      "translation": rng.uniform(-50.0, 50.0, 3).tolist(), "faces": faces})

    for _ in range(16):
        R = rng.uniform(20.0, 200.0) * (1 if rng.uniform() < 0.5 else -1)
        place([{"type": "SphericalFace", "kw": {"curvature": float(R), "z_height": 0.0},
                "owner": {"diameter": 25.0}, "material": "glass"}])
    for _ in range(16):
        R = rng.uniform(20.0, 200.0) * (1 if rng.uniform() < 0.5 else -1)
        place([{"type": "ConicRevolutionFace", "kw": {"curvature": float(R), "z_height": 0.0,
                                                      "conic_const": float(rng.uniform(-2.0, 0.0))},
                "shape": circ, "material": "mirror"}])
    for _ in range(16):
        coefs = []
        for noll in range(1, 16):
            n, m = noll_to_nm(noll)
            coefs.append([ansi_j(n, m), float(rng.normal(0.0, 5e-4))])
        place([{"type": "DistortionFace", "kw": {"accuracy": 1e-6},
                "base_face": {"type": "ShapedPlanarFace", "kw": {"z_height": 0.0}, "shape": circ},
                "distortion": {"type": "ZernikeDistortion", "coefs": coefs, "kw": {"unit_radius": 12.5}},
                "shape": circ, "material": "glass"}])
    for _ in range(8):
        c = np.zeros((5, 5))
        for i in range(5):
            for j in range(5 - i):
                c[i, j] = rng.normal(0.0, 1e-4)
        R = rng.uniform(50.0, 200.0) * (1 if rng.uniform() < 0.5 else -1)
        place([{"type": "ExtendedPolynomialFace", "kw": {"norm_radius": 12.5},
                "attrs": {"curvature": float(R), "conic_const": 0.0, "z_height": 0.0, "coefs": c.tolist()},
                "shape": circ, "material": "glass"}])
    for _ in range(8):
        # one face of a 90 degree prism: the hypotenuse square in the plane x = z
        s = 10.0
        place([{"type": "OrientedPolygonFace",
                "kw": {"origin": [0.0, 0.0, 0.0], "x_axis": [1.0 / math.sqrt(2), 0.0, 1.0 / math.sqrt(2)],
                       "normal": [1.0 / math.sqrt(2), 0.0, -1.0 / math.sqrt(2)],
                       "xy_points": [[-s, -s], [s, -s], [s, s], [-s, s]]},
                "material": "glass"}])
    return {"materials": mats, "lists": lists}


CONFIG3_BLOCK = 65536


def config3_rays(ray_dtype, n=16777216, seed=3, first_block=0):
    """Rays in blocks of 65,536 with one PCG64 stream per block, so a
    subsample taken from the first blocks is the same rays as in the full set."""
    n_blocks = (n + CONFIG3_BLOCK - 1) // CONFIG3_BLOCK
    seqs = np.random.SeedSequence(seed).spawn(first_block + n_blocks)[first_block:]
    rays = np.zeros(n, dtype=ray_dtype)
    for b, ss in enumerate(seqs):
        lo, hi = b * CONFIG3_BLOCK, min(n, (b + 1) * CONFIG3_BLOCK)
        m = hi - lo
        rng = np.random.Generator(np.random.PCG64(ss))
        g = rng.standard_normal((CONFIG3_BLOCK, 2))[:m] * 0.05
        xy = rng.uniform(-10.0, 10.0, (CONFIG3_BLOCK, 2))[:m]
        d = np.concatenate([g, np.ones((m, 1))], axis=1)
        d /= np.linalg.norm(d, axis=1)[:, None]
        origin = np.concatenate([xy, np.full((m, 1), -60.0)], axis=1)
        e1 = np.cross(np.array([0.0, 1.0, 0.0]), d)
        e1 /= np.linalg.norm(e1, axis=1)[:, None]
        fill_rays(rays[lo:hi], origin, d, e1)
    rays['ray_ident'] = np.arange(n, dtype=np.uint32) + np.uint32(first_block * CONFIG3_BLOCK)
    return rays, np.array([0.8])


CONFIG3 = {"recursion_limit": 12, "max_length": 1000.0, "e2_terminate": 1e-6}


def subsample(rays, wavelengths, idx, per_ray_wavelength):
    """Rays `idx` of a workload with ray_ident / wavelength_idx kept consistent."""
    sub = rays[idx].copy()
    if per_ray_wavelength:
        wl = np.asarray(wavelengths)[sub['wavelength_idx']]
        sub['wavelength_idx'] = np.arange(len(sub), dtype=np.uint32)
        return sub, wl
    return sub, np.asarray(wavelengths)


def spec_copy(spec):
    return copy.deepcopy(spec)


# ---- configuration 4 (differentiable lens) ---------------------------------------------
# A four-element, eight-face Cooke-triplet-like objective (glasses 1.62 / 1.62 /
# 1.52 and a 1.62 field element), even aspheres throughout.  Optical radii
# (positive: centre of curvature behind the vertex) are stored with raypier's
# sign, curvature = -R.  Nominal best focus for the 8 mm collimated beam lies
# 39.4 mm behind the last vertex.
LENS4_RADII = [22.0, -400.0, -28.0, 22.0, 60.0, -25.0, 30.0, 45.0]
LENS4_CONIC = [-0.20, 0.10, 0.15, -0.10, 0.20, -0.15, 0.10, -0.20]
LENS4_A4 = [2.0e-6, -1.0e-6, 1.5e-6, -2.0e-6, 1.0e-6, 2.0e-6, -1.5e-6, 1.0e-6]
LENS4_A6 = [-1.0e-8, 2.0e-8, -1.5e-8, 1.0e-8, -2.0e-8, 1.5e-8, 1.0e-8, -1.0e-8]
LENS4_THICKNESS = [3.5, 4.0, 1.2, 4.0, 3.0, 1.0, 2.5, 39.4]
LENS4_SEMI = [9.0, 9.0, 8.0, 8.0, 8.0, 8.0, 8.0, 8.0]
LENS4_INDEX = [1.0, 1.62, 1.0, 1.62, 1.0, 1.52, 1.0, 1.62, 1.0]
CONFIG4 = {"n_rays": 262144, "beam_radius": 4.0, "wavelength": 0.587, "z_start": -10.0, "max_length": 1000.0,
           "atol": 1.0e-8, "tolerance": 1.0e-4, "perturbation": 0.02, "seed": 4, "fd_step": 1.0e-6}


def config4_nominal():
    """The 40 nominal parameters: curvature[8] (raypier sign), conic[8], A4[8], A6[8], thickness[8]."""
    return np.array([-r for r in LENS4_RADII] + LENS4_CONIC + LENS4_A4 + LENS4_A6 + LENS4_THICKNESS,
                    dtype=np.double)


def config4_params(seed=None):
    """Nominal parameters with seeded uniform perturbations of +-2 %."""
    rng = np.random.Generator(np.random.PCG64(CONFIG4["seed"] if seed is None else seed))
    p = config4_nominal()
    return p * (1.0 + rng.uniform(-CONFIG4["perturbation"], CONFIG4["perturbation"], p.shape[0]))


def config4_rays(ray_dtype, n=None):
    """Collimated rays on a hexagonal grid filling the 8 mm beam, starting at z = -10."""
    n = n or CONFIG4["n_rays"]
    x, y = hex_grid(max(n, 7), CONFIG4["beam_radius"])
    x, y = x[:n], y[:n]
    rays = np.zeros(n, dtype=ray_dtype)
    origin = np.stack([x, y, np.full(n, CONFIG4["z_start"])], axis=1)
    fill_rays(rays, origin, (0.0, 0.0, 1.0), (1.0, 0.0, 0.0))
    return rays, np.array([CONFIG4["wavelength"]])


def config4_spec(params):
    """The lens as an ordinary raypier scene: one face list, every surface an
    AsphericFace with its normal turned to -z and a DielectricMaterial whose
    outside is the medium in front of it, then the image plane (a detector)."""
    n = len(LENS4_RADII)
    params = np.asarray(params, dtype=np.double)
    faces, mats = [], {"image": {"type": "OpaqueMaterial"}}
    z = 0.0
    for k in range(n):
        mats[f"s{k}"] = {"type": "DielectricMaterial",
                         "kw": {"n_inside": LENS4_INDEX[k + 1], "n_outside": LENS4_INDEX[k]}}
        faces.append({"type": "AsphericFace",
                      "kw": {"curvature": float(params[k]), "z_height": z, "conic_const": float(params[n + k]),
                             "A4": float(params[2 * n + k]), "A6": float(params[3 * n + k]),
                             "atol": CONFIG4["atol"], "invert_normal": 1},
                      "shape": {"type": "CircleShape", "kw": {"radius": LENS4_SEMI[k]}},
                      "material": f"s{k}"})
        z += float(params[4 * n + k])
    faces.append({"type": "CircularFace", "kw": {"z_plane": z},
                  "owner": {"diameter": 1.0e9, "offset": 0.0}, "material": "image"})
    return {"materials": mats, "lists": [{"translation": [0, 0, 0], "faces": faces}]}


# ---- configuration 5 (serving) -----------------------------------------------------
CONFIG5 = {"n_jobs": 10000, "rate": 200.0, "seed": 5, "min_rays": 1000, "max_rays": 4000000,
           "wl_range": (0.4, 1.0), "n_wavelengths": 256, "hbm_budget": 120 * 10**9, "n_systems": 256,
           "recursion_limit": 8, "max_length": 1000.0, "e2_terminate": 1e-6}


def config5_system(rng, n_elements, entrance=False):
    """A random coaxial system of `n_elements` singlets (2 faces each) drawn
    from configuration 2's face mix (spherical, conic, aspheric, plane), crown
    or flint with Sellmeier dispersion and the materials' default Fresnel
    thresholds, then (`entrance`) one more air-to-glass surface whose glass
    runs on to the detector, then the detector: 2 n_elements + 1 (+ 1) faces.
    Every face's normal points to +z at its vertex, so a face's material has
    the medium in front as `inside` (DielectricMaterial's out-to-in test is
    normal . d < 0)."""
    mats = {"detector": {"type": "OpaqueMaterial"}}
    for g in ("crown", "flint"):
        mats[f"in_{g}"] = {"type": "FullDielectricDispersiveMaterial",
                           "kw": {"dispersion_inside": "air", "dispersion_outside": g}}
        mats[f"out_{g}"] = {"type": "FullDielectricDispersiveMaterial",
                            "kw": {"dispersion_inside": g, "dispersion_outside": "air"}}
    circ = {"type": "CircleShape", "kw": {"radius": 12.5}}
    faces, z = [], 0.0

    def surface(z_height, mat):
        kind = rng.integers(0, 4)
        R = float(rng.uniform(60.0, 400.0)) * (1.0 if rng.uniform() < 0.5 else -1.0)
        if kind == 0:
            return {"type": "SphericalFace", "kw": {"curvature": -R, "z_height": z_height},
                    "owner": {"diameter": 25.0}, "material": mat}
        if kind == 1:
            return {"type": "ConicRevolutionFace", "kw": {"curvature": -R, "z_height": z_height,
                                                          "conic_const": float(rng.uniform(-1.5, 0.5))},
                    "shape": circ, "material": mat}
        if kind == 2:
            return {"type": "AsphericFace", "kw": {"curvature": -R, "z_height": z_height,
                                                   "conic_const": float(rng.uniform(-1.0, 0.0)),
                                                   "A4": float(rng.normal(0.0, 1e-6)),
                                                   "A6": float(rng.normal(0.0, 1e-9))},
                    "shape": circ, "material": mat}
        return {"type": "ShapedPlanarFace", "kw": {"z_height": z_height}, "shape": circ, "material": mat}

    for _ in range(n_elements):
        g = "crown" if rng.uniform() < 0.5 else "flint"
        faces.append(surface(z, f"in_{g}"))
        z += float(rng.uniform(4.0, 8.0))
        faces.append(surface(z, f"out_{g}"))
        z += float(rng.uniform(3.0, 10.0))
    if entrance:
        faces.append(surface(z, "in_crown" if rng.uniform() < 0.5 else "in_flint"))
        z += float(rng.uniform(3.0, 10.0))
    faces.append({"type": "CircularFace", "kw": {"z_plane": z + 20.0}, "owner": {"diameter": 400.0, "offset": 0.0},
                  "material": "detector"})
    return {"curves": {"crown": CROWN, "flint": FLINT, "air": AIR}, "materials": mats,
            "lists": [{"translation": [0, 0, 0], "faces": faces}]}


def config5_jobs(n_jobs=None, seed=None):
    """The seeded job stream: (arrival time s, system index, n_rays, source seed,
    source type, wavelengths), with `CONFIG5["n_systems"]` distinct systems
    of 2-40 faces (uniform) that jobs draw from, arrivals Poisson at
    CONFIG5["rate"]/s and ray counts log-uniform over [1e3, 4e6]."""
    C = CONFIG5
    n_jobs = C["n_jobs"] if n_jobs is None else n_jobs
    rng = np.random.Generator(np.random.PCG64(C["seed"] if seed is None else seed))
    systems = []
    for _ in range(C["n_systems"]):
        lens_faces = int(rng.integers(2, 41)) - 1  # 2-40 faces with the detector
        systems.append(config5_system(rng, lens_faces // 2, entrance=lens_faces % 2 == 1))
    t = np.cumsum(rng.exponential(1.0 / C["rate"], n_jobs))
    sys_idx = rng.integers(0, len(systems), n_jobs)
    n_rays = np.exp(rng.uniform(math.log(C["min_rays"]), math.log(C["max_rays"]), n_jobs)).astype(np.int64)
    seeds = rng.integers(1, 2**62, n_jobs)
    kinds = rng.integers(1, 3, n_jobs)  # point cone or collimated disc
    wls = [np.sort(rng.uniform(C["wl_range"][0], C["wl_range"][1], C["n_wavelengths"])) for _ in range(n_jobs)]
    return systems, [{"t": float(t[k]), "system": int(sys_idx[k]), "n_rays": int(n_rays[k]), "seed": int(seeds[k]),
                      "source": int(kinds[k]), "wavelengths": wls[k]} for k in range(n_jobs)]
