"""Generate the golden vectors in tests/golden/ by running the reference
raypier tracer (its Cython core built from source by oracle/build_ref.py).

Run in a container that has the reference sources and Cython:

    python oracle/build_ref.py && python tests/golden/make_golden.py
    python tests/golden/make_golden.py --lens     # only the configuration-4 lens case
    python tests/golden/make_golden.py --coated   # only the coated-material cases
    python tests/golden/make_golden.py --faces2   # only the second face set
    python tests/golden/make_golden.py --sequential  # only the trace_ray_sequence case
    python tests/golden/make_golden.py --gausslets   # only the Gausslet cases
    python tests/golden/make_golden.py --capture     # only the post-trace capture case
    python tests/golden/make_golden.py --fields      # only the E-field summation cases
    python tests/golden/make_golden.py --fields2     # only the decomposition helpers of cfields

Every fixture stores the scene description (the JSON spec understood by
raypier_optics_gb300.workloads.build_scene), the inputs, and the reference's
outputs.  The tests rebuild the same scene with this package's classes and
compare the oracle and the GPU path against these outputs.
"""
from __future__ import annotations

import contextlib
import hashlib
import io
import json
import math
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)
sys.path.insert(0, os.path.join(REPO, "oracle"))

import build_ref  # noqa: E402
from raypier_optics_gb300 import workloads as W  # noqa: E402

RNG_SEED = 20261203


# ---- scene zoos -----------------------------------------------------------------------
def _glass(name="glass", n_in=1.5, n_out=1.0, thr=-1.0):
    return {"type": "FullDielectricMaterial", "kw": {"n_inside": n_in, "n_outside": n_out,
                                                     "reflection_threshold": thr, "transmission_threshold": thr}}


CIRC8 = {"type": "CircleShape", "kw": {"radius": 8.0, "centre": [1.0, -1.0]}}
RECT = {"type": "RectangleShape", "kw": {"width": 10.0, "height": 6.0}}
PENTAGON = {"type": "PolygonShape", "coordinates": [[9.0 * math.cos(a), 9.0 * math.sin(a)]
                                                    for a in np.linspace(0, 2 * math.pi, 6)[:-1]]}


def zernike15(rng, scale):
    return [[W.ansi_j(*W.noll_to_nm(j)), float(rng.normal(0.0, scale))] for j in range(1, 16)]


def face_zoo(rng):
    """One spec per face type (plus shape and sign variants)."""
    circ12 = {"type": "CircleShape", "kw": {"radius": 12.0}}
    faces = {
        "circular": {"type": "CircularFace", "kw": {"z_plane": 0.0}, "owner": {"diameter": 20.0, "offset": 1.0}},
        "circular_inv": {"type": "CircularFace", "kw": {"z_plane": 2.0, "invert_normals": 1},
                         "owner": {"diameter": 20.0, "offset": 0.0}},
        "rectangular": {"type": "RectangularFace", "kw": {"z_plane": 0.0},
                        "owner": {"length": 10.0, "width": 6.0, "offset": 1.0}},
        "planar_circle": {"type": "ShapedPlanarFace", "kw": {"z_height": 1.0}, "shape": CIRC8},
        "planar_rect_not_circle": {"type": "ShapedPlanarFace", "kw": {"z_height": 0.0},
                                   "shape": {"type": "and", "a": RECT,
                                             "b": {"type": "not", "a": {"type": "CircleShape",
                                                                        "kw": {"radius": 2.0}}}}},
        "planar_polygon_xor": {"type": "ShapedPlanarFace", "kw": {"z_height": 0.0},
                               "shape": {"type": "xor", "a": PENTAGON, "b": {"type": "CircleShape",
                                                                             "kw": {"radius": 3.0}}}},
        "planar_or": {"type": "ShapedPlanarFace", "kw": {"z_height": 0.0},
                      "shape": {"type": "or", "a": CIRC8, "b": RECT}},
        "spherical_pos": {"type": "SphericalFace", "kw": {"curvature": 30.0, "z_height": 0.0},
                          "owner": {"diameter": 20.0}},
        "spherical_neg": {"type": "SphericalFace", "kw": {"curvature": -30.0, "z_height": 0.0, "invert_normal": 1},
                          "owner": {"diameter": 20.0}},
        "shaped_spherical": {"type": "ShapedSphericalFace", "kw": {"curvature": 40.0, "z_height": 0.0},
                             "shape": RECT},
        "conic_mirror": {"type": "ConicRevolutionFace", "kw": {"curvature": 40.0, "conic_const": -1.5},
                         "shape": circ12, "material": "mirror"},
        "conic_inv": {"type": "ConicRevolutionFace", "kw": {"curvature": -25.0, "conic_const": -0.5,
                                                            "invert_normals": 1}, "shape": circ12},
        "aspheric": {"type": "AsphericFace", "kw": {"curvature": -50.0, "conic_const": -0.6, "A4": 1e-5,
                                                    "A6": -2e-8, "A8": 5e-11, "A10": 1e-14, "A12": -1e-17},
                     "shape": circ12},
        "aspheric_pos": {"type": "AsphericFace", "kw": {"curvature": 70.0, "conic_const": 0.3, "A4": -2e-6,
                                                        "invert_normals": 1}, "shape": circ12},
        "extpoly": {"type": "ExtendedPolynomialFace", "kw": {"norm_radius": 10.0},
                    "attrs": {"curvature": 60.0, "conic_const": -0.2, "z_height": 0.5,
                              "coefs": rng.normal(0.0, 1e-3, (3, 3)).tolist()}, "shape": circ12},
        "extpoly_inv": {"type": "ExtendedPolynomialFace", "kw": {"norm_radius": 12.0, "invert_normals": 1},
                        "attrs": {"curvature": -80.0, "conic_const": 0.0, "z_height": 0.0,
                                  "coefs": rng.normal(0.0, 1e-4, (5, 5)).tolist()}, "shape": circ12},
        "zernike_plane": {"type": "DistortionFace", "kw": {"accuracy": 1e-6},
                          "base_face": {"type": "ShapedPlanarFace", "kw": {"z_height": 0.0}, "shape": circ12},
                          "distortion": {"type": "ZernikeDistortion", "coefs": zernike15(rng, 2e-3),
                                         "kw": {"unit_radius": 10.0}}, "shape": circ12},
        "j7_sphere": {"type": "DistortionFace", "kw": {"accuracy": 1e-7},
                      "base_face": {"type": "ShapedSphericalFace", "kw": {"curvature": 80.0}, "shape": circ12},
                      "distortion": {"type": "SimpleTestZernikeJ7", "kw": {"unit_radius": 10.0,
                                                                           "amplitude": 1e-3}},
                      "shape": circ12},
        "oriented_polygon": {"type": "OrientedPolygonFace",
                             "kw": {"origin": [0.5, 0.0, 0.0], "normal": [0.1, 0.0, -1.0],
                                    "x_axis": [1.0, 0.0, 0.1],
                                    "xy_points": [[-8.0, -6.0], [9.0, -5.0], [0.0, 9.0]]}},
        "polygon": {"type": "PolygonFace", "kw": {"z_plane": 0.0, "xy_points": PENTAGON["coordinates"]}},
        "elliptical": {"type": "ElipticalPlaneFace", "kw": {"g_x": 0.1, "g_y": -0.05},
                       "owner": {"diameter": 20.0}},
    }
    return faces


def face_scene(face):
    face = dict(face)
    face.setdefault("material", "glass")
    rot = W._random_rotation(np.random.Generator(np.random.PCG64(7)))
    small = np.eye(3) + 0.05 * (rot - np.eye(3))
    q, r = np.linalg.qr(small)
    q = q * np.sign(np.diag(r))[None, :]
    return {"materials": {"glass": _glass(), "mirror": {"type": "PECMaterial"},
                          "detector": {"type": "OpaqueMaterial"}},
            "lists": [{"rotation": q.tolist(), "translation": [0.3, -0.2, 20.0], "faces": [face]},
                      {"translation": [0, 0, 60.0], "faces": [
                          {"type": "CircularFace", "kw": {"z_plane": 0.0},
                           "owner": {"diameter": 400.0, "offset": 0.0}, "material": "detector"}]}]}


def ellipse_trans(f1, f2):
    """The owner's ellipse_trans of an ellipsoid with foci f1, f2 (ellipsoids.py
    config_trans): the face-list frame -> a frame with the major axis along x
    and the centre at the origin, with its exact inverse."""
    f1, f2 = np.asarray(f1, dtype=float), np.asarray(f2, dtype=float)
    c = (f1 + f2) / 2
    ex = (f2 - f1) / np.linalg.norm(f2 - f1)
    ey = np.cross([0.0, 0.0, 1.0], ex)
    ey /= np.linalg.norm(ey)
    ez = np.cross(ex, ey)
    R = np.stack([ex, ey, ez])
    M = np.eye(4)
    M[:3, :3] = R
    M[:3, 3] = -R @ c
    Mi = np.eye(4)
    Mi[:3, :3] = R.T
    Mi[:3, 3] = c
    return {"matrix": M.tolist(), "inverse": Mi.tolist()}


def face_zoo2():
    """The faces of the second set: off-axis paraboloid, ellipsoid, saddle,
    cylinder and axicon (cfaces.pyx:1224-1680)."""
    circ12 = {"type": "CircleShape", "kw": {"radius": 12.0}}
    f1, f2, size = (-4.0, 1.0, 2.0), (5.0, -2.0, 28.0), 60.0
    h = float(np.linalg.norm(np.subtract(f2, f1)))
    axes = [size / 2.0, 0.5 * math.sqrt(size ** 2 - h ** 2)]
    return {
        "oap": {"type": "OffAxisParabolicFace", "attrs": {"EFL": 12.0, "diameter": 30.0}, "material": "mirror",
                "rotate": False},
        "ellipsoid": {"type": "EllipsoidalFace", "material": "mirror",
                      "owner": {"ellipse_trans": ellipse_trans(f1, f2), "axes": axes, "X_bounds": [-20.0, 20.0],
                                "Y_bounds": [-20.0, 20.0], "Z_bounds": [2.0, 40.0]}},
        "saddle": {"type": "SaddleFace", "kw": {"z_height": 0.5, "curvature": 0.02}, "shape": circ12},
        "saddle_rect": {"type": "SaddleFace", "kw": {"z_height": -1.0, "curvature": -0.01}, "shape": RECT},
        "cylinder": {"type": "CylindericalFace", "kw": {"z_height": 0.0, "radius": 30.0}, "shape": circ12},
        "cylinder_neg": {"type": "CylindericalFace", "kw": {"z_height": 1.0, "radius": -25.0, "invert_normal": 1},
                         "shape": RECT},
        "axicon": {"type": "AxiconFace", "kw": {"z_height": 1.0, "gradient": 0.3}, "shape": circ12},
        "axicon_neg": {"type": "AxiconFace", "kw": {"z_height": -1.0, "gradient": -0.2}, "shape": PENTAGON},
    }


def face_scene2(face):
    face = dict(face)
    rotate = face.pop("rotate", True)
    spec = face_scene(face)
    if not rotate:
        spec["lists"][0].pop("rotation")
    return spec

def material_zoo():
    crown1 = {"formula_id": 1, "coefs": [0.0, 1.03961212, 0.0774596669, 0.231792344, 0.141484679, 1.01046945,
                                         10.1779013], "absorption": 2.0}
    poly3 = {"formula_id": 3, "coefs": [2.2, 0.011, 2.0, -0.01, -2.0, 1e-4, -4.0], "wavelength_min": 0.3}
    const0 = {"formula_id": 0, "coefs": [1.33], "absorption": 0.5}
    return {"curves": {"crown": W.CROWN, "flint": W.FLINT, "air": W.AIR, "crown1": crown1, "poly3": poly3,
                       "water": const0},
            "materials": {
                "opaque": {"type": "OpaqueMaterial"},
                "transparent": {"type": "TransparentMaterial"},
                "pec": {"type": "PECMaterial"},
                "partial": {"type": "PartiallyReflectiveMaterial", "kw": {"reflectivity": 0.3}},
                "linpol": {"type": "LinearPolarisingMaterial"},
                "waveplate": {"type": "WaveplateMaterial", "kw": {"retardance": 0.25, "fast_axis": [1.0, 1.0, 0.0]}},
                "dielectric": {"type": "DielectricMaterial", "kw": {"n_inside": [1.5, 0.01], "n_outside": 1.0}},
                "full_default": {"type": "FullDielectricMaterial", "kw": {"n_inside": 1.7, "n_outside": 1.0}},
                "full_split": {"type": "FullDielectricMaterial",
                               "kw": {"n_inside": [1.6, 0.02], "n_outside": 1.1,
                                      "reflection_threshold": -1.0, "transmission_threshold": -1.0}},
                "disp_sellmeier1": {"type": "FullDielectricDispersiveMaterial",
                                    "kw": {"dispersion_inside": "crown1", "dispersion_outside": "air",
                                           "reflection_threshold": -1.0, "transmission_threshold": -1.0}},
                "disp_sellmeier2": {"type": "FullDielectricDispersiveMaterial",
                                    "kw": {"dispersion_inside": "flint", "dispersion_outside": "crown"}},
                "disp_poly3": {"type": "FullDielectricDispersiveMaterial",
                               "kw": {"dispersion_inside": "poly3", "dispersion_outside": "water",
                                      "reflection_threshold": -1.0, "transmission_threshold": -1.0}},
                "aperture_circ": {"type": "CircularApertureMaterial",
                                  "kw": {"outer_radius": 15.0, "radius": 6.0, "edge_width": 1.5,
                                         "origin": [0.0, 0.0, 20.0]}},
                "aperture_circ_inv": {"type": "CircularApertureMaterial",
                                      "kw": {"outer_radius": 14.0, "radius": 4.0, "edge_width": 1.0,
                                             "origin": [0.5, 0.0, 20.0], "invert": 1}},
                "aperture_rect": {"type": "RectangularApertureMaterial",
                                  "kw": {"outer_width": 20.0, "outer_height": 16.0, "width": 8.0, "height": 5.0,
                                         "edge_width": 1.0, "origin": [0.0, 0.0, 20.0]}},
            }}


def coated_zoo():
    """Materials added after the first zoo -- thin-film coatings
    (SingleLayerCoatedMaterial, CoatedDispersiveMaterial) and diffraction
    gratings -- in their own fixtures."""
    crown1 = material_zoo()["curves"]["crown1"]
    mgf2 = {"formula_id": 0, "coefs": [1.38]}
    film = {"formula_id": 0, "coefs": [2.05], "absorption": 0.8}
    return {"curves": {"crown1": crown1, "flint": W.FLINT, "crown": W.CROWN, "air": W.AIR, "mgf2": mgf2,
                       "film": film},
            "materials": {
                "coated_single": {"type": "SingleLayerCoatedMaterial",
                                  "kw": {"n_inside": 1.5, "n_outside": 1.0, "n_coating": 1.38, "thickness": 0.1,
                                         "reflection_threshold": -1.0, "transmission_threshold": -1.0}},
                "coated_single_abs": {"type": "SingleLayerCoatedMaterial",
                                      "kw": {"n_inside": [1.7, 0.01], "n_outside": 1.0, "n_coating": [2.1, 0.005],
                                             "thickness": 0.35, "reflection_threshold": -1.0,
                                             "transmission_threshold": -1.0}},
                "coated_disp": {"type": "CoatedDispersiveMaterial",
                                "kw": {"dispersion_inside": "crown1", "dispersion_outside": "air",
                                       "dispersion_coating": "mgf2", "coating_thickness": 0.2,
                                       "reflection_threshold": -1.0, "transmission_threshold": -1.0}},
                "coated_disp_default": {"type": "CoatedDispersiveMaterial",
                                        "kw": {"dispersion_inside": "flint", "dispersion_outside": "crown",
                                               "dispersion_coating": "film", "coating_thickness": 0.15}},
                "grating": {"type": "DiffractionGratingMaterial",
                            "kw": {"lines_per_mm": 600.0, "order": 1, "efficiency": 0.8,
                                   "origin": [0.3, -0.2, 20.0]}},
                "grating_m2": {"type": "DiffractionGratingMaterial",
                               "kw": {"lines_per_mm": 1200.0, "order": -2, "efficiency": 1.0}},
            }}


def material_scene(mat_name, zoo=None):
    zoo = zoo or material_zoo()
    spec = {"curves": zoo["curves"], "materials": {mat_name: zoo["materials"][mat_name],
                                                   "detector": {"type": "OpaqueMaterial"}},
            "lists": [{"translation": [0, 0, 20.0], "faces": [
                {"type": "CircularFace", "kw": {"z_plane": 0.0}, "owner": {"diameter": 40.0, "offset": 0.0},
                 "material": mat_name}]},
                      {"translation": [0, 0, 0.0], "faces": [
                          {"type": "CircularFace", "kw": {"z_plane": -30.0},
                           "owner": {"diameter": 400.0, "offset": 0.0}, "material": "detector"},
                          {"type": "CircularFace", "kw": {"z_plane": 70.0, "invert_normals": 1},
                           "owner": {"diameter": 400.0, "offset": 0.0}, "material": "detector"}]}]}
    return spec


def random_rays(ray_dtype, rng, n, z0, zdir, tilt, spread, per_ray_wl=False, wl_range=(0.45, 0.9)):
    th = rng.uniform(0.0, tilt, n)
    ph = rng.uniform(0.0, 2 * math.pi, n)
    d = np.stack([np.sin(th) * np.cos(ph), np.sin(th) * np.sin(ph), zdir * np.cos(th)], axis=1)
    o = np.stack([rng.uniform(-spread, spread, n), rng.uniform(-spread, spread, n), np.full(n, z0)], axis=1)
    e1 = np.cross(np.array([0.0, 1.0, 0.0]), d)
    e1 /= np.linalg.norm(e1, axis=1)[:, None]
    rays = np.zeros(n, dtype=ray_dtype)
    W.fill_rays(rays, o, d, e1)
    rays['E1_amp'] = rng.normal(0, 1, n) + 1j * rng.normal(0, 1, n)
    rays['E2_amp'] = rng.normal(0, 1, n) + 1j * rng.normal(0, 1, n)
    rays['phase'] = rng.uniform(0, 1, n)
    rays['accumulated_path'] = rng.uniform(0, 5, n)
    rays['ray_type_id'] = rng.integers(0, 4, n)
    if per_ray_wl:
        rays['wavelength_idx'] = np.arange(n, dtype=np.uint32)
        return rays, rng.uniform(wl_range[0], wl_range[1], n)
    return rays, np.array([0.55])


# ---- running the reference --------------------------------------------------------------
def run_reference(ref, spec, rays, wl, recursion_limit, max_length):
    lists = W.build_scene(spec, ref)
    rc = ref.ctracer.RayCollection.from_array(rays.copy())
    rc.wavelengths = np.asarray(wl, dtype=np.double)
    with contextlib.redirect_stdout(io.StringIO()):
        traced, all_faces = ref.tracer.trace_rays(rc, lists, recursion_limit=recursion_limit, max_length=max_length)
    gens = [t.copy_as_array() for t in traced]
    counts = np.array([f.count for f in all_faces], dtype=np.uint32)
    return gens, counts


def save_trace_case(path, spec, rays, wl, params, gens, counts):
    offs = np.cumsum([0] + [len(g) for g in gens]).astype(np.uint64)
    out = np.concatenate(gens) if gens else np.zeros(0, dtype=rays.dtype)
    np.savez_compressed(path, spec=np.array(json.dumps(spec)), params=np.array(json.dumps(params)),
                        rays=rays, wl=np.asarray(wl, dtype=np.double), out=out, offsets=offs, counts=counts)


def index_digest(gens):
    h = hashlib.sha256()
    for g in gens:
        for f in ("wavelength_idx", "parent_idx", "end_face_idx", "ray_ident", "ray_type_id"):
            h.update(np.ascontiguousarray(g[f]).tobytes())
    return h.hexdigest()


def full_digest(g):
    return hashlib.sha256(np.ascontiguousarray(g).tobytes()).hexdigest()


def main():
    ref = build_ref.load()
    rdt = ref.ctracer.ray_dtype
    rng = np.random.Generator(np.random.PCG64(RNG_SEED))
    out_dir = HERE

    # configuration 1: full-size digests and a 64-ray subset in full
    spec1 = W.config1_spec()
    rays1, wl1 = W.config1_rays(rdt)
    P1 = dict(W.CONFIG1)
    gens, counts = run_reference(ref, spec1, rays1, wl1, P1["recursion_limit"], P1["max_length"])
    with open(os.path.join(out_dir, "config1_full.json"), "w") as f:
        json.dump({"n_rays": int(len(rays1)), "gen_sizes": [len(g) for g in gens],
                   "segments": int(sum(len(g) for g in gens)), "face_counts": counts.tolist(),
                   "index_sha256": index_digest(gens), "gen_sha256": [full_digest(g) for g in gens],
                   "params": P1}, f, indent=1)
    sub = rays1[::64].copy()
    sub['ray_ident'] = np.arange(len(sub), dtype=np.uint32) * 64
    gens, counts = run_reference(ref, spec1, sub, wl1, P1["recursion_limit"], P1["max_length"])
    save_trace_case(os.path.join(out_dir, "config1_sub64.npz"), spec1, sub, wl1, P1, gens, counts)

    # configuration 2: 24 rays spread over the 1,048,576-ray set
    rays2, wl2 = W.config2_rays(rdt)
    idx = np.linspace(0, len(rays2) - 1, 24).astype(np.int64)
    sub, swl = W.subsample(rays2, wl2, idx, per_ray_wavelength=True)
    P2 = dict(W.CONFIG2)
    gens, counts = run_reference(ref, W.config2_spec(), sub, swl, P2["recursion_limit"], P2["max_length"])
    save_trace_case(os.path.join(out_dir, "config2_sub24.npz"), W.config2_spec(), sub, swl, P2, gens, counts)

    # configuration 3: the first 48 rays of the 16,777,216-ray set
    rays3, wl3 = W.config3_rays(rdt, 48)
    P3 = dict(W.CONFIG3)
    gens, counts = run_reference(ref, W.config3_spec(), rays3, wl3, P3["recursion_limit"], P3["max_length"])
    save_trace_case(os.path.join(out_dir, "config3_sub48.npz"), W.config3_spec(), rays3, wl3, P3, gens, counts)

    # face zoo: each face type in its own scene, rays from both sides
    zoo = face_zoo(rng)
    units = {}
    for name, face in zoo.items():
        spec = face_scene(face)
        r1, wl = random_rays(rdt, rng, 40, -10.0, +1.0, 0.35, 13.0)
        r2, _ = random_rays(rdt, rng, 24, 45.0, -1.0, 0.35, 13.0)
        rays = np.concatenate([r1, r2])
        rays['ray_ident'] = np.arange(len(rays), dtype=np.uint32)
        params = {"recursion_limit": 4, "max_length": 200.0, "e2_terminate": 0.0}
        gens, counts = run_reference(ref, spec, rays, wl, params["recursion_limit"], params["max_length"])
        save_trace_case(os.path.join(out_dir, f"face_{name}.npz"), spec, rays, wl, params, gens, counts)
        # unit calls on the same face: intersect (base and non-base rays) and normals
        lists = W.build_scene(spec, ref)
        f = lists[0].faces[0]
        f.update()
        p1 = np.stack([rng.uniform(-14, 14, 64), rng.uniform(-14, 14, 64), rng.uniform(-30, -2, 64)], axis=1)
        p2 = np.stack([rng.uniform(-14, 14, 64), rng.uniform(-14, 14, 64), rng.uniform(2, 60, 64)], axis=1)
        p2[:8] = p1[:8] + np.array([0, 0, 80.0])
        d_base = np.array([f.intersect(tuple(a), tuple(b), 1) for a, b in zip(p1, p2)])
        d_free = np.array([f.intersect(tuple(a), tuple(b), 0) for a, b in zip(p1, p2)])
        pts = np.stack([rng.uniform(-9, 9, 32), rng.uniform(-9, 9, 32), rng.uniform(-1, 1, 32)], axis=1)
        nrm = np.array([f.compute_normal(tuple(p)) for p in pts])
        units[f"face_{name}_p1"] = p1
        units[f"face_{name}_p2"] = p2
        units[f"face_{name}_dist_base"] = d_base
        units[f"face_{name}_dist_free"] = d_free
        units[f"face_{name}_pts"] = pts
        units[f"face_{name}_normal"] = nrm
        shape = getattr(f, "shape", None)
        if shape is not None:
            xy = rng.uniform(-11, 11, (200, 2))
            units[f"face_{name}_xy"] = xy
            units[f"face_{name}_inside"] = np.array([bool(shape.point_inside(x, y)) for x, y in xy])
        if hasattr(f, "distortion") and f.distortion is not None:
            x = np.concatenate([[0.0, 1e-9], rng.uniform(-12, 12, 98)])
            y = np.concatenate([[0.0, 0.0], rng.uniform(-12, 12, 98)])
            units[f"face_{name}_dist_x"] = x
            units[f"face_{name}_dist_y"] = y
            units[f"face_{name}_dist_zg"] = np.asarray(f.distortion.z_offset_and_gradient(x, y))
            units[f"face_{name}_dist_z"] = np.asarray(f.distortion.z_offset(x, y))

    # material zoo: each material on a plane, rays from both sides at up to 70 degrees
    mz = material_zoo()
    for name in mz["materials"]:
        spec = material_scene(name)
        per_ray = name.startswith("disp_")
        r1, wla = random_rays(rdt, rng, 40, 0.0, +1.0, 1.2, 12.0, per_ray_wl=per_ray)
        r2, wlb = random_rays(rdt, rng, 24, 40.0, -1.0, 1.2, 12.0, per_ray_wl=per_ray)
        rays = np.concatenate([r1, r2])
        rays['ray_ident'] = np.arange(len(rays), dtype=np.uint32)
        if per_ray:
            rays['wavelength_idx'] = np.arange(len(rays), dtype=np.uint32)
            wl = np.concatenate([wla, wlb])
        else:
            wl = wla
        params = {"recursion_limit": 3, "max_length": 300.0, "e2_terminate": 0.0}
        gens, counts = run_reference(ref, spec, rays, wl, params["recursion_limit"], params["max_length"])
        save_trace_case(os.path.join(out_dir, f"mat_{name}.npz"), spec, rays, wl, params, gens, counts)
        # eval_child_ray unit calls with random orientations
        lists = W.build_scene(spec, ref)
        mat = lists[0].faces[0].material
        mat.wavelengths = np.asarray(wl, dtype=np.double)
        rc = ref.ctracer.RayCollection.from_array(rays.copy())
        nrm = rng.normal(0, 1, (len(rays), 3))
        nrm[:4] = rays['direction'][:4]          # normal incidence cases
        tng = rng.normal(0, 1, (len(rays), 3))
        pts = rng.uniform(-10, 10, (len(rays), 3))
        pts[:, 2] += 20.0
        kids, nk = [], []
        for i in range(len(rays)):
            out = ref.ctracer.RayCollection(2)
            mat.eval_child_ray(rc[i], i, tuple(pts[i]), tuple(nrm[i]), tuple(tng[i]), out)
            a = out.copy_as_array()
            nk.append(len(a))
            kids.append(a)
        units[f"mat_{name}_normals"] = nrm
        units[f"mat_{name}_tangents"] = tng
        units[f"mat_{name}_points"] = pts
        units[f"mat_{name}_nkids"] = np.array(nk)
        units[f"mat_{name}_kids"] = np.concatenate(kids) if kids else np.zeros(0, rdt)

    # Convert_to_SP
    rays, _ = random_rays(rdt, rng, 64, 0.0, 1.0, 1.0, 5.0)
    nrm = rng.normal(0, 1, (64, 3))
    nrm[:4] = rays['direction'][:4]
    rc = ref.ctracer.RayCollection.from_array(rays.copy())
    sp = [ref.cmaterials.Convert_to_SP(rc[i], tuple(nrm[i])) for i in range(64)]
    units["sp_rays"] = rays
    units["sp_normals"] = nrm
    tmp = ref.ctracer.RayCollection(64)
    for r in sp:
        tmp.add_ray(r)
    units["sp_out"] = tmp.copy_as_array()

    # dispersion curves
    wl = np.linspace(0.35, 1.6, 60)
    for name, c in material_zoo()["curves"].items():
        curve = W._make_curve(c, ref)
        units[f"curve_{name}_n"] = np.asarray(curve.evaluate_n(wl))
    units["curve_wl"] = wl
    units["curve_specs"] = np.array(json.dumps(material_zoo()["curves"]))

    np.savez_compressed(os.path.join(out_dir, "units.npz"), **units)
    np.savez_compressed(os.path.join(out_dir, "face_zoo_specs.npz"),
                        specs=np.array(json.dumps({k: face_scene(v) for k, v in zoo.items()})))
    lens_case(ref, out_dir)
    coated_case(ref, out_dir)
    faces2_case(ref, out_dir)
    sequential_case(ref, out_dir)
    gausslet_cases(ref, out_dir)
    capture_cases(ref, out_dir)
    field_cases(ref, out_dir)
    print("golden vectors written to", out_dir)


def coated_case(ref, out_dir):
    """The coated materials: trace cases mat_<name>.npz and eval_child_ray
    unit vectors in units_coated.npz, with their own random stream."""
    rdt = ref.ctracer.ray_dtype
    rng = np.random.Generator(np.random.PCG64(RNG_SEED + 41))
    zoo = coated_zoo()
    units = {}
    for name in zoo["materials"]:
        spec = material_scene(name, zoo)
        per_ray = name.startswith("coated_disp")
        r1, wla = random_rays(rdt, rng, 40, 0.0, +1.0, 1.2, 12.0, per_ray_wl=True, wl_range=(0.4, 1.0))
        r2, wlb = random_rays(rdt, rng, 24, 40.0, -1.0, 1.2, 12.0, per_ray_wl=True, wl_range=(0.4, 1.0))
        rays = np.concatenate([r1, r2])
        rays['ray_ident'] = np.arange(len(rays), dtype=np.uint32)
        rays['wavelength_idx'] = np.arange(len(rays), dtype=np.uint32)
        wl = np.concatenate([wla, wlb])
        params = {"recursion_limit": 3, "max_length": 300.0, "e2_terminate": 0.0}
        gens, counts = run_reference(ref, spec, rays, wl, params["recursion_limit"], params["max_length"])
        save_trace_case(os.path.join(out_dir, f"mat_{name}.npz"), spec, rays, wl, params, gens, counts)
        lists = W.build_scene(spec, ref)
        mat = lists[0].faces[0].material
        mat.wavelengths = np.asarray(wl, dtype=np.double)
        rc = ref.ctracer.RayCollection.from_array(rays.copy())
        nrm = rng.normal(0, 1, (len(rays), 3))
        nrm[:4] = rays['direction'][:4]
        tng = rng.normal(0, 1, (len(rays), 3))
        pts = rng.uniform(-10, 10, (len(rays), 3))
        pts[:, 2] += 20.0
        kids, nk = [], []
        for i in range(len(rays)):
            out = ref.ctracer.RayCollection(2)
            mat.eval_child_ray(rc[i], i, tuple(pts[i]), tuple(nrm[i]), tuple(tng[i]), out)
            a = out.copy_as_array()
            nk.append(len(a))
            kids.append(a)
        units[f"mat_{name}_normals"] = nrm
        units[f"mat_{name}_tangents"] = tng
        units[f"mat_{name}_points"] = pts
        units[f"mat_{name}_nkids"] = np.array(nk)
        units[f"mat_{name}_kids"] = np.concatenate(kids) if kids else np.zeros(0, rdt)
    np.savez_compressed(os.path.join(out_dir, "units_coated.npz"), **units)


def faces2_case(ref, out_dir):
    """The second face set: trace cases face_<name>.npz, unit vectors in
    units_faces2.npz and the scene specs in face_zoo2_specs.npz, with their
    own random stream."""
    rdt = ref.ctracer.ray_dtype
    rng = np.random.Generator(np.random.PCG64(RNG_SEED + 77))
    zoo = face_zoo2()
    units = {}
    specs = {}
    for name, face in zoo.items():
        spec = face_scene2(face)
        specs[name] = spec
        r1, wl = random_rays(rdt, rng, 40, -10.0, +1.0, 0.35, 13.0)
        r2, _ = random_rays(rdt, rng, 24, 45.0, -1.0, 0.35, 13.0)
        if name == "oap":  # axis-parallel rays take the reference's linear-root branch
            r1['direction'][:6] = (0.0, 0.0, 1.0)
            r1['E_vector'][:6] = (1.0, 0.0, 0.0)
            r1['origin'][:6, 0] = rng.uniform(9.5, 14.5, 6)
            r1['origin'][:6, 1] = rng.uniform(-2.5, 2.5, 6)
        rays = np.concatenate([r1, r2])
        rays['ray_ident'] = np.arange(len(rays), dtype=np.uint32)
        params = {"recursion_limit": 4, "max_length": 200.0, "e2_terminate": 0.0}
        gens, counts = run_reference(ref, spec, rays, wl, params["recursion_limit"], params["max_length"])
        save_trace_case(os.path.join(out_dir, f"face_{name}.npz"), spec, rays, wl, params, gens, counts)
        lists = W.build_scene(spec, ref)
        f = lists[0].faces[0]
        f.update()
        p1 = np.stack([rng.uniform(-14, 14, 64), rng.uniform(-14, 14, 64), rng.uniform(-30, -2, 64)], axis=1)
        p2 = np.stack([rng.uniform(-14, 14, 64), rng.uniform(-14, 14, 64), rng.uniform(2, 60, 64)], axis=1)
        if name == "oap":
            p1[:8, 0] = rng.uniform(9.5, 14.5, 8)
            p1[:8, 1] = rng.uniform(-2.5, 2.5, 8)
        p2[:8] = p1[:8] + np.array([0, 0, 80.0])
        p2[8:12, 0] = p1[8:12, 0]   # d.x == 0 only
        p2[12:16, 1] = p1[12:16, 1]  # d.y == 0 only
        d_base = np.array([f.intersect(tuple(a), tuple(b), 1) for a, b in zip(p1, p2)])
        d_free = np.array([f.intersect(tuple(a), tuple(b), 0) for a, b in zip(p1, p2)])
        pts = np.stack([rng.uniform(-9, 9, 32), rng.uniform(-9, 9, 32), rng.uniform(-1, 1, 32)], axis=1)
        nrm = np.array([f.compute_normal(tuple(p)) for p in pts])
        units[f"face_{name}_p1"] = p1
        units[f"face_{name}_p2"] = p2
        units[f"face_{name}_dist_base"] = d_base
        units[f"face_{name}_dist_free"] = d_free
        units[f"face_{name}_pts"] = pts
        units[f"face_{name}_normal"] = nrm
    np.savez_compressed(os.path.join(out_dir, "units_faces2.npz"), **units)
    np.savez_compressed(os.path.join(out_dir, "face_zoo2_specs.npz"), specs=np.array(json.dumps(specs)))


def sequential_case(ref, out_dir):
    """core/tracer.py trace_ray_sequence on the configuration-1 lens: each
    face list appears twice in the sequence, so face.idx is each face's last
    position in the chained face list, as the reference assigns it."""
    rdt = ref.ctracer.ray_dtype
    rng = np.random.Generator(np.random.PCG64(RNG_SEED + 91))
    spec = W.config1_spec()
    seq = [[0, 0], [0, 1], [1, 0], [1, 1], [2, 0]]
    rays, wl = random_rays(rdt, rng, 64, -5.0, +1.0, 0.2, 6.0)
    rays['ray_ident'] = np.arange(len(rays), dtype=np.uint32)
    params = {"recursion_limit": 10, "max_length": 1000.0, "sequence": seq}
    lists = W.build_scene(spec, ref)
    rc = ref.ctracer.RayCollection.from_array(rays.copy())
    rc.wavelengths = np.asarray(wl, dtype=np.double)
    with contextlib.redirect_stdout(io.StringIO()):
        traced, all_faces = ref.tracer.trace_ray_sequence(rc, [(lists[l], f) for l, f in seq],
                                                          recursion_limit=params["recursion_limit"],
                                                          max_length=params["max_length"])
    gens = [t.copy_as_array() for t in traced]
    counts = np.array([f.count for f in all_faces], dtype=np.uint32)
    save_trace_case(os.path.join(out_dir, "seq_config1.npz"), spec, rays, wl, params, gens, counts)


def gausslets_from_rays(ref, rays, wl, radius=0.05, working_dist=0.0, gausslet_bit=False):
    """Gausslets of the reference built from rays: GaussletCollection.from_rays
    then config_parabasal_rays (ctracer.pyx:1320-1343, 1430-1476)."""
    r = rays.copy()
    if gausslet_bit:
        r['ray_type_id'] |= 2
    gc = ref.ctracer.GaussletCollection.from_rays(r)
    gc.config_parabasal_rays(np.asarray(wl, dtype=np.double), radius, working_dist)
    return gc.copy_as_array()


def run_reference_gausslets(ref, spec, gausslets, wl, recursion_limit, max_length, sequence=None):
    lists = W.build_scene(spec, ref)
    gc = ref.ctracer.GaussletCollection.from_array(gausslets.copy())
    gc.wavelengths = np.asarray(wl, dtype=np.double)
    with contextlib.redirect_stdout(io.StringIO()):
        if sequence is None:
            traced, all_faces = ref.tracer.trace_rays(gc, lists, recursion_limit=recursion_limit,
                                                      max_length=max_length)
        else:
            traced, all_faces = ref.tracer.trace_ray_sequence(gc, [(lists[l], f) for l, f in sequence],
                                                              recursion_limit=recursion_limit,
                                                              max_length=max_length)
    gens = [t.copy_as_array() for t in traced]
    counts = np.array([f.count for f in all_faces], dtype=np.uint32)
    return gens, counts


def gausslet_cases(ref, out_dir):
    """Gausslet tracing (trace_gausslet_c / trace_one_face_gausslet_c): trace
    cases gauss_<name>.npz and eval_parabasal_ray unit vectors in
    units_gausslet.npz, with their own random stream."""
    gdt = ref.ctracer.gausslet_dtype
    rdt = ref.ctracer.ray_dtype
    rng = np.random.Generator(np.random.PCG64(RNG_SEED + 123))
    cases = {}
    # the configuration-1 lens, non-sequential and sequential
    spec1 = W.config1_spec()
    r, wl = random_rays(rdt, rng, 48, -5.0, +1.0, 0.15, 5.0)
    cases["config1"] = (spec1, gausslets_from_rays(ref, r, wl, 0.05, 2.0), wl,
                        {"recursion_limit": 6, "max_length": 1000.0})
    cases["seq_config1"] = (spec1, gausslets_from_rays(ref, r, wl, 0.02, -1.0), wl,
                            {"recursion_limit": 10, "max_length": 1000.0,
                             "sequence": [[0, 0], [0, 1], [1, 0], [1, 1], [2, 0]]})
    # each parabasal evaluation: base (PEC, dispersive, partial), dielectric, coatings, grating
    zoo = material_zoo()
    czoo = coated_zoo()
    for name, z in (("pec", zoo), ("disp_sellmeier1", zoo), ("partial", zoo), ("full_split", zoo),
                    ("dielectric", zoo), ("coated_single", czoo), ("coated_disp", czoo), ("grating", czoo),
                    ("grating_m2", czoo)):
        spec = material_scene(name, z)
        r1, wla = random_rays(rdt, rng, 24, 0.0, +1.0, 0.6, 10.0, per_ray_wl=True, wl_range=(0.4, 1.0))
        r2, wlb = random_rays(rdt, rng, 16, 40.0, -1.0, 0.6, 10.0, per_ray_wl=True, wl_range=(0.4, 1.0))
        rays = np.concatenate([r1, r2])
        rays['ray_ident'] = np.arange(len(rays), dtype=np.uint32)
        rays['wavelength_idx'] = np.arange(len(rays), dtype=np.uint32)
        wl = np.concatenate([wla, wlb])
        cases["mat_" + name] = (spec, gausslets_from_rays(ref, rays, wl, 0.1, 0.5), wl,
                                {"recursion_limit": 3, "max_length": 300.0})
    # decomposition: a ResampleGaussletMaterial plane between two detectors
    spec = material_scene("resample", {"curves": {}, "materials": {
        "resample": {"type": "ResampleGaussletMaterial", "kw": {"eval_func": "resample_shift"}}}})
    r, wl = random_rays(rdt, rng, 32, 0.0, +1.0, 0.5, 10.0)
    g = gausslets_from_rays(ref, r, wl, 0.05, 0.0, gausslet_bit=True)
    g['base_ray']['ray_type_id'][::4] &= ~np.uint32(2)  # some are not captured
    cases["resample"] = (spec, g, wl, {"recursion_limit": 4, "max_length": 300.0})
    for name, (spec, g, wl, params) in cases.items():
        gens, counts = run_reference_gausslets(ref, spec, g, wl, params["recursion_limit"], params["max_length"],
                                               params.get("sequence"))
        offs = np.cumsum([0] + [len(x) for x in gens]).astype(np.uint64)
        out = np.concatenate(gens) if gens else np.zeros(0, dtype=gdt)
        np.savez_compressed(os.path.join(out_dir, f"gauss_{name}.npz"), spec=np.array(json.dumps(spec)),
                            params=np.array(json.dumps(params)), gausslets=g, wl=np.asarray(wl, dtype=np.double),
                            out=out, offsets=offs, counts=counts)
    # eval_parabasal_ray unit calls of every material
    units = {}
    allm = dict(zoo["materials"])
    allm.update(czoo["materials"])
    curves = dict(zoo["curves"])
    curves.update(czoo["curves"])
    for name, mspec in allm.items():
        spec = {"curves": curves, "materials": {name: mspec, "detector": {"type": "OpaqueMaterial"}},
                "lists": [{"faces": [{"type": "CircularFace", "kw": {"z_plane": 0.0},
                                      "owner": {"diameter": 40.0, "offset": 0.0}, "material": name}]}]}
        lists = W.build_scene(spec, ref)
        mat = lists[0].faces[0].material
        n = 32
        wl = rng.uniform(0.45, 0.9, n)
        mat.wavelengths = wl
        base, _ = random_rays(rdt, rng, n, 0.0, 1.0, 0.8, 5.0, per_ray_wl=True)
        base['wavelength_idx'] = np.arange(n, dtype=np.uint32)
        base['refractive_index'] = rng.uniform(1.0, 1.7, n) + 0j
        dirs = rng.normal(0, 1, (n, 3))
        dirs[:, 2] = np.abs(dirs[:, 2]) + 0.5
        dirs[n // 2:, 2] *= -1
        pts = rng.uniform(-5, 5, (n, 3))
        nrm = rng.normal(0, 1, (n, 3))
        nrm[:, 2] = np.abs(nrm[:, 2]) + 1.0
        tng = rng.normal(0, 1, (n, 3))
        refl = (np.arange(n) % 2).astype(bool)
        rc = ref.ctracer.RayCollection.from_array(base.copy())
        out = np.zeros(n, dtype=ref.ctracer.para_dtype)
        for i in range(n):
            p = mat.eval_parabasal_ray(rc[i], tuple(dirs[i]), tuple(pts[i]), tuple(nrm[i]), tuple(tng[i]),
                                       bool(refl[i]))
            out[i] = (p.origin, p.direction, p.normal, p.length)
        units[f"para_{name}_spec"] = np.array(json.dumps(spec))
        units[f"para_{name}_wl"] = wl
        units[f"para_{name}_base"] = base
        units[f"para_{name}_dirs"] = dirs
        units[f"para_{name}_points"] = pts
        units[f"para_{name}_normals"] = nrm
        units[f"para_{name}_tangents"] = tng
        units[f"para_{name}_refl"] = refl
        units[f"para_{name}_out"] = out
    np.savez_compressed(os.path.join(out_dir, "units_gausslet.npz"), **units)


def capture_cases(ref, out_dir):
    """select_ray_intersections / select_gausslet_intersections on traced
    generations of the configuration-1 lens (three wavelengths listed out of
    order, so the merge onto unique values is exercised)."""
    rdt = ref.ctracer.ray_dtype
    rng = np.random.Generator(np.random.PCG64(RNG_SEED + 211))
    spec = W.config1_spec()
    wl = np.array([0.65, 0.45, 0.55])
    rays, _ = random_rays(rdt, rng, 64, -5.0, +1.0, 0.12, 6.0)
    rays['wavelength_idx'] = rng.integers(0, 3, len(rays))
    params = {"recursion_limit": 5, "max_length": 1000.0}
    lists = W.build_scene(spec, ref)
    rc = ref.ctracer.RayCollection.from_array(rays.copy())
    rc.wavelengths = wl
    with contextlib.redirect_stdout(io.StringIO()):
        traced, _ = ref.tracer.trace_rays(rc, lists, recursion_limit=params["recursion_limit"],
                                          max_length=params["max_length"])
    out = {}
    for li in (1, 2):
        sel = ref.ctracer.select_ray_intersections(lists[li], traced)
        out[f"rays_list{li}"] = sel.copy_as_array()
        out[f"rays_list{li}_wl"] = np.asarray(sel.wavelengths)
    gens = [t.copy_as_array() for t in traced]
    offs = np.cumsum([0] + [len(g) for g in gens]).astype(np.uint64)
    g = gausslets_from_rays(ref, rays, wl, 0.05, 1.0)
    gc = ref.ctracer.GaussletCollection.from_array(g.copy())
    gc.wavelengths = wl
    lists = W.build_scene(spec, ref)
    with contextlib.redirect_stdout(io.StringIO()):
        gtraced, _ = ref.tracer.trace_rays(gc, lists, recursion_limit=params["recursion_limit"],
                                           max_length=params["max_length"])
    for li in (1, 2):
        sel = ref.ctracer.select_gausslet_intersections(lists[li], gtraced)
        out[f"gausslets_list{li}"] = sel.copy_as_array()
        out[f"gausslets_list{li}_wl"] = np.asarray(sel.wavelengths)
    ggens = [t.copy_as_array() for t in gtraced]
    goffs = np.cumsum([0] + [len(x) for x in ggens]).astype(np.uint64)
    np.savez_compressed(os.path.join(out_dir, "units_capture.npz"), spec=np.array(json.dumps(spec)),
                        params=np.array(json.dumps(params)), wl=wl, rays=rays, gens=np.concatenate(gens),
                        offsets=offs, gausslets=g, ggens=np.concatenate(ggens), goffsets=goffs, **out)


def hex_field(rdt, radius, spacing, z0=0.0):
    """Rays on a hexagonal lattice travelling along +z, with the indices of
    each ray's six lattice neighbours (-1 where the lattice ends)."""
    m = int(radius / spacing) + 2
    i, j = np.meshgrid(np.arange(-m, m + 1), np.arange(-m, m + 1))
    x = (i + 0.5 * j).reshape(-1) * spacing
    y = (j * math.sqrt(3.0) / 2.0).reshape(-1) * spacing
    keep = x * x + y * y <= radius * radius
    x, y = x[keep], y[keep]
    n = len(x)
    rays = np.zeros(n, dtype=rdt)
    W.fill_rays(rays, np.stack([x, y, np.full(n, z0)], axis=1), (0.0, 0.0, 1.0), (1.0, 0.0, 0.0))
    nb = np.full((n, 6), -1, dtype=np.int32)
    for k in range(n):
        for a in range(6):
            ang = a * math.pi / 3.0
            tx, ty = x[k] + spacing * math.cos(ang), y[k] + spacing * math.sin(ang)
            hit = np.flatnonzero(np.hypot(x - tx, y - ty) < 1e-6 * spacing)
            if hit.size:
                nb[k, a] = hit[0]
    return rays, nb


def field_cases(ref, out_dir):
    """The E-field consumers (cfields.pyx, core/fields.py): single-call
    evaluate_modes and sum_gaussian_modes vectors, eval_Efield_from_gausslets
    of a gausslet beam before and after the configuration-1 lens,
    EFieldSummation at a non-zero time, and eval_Efield_from_rays of a
    hexagonal ray field."""
    rdt = ref.ctracer.ray_dtype
    rng = np.random.Generator(np.random.PCG64(RNG_SEED + 307))
    u = {}
    # evaluate_modes on random parabasal offsets
    x = rng.normal(0, 0.1, (64, 6))
    y = rng.normal(0, 0.1, (64, 6))
    dx = rng.normal(0, 1e-3, (64, 6))
    dy = rng.normal(0, 1e-3, (64, 6))
    u.update(modes_x=x, modes_y=y, modes_dx=dx, modes_dy=dy,
             modes_out=np.asarray(ref.cfields.evaluate_modes(x, y, dx, dy, 1.3)))
    # sum_gaussian_modes on random modes (positive widths) near their origins
    n = 48
    r, _ = random_rays(rdt, rng, n, 0.0, 1.0, 0.05, 0.5, per_ray_wl=True, wl_range=(0.5, 0.9))
    r['wavelength_idx'] = rng.integers(0, 3, n)
    r['refractive_index'] = 1.0 + 1e-4j
    modes = rng.normal(0, 0.01, (n, 3)) + 1j * np.column_stack([rng.uniform(20, 40, n), rng.uniform(-2, 2, n),
                                                                 rng.uniform(20, 40, n)])
    wl = np.array([0.6, 0.55, 0.8])
    pts = np.column_stack([rng.uniform(-0.6, 0.6, 300), rng.uniform(-0.6, 0.6, 300), rng.uniform(-1, 30, 300)])
    rc = ref.ctracer.RayCollection.from_array(r.copy())
    u.update(sum_rays=r, sum_modes=modes, sum_wl=wl, sum_points=pts,
             sum_E=np.asarray(ref.cfields.sum_gaussian_modes(rc, modes, wl, pts, 0.0)),
             sum_E_t=np.asarray(ref.cfields.sum_gaussian_modes(rc, modes, wl, pts, 2.5)))
    # a gausslet beam: on its own, and after the configuration-1 lens
    rays, nb = hex_field(rdt, 2.0, 0.4)
    wl = np.array([0.6])
    g = gausslets_from_rays(ref, rays, wl, 0.25, 0.0)
    gc = ref.ctracer.GaussletCollection.from_array(g.copy())
    gc.wavelengths = wl
    gx, gy = np.meshgrid(np.linspace(-2.5, 2.5, 15), np.linspace(-2.5, 2.5, 15))
    plane = np.column_stack([gx.reshape(-1), gy.reshape(-1), np.full(gx.size, 10.0)])
    u.update(beam_gausslets=g, beam_wl=wl, beam_points=plane,
             beam_E=np.asarray(ref.fields.eval_Efield_from_gausslets(gc, plane)))
    lists = W.build_scene(W.config1_spec(), ref)
    gc = ref.ctracer.GaussletCollection.from_array(g.copy())
    gc.wavelengths = wl
    with contextlib.redirect_stdout(io.StringIO()):
        traced, _ = ref.tracer.trace_rays(gc, lists, recursion_limit=4, max_length=1000.0)
    after = traced[3].copy_as_array()   # the gausslets leaving the lens towards the detector
    fx, fz = np.meshgrid(np.linspace(-0.3, 0.3, 13), np.linspace(60.0, 110.0, 11))
    focus = np.column_stack([fx.reshape(-1), np.zeros(fx.size), fz.reshape(-1)])
    lens_gc = ref.ctracer.GaussletCollection.from_array(after.copy())
    lens_gc.wavelengths = wl
    summ = ref.fields.EFieldSummation(lens_gc)
    u.update(lens_gausslets=after, lens_points=focus,
             lens_E=np.asarray(ref.fields.eval_Efield_from_gausslets(lens_gc, focus)),
             lens_E_t=np.asarray(summ.evaluate(focus.copy(), time_ps=0.7)))
    # a ray field with lattice neighbours
    rc = ref.ctracer.RayCollection.from_array(rays.copy())
    rc.neighbours = nb
    u.update(rf_rays=rays, rf_neighbours=nb, rf_points=plane,
             rf_E=np.asarray(ref.fields.eval_Efield_from_rays(rc, plane, wl, blending=1.0)))
    np.savez_compressed(os.path.join(out_dir, "units_fields.npz"), **u)


def field_decomp_cases(ref, out_dir):
    """The decomposition helpers of cfields.pyx: calc_mode_curvature on random
    slopes and second derivatives, build_interaction_matrix of modes on a
    hexagonal lattice against a finer square grid of test points (its output
    buffer estimate, 176 entries per mode, covers the ~80 pairs per mode), and
    apply_mode_curvature on a gausslet beam."""
    rdt = ref.ctracer.ray_dtype
    rng = np.random.Generator(np.random.PCG64(RNG_SEED + 311))
    u = {}
    n = 40
    dx, dy = rng.normal(0, 0.05, n), rng.normal(0, 0.05, n)
    dx2, dy2, dxdy = rng.normal(0, 0.02, n), rng.normal(0, 0.02, n), rng.normal(0, 0.01, n)
    rx, ry = rng.uniform(-1, 1, n), rng.uniform(-1, 1, n)
    u.update(mc_rx=rx, mc_ry=ry, mc_dx=dx, mc_dy=dy, mc_dx2=dx2, mc_dy2=dy2, mc_dxdy=dxdy)
    for k, v in zip("ABCXYZ", ref.cfields.calc_mode_curvature(rx, ry, dx, dy, dx2, dy2, dxdy)):
        u["mc_" + k] = np.asarray(v)
    # interaction matrix: modes 0.1 mm apart, test points every 0.05 mm
    rays, _ = hex_field(rdt, 0.6, 0.1)
    mx, my = rays['origin'][:, 0].copy(), rays['origin'][:, 1].copy()
    m = len(mx)
    A, B, C, X, Y, Z = ref.cfields.calc_mode_curvature(mx, my, rng.normal(0, 0.02, m), rng.normal(0, 0.02, m),
                                                       rng.normal(0, 0.5, m), rng.normal(0, 0.5, m),
                                                       rng.normal(0, 0.2, m))
    g = np.linspace(-0.7, 0.7, 29)
    tx, ty = [v.reshape(-1).copy() for v in np.meshgrid(g, g)]
    args = dict(wavelength=0.6, spacing=0.1, max_spacing=0.25, blending=1.0, test_spacing=0.05)
    data, (xi, xj) = ref.cfields.build_interaction_matrix(mx, my, tx, ty, np.asarray(A), np.asarray(B),
                                                           np.asarray(C), np.asarray(X), np.asarray(Y),
                                                           np.asarray(Z), args["wavelength"], args["spacing"],
                                                           args["max_spacing"], args["blending"],
                                                           args["test_spacing"])
    u.update(im_rx=mx, im_ry=my, im_tx=tx, im_ty=ty, im_A=np.asarray(A), im_B=np.asarray(B), im_C=np.asarray(C),
             im_X=np.asarray(X), im_Y=np.asarray(Y), im_Z=np.asarray(Z),
             im_args=np.array([args[k] for k in ("wavelength", "spacing", "max_spacing", "blending",
                                                   "test_spacing")]),
             im_data=np.asarray(data), im_i=np.asarray(xi).astype(np.uint64), im_j=np.asarray(xj).astype(np.uint64))
    # apply_mode_curvature on a gausslet beam
    beam, _ = hex_field(rdt, 2.0, 0.4)
    gl = gausslets_from_rays(ref, beam, np.array([0.6]), 0.25, 0.0)
    k = len(gl)
    cA, cB, cC = rng.normal(0, 0.01, k), rng.normal(0, 0.005, k), rng.normal(0, 0.01, k)
    gc = ref.ctracer.GaussletCollection.from_array(gl.copy())
    ref.cfields.apply_mode_curvature(gc, cA, cB, cC)
    u.update(ac_gausslets=gl, ac_A=cA, ac_B=cB, ac_C=cC, ac_out=gc.copy_as_array())
    np.savez_compressed(os.path.join(out_dir, "units_fields2.npz"), **u)


def lens_case(ref, out_dir):
    """Configuration 4: the perturbed eight-surface lens as an ordinary scene
    (AsphericFace + DielectricMaterial, image plane), 64 rays of the 262,144-ray
    grid, traced by the reference's trace_rays."""
    rays4, wl4 = W.config4_rays(ref.ctracer.ray_dtype)
    idx = np.linspace(0, len(rays4) - 1, 64).astype(np.int64)
    sub = rays4[idx].copy()
    spec = W.config4_spec(W.config4_params())
    P4 = {"recursion_limit": 10, "max_length": W.CONFIG4["max_length"], "e2_terminate": 0.0}
    gens, counts = run_reference(ref, spec, sub, wl4, P4["recursion_limit"], P4["max_length"])
    save_trace_case(os.path.join(out_dir, "config4_sub64.npz"), spec, sub, wl4, P4, gens, counts)


if __name__ == "__main__":
    if sys.argv[1:] == ["--lens"]:
        lens_case(build_ref.load(), HERE)
    elif sys.argv[1:] == ["--coated"]:
        coated_case(build_ref.load(), HERE)
    elif sys.argv[1:] == ["--faces2"]:
        faces2_case(build_ref.load(), HERE)
    elif sys.argv[1:] == ["--sequential"]:
        sequential_case(build_ref.load(), HERE)
    elif sys.argv[1:] == ["--gausslets"]:
        gausslet_cases(build_ref.load(), HERE)
    elif sys.argv[1:] == ["--capture"]:
        capture_cases(build_ref.load(), HERE)
    elif sys.argv[1:] == ["--fields"]:
        field_cases(build_ref.load(), HERE)
    elif sys.argv[1:] == ["--fields2"]:
        field_decomp_cases(build_ref.load(), HERE)
    else:
        main()
