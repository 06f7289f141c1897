"""GPU parity: the sm_103a plain FP64 path against the reference's golden
vectors and against the C oracle, through the same API a reference user
calls (trace_rays / trace_segment / the single-plugin methods).

Tolerances: every index field (end_face_idx, parent_idx, ray_ident,
wavelength_idx, ray_type_id), the generation sizes and the face hit counts
are bit-exact; every floating-point field agrees within rtol=1e-9
(atol=1e-12 for values at zero)."""
import hashlib
import json
import os

import numpy as np
import pytest

import oracle
from helpers import (GOLDEN, assert_generations, assert_records, build, face_unit_names, load_case, oracle_trace_parallel,
                     load_face_specs, load_units, material_unit_names, tables_for, trace_case_names)
from raypier_optics_gb300 import cmaterials, ctracer, scene, tracer, unitcalls
from raypier_optics_gb300 import workloads as W
from raypier_optics_gb300.ctracer import RayCollection

pytestmark = pytest.mark.gpu


def gpu_trace(spec, rays, wl, recursion_limit, max_length, e2=0.0):
    lists, _ = build(spec)
    rc = RayCollection.from_array(rays)
    rc.wavelengths = wl
    traced, faces = tracer.trace_rays(rc, lists, recursion_limit=recursion_limit, max_length=max_length,
                                      e2_terminate=e2)
    return [t.copy_as_array() for t in traced], np.array([f.count for f in faces])


@pytest.mark.parametrize("name", trace_case_names())
def test_gpu_trace_matches_reference_golden(name):
    c = load_case(name)
    p = c["params"]
    gens, counts = gpu_trace(c["spec"], c["rays"], c["wl"], p["recursion_limit"], p["max_length"])
    assert_generations(gens, c["gens"], what=name)
    np.testing.assert_array_equal(counts, c["counts"])


def test_gpu_config1_full_size_matches_reference_digest_and_oracle():
    ref = json.load(open(os.path.join(GOLDEN, "config1_full.json")))
    rays, wl = W.config1_rays(ctracer.ray_dtype)
    gens, counts = gpu_trace(W.config1_spec(), rays, wl, 6, 1000.0, 1e-6)
    assert [len(g) for g in gens] == ref["gen_sizes"]
    assert counts.tolist() == ref["face_counts"]
    h = hashlib.sha256()
    for g in gens:
        for f in ("wavelength_idx", "parent_idx", "end_face_idx", "ray_ident", "ray_type_id"):
            h.update(np.ascontiguousarray(g[f]).tobytes())
    assert h.hexdigest() == ref["index_sha256"]
    tables, _, _ = tables_for(W.config1_spec())
    ogens, _ = oracle.trace_rays(tables, wl, rays, 6, 1000.0, 1e-6)
    assert_generations(gens, ogens, what="config1")


@pytest.mark.parametrize("n", [1, 127, 128, 129, 4097, 65536])
def test_gpu_config1_ragged_sizes_match_oracle(n):
    rays, wl = W.config1_rays(ctracer.ray_dtype, max(n, 4096))
    rays = rays[:n]
    gens, _ = gpu_trace(W.config1_spec(), rays, wl, 6, 1000.0)
    tables, _, _ = tables_for(W.config1_spec())
    ogens, _ = oracle.trace_rays(tables, wl, rays, 6, 1000.0)
    assert_generations(gens, ogens, what=f"config1 n={n}")


def test_gpu_empty_input():
    rays = np.zeros(0, dtype=ctracer.ray_dtype)
    gens, counts = gpu_trace(W.config1_spec(), rays, np.array([0.55]), 6, 1000.0)
    assert gens == [] and counts.sum() == 0


def test_gpu_all_rays_miss():
    rays, wl = W.config1_rays(ctracer.ray_dtype, 300)
    rays['direction'] = (0.0, 0.0, -1.0)
    gens, counts = gpu_trace(W.config1_spec(), rays, wl, 6, 1000.0)
    assert len(gens) == 1 and counts.sum() == 0
    assert np.all(gens[0]['end_face_idx'] == 0xFFFFFFFF)
    assert np.all(gens[0]['length'] == 1000.0)


def test_gpu_config2_subsample_with_termination_matches_oracle():
    rays, wl = W.config2_rays(ctracer.ray_dtype, 1 << 20)
    idx = np.arange(0, 1 << 20, 256)
    sub, swl = W.subsample(rays, wl, idx, per_ray_wavelength=True)
    gens, counts = gpu_trace(W.config2_spec(), sub, swl, 8, 1000.0, 1e-6)
    tables, _, _ = tables_for(W.config2_spec())
    ogens, ocounts = oracle.trace_rays(tables, swl, sub, 8, 1000.0, 1e-6)
    assert_generations(gens, ogens, what="config2 subsample")
    np.testing.assert_array_equal(counts, ocounts[:tables.n_faces])


def test_gpu_config3_subsample_matches_oracle():
    rays, wl = W.config3_rays(ctracer.ray_dtype, 1024)
    gens, counts = gpu_trace(W.config3_spec(), rays, wl, 12, 1000.0, 1e-6)
    tables, _, _ = tables_for(W.config3_spec())
    ogens, ocounts = oracle.trace_rays(tables, wl, rays, 12, 1000.0, 1e-6)
    assert_generations(gens, ogens, what="config3 subsample")
    np.testing.assert_array_equal(counts, ocounts[:tables.n_faces])


def test_gpu_config3_65536_rays_match_oracle():
    """The 64-face clutter scene (Zernike-distorted planes, polynomial faces,
    prisms, spheres, conic mirrors; 12 generations) on the first 65,536 rays
    of its 16,777,216-ray workload: hit face, parent, ray count and
    termination bit-exact, floats within 1e-9, face hit counts equal."""
    rays, wl = W.config3_rays(ctracer.ray_dtype, 65536)
    gens, counts = gpu_trace(W.config3_spec(), rays, wl, 12, 1000.0, 1e-6)
    tables, _, _ = tables_for(W.config3_spec())
    ogens, ocounts = oracle_trace_parallel(tables, wl, rays, 12, 1000.0, 1e-6, counts=True)
    assert_generations(gens, ogens, what="config3 65536 rays")
    np.testing.assert_array_equal(counts, ocounts[:tables.n_faces])


def test_gpu_trace_segment_mutates_input_and_appends_children_in_order():
    c = load_case("config2_sub24")
    lists, all_faces = build(c["spec"])
    rc = RayCollection.from_array(c["rays"])
    rc.wavelengths = c["wl"]
    children = ctracer.trace_segment(rc, lists, all_faces, max_length=1000.0)
    tables, _, _ = tables_for(c["spec"])
    mutated, kids, ocounts = oracle.trace_segment(tables, c["wl"], c["rays"], 1000.0)
    assert_records(rc.copy_as_array(), mutated, what="mutated input")
    assert_records(children.copy_as_array(), kids, what="children")
    assert children.parent is rc
    np.testing.assert_array_equal([f.count for f in all_faces], ocounts[:tables.n_faces])


def test_gpu_trace_segment_loop_uploads_scene_once():
    """A caller's own generation loop over trace_segment (the reference's
    core/tracer.py:36-45 loop) uploads the scene once; a changed face
    parameter uploads a new one, and every generation still equals the
    oracle's."""
    from raypier_optics_gb300 import runtime
    c = load_case("config2_sub24")
    lists, all_faces = build(c["spec"])
    ctx = runtime.get_context()

    def run_loop(n_gens):
        rc = RayCollection.from_array(c["rays"])
        rc.wavelengths = c["wl"]
        tables = scene.compile_scene(lists)
        host = c["rays"]
        for g in range(n_gens):
            if rc.n_rays == 0:
                break
            kids = ctracer.trace_segment(rc, lists, all_faces, max_length=1000.0)
            mutated, okids, _ = oracle.trace_segment(tables, c["wl"], host, 1000.0)
            assert_records(rc.copy_as_array(), mutated, what=f"generation {g} input")
            assert_records(kids.copy_as_array(), okids, what=f"generation {g} children")
            rc, host = kids, okids

    all_faces[0].curvature *= 1.001   # a scene no earlier test uploaded
    before = getattr(ctx, "scene_uploads", 0)
    run_loop(4)
    assert ctx.scene_uploads - before == 1
    all_faces[0].curvature *= 1.01
    all_faces[0].update()
    run_loop(3)
    assert ctx.scene_uploads - before == 2


def test_gpu_trace_one_face_segment_matches_oracle():
    c = load_case("config2_sub24")
    lists, all_faces = build(c["spec"])
    rc = RayCollection.from_array(c["rays"])
    rc.wavelengths = c["wl"]
    kids = ctracer.trace_one_face_segment(rc, lists[0], 0, all_faces, max_length=1000.0)
    tables = scene.compile_scene([lists[0]])
    mutated, okids, _ = oracle.trace_segment(tables, c["wl"], c["rays"], 1000.0, one_list=0, one_face=0)
    assert_records(rc.copy_as_array(), mutated, what="mutated input")
    assert_records(kids.copy_as_array(), okids, what="children")


# ---- single-plugin calls against the reference's unit outputs ----------------------------
UNITS = load_units()
FACE_NAMES = face_unit_names(UNITS)
FACE_SPECS = load_face_specs()


@pytest.mark.parametrize("name", FACE_NAMES)
def test_gpu_face_intersect_and_normal_match_reference(name):
    lists, _ = build(FACE_SPECS[name])
    f = lists[0].faces[0]
    p1, p2 = UNITS[f"face_{name}_p1"], UNITS[f"face_{name}_p2"]
    np.testing.assert_allclose(unitcalls.face_intersect(f, p1, p2, 1), UNITS[f"face_{name}_dist_base"],
                               rtol=1e-9, atol=1e-12)
    np.testing.assert_allclose(unitcalls.face_intersect(f, p1, p2, 0), UNITS[f"face_{name}_dist_free"],
                               rtol=1e-9, atol=1e-12)
    np.testing.assert_allclose(unitcalls.face_normal(f, UNITS[f"face_{name}_pts"]), UNITS[f"face_{name}_normal"],
                               rtol=1e-9, atol=1e-12)
    if f"face_{name}_xy" in UNITS:
        np.testing.assert_array_equal(unitcalls.shape_inside(f.shape, UNITS[f"face_{name}_xy"]),
                                      UNITS[f"face_{name}_inside"])
    if f"face_{name}_dist_zg" in UNITS:
        out = unitcalls.distortion_eval(f.distortion, UNITS[f"face_{name}_dist_x"], UNITS[f"face_{name}_dist_y"])
        np.testing.assert_allclose(out[:, :3], UNITS[f"face_{name}_dist_zg"], rtol=1e-9, atol=1e-15)
        np.testing.assert_allclose(out[:, 3], UNITS[f"face_{name}_dist_z"], rtol=1e-9, atol=1e-15)


MAT_NAMES = material_unit_names(UNITS)


@pytest.mark.parametrize("name", MAT_NAMES)
def test_gpu_material_eval_matches_reference(name):
    c = load_case("mat_" + name)
    lists, _ = build(c["spec"])
    mat = lists[0].faces[0].material
    mat.wavelengths = c["wl"]
    rays = [ctracer.Ray() for _ in range(len(c["rays"]))]
    for r, rec in zip(rays, c["rays"]):
        r.ray[()] = rec
    kids = unitcalls.eval_child_rays(mat, rays, np.arange(len(rays)), UNITS[f"mat_{name}_points"],
                                     UNITS[f"mat_{name}_normals"], UNITS[f"mat_{name}_tangents"])
    nk = [len(k) for k in kids]
    np.testing.assert_array_equal(nk, UNITS[f"mat_{name}_nkids"])
    got = np.array([k.ray for ks in kids for k in ks], dtype=ctracer.ray_dtype).reshape(-1)
    assert_records(got, UNITS[f"mat_{name}_kids"], what=name)


def test_gpu_convert_to_sp_matches_reference():
    rays = [ctracer.Ray() for _ in range(len(UNITS["sp_rays"]))]
    for r, rec in zip(rays, UNITS["sp_rays"]):
        r.ray[()] = rec
    out = unitcalls.convert_to_sp(rays, UNITS["sp_normals"])
    got = np.array([r.ray for r in out], dtype=ctracer.ray_dtype).reshape(-1)
    assert_records(got, UNITS["sp_out"], what="Convert_to_SP")


def test_gpu_dispersion_curves_match_reference():
    specs = json.loads(str(UNITS["curve_specs"]))
    wl = UNITS["curve_wl"]
    for name, spec in specs.items():
        curve = cmaterials.BaseDispersionCurve(spec["formula_id"], spec["coefs"], spec.get("absorption", 0.0),
                                               spec.get("wavelength_min", 0.1), spec.get("wavelength_max", 1e6))
        np.testing.assert_allclose(curve.evaluate_n(wl), UNITS[f"curve_{name}_n"], rtol=1e-12, atol=0)


def test_gpu_wavelength_out_of_range_raises():
    curve = cmaterials.BaseDispersionCurve(2, W.CROWN["coefs"], wavelength_min=0.4, wavelength_max=0.7)
    with pytest.raises(ValueError):
        curve.evaluate_n([0.3])
