"""Host-side logic that needs no GPU: the ray record layout, RayCollection,
shapes, Zernike indexing, the scene compiler, the workloads, and the rule
that the tracing path fails loudly instead of falling back to the CPU."""
import json
import math
import os

import numpy as np
import pytest

from helpers import GOLDEN, NS, build, load_case
from raypier_optics_gb300 import (_native, cdistortions, cfaces, cmaterials, cshapes, ctracer, runtime,
                                  scene, tracer)
from raypier_optics_gb300 import workloads as W


def test_ray_dtype_is_the_reference_layout():
    ref_dtype = load_case("config1_sub64")["rays"].dtype
    golden_dtype = np.load(os.path.join(GOLDEN, "config1_sub64.npz"))["rays"].dtype
    assert ctracer.ray_dtype.itemsize == 188 == golden_dtype.itemsize
    assert ctracer.ray_dtype.descr == golden_dtype.descr
    assert ref_dtype == ctracer.ray_dtype


def test_raycollection_host_operations():
    rc = ctracer.RayCollection(2)
    assert rc.n_rays == 0 and len(rc) == 0
    for i in range(5):
        rc.add_ray(ctracer.Ray(origin=(i, 0, 0), direction=(0, 0, 1), ray_ident=i))
    assert rc.n_rays == 5 and rc.max_size >= 5
    np.testing.assert_array_equal(rc.ray_ident, np.arange(5))
    np.testing.assert_array_equal(rc.origin[:, 0], np.arange(5))
    rc[2] = ctracer.Ray(origin=(9, 9, 9))
    assert rc[2].origin == (9.0, 9.0, 9.0)
    with pytest.raises(IndexError):
        rc[5]
    with pytest.raises(TypeError):
        rc.add_ray_list([ctracer.Ray(), "not a ray"])
    arr = rc.copy_as_array()
    rc2 = ctracer.RayCollection.from_array(arr)
    assert rc2.copy_as_array().tobytes() == arr.tobytes()
    rc2.reset_length(12.5)
    assert np.all(rc2.length == 12.5)
    rc2.clear_ray_list()
    assert rc2.n_rays == 0
    rc.wavelengths = [0.5, 0.6]
    child = ctracer.RayCollection(0)
    child.parent = rc
    np.testing.assert_array_equal(child.wavelengths, [0.5, 0.6])
    t = rc.termination
    assert t.shape == (5, 3)


def test_ray_polarisation_helpers():
    r = ctracer.Ray(direction=(0, 0, 1), E_vector=(1, 0, 0), E1_amp=1.0, E2_amp=1.0j, refractive_index=1.5)
    assert math.isclose(r.power, 3.0)
    assert math.isclose(r.amplitude, math.sqrt(2))
    assert math.isclose(abs(r.ellipticity), 1.0)
    r.project_E(0, 1, 0)
    assert np.allclose(r.E_vector, (0, 1, 0)) or np.allclose(r.E_vector, (0, -1, 0))


def test_ansi_zernike_indices():
    # ANSI j -> (n, m): j = (n(n+2) + m) / 2 (raypier/distortions.py:64,83)
    for j in range(20):
        n, m, k = cdistortions.eval_nmk(j)
        assert (n * (n + 2) + m) // 2 == j
        assert abs(m) <= n and (n - m) % 2 == 0
        assert k == (n // 2) * (n // 2 + 1) + abs(m)
    assert [W.ansi_j(*W.noll_to_nm(j)) for j in range(1, 16)] == \
        [0, 2, 1, 4, 3, 5, 7, 8, 6, 9, 12, 13, 11, 14, 10]


def test_shapes_host_predicate_matches_reference():
    units = np.load(os.path.join(GOLDEN, "units.npz"))
    specs = json.loads(str(np.load(os.path.join(GOLDEN, "face_zoo_specs.npz"))["specs"]))
    checked = 0
    for name, spec in specs.items():
        if f"face_{name}_xy" not in units.files:
            continue
        lists, _ = build(spec)
        shape = lists[0].faces[0].shape
        got = np.array([bool(shape.point_inside(x, y)) for x, y in units[f"face_{name}_xy"]])
        np.testing.assert_array_equal(got, units[f"face_{name}_inside"], err_msg=name)
        checked += 1
    assert checked >= 10


def test_scene_compiler_packs_parameters():
    lists, faces = build(W.config2_spec())
    t = scene.compile_scene(lists)
    assert t.n_faces == 11 and t.faces.shape[0] == 11 and t.lists.shape[0] == 5
    assert list(t.lists["first_face"]) == [0, 3, 6, 8, 10]
    sph = t.faces[0]
    assert sph["type"] == cfaces.SPHERICAL and tuple(sph["p"][:3]) == (50.0, -100.0, 0.0)
    assert sph["invert_normal"] == 1
    asp = t.faces[6]
    assert asp["type"] == cfaces.ASPHERIC
    assert asp["p"][11] == 4.0 and asp["p"][12] == math.pow(80.0, 3.0)
    assert asp["shape"] >= 0 and t.shape_ops[asp["shape"]]["op"] == cshapes.OP_CIRCLE
    # 4 dispersive materials + detector, 3 curves
    assert t.materials.shape[0] == 4 and t.dispersions.shape[0] == 3
    assert t.lists[1]["trans"]["t"][2] == 30.0 and t.lists[1]["inv_trans"]["t"][2] == -30.0


def test_scene_compiler_extended_polynomial_and_distortion_records():
    lists, _ = build(W.config3_spec())
    t = scene.compile_scene(lists)
    assert t.n_faces == 64 and t.faces.shape[0] == 64 + 16  # 16 DistortionFace base records
    ep = [f for f in t.faces[:64] if f["type"] == cfaces.EXTPOLY]
    assert len(ep) == 8
    obj = [f for fl in lists for f in fl.faces if isinstance(f, cfaces.ExtendedPolynomialFace)][0]
    rec = ep[0]
    assert rec["p"][0] == -obj.curvature and rec["p"][1] == obj.conic_const + 1.0
    assert (rec["n_aux0"], rec["n_aux1"]) == (5, 5)
    dist = [f for f in t.faces[:64] if f["type"] == cfaces.DISTORTION]
    assert all(f["base"] >= 64 for f in dist)
    assert all(t.faces[f["base"]]["type"] == cfaces.SHAPED_PLANAR for f in dist)
    assert t.distortions.shape[0] == 16 and all(t.distortions["n_coefs"] == 15)


def test_unsupported_types_raise_not_implemented():
    class CustomFace(ctracer.Face):
        pass

    class CustomMaterial(ctracer.InterfaceMaterial):
        pass

    fl = ctracer.FaceList()
    fl.faces = [CustomFace()]
    with pytest.raises(NotImplementedError):
        scene.compile_scene([fl])
    fl.faces = [cfaces.CircularFace(material=CustomMaterial())]
    with pytest.raises(NotImplementedError):
        scene.compile_scene([fl])
    curve = cmaterials.BaseDispersionCurve(5, [1.0, 0.1, 2.0])
    fl.faces = [cfaces.CircularFace(material=cmaterials.FullDielectricDispersiveMaterial(dispersion_inside=curve))]
    with pytest.raises(NotImplementedError):
        scene.compile_scene([fl])


def test_material_argument_errors_match_reference():
    with pytest.raises(ValueError):
        cmaterials.BaseDispersionCurve(4, [1.0])          # cmaterials.pyx:199-200
    with pytest.raises(ValueError):
        cmaterials.PartiallyReflectiveMaterial(reflectivity=1.5)
    curve = cmaterials.BaseDispersionCurve(2, W.CROWN["coefs"], wavelength_min=0.4, wavelength_max=0.7)
    with pytest.raises(ValueError):
        curve._check_range([0.8])
    m = cmaterials.FullDielectricDispersiveMaterial(dispersion_inside=curve)
    with pytest.raises(ValueError):
        m.wavelengths = np.array([0.3])


def test_face_defaults_follow_reference_constructors():
    f = cfaces.CircularFace(diameter=99.0)   # diameter comes from the owner, not the keyword
    assert f.diameter == 0.0 and f.tolerance == 0.0001 and isinstance(f.material, cmaterials.PECMaterial)
    s = cfaces.SphericalFace()
    assert s.curvature == 25.0
    e = cfaces.ExtendedPolynomialFace(curvature=10.0, conic_const=-1.0)
    assert e.curvature == 10.0 and e.conic_const == -1.0 and e.norm_radius == 100.0
    o = cfaces.OrientedPolygonFace(normal=(0, 0, 2), x_axis=(2, 0, 0))
    assert np.allclose(o.normal, (0, 0, 1)) and np.allclose(o._y_axis, (0, 1, 0))


def test_workloads_are_deterministic():
    a, wa = W.config2_rays(ctracer.ray_dtype, 1000)
    b, wb = W.config2_rays(ctracer.ray_dtype, 1000)
    assert a.tobytes() == b.tobytes() and np.array_equal(wa, wb)
    d = a['direction']
    assert np.allclose(np.linalg.norm(d, axis=1), 1.0)
    assert np.all(d[:, 2] >= math.cos(0.1) - 1e-12)
    c3a, _ = W.config3_rays(ctracer.ray_dtype, 10)
    c3b, _ = W.config3_rays(ctracer.ray_dtype, 70000)
    assert c3a.tobytes() == c3b[:10].tobytes()
    x, y = W.hex_grid(4096, 5.0)
    r = np.hypot(x, y)
    assert len(x) == 4096 and math.isclose(r.max(), 5.0) and np.all(np.diff(np.round(r, 9)) >= 0)


def test_tracing_without_a_gpu_fails_loudly(monkeypatch):
    """No CPU fallback: without a device the C ABI reports an error."""
    try:
        ctx = runtime.Context(0)
    except _native.RPError:
        ctx = None
    if ctx is not None:
        pytest.skip("a GPU is present")
    lists, _ = build(W.config1_spec())
    rays, wl = W.config1_rays(ctracer.ray_dtype, 16)
    rc = ctracer.RayCollection.from_array(rays)
    rc.wavelengths = wl
    with pytest.raises(_native.RPError):
        tracer.trace_rays(rc, lists, recursion_limit=2, max_length=100.0)
