"""E-field summation over Gaussian modes (cfields.pyx:49-234,
core/fields.py:83-277) against the reference's own outputs: single-call
evaluate_modes / sum_gaussian_modes vectors, a gausslet beam before and after
the configuration-1 lens (eval_Efield_from_gausslets, EFieldSummation at a
non-zero time) and a hexagonal ray field (eval_Efield_from_rays).

The oracle reproduces the reference bit for bit on x86-64.  The GPU sums the
same terms in the same order with its own exp / sincos / complex square root
and Smith complex division, so its fields agree to
|E - E_ref| <= FIELD_RTOL * max |E_ref| (per case)."""
import os

import numpy as np
import pytest

import oracle
from helpers import GOLDEN, X86
from raypier_optics_gb300 import ctracer, fields

U = dict(np.load(os.path.join(GOLDEN, "units_fields.npz")))
FIELD_RTOL = 1e-9
MODES_RTOL = 1e-12


def _close(got, exp, rtol):
    scale = np.max(np.abs(exp))
    err = np.max(np.abs(got - exp))
    assert err <= rtol * scale, (err, scale)


def _oracle_from_gausslets(g, wl, points, time_ps=0.0):
    rays, x, y, dx, dy = oracle.gausslet_samples(g)
    modes = oracle.evaluate_modes(x, y, dx, dy, 1.0)
    return oracle.sum_gaussian_modes(np.ascontiguousarray(rays), modes, wl, points, time_ps)


def _eq(got, exp):
    if X86:
        assert np.array_equal(got, exp)
    else:
        _close(got, exp, 1e-12)


def test_oracle_evaluate_modes_matches_reference():
    _eq(oracle.evaluate_modes(U["modes_x"], U["modes_y"], U["modes_dx"], U["modes_dy"], 1.3), U["modes_out"])


def test_oracle_sum_gaussian_modes_matches_reference():
    r = U["sum_rays"].astype(ctracer.ray_dtype)
    for t, key in ((0.0, "sum_E"), (2.5, "sum_E_t")):
        _eq(oracle.sum_gaussian_modes(r, U["sum_modes"], U["sum_wl"], U["sum_points"], t), U[key])


def test_oracle_field_pipelines_match_reference():
    g = U["beam_gausslets"].astype(ctracer.gausslet_dtype)
    _eq(_oracle_from_gausslets(g, U["beam_wl"], U["beam_points"]), U["beam_E"])
    g = U["lens_gausslets"].astype(ctracer.gausslet_dtype)
    _eq(_oracle_from_gausslets(g, U["beam_wl"], U["lens_points"]), U["lens_E"])
    _eq(_oracle_from_gausslets(g, U["beam_wl"], U["lens_points"], 0.7), U["lens_E_t"])
    rays, x, y, dx, dy = oracle.ray_samples(U["rf_rays"].astype(ctracer.ray_dtype), U["rf_neighbours"])
    _eq(oracle.sum_gaussian_modes(rays, oracle.evaluate_modes(x, y, dx, dy, 1.0), U["beam_wl"], U["rf_points"]),
        U["rf_E"])


def test_child_neighbours_follow_parent_and_type():
    parent = ctracer.RayCollection.from_array(np.zeros(3, dtype=ctracer.ray_dtype))
    parent.neighbours = np.array([[1, -1], [0, 2], [1, -1]], dtype=np.int32)
    kids = np.zeros(5, dtype=ctracer.ray_dtype)
    kids['parent_idx'] = [0, 0, 1, 1, 2]
    kids['ray_type_id'] = [1, 0, 1, 0, 0]
    child = ctracer.RayCollection.from_array(kids)
    child.parent = parent
    np.testing.assert_array_equal(child.neighbours, [[2, -1], [3, -1], [0, -1], [1, 4], [3, -1]])


@pytest.mark.gpu
def test_gpu_evaluate_modes_matches_reference():
    from raypier_optics_gb300 import cfields
    got = cfields.evaluate_modes(U["modes_x"], U["modes_y"], U["modes_dx"], U["modes_dy"], 1.3)
    np.testing.assert_allclose(got, U["modes_out"], rtol=MODES_RTOL, atol=0)


@pytest.mark.gpu
def test_gpu_evaluate_modes_raises_on_a_degenerate_fit():
    from raypier_optics_gb300 import cfields
    z = np.zeros((2, 6))
    with pytest.raises(ZeroDivisionError):
        cfields.evaluate_modes(z, z, z, z)


@pytest.mark.gpu
def test_gpu_sum_gaussian_modes_matches_reference():
    from raypier_optics_gb300 import cfields
    rc = ctracer.RayCollection.from_array(U["sum_rays"].astype(ctracer.ray_dtype))
    for t, key in ((0.0, "sum_E"), (2.5, "sum_E_t")):
        _close(cfields.sum_gaussian_modes(rc, U["sum_modes"], U["sum_wl"], U["sum_points"], t), U[key], FIELD_RTOL)


@pytest.mark.gpu
def test_gpu_eval_efield_from_gausslets_matches_reference():
    for gkey, pkey, ekey in (("beam_gausslets", "beam_points", "beam_E"), ("lens_gausslets", "lens_points", "lens_E")):
        gc = ctracer.GaussletCollection.from_array(U[gkey].astype(ctracer.gausslet_dtype))
        gc.wavelengths = U["beam_wl"]
        _close(fields.eval_Efield_from_gausslets(gc, U[pkey]), U[ekey], FIELD_RTOL)


@pytest.mark.gpu
def test_gpu_efield_summation_at_a_time_matches_reference():
    gc = ctracer.GaussletCollection.from_array(U["lens_gausslets"].astype(ctracer.gausslet_dtype))
    gc.wavelengths = U["beam_wl"]
    s = fields.EFieldSummation(gc)
    _close(s.evaluate(U["lens_points"], time_ps=0.7), U["lens_E_t"], FIELD_RTOL)
    _close(s.evaluate(U["lens_points"]), U["lens_E"], FIELD_RTOL)


@pytest.mark.gpu
def test_gpu_eval_efield_from_rays_matches_reference():
    rc = ctracer.RayCollection.from_array(U["rf_rays"].astype(ctracer.ray_dtype))
    rc.neighbours = U["rf_neighbours"]
    _close(fields.eval_Efield_from_rays(rc, U["rf_points"], U["beam_wl"]), U["rf_E"], FIELD_RTOL)


def test_oracle_sphere_projection_keeps_the_rays_that_meet_it():
    r = U["rf_rays"].astype(ctracer.ray_dtype)
    c = r["origin"].mean(axis=0) + np.array([0.0, 0.0, 5.0])
    radius = float(np.max(np.linalg.norm(r["origin"] - c, axis=1))) * 0.9
    got = oracle.project_to_sphere(r, c, radius)
    assert 0 < len(got) <= len(r)
    np.testing.assert_allclose(np.linalg.norm(got["origin"] - c, axis=1), radius, rtol=1e-12)


@pytest.mark.gpu
def test_gpu_wavefront_samples_match_the_oracle():
    """The device's neighbour samples (the mode fit's input) against the
    oracle's restatement of core/fields.py:80-148, bit for bit: the same
    operations in the same order, FP64 without contraction."""
    g = U["lens_gausslets"].astype(ctracer.gausslet_dtype)
    exp = oracle.gausslet_samples(g)
    got = fields.evaluate_neighbours_gc(ctracer.GaussletCollection.from_array(g))
    np.testing.assert_array_equal(got[0], exp[0])
    for a, b in zip(got[1:], exp[1:]):
        np.testing.assert_array_equal(a, b)
    r = U["rf_rays"].astype(ctracer.ray_dtype)
    exp = oracle.ray_samples(r, U["rf_neighbours"])
    got = fields.evaluate_neighbours(r, U["rf_neighbours"])
    assert len(got[0]) == len(exp[0]) and len(exp[0]) > 0
    np.testing.assert_array_equal(got[0], exp[0])
    for a, b in zip(got[1:], exp[1:]):
        np.testing.assert_array_equal(a, b)


@pytest.mark.gpu
def test_gpu_neighbour_index_outside_the_lattice_raises():
    r = U["rf_rays"].astype(ctracer.ray_dtype)
    nb = np.array(U["rf_neighbours"], dtype=np.int32, copy=True)
    nb[0, 0] = len(r)
    with pytest.raises(IndexError):
        fields.evaluate_neighbours(r, nb)


@pytest.mark.gpu
def test_gpu_sphere_projection_matches_the_oracle():
    r = U["rf_rays"].astype(ctracer.ray_dtype)
    c = r["origin"].mean(axis=0) + np.array([0.0, 0.0, 5.0])
    # rays further from the axis than the radius (they run along z) miss the sphere
    radius = float(np.max(np.linalg.norm(r["origin"][:, :2] - c[:2], axis=1))) * 0.6
    exp = oracle.project_to_sphere(r, c, radius)
    got = fields.project_to_sphere(r, c, radius)
    assert 0 < len(exp) < len(r)
    np.testing.assert_array_equal(got, exp)


@pytest.mark.gpu
def test_gpu_efield_from_projected_rays_matches_the_oracle():
    """eval_Efield_from_rays with an exit-pupil sphere every ray meets."""
    rc = ctracer.RayCollection.from_array(U["rf_rays"].astype(ctracer.ray_dtype))
    rc.neighbours = U["rf_neighbours"]
    r = rc.copy_as_array()
    c = r["origin"].mean(axis=0) - 50.0 * r["direction"].mean(axis=0)
    radius = float(np.min(np.linalg.norm(r["origin"] - c, axis=1))) * 0.5
    proj = oracle.project_to_sphere(r, c, radius)
    assert len(proj) == len(r)
    rays, x, y, dx, dy = oracle.ray_samples(proj, U["rf_neighbours"])
    exp = oracle.sum_gaussian_modes(rays, oracle.evaluate_modes(x, y, dx, dy, 1.0), U["beam_wl"], U["rf_points"])
    got = fields.eval_Efield_from_rays(rc, U["rf_points"], U["beam_wl"], exit_pupil_offset=radius,
                                       exit_pupil_centre=c)
    _close(got, exp, FIELD_RTOL)


@pytest.mark.gpu
def test_gpu_efield_summation_exposes_modes_and_base_rays():
    g = U["lens_gausslets"].astype(ctracer.gausslet_dtype)
    gc = ctracer.GaussletCollection.from_array(g)
    gc.wavelengths = U["beam_wl"]
    s = fields.EFieldSummation(gc)
    rays, x, y, dx, dy = oracle.gausslet_samples(g)
    np.testing.assert_allclose(s.modes, oracle.evaluate_modes(x, y, dx, dy, 1.0), rtol=MODES_RTOL, atol=0)
    np.testing.assert_array_equal(s.base_rays.copy_as_array(), rays)
    np.testing.assert_allclose(fields.ExtractGamma(gc), s.modes, rtol=0, atol=0)


def test_gamma_propagates_the_mode_matrix():
    """Gamma(z) equals G (1 + z G)^-1 for the symmetric 2 x 2 mode matrix."""
    rng = np.random.default_rng(3)
    for _ in range(20):
        A, B, C = rng.normal(size=3) + 1j * rng.uniform(0.1, 1.0, size=3)
        z = rng.uniform(-2, 2)
        G = np.array([[A, B], [B, C]])
        exp = G @ np.linalg.inv(np.eye(2) + z * G)
        got = fields.Gamma(z, A, B, C)
        np.testing.assert_allclose([got[0], got[1], got[2]], [exp[0, 0], exp[0, 1], exp[1, 1]], rtol=1e-12)


def test_find_ray_gen_follows_the_chain_of_waypoints():
    def gen(origin, direction, length):
        a = np.zeros(4, dtype=ctracer.ray_dtype)
        a["origin"] = origin
        a["direction"] = direction
        a["length"] = length
        return ctracer.RayCollection.from_array(a)
    gens = [gen([0, 0, 0], [0, 0, 1], 10.0), gen([0, 0, 10], [0, 0, 1], 10.0), gen([0, 0, 20], [0, 0, 1], 10.0)]
    assert fields.find_ray_gen([0, 0, 1], gens) == 0
    assert fields.find_ray_gen([0, 0, 9], gens) == 0
    assert fields.find_ray_gen([0, 0, 11], gens) == 1
    assert fields.find_ray_gen([0, 0, 19], gens) == 1
    assert fields.find_ray_gen([0, 0, 21], gens) == 2
    assert fields.find_ray_gen([0, 0, 40], gens) == -1
