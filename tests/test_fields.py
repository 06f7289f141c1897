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
    rays, x, y, dx, dy = fields.evaluate_neighbours_gc(g)
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
    rays, x, y, dx, dy = fields.evaluate_neighbours(U["rf_rays"].astype(ctracer.ray_dtype), U["rf_neighbours"])
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
