"""The decomposition helpers of cfields.pyx (232-426) against the reference's
own outputs: calc_mode_curvature, build_interaction_matrix and
apply_mode_curvature.

The curvature and the tilted parabasal directions use only +, -, *, / and
sqrt, which round the same on the GPU as in the reference's C, so they are
compared bit for bit.  The interaction matrix has the reference's pairs in
the reference's order (exact indices); its entries are complex exponentials
of FP64 phases, evaluated with the GPU's own exp / sincos / complex square
root, and agree to |U - U_ref| <= FIELD_RTOL * max |U_ref|."""
import os

import numpy as np
import pytest

import oracle
from helpers import GOLDEN, X86
from raypier_optics_gb300 import ctracer

U = dict(np.load(os.path.join(GOLDEN, "units_fields2.npz")))
FIELD_RTOL = 1e-9
MC_KEYS = ("mc_rx", "mc_ry", "mc_dx", "mc_dy", "mc_dx2", "mc_dy2", "mc_dxdy")
IM_KEYS = ("im_rx", "im_ry", "im_tx", "im_ty", "im_A", "im_B", "im_C", "im_X", "im_Y", "im_Z")


def _eq(got, exp):
    if X86:
        assert np.array_equal(got, exp)
    else:
        np.testing.assert_allclose(got, exp, rtol=1e-13, atol=1e-15)


def _check_matrix(got, rtol):
    data, (i, j) = got
    assert data.dtype == np.complex128 and len(data) == len(U["im_data"])
    np.testing.assert_array_equal(i, U["im_i"])
    np.testing.assert_array_equal(j, U["im_j"])
    scale = np.max(np.abs(U["im_data"]))
    assert np.max(np.abs(data - U["im_data"])) <= rtol * scale


def test_oracle_mode_curvature_matches_reference():
    got = oracle.calc_mode_curvature(*[U[k] for k in MC_KEYS])
    for v, k in zip(got, "ABCXYZ"):
        _eq(v, U["mc_" + k])


def test_oracle_interaction_matrix_matches_reference():
    data, (i, j) = oracle.build_interaction_matrix(*[U[k] for k in IM_KEYS], *U["im_args"])
    np.testing.assert_array_equal(i, U["im_i"])
    np.testing.assert_array_equal(j, U["im_j"])
    _eq(data, U["im_data"])


def test_oracle_interaction_matrix_is_row_major_and_within_reach():
    data, (i, j) = oracle.build_interaction_matrix(*[U[k] for k in IM_KEYS], *U["im_args"])
    key = i.astype(np.int64) * len(U["im_tx"]) + j.astype(np.int64)
    assert np.all(np.diff(key) > 0)
    d2 = (U["im_tx"][j] - U["im_rx"][i]) ** 2 + (U["im_ty"][j] - U["im_ry"][i]) ** 2
    assert np.all(d2 <= U["im_args"][2] ** 2)


def test_oracle_apply_mode_curvature_matches_reference():
    got = oracle.apply_mode_curvature(U["ac_gausslets"], U["ac_A"], U["ac_B"], U["ac_C"])
    if X86:
        assert got.tobytes() == U["ac_out"].tobytes()
    else:
        np.testing.assert_allclose(got['para_rays']['direction'], U["ac_out"]['para_rays']['direction'],
                                   rtol=1e-13, atol=1e-15)


@pytest.mark.gpu
def test_gpu_mode_curvature_matches_reference():
    from raypier_optics_gb300 import cfields
    got = cfields.calc_mode_curvature(*[U[k] for k in MC_KEYS])
    for v, k in zip(got, "ABCXYZ"):
        assert np.array_equal(v, U["mc_" + k]), k


@pytest.mark.gpu
def test_gpu_mode_curvature_of_no_points():
    from raypier_optics_gb300 import cfields
    got = cfields.calc_mode_curvature(*[np.zeros(0)] * 7)
    assert [v.shape for v in got] == [(0,), (0,), (0,), (0, 3), (0, 3), (0, 3)]


@pytest.mark.gpu
def test_gpu_interaction_matrix_matches_reference():
    from raypier_optics_gb300 import cfields
    _check_matrix(cfields.build_interaction_matrix(*[U[k] for k in IM_KEYS], *U["im_args"]), FIELD_RTOL)


@pytest.mark.gpu
def test_gpu_interaction_matrix_grows_past_a_short_estimate():
    # a test_spacing far above the real one makes the reference's size
    # estimate one entry per mode; the result is still every pair
    from raypier_optics_gb300 import cfields
    args = list(U["im_args"])
    args[4] = 100.0
    _check_matrix(cfields.build_interaction_matrix(*[U[k] for k in IM_KEYS], *args), FIELD_RTOL)


def _no_pair_case():
    # test points moved off the lattice by 0.013 mm, reach 1 um: no pair
    arrays = [U[k] for k in IM_KEYS]
    arrays[2] = arrays[2] + 0.013
    arrays[3] = arrays[3] + 0.013
    args = list(U["im_args"])
    args[2] = 1e-3
    return arrays, args


def test_oracle_interaction_matrix_without_pairs():
    arrays, args = _no_pair_case()
    data, (i, j) = oracle.build_interaction_matrix(*arrays, *args)
    assert len(data) == len(i) == len(j) == 0


@pytest.mark.gpu
def test_gpu_interaction_matrix_without_pairs():
    from raypier_optics_gb300 import cfields
    arrays, args = _no_pair_case()
    data, (i, j) = cfields.build_interaction_matrix(*arrays, *args)
    assert len(data) == len(i) == len(j) == 0


@pytest.mark.gpu
def test_gpu_apply_mode_curvature_matches_reference():
    from raypier_optics_gb300 import cfields
    gc = ctracer.GaussletCollection.from_array(U["ac_gausslets"].astype(ctracer.gausslet_dtype))
    cfields.apply_mode_curvature(gc, U["ac_A"], U["ac_B"], U["ac_C"])
    got = gc.copy_as_array()
    assert got.tobytes() == U["ac_out"].astype(ctracer.gausslet_dtype).tobytes()


def test_short_arrays_raise_before_any_device_work():
    # the reference's bounds-checked buffers raise IndexError; here the
    # check comes before the library is touched, so it holds without a GPU
    from raypier_optics_gb300 import cfields
    with pytest.raises(IndexError):
        cfields.calc_mode_curvature(np.zeros(4), np.zeros(4), np.zeros(3), np.zeros(4), np.zeros(4), np.zeros(4),
                                    np.zeros(4))
    a = [U[k] for k in IM_KEYS]
    a[4] = a[4][:-1]
    with pytest.raises(IndexError):
        cfields.build_interaction_matrix(*a, *U["im_args"])
    gc = ctracer.GaussletCollection.from_array(U["ac_gausslets"].astype(ctracer.gausslet_dtype))
    with pytest.raises(IndexError):
        cfields.apply_mode_curvature(gc, U["ac_A"][:-1], U["ac_B"], U["ac_C"])
