"""Post-trace ray capture: select_ray_intersections and
select_gausslet_intersections (ctracer.pyx:1981-2058) on traced generations of
the configuration-1 lens, against the reference's own outputs: the oracle on
the CPU, the GPU path through the package's functions."""
import json
import os

import numpy as np
import pytest

import oracle
from helpers import GOLDEN, X86, assert_gausslets, assert_records, build, tables_for
from raypier_optics_gb300 import ctracer

U = dict(np.load(os.path.join(GOLDEN, "units_capture.npz")))
SPEC = json.loads(str(U["spec"]))


def _gens(key, okey, dtype):
    offs = U[okey].astype(np.int64)
    arr = U[key].astype(dtype)
    return [arr[offs[g]:offs[g + 1]] for g in range(len(offs) - 1)]


@pytest.mark.parametrize("li", [1, 2])
def test_oracle_select_ray_intersections_matches_reference(li):
    tables, _, _ = tables_for(SPEC)
    gens = _gens("gens", "offsets", ctracer.ray_dtype)
    recs, wl = oracle.select_ray_intersections(tables, li, [(g, U["wl"]) for g in gens])
    np.testing.assert_array_equal(wl, U[f"rays_list{li}_wl"])
    assert_records(recs, U[f"rays_list{li}"].astype(ctracer.ray_dtype), exact=X86, what=f"list {li}")


@pytest.mark.gpu
@pytest.mark.parametrize("li", [1, 2])
def test_gpu_select_ray_intersections_matches_reference(li):
    lists, _ = build(SPEC)
    cols = []
    for g in _gens("gens", "offsets", ctracer.ray_dtype):
        rc = ctracer.RayCollection.from_array(g)
        rc.wavelengths = U["wl"]
        cols.append(rc)
    sel = ctracer.select_ray_intersections(lists[li], cols)
    np.testing.assert_array_equal(sel.wavelengths, U[f"rays_list{li}_wl"])
    assert_records(sel.copy_as_array(), U[f"rays_list{li}"].astype(ctracer.ray_dtype), what=f"list {li}")


@pytest.mark.gpu
@pytest.mark.parametrize("li", [1, 2])
def test_gpu_select_gausslet_intersections_matches_reference(li):
    lists, _ = build(SPEC)
    cols = []
    for g in _gens("ggens", "goffsets", ctracer.gausslet_dtype):
        gc = ctracer.GaussletCollection.from_array(g)
        gc.wavelengths = U["wl"]
        cols.append(gc)
    sel = ctracer.select_gausslet_intersections(lists[li], cols)
    np.testing.assert_array_equal(sel.wavelengths, U[f"gausslets_list{li}_wl"])
    assert_gausslets(sel.copy_as_array(), U[f"gausslets_list{li}"].astype(ctracer.gausslet_dtype),
                     what=f"list {li}")
