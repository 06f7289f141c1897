"""Gausslet tracing (trace_gausslet_c / trace_one_face_gausslet_c with
trace_parabasal_rays, ctracer.pyx:2214-2385; eval_parabasal_ray_c of every
material) against the reference's own traces: the oracle on the CPU and the
GPU path through the package's trace_rays / trace_ray_sequence.  Cases: the
configuration-1 lens (non-sequential and sequential), one plane per
parabasal rule (base reflection / pass-through, dielectric, coatings,
gratings) and a ResampleGaussletMaterial decomposition."""
from itertools import chain

import numpy as np
import pytest

import oracle
from helpers import (NS, X86, assert_gausslet_generations, gausslet_case_names, load_gausslet_case, tables_for)
from raypier_optics_gb300 import ctracer, scene
from raypier_optics_gb300 import workloads as W

CASES = gausslet_case_names()


def _resample(records):
    gc = ctracer.GaussletCollection.from_array(records)
    return W.resample_shift(gc).copy_as_array()


def _scene(c):
    """Face lists with face.idx as the reference's driver assigns it (the
    chained face lists of a sequence repeat lists)."""
    lists = W.build_scene(c["spec"], NS)
    seq = c["params"].get("sequence")
    chained = list(chain(*(lists[l].faces for l, _ in seq))) if seq else [f for fl in lists for f in fl.faces]
    for i, f in enumerate(chained):
        f.idx = i
        f.update()
    return lists, chained


def test_gausslet_record_layout():
    assert ctracer.gausslet_dtype.itemsize == 668 and ctracer.para_dtype.itemsize == 80


@pytest.mark.parametrize("name", CASES)
def test_oracle_gausslet_trace_matches_reference(name):
    c = load_gausslet_case(name)
    lists, chained = _scene(c)
    tables = scene.compile_scene(lists)
    P = c["params"]
    decompose = {m: _resample for m, obj in enumerate(tables.material_objects)
                 if type(obj).__name__ == "ResampleGaussletMaterial"}
    gens, counts = oracle.trace_gausslets(tables, c["wl"], c["gausslets"], P["recursion_limit"], P["max_length"],
                                          decompose=decompose, sequence=P.get("sequence"))
    assert_gausslet_generations(gens, c["gens"], exact=X86, what=name)
    rec_of = {id(f): k for k, f in enumerate(tables.face_objects)}
    assert [int(counts[rec_of[id(f)]]) for f in chained] == c["counts"].tolist()


def test_oracle_eval_parabasal_matches_reference():
    u = dict(np.load(oracle.os.path.join(oracle.REPO, "tests", "golden", "units_gausslet.npz")))
    names = sorted({k[len("para_"):-len("_out")] for k in u if k.startswith("para_") and k.endswith("_out")})
    assert len(names) >= 15
    import json
    for name in names:
        tables, _, _ = tables_for(json.loads(str(u[f"para_{name}_spec"])))
        base = u[f"para_{name}_base"].astype(ctracer.ray_dtype)
        got = np.zeros(len(base), dtype=ctracer.para_dtype)
        for i in range(len(base)):
            got[i] = oracle.eval_parabasal(tables, u[f"para_{name}_wl"], 0, base[i], u[f"para_{name}_dirs"][i],
                                           u[f"para_{name}_points"][i], u[f"para_{name}_normals"][i],
                                           u[f"para_{name}_tangents"][i], int(u[f"para_{name}_refl"][i]))
        exp = u[f"para_{name}_out"].astype(ctracer.para_dtype)
        for f in ("origin", "direction", "normal", "length"):
            if X86:
                assert np.array_equal(got[f], exp[f], equal_nan=True), (name, f)
            else:
                np.testing.assert_allclose(got[f], exp[f], rtol=1e-12, atol=1e-15, err_msg=f"{name} {f}")


@pytest.mark.gpu
@pytest.mark.parametrize("name", CASES)
def test_gpu_gausslet_trace_matches_reference(name):
    from raypier_optics_gb300 import tracer
    c = load_gausslet_case(name)
    lists = W.build_scene(c["spec"], NS)
    gc = ctracer.GaussletCollection.from_array(c["gausslets"].copy())
    gc.wavelengths = c["wl"]
    P = c["params"]
    if P.get("sequence"):
        traced, all_faces = tracer.trace_ray_sequence(gc, [(lists[l], f) for l, f in P["sequence"]],
                                                      recursion_limit=P["recursion_limit"],
                                                      max_length=P["max_length"])
    else:
        traced, all_faces = tracer.trace_rays(gc, lists, recursion_limit=P["recursion_limit"],
                                              max_length=P["max_length"])
    assert_gausslet_generations([t.copy_as_array() for t in traced], c["gens"], what=name)
    assert [f.count for f in all_faces] == c["counts"].tolist()


# (case, radius, working distance) of the reference's config_parabasal_rays
# call that made each golden case's input gausslets (tests/golden/make_golden.py)
PARABASAL_CASES = [("config1", 0.05, 2.0), ("seq_config1", 0.02, -1.0), ("mat_dielectric", 0.1, 0.5),
                   ("mat_grating", 0.1, 0.5)]


@pytest.mark.gpu
@pytest.mark.parametrize("name,radius,wd", PARABASAL_CASES)
def test_gpu_config_parabasal_rays_matches_reference(name, radius, wd):
    """GaussletCollection.config_parabasal_rays on the device reproduces the
    reference's parabasal rays bit for bit (cos / sin of the three angles from
    the host C library, every other operation in the reference's order)."""
    c = load_gausslet_case(name)
    exp = c["gausslets"]
    gc = ctracer.GaussletCollection.from_rays(np.ascontiguousarray(exp["base_ray"]))
    gc.config_parabasal_rays(c["wl"], radius, wd)
    got = gc.copy_as_array()
    for f in ("origin", "direction", "normal", "length"):
        np.testing.assert_array_equal(got["para_rays"][f], exp["para_rays"][f], err_msg=f"{name}: parabasal {f}")
    np.testing.assert_array_equal(got["base_ray"], exp["base_ray"])


@pytest.mark.gpu
def test_gpu_total_power_sums_the_base_rays():
    c = load_gausslet_case("config1")
    g = c["gausslets"]
    gc = ctracer.GaussletCollection.from_array(np.concatenate([g] * 50))
    b = gc.copy_as_array()["base_ray"]
    n = b["refractive_index"].real
    exp = float(np.sum((np.abs(b["E1_amp"]) ** 2 + np.abs(b["E2_amp"]) ** 2) * n))
    assert gc.total_power == pytest.approx(exp, rel=1e-13)
    assert ctracer.GaussletCollection(0).total_power == 0.0
