"""The C oracle (oracle/rp_oracle.c) against the reference's golden vectors.

These run on the CPU only.  On x86-64 the oracle, built with the reference's
own flags, must reproduce the reference byte for byte; elsewhere (another
libm) indices must still match exactly and floats within the parity
tolerance."""
import hashlib
import json
import os

import numpy as np
import pytest

import oracle
from helpers import (GOLDEN, X86, assert_generations, assert_records, face_unit_names, load_case,
                     load_face_specs, load_units, material_unit_names, tables_for, trace_case_names)
from raypier_optics_gb300 import ctracer, workloads as W


@pytest.mark.parametrize("name", trace_case_names())
def test_oracle_trace_matches_reference(name):
    c = load_case(name)
    tables, lists, all_faces = tables_for(c["spec"])
    p = c["params"]
    gens, counts = oracle.trace_rays(tables, c["wl"], c["rays"], p["recursion_limit"], p["max_length"], 0.0)
    assert_generations(gens, c["gens"], exact=X86, what=name)
    np.testing.assert_array_equal(counts[:tables.n_faces], c["counts"])


def _index_digest(gens):
    h = hashlib.sha256()
    for g in gens:
        for f in ("wavelength_idx", "parent_idx", "end_face_idx", "ray_ident", "ray_type_id"):
            h.update(np.ascontiguousarray(g[f]).tobytes())
    return h.hexdigest()


def test_oracle_config1_full_size_digest():
    ref = json.load(open(os.path.join(GOLDEN, "config1_full.json")))
    rays, wl = W.config1_rays(ctracer.ray_dtype)
    tables, _, _ = tables_for(W.config1_spec())
    p = ref["params"]
    gens, counts = oracle.trace_rays(tables, wl, rays, p["recursion_limit"], p["max_length"], 0.0)
    assert [len(g) for g in gens] == ref["gen_sizes"] == [4096, 8192, 8192, 16384, 24576, 40960]
    assert sum(len(g) for g in gens) == ref["segments"] == 102400
    assert counts[:tables.n_faces].tolist() == ref["face_counts"]
    assert _index_digest(gens) == ref["index_sha256"]
    if X86:
        assert [hashlib.sha256(np.ascontiguousarray(g).tobytes()).hexdigest() for g in gens] == ref["gen_sha256"]


def test_oracle_termination_rule_is_inactive_on_config1():
    rays, wl = W.config1_rays(ctracer.ray_dtype, 512)
    tables, _, _ = tables_for(W.config1_spec())
    a, _ = oracle.trace_rays(tables, wl, rays, 6, 1000.0, 0.0)
    b, _ = oracle.trace_rays(tables, wl, rays, 6, 1000.0, 1e-6)
    assert [len(g) for g in a] == [len(g) for g in b]


def test_oracle_termination_drops_weak_children_stably():
    c = load_case("config2_sub24")
    tables, _, _ = tables_for(c["spec"])
    p = c["params"]
    full, _ = oracle.trace_rays(tables, c["wl"], c["rays"], 4, p["max_length"], 0.0)
    term, _ = oracle.trace_rays(tables, c["wl"], c["rays"], 4, p["max_length"], 0.1)
    # generation 1 is the children of generation 0: the kept ones are the strong
    # ones, in the same order
    e2 = lambda g: (np.abs(g["E1_amp"]) ** 2 + np.abs(g["E2_amp"]) ** 2)
    keep = full[1][~(e2(full[1]) < 0.1)]
    np.testing.assert_array_equal(term[1]["parent_idx"], keep["parent_idx"])
    np.testing.assert_array_equal(term[1]["ray_type_id"], keep["ray_type_id"])
    assert len(term[1]) < len(full[1])


UNITS = load_units()


@pytest.mark.parametrize("name", material_unit_names(UNITS))
def test_oracle_material_eval_matches_reference(name):
    """eval_child_ray of every material (random orientations, normal incidence
    among them) against the reference's own calls."""
    c = load_case("mat_" + name)
    tables, lists, _ = tables_for(c["spec"])
    mat_idx = 0  # the material of the case's first face is the first in the table
    kids = oracle.eval_child_rays(tables, c["wl"], mat_idx, c["rays"], np.arange(len(c["rays"])),
                                  UNITS[f"mat_{name}_points"], UNITS[f"mat_{name}_normals"],
                                  UNITS[f"mat_{name}_tangents"])
    np.testing.assert_array_equal([len(k) for k in kids], UNITS[f"mat_{name}_nkids"])
    got = np.concatenate(kids) if kids else np.zeros(0, dtype=ctracer.ray_dtype)
    assert_records(got, UNITS[f"mat_{name}_kids"], exact=X86, what=name)


@pytest.mark.parametrize("name", face_unit_names(UNITS))
def test_oracle_face_intersect_and_normal_match_reference(name):
    """Face.intersect (base and non-base rays, axis-parallel segments among
    them) and Face.compute_normal of every face type against the reference's
    own calls; NaN where the reference returns NaN."""
    tables, lists, _ = tables_for(load_face_specs()[name])
    p1, p2 = UNITS[f"face_{name}_p1"], UNITS[f"face_{name}_p2"]
    got = [oracle.face_intersect(tables, 0, p1, p2, 1), oracle.face_intersect(tables, 0, p1, p2, 0),
           oracle.face_normal(tables, 0, UNITS[f"face_{name}_pts"])]
    exp = [UNITS[f"face_{name}_dist_base"], UNITS[f"face_{name}_dist_free"], UNITS[f"face_{name}_normal"]]
    for a, b in zip(got, exp):
        if X86:
            assert np.array_equal(a, b, equal_nan=True), (name, a, b)
        else:
            np.testing.assert_allclose(a, b, rtol=1e-12, atol=1e-15)
