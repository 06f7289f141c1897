"""Shared test utilities: golden-case loading, scene construction with this
package's classes, and record comparison at the parity tolerances
(indices bit-exact; floating point within 1e-9 relative)."""
from __future__ import annotations

import glob
import json
import os
import platform
import types

import numpy as np

from raypier_optics_gb300 import cdistortions, cfaces, cmaterials, cshapes, ctracer, scene
from raypier_optics_gb300 import workloads as W

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
NS = types.SimpleNamespace(ctracer=ctracer, cfaces=cfaces, cmaterials=cmaterials, cshapes=cshapes,
                           cdistortions=cdistortions)
INDEX_FIELDS = ("wavelength_idx", "parent_idx", "end_face_idx", "ray_ident", "ray_type_id")
FLOAT_FIELDS = ("origin", "direction", "normal", "E_vector", "refractive_index", "E1_amp", "E2_amp",
                "length", "phase", "accumulated_path")
# parity tolerance for floating-point fields (positions, directions, fields, OPL)
RTOL = 1e-9
ATOL = 1e-12
X86 = platform.machine() in ("x86_64", "AMD64")


def trace_case_names():
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "*.npz"))
                  if not os.path.basename(p).startswith(("units", "face_zoo", "seq_", "gauss_")))


def load_units():
    """The reference's single-call outputs: units.npz plus the coated-material
    vectors of units_coated.npz and the second face set of units_faces2.npz,
    as one mapping."""
    out = dict(np.load(os.path.join(GOLDEN, "units.npz")))
    for extra in ("units_coated.npz", "units_faces2.npz"):
        out.update(dict(np.load(os.path.join(GOLDEN, extra))))
    return out


def load_face_specs():
    """Scene spec of every face-zoo case, keyed by face name."""
    specs = {}
    for f in ("face_zoo_specs.npz", "face_zoo2_specs.npz"):
        specs.update(json.loads(str(np.load(os.path.join(GOLDEN, f))["specs"])))
    return specs


def face_unit_names(units):
    return sorted({k[len("face_"):-len("_dist_base")] for k in units
                   if k.startswith("face_") and k.endswith("_dist_base")})


def material_unit_names(units):
    return sorted({k[len("mat_"):-len("_nkids")] for k in units if k.startswith("mat_") and k.endswith("_nkids")})


def load_case(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    spec = json.loads(str(z["spec"]))
    params = json.loads(str(z["params"]))
    offs = z["offsets"].astype(np.int64)
    out = z["out"]
    gens = [out[offs[g]:offs[g + 1]] for g in range(len(offs) - 1)]
    return dict(spec=spec, params=params, rays=z["rays"].astype(ctracer.ray_dtype), wl=z["wl"], gens=gens,
                counts=z["counts"])


def build(spec):
    """Face lists for `spec` with face.idx assigned and params pulled, as
    trace_rays does (core/tracer.py:28-34)."""
    lists = W.build_scene(spec, NS)
    all_faces = [f for fl in lists for f in fl.faces]
    for i, f in enumerate(all_faces):
        f.idx = i
        f.update()
    return lists, all_faces


def tables_for(spec):
    lists, all_faces = build(spec)
    return scene.compile_scene(lists), lists, all_faces


def assert_records(got, exp, exact=False, what=""):
    assert len(got) == len(exp), f"{what}: {len(got)} rays vs {len(exp)}"
    for f in INDEX_FIELDS:
        np.testing.assert_array_equal(got[f], exp[f], err_msg=f"{what}: field {f}")
    for f in FLOAT_FIELDS:
        a, b = got[f], exp[f]
        if exact:
            a8 = np.ascontiguousarray(a).view(np.uint8)
            b8 = np.ascontiguousarray(b).view(np.uint8)
            assert np.array_equal(a8, b8), f"{what}: field {f} differs"
        else:
            np.testing.assert_allclose(a, b, rtol=RTOL, atol=ATOL, equal_nan=True, err_msg=f"{what}: field {f}")


def assert_generations(got_gens, exp_gens, exact=False, what=""):
    assert [len(g) for g in got_gens] == [len(g) for g in exp_gens], \
        f"{what}: generation sizes {[len(g) for g in got_gens]} vs {[len(g) for g in exp_gens]}"
    for g, (a, b) in enumerate(zip(got_gens, exp_gens)):
        assert_records(a, b, exact=exact, what=f"{what} gen {g}")


def gausslet_case_names():
    return sorted(os.path.basename(p)[len("gauss_"):-4] for p in glob.glob(os.path.join(GOLDEN, "gauss_*.npz")))


def load_gausslet_case(name):
    z = np.load(os.path.join(GOLDEN, f"gauss_{name}.npz"))
    offs = z["offsets"].astype(np.int64)
    out = z["out"].astype(ctracer.gausslet_dtype)
    return dict(spec=json.loads(str(z["spec"])), params=json.loads(str(z["params"])),
                gausslets=z["gausslets"].astype(ctracer.gausslet_dtype), wl=z["wl"],
                gens=[out[offs[g]:offs[g + 1]] for g in range(len(offs) - 1)], counts=z["counts"])


def assert_gausslets(got, exp, exact=False, what=""):
    assert len(got) == len(exp), f"{what}: {len(got)} gausslets vs {len(exp)}"
    assert_records(np.ascontiguousarray(got["base_ray"]), np.ascontiguousarray(exp["base_ray"]), exact=exact,
                   what=what + " base")
    for f in ("origin", "direction", "normal", "length"):
        a, b = got["para_rays"][f], exp["para_rays"][f]
        if exact:
            assert np.array_equal(np.ascontiguousarray(a).view(np.uint8), np.ascontiguousarray(b).view(np.uint8)), \
                f"{what}: parabasal {f} differs"
        else:
            np.testing.assert_allclose(a, b, rtol=RTOL, atol=ATOL, equal_nan=True, err_msg=f"{what}: parabasal {f}")


def assert_gausslet_generations(got_gens, exp_gens, exact=False, what=""):
    assert [len(g) for g in got_gens] == [len(g) for g in exp_gens], \
        f"{what}: generation sizes {[len(g) for g in got_gens]} vs {[len(g) for g in exp_gens]}"
    for g, (a, b) in enumerate(zip(got_gens, exp_gens)):
        assert_gausslets(a, b, exact=exact, what=f"{what} gen {g}")


def oracle_trace_parallel(tables, wavelengths, records, recursion_limit, max_length, e2_terminate=0.0, chunks=None,
                          counts=False):
    """The oracle's trace of `records`, cut into contiguous chunks traced on
    threads (the oracle is re-entrant and ctypes releases the GIL around each
    call), merged back into the single-trace order with parent indices
    rebased.  Returns the generations (and, with counts=True, also the
    per-face hit counts summed over the chunks).  Every ray's children depend
    on that ray alone, so the merge equals one trace of all the rays."""
    import oracle
    from concurrent.futures import ThreadPoolExecutor
    from raypier_optics_gb300 import shard
    n = len(records)
    k = chunks or max(1, min(os.cpu_count() or 1, 32, (n + 1023) // 1024))
    bounds = [shard.shard_bounds(n, k, r) for r in range(k)]

    def one(b):
        lo, hi = b
        return oracle.trace_rays(tables, wavelengths, np.ascontiguousarray(records[lo:hi]), recursion_limit,
                                 max_length, e2_terminate)

    with ThreadPoolExecutor(k) as ex:
        per = list(ex.map(one, bounds))
    gens = shard.merge_generations([p[0] for p in per])
    if counts:
        return gens, np.sum([np.asarray(p[1], dtype=np.int64) for p in per], axis=0)
    return gens
