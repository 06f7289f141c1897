"""The mixed FP32/FP64 path against the FP64 oracle.

Directions, normals and the polarisation / Fresnel arithmetic are FP32; ray
positions, distances (quadratic roots, last asphere Newton step) and the
optical path stay FP64.  Index fields agree with the oracle except for rays
that graze an edge, so the checks are statistical: generation sizes within
0.1 %, index agreement above 99.9 %, and the float error bounds below on the
rays whose indices agree."""
import numpy as np
import pytest

import oracle
from helpers import build, load_case, tables_for, trace_case_names
from raypier_optics_gb300 import ctracer, precision, tracer
from raypier_optics_gb300 import workloads as W
from raypier_optics_gb300.ctracer import RayCollection

pytestmark = pytest.mark.gpu

# bounds asserted on the rays whose indices match the FP64 oracle
POSITION_NM_P99 = 100.0
OPL_NM_P99 = 10.0
DIRECTION_RAD_P99 = 1e-5


def mixed_trace(spec, rays, wl, P):
    lists, _ = build(spec)
    rc = RayCollection.from_array(rays)
    rc.wavelengths = wl
    traced, _ = tracer.trace_rays(rc, lists, recursion_limit=P["recursion_limit"], max_length=P["max_length"],
                                  flags=tracer.RP_TRACE_MIXED, e2_terminate=P["e2_terminate"])
    return [t.copy_as_array() for t in traced]


@pytest.mark.parametrize("config", ["config1", "config2"])
def test_mixed_path_accuracy_against_oracle(config):
    if config == "config1":
        rays, wl = W.config1_rays(ctracer.ray_dtype)
        spec, P = W.config1_spec(), W.CONFIG1
    else:
        rays, wl = W.config2_rays(ctracer.ray_dtype, 1 << 20)
        rays, wl = W.subsample(rays, wl, np.arange(0, 1 << 20, 256), per_ray_wavelength=True)
        spec, P = W.config2_spec(), W.CONFIG2
    gens = mixed_trace(spec, rays, wl, P)
    tables, _, _ = tables_for(spec)
    ogens, _ = oracle.trace_rays(tables, wl, rays, P["recursion_limit"], P["max_length"], P["e2_terminate"])
    sizes, osizes = [len(g) for g in gens], [len(g) for g in ogens]
    assert len(sizes) == len(osizes)
    assert all(abs(a - b) <= max(2, 1e-3 * b) for a, b in zip(sizes, osizes)), (sizes, osizes)
    st = precision.compare_traces(gens, ogens)
    print(config, st)
    assert st["index_agreement"] > 0.999
    assert st["position_nm"]["p99"] < POSITION_NM_P99
    assert st["opl_nm"]["p99"] < OPL_NM_P99
    assert st["direction_rad"]["p99"] < DIRECTION_RAD_P99


def test_mixed_path_config3_runs_and_mostly_agrees():
    rays, wl = W.config3_rays(ctracer.ray_dtype, 512)
    gens = mixed_trace(W.config3_spec(), rays, wl, W.CONFIG3)
    tables, _, _ = tables_for(W.config3_spec())
    ogens, _ = oracle.trace_rays(tables, wl, rays, 12, 1000.0, 1e-6)
    st = precision.compare_traces(gens, ogens)
    print("config3", st)
    assert st["index_agreement"] > 0.99


@pytest.mark.parametrize("name", [n for n in trace_case_names() if n.startswith(("face_", "mat_"))])
def test_mixed_path_on_every_face_and_material_case(name):
    """Each face and material type through the mixed kernel (its float-float
    code where it has one, its FP64 code otherwise) against the reference's
    golden trace of the same rays."""
    c = load_case(name)
    P = dict(c["params"])
    P.setdefault("e2_terminate", 0.0)
    gens = mixed_trace(c["spec"], c["rays"], c["wl"], P)
    st = precision.compare_traces(gens, c["gens"])
    sizes, osizes = [len(g) for g in gens], [len(g) for g in c["gens"]]
    assert len(sizes) == len(osizes) and all(abs(a - b) <= 2 for a, b in zip(sizes, osizes)), (sizes, osizes)
    assert st["index_agreement"] > 0.97, st
    if st["position_nm"]["p99"] is not None:
        assert st["position_nm"]["p99"] < POSITION_NM_P99, st
        assert st["opl_nm"]["p99"] < OPL_NM_P99, st
