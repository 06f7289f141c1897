"""The trace-job server (configuration 5): a job's result equals the same
trace run through rp_trace_rays (its generations advanced in batched steps
with other jobs' rays sharing the kernels' launches), is the same alone and
among other jobs, and the HBM budget holds jobs back."""
import ctypes

import numpy as np
import pytest

from raypier_optics_gb300 import _native, ctracer, runtime, serve, tracer
from raypier_optics_gb300 import workloads as W

pytestmark = pytest.mark.gpu

FLOAT_RTOL = 1e-9  # host-side sums (another order) against the device's fixed-order tallies


@pytest.fixture(scope="module")
def stream():
    systems, jobs = W.config5_jobs(64, seed=11)
    return [serve.CompiledSystem(s) for s in systems[:16]], jobs


def trace_reference(system, src, wl, flags):
    """The job's rays generated into a device buffer, traced by trace_rays,
    tallied on the host."""
    ctx = runtime.get_context()
    buf = runtime.DeviceRays(ctx, src.n_rays)
    _native.check(ctx.lib.rp_source_generate(ctx.handle, ctypes.byref(src), len(wl), buf.handle),
                  "rp_source_generate")
    recs = np.zeros(src.n_rays, dtype=ctracer.ray_dtype)
    buf.download(recs, src.n_rays)
    buf.free()
    rc = ctracer.RayCollection.from_array(recs)
    rc.wavelengths = wl
    traced, faces = tracer.trace_rays(rc, W.build_scene(system.spec, serve._ns()), recursion_limit=8,
                                      max_length=1000.0, flags=flags, e2_terminate=1e-6)
    gens = [t.copy_as_array() for t in traced]
    hits = np.concatenate([g[g["end_face_idx"] == system.detector] for g in gens])
    p = hits["origin"] + hits["direction"] * hits["length"][:, None]
    power = (np.abs(hits["E1_amp"]) ** 2 + np.abs(hits["E2_amp"]) ** 2) * hits["refractive_index"].real
    return {"generations": len(gens), "segments": sum(len(g) for g in gens), "detector_hits": len(hits),
            "detector_power": power.sum(), "sum_x": p[:, 0].sum(), "sum_y": p[:, 1].sum(),
            "sum_xx": (p[:, 0] ** 2).sum(), "sum_yy": (p[:, 1] ** 2).sum(),
            "face_counts": np.array([f.count for f in faces], dtype=np.uint32)}


@pytest.mark.parametrize("flags,step_groups", [(0, None), (1, None), (1, 24)],
                         ids=["plain_fp64", "mixed", "mixed_in_chunks"])
def test_job_matches_trace_rays(flags, step_groups):
    """A job through the server against the same rays through trace_rays; in
    chunks: every generation of more than 24 groups (3,072 rays) traced over
    several steps of at most 24 groups (at least 8)."""
    spec = W.config5_system(np.random.Generator(np.random.PCG64(3)), 4)
    system = serve.CompiledSystem(spec)
    system.spec = spec
    wl = np.linspace(0.45, 0.95, 32)
    src = serve.source_desc(serve.RP_SOURCE_POINT_CONE, 20000, 1234)
    srv = serve.Server(lanes=1)
    if step_groups:
        srv.set_step_groups(step_groups, 8)
    jid = srv.submit(system, src, wl, flags=flags)
    got = srv.wait(jid, system.n_faces)
    srv.close()
    ref = trace_reference(system, src, wl, flags)
    assert got["status"] == 0
    for k in ("generations", "segments", "detector_hits"):
        assert got[k] == ref[k], k
    np.testing.assert_array_equal(got["face_counts"], ref["face_counts"])
    for k in ("detector_power", "sum_x", "sum_y", "sum_xx", "sum_yy"):
        assert got[k] == pytest.approx(ref[k], rel=FLOAT_RTOL, abs=1e-9), k
    assert ref["detector_hits"] > 0


def test_results_are_the_same_alone_and_in_the_mix(stream):
    systems, jobs = stream
    jobs = [dict(j, n_rays=min(j["n_rays"], 300000), system=j["system"] % len(systems)) for j in jobs]
    probe = jobs[:6]
    # alone: one job in flight at a time
    srv = serve.Server(lanes=1)
    alone = []
    for j in probe:
        jid = srv.submit(systems[j["system"]], serve.source_desc(j["source"], j["n_rays"], j["seed"]), j["wavelengths"])
        alone.append(srv.wait(jid, systems[j["system"]].n_faces))
    srv.close()
    # in the mix: up to eight jobs in flight, the probes among other jobs, all submitted at once
    srv = serve.Server(lanes=8)
    ids = []
    for k, j in enumerate(jobs[:30]):
        ids.append(srv.submit(systems[j["system"]], serve.source_desc(j["source"], j["n_rays"], j["seed"]),
                              j["wavelengths"]))
    mixed = [srv.wait(i, systems[j["system"]].n_faces) for i, j in zip(ids, jobs[:30])]
    srv.close()
    overlap = sum(1 for a in mixed for b in mixed if a is not b and a["t_start_ms"] < b["t_done_ms"]
                  and b["t_start_ms"] < a["t_done_ms"])
    assert overlap > 0, "jobs did not run concurrently"
    for a, b in zip(alone, mixed[:6]):
        assert a["status"] == b["status"] == 0
        for k in ("generations", "segments", "detector_hits", "detector_power", "sum_x", "sum_y", "sum_xx", "sum_yy"):
            assert a[k] == b[k], k
        np.testing.assert_array_equal(a["face_counts"], b["face_counts"])


def test_budget_holds_jobs_back(stream):
    systems, _ = stream
    wl = np.linspace(0.5, 0.9, 8)
    n = 100000
    est = n * 188 * 6
    srv = serve.Server(lanes=4, hbm_budget=int(est * 1.5))
    ids = [srv.submit(systems[k], serve.source_desc(serve.RP_SOURCE_COLLIMATED_DISC, n, 77 + k), wl)
           for k in range(4)]
    res = [srv.wait(i, systems[k].n_faces) for k, i in enumerate(ids)]
    srv.close()
    assert all(r["status"] == 0 for r in res)
    iv = sorted((r["t_start_ms"], r["t_done_ms"]) for r in res)
    for (s0, e0), (s1, e1) in zip(iv, iv[1:]):
        assert s1 >= e0, "two jobs ran together beyond the budget"


def test_submit_rejects_a_bad_source(stream):
    systems, _ = stream
    srv = serve.Server(lanes=1)
    src = serve.source_desc(7, 10, 1)
    with pytest.raises(_native.RPError):
        srv.submit(systems[0], src, np.array([0.5]))
    srv.close()
