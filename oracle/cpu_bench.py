"""CPU timing of the reference tracing path, for bench.py's CPU-baseline leg
and its reference arm.

TEST/BENCH INFRASTRUCTURE ONLY.  Times the reference's own Cython tracer
(oracle/_ref, built from the reference sources by oracle/build_ref.py) when it
is available -- kind "reference" -- and otherwise the C restatement
(oracle/rp_oracle.c) -- kind "port".  Rays are independent, so the sample is
cut into contiguous shards traced by a pool of worker processes (spawned, so
no process is forked after a GPU context exists).
"""
from __future__ import annotations

import contextlib
import io
import multiprocessing as mp
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)


def _setup_path():
    for p in (REPO, HERE):
        if p not in sys.path:
            sys.path.insert(0, p)


def reference_available() -> bool:
    _setup_path()
    import build_ref
    try:
        return build_ref.have_built() or build_ref.build()
    except Exception:
        return False


def _worker(args):
    kind, config, records, wl = args
    _setup_path()
    from raypier_optics_gb300 import workloads as W
    spec = {"config1": W.config1_spec, "config2": W.config2_spec, "config3": W.config3_spec}[config]()
    P = {"config1": W.CONFIG1, "config2": W.CONFIG2, "config3": W.CONFIG3}[config]
    t0 = time.perf_counter()
    if kind == "reference":
        import build_ref
        ref = build_ref.load()
        lists = W.build_scene(spec, ref)
        rc = ref.ctracer.RayCollection.from_array(records.astype(ref.ctracer.ray_dtype))
        rc.wavelengths = wl
        t0 = time.perf_counter()
        with contextlib.redirect_stdout(io.StringIO()):
            traced, _ = ref.tracer.trace_rays(rc, lists, recursion_limit=P["recursion_limit"],
                                              max_length=P["max_length"])
        # the reference applies no |E|^2 rule; its segment count is the work it did
        segs = sum(t.n_rays for t in traced)
    else:
        import types
        import oracle
        from raypier_optics_gb300 import cdistortions, cfaces, cmaterials, cshapes, ctracer, scene
        ns = types.SimpleNamespace(ctracer=ctracer, cfaces=cfaces, cmaterials=cmaterials, cshapes=cshapes,
                                   cdistortions=cdistortions)
        lists = W.build_scene(spec, ns)
        faces = [f for fl in lists for f in fl.faces]
        for i, f in enumerate(faces):
            f.idx = i
            f.update()
        tables = scene.compile_scene(lists)
        oracle.load()
        t0 = time.perf_counter()
        gens, _ = oracle.trace_rays(tables, wl, records, P["recursion_limit"], P["max_length"], 0.0)
        segs = sum(len(g) for g in gens)
    return segs, time.perf_counter() - t0


def time_cpu(config, records, wl, per_ray_wl, processes=None, shards=None, kind=None):
    """Traces `records` on the host in `shards` shards over `processes`
    processes; returns dict(value=segments/s, segments, seconds, cores, kind)."""
    _setup_path()
    if kind is None:
        kind = "reference" if reference_available() else "port"
    if kind == "port":
        import oracle
        oracle.build()
    P = processes or len(os.sched_getaffinity(0))
    n = records.shape[0]
    shards = shards or max(P, 1)
    bounds = np.linspace(0, n, shards + 1).astype(np.int64)
    jobs = []
    for a, b in zip(bounds[:-1], bounds[1:]):
        rec = records[a:b].copy()
        w = np.asarray(wl)
        if per_ray_wl:
            w = w[rec['wavelength_idx']]
            rec['wavelength_idx'] = np.arange(len(rec), dtype=np.uint32)
        jobs.append((kind, config, rec, w))
    ctx = mp.get_context("spawn")
    t0 = time.perf_counter()
    with ctx.Pool(P) as pool:
        res = pool.map(_worker, jobs, chunksize=1)
    wall = time.perf_counter() - t0
    segs = sum(r[0] for r in res)
    busy = max(r[1] for r in res)
    # shards run concurrently, one per process: the slowest shard's trace time
    # (process start-up and scene construction excluded) is the sample's time
    return {"value": segs / busy, "segments": int(segs), "seconds": busy, "wall_seconds": wall, "cores": P,
            "kind": kind}


# Arm Ltd. (implementer 0x41) core part numbers of the server cores this may run on
_ARM_PARTS = {"0xd0c": "Arm Neoverse-N1", "0xd40": "Arm Neoverse-V1", "0xd49": "Arm Neoverse-N2",
              "0xd4f": "Arm Neoverse-V2 (NVIDIA Grace)", "0xd8e": "Arm Neoverse-N3", "0xd84": "Arm Neoverse-V3"}


def cpu_model() -> str:
    """The host CPU's name: /proc/cpuinfo's model name on x86, the Arm core
    named from its part number on aarch64."""
    part = None
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                key = line.lower().split(":", 1)[0].strip()
                if key == "model name":
                    return line.split(":", 1)[1].strip()
                if key == "cpu part" and part is None:
                    part = line.split(":", 1)[1].strip().lower()
    except OSError:
        pass
    if part is not None:
        return _ARM_PARTS.get(part, f"Arm core part {part}")
    import platform
    return platform.processor() or platform.machine()


# ---- the paths beside the headline trace (bench.py's extras leg) --------------------
def _gausslet_worker(args):
    records, wl, seq = args
    _setup_path()
    import build_ref
    from raypier_optics_gb300 import workloads as W
    ref = build_ref.load()
    lists = W.build_scene(W.config1_spec(), ref)
    gc = ref.ctracer.GaussletCollection.from_array(records.astype(ref.ctracer.gausslet_dtype))
    gc.wavelengths = wl
    t0 = time.perf_counter()
    with contextlib.redirect_stdout(io.StringIO()):
        if seq:
            traced, _ = ref.tracer.trace_ray_sequence(gc, [(lists[l], f) for l, f in seq], recursion_limit=10,
                                                      max_length=1000.0)
        else:
            traced, _ = ref.tracer.trace_rays(gc, lists, recursion_limit=6, max_length=1000.0)
    return sum(t.n_rays for t in traced), time.perf_counter() - t0


def _sequence_worker(args):
    records, wl, seq = args
    _setup_path()
    import build_ref
    from raypier_optics_gb300 import workloads as W
    ref = build_ref.load()
    lists = W.build_scene(W.config1_spec(), ref)
    rc = ref.ctracer.RayCollection.from_array(records.astype(ref.ctracer.ray_dtype))
    rc.wavelengths = wl
    t0 = time.perf_counter()
    with contextlib.redirect_stdout(io.StringIO()):
        traced, _ = ref.tracer.trace_ray_sequence(rc, [(lists[l], f) for l, f in seq], recursion_limit=10,
                                                  max_length=1000.0)
    return sum(t.n_rays for t in traced), time.perf_counter() - t0


def _pool_time(worker, records, wl, seq, processes=None):
    P = processes or len(os.sched_getaffinity(0))
    bounds = np.linspace(0, records.shape[0], P + 1).astype(np.int64)
    jobs = [(records[a:b].copy(), np.asarray(wl), seq) for a, b in zip(bounds[:-1], bounds[1:]) if b > a]
    with mp.get_context("spawn").Pool(len(jobs)) as pool:
        res = pool.map(worker, jobs, chunksize=1)
    segs = sum(r[0] for r in res)
    busy = max(r[1] for r in res)
    return {"value": segs / busy, "segments": int(segs), "seconds": busy, "cores": len(jobs), "kind": "reference"}


def time_gausslets_cpu(records, wl, seq=None):
    """The reference's Gausslet trace (config-1 lens) of `records`, gausslet
    segments per second over the host cores.  None without the reference."""
    if not reference_available():
        return None
    return _pool_time(_gausslet_worker, records, wl, seq)


def time_sequence_cpu(records, wl, seq):
    """The reference's trace_ray_sequence of rays through the config-1 lens."""
    if not reference_available():
        return None
    return _pool_time(_sequence_worker, records, wl, seq)


def time_field_cpu(rays, modes, wl, points):
    """The reference's sum_gaussian_modes (OpenMP over the points) in this
    process: mode evaluations per second.  None without the reference."""
    if not reference_available():
        return None
    _setup_path()
    import build_ref
    ref = build_ref.load()
    rc = ref.ctracer.RayCollection.from_array(np.ascontiguousarray(rays).astype(ref.ctracer.ray_dtype))
    t0 = time.perf_counter()
    ref.cfields.sum_gaussian_modes(rc, np.ascontiguousarray(modes), np.asarray(wl, dtype=np.double),
                                   np.ascontiguousarray(points), 0.0)
    dt = time.perf_counter() - t0
    return {"value": len(rays) * len(points) / dt, "evaluations": int(len(rays) * len(points)), "seconds": dt,
            "cores": len(os.sched_getaffinity(0)), "kind": "reference"}


def time_interaction_cpu(rx, ry, tx, ty, A, B, C, X, Y, Z, wavelength, spacing, max_spacing, blending, test_spacing):
    """The reference's build_interaction_matrix (one thread) in this process:
    mode-point pairs tested per second.  None without the reference."""
    if not reference_available():
        return None
    _setup_path()
    import build_ref
    ref = build_ref.load()
    a = [np.ascontiguousarray(v, dtype=np.double) for v in (rx, ry, tx, ty, A, B, C, X, Y, Z)]
    t0 = time.perf_counter()
    ref.cfields.build_interaction_matrix(*a, wavelength, spacing, max_spacing, blending, test_spacing)
    dt = time.perf_counter() - t0
    return {"value": len(rx) * len(tx) / dt, "pairs": int(len(rx) * len(tx)), "seconds": dt, "cores": 1,
            "kind": "reference"}
