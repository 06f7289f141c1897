"""Serving: a stream of trace jobs through the library's job server.

``Server`` wraps rp_server: up to ``lanes`` jobs in flight on one device
under one HBM budget, admitted as slots and memory free up; every step of
the server advances all of them by one generation in shared launches of the
mixed-path kernels (continuous batching of generations).  ``run_stream`` replays a timed job stream (configuration 5: Poisson
arrivals, systems of 2-40 faces, log-uniform ray counts) against a server and
returns each job's latency and result.
"""
from __future__ import annotations

import ctypes
import threading
import time
import types

import numpy as np

from . import _native, scene

RP_SOURCE_POINT_CONE = 1
RP_SOURCE_COLLIMATED_DISC = 2


def _ns():
    from . import cdistortions, cfaces, cmaterials, cshapes, ctracer
    return types.SimpleNamespace(ctracer=ctracer, cfaces=cfaces, cmaterials=cmaterials, cshapes=cshapes,
                                 cdistortions=cdistortions)


class CompiledSystem:
    """A scene spec compiled to tables once, submitted by many jobs."""

    def __init__(self, spec):
        from . import workloads as W
        lists = W.build_scene(spec, _ns())
        faces = [f for fl in lists for f in fl.faces]
        for i, f in enumerate(faces):
            f.idx = i
            f.update()
        self.spec = spec
        self.tables = scene.compile_scene(lists)
        self.desc = self.tables.desc()
        self.n_faces = len(faces)
        self.detector = len(faces) - 1  # the last face of the specs here is the detector


def source_desc(kind, n_rays, seed, origin=(0.0, 0.0, -200.0), half_angle=0.05, radius=8.0):
    s = _native.SourceDesc()
    s.type = kind
    s.n_rays = n_rays
    s.seed = seed
    s.origin[:] = origin
    s.half_angle = half_angle
    s.radius = radius
    return s


class Server:
    def __init__(self, device=0, hbm_budget=0, lanes=4):
        self.lib = _native.load()
        h = ctypes.c_void_p()
        _native.check(self.lib.rp_server_create(device, int(hbm_budget), lanes, ctypes.byref(h)), "rp_server_create")
        self.handle = h

    def submit(self, system: CompiledSystem, source, wavelengths, recursion_limit=8, max_length=1000.0,
               flags=1, e2_terminate=1e-6) -> int:
        wl = np.ascontiguousarray(wavelengths, dtype=np.double)
        jd = _native.JobDesc()
        jd.scene = ctypes.cast(ctypes.pointer(system.desc), ctypes.c_void_p)
        jd.wavelengths = wl.ctypes.data
        jd.n_wl = wl.shape[0]
        jd.source = source
        jd.recursion_limit = recursion_limit
        jd.max_length = max_length
        jd.flags = flags
        jd.detector_face = system.detector
        jd.e2_terminate = e2_terminate
        jid = ctypes.c_uint64()
        _native.check(self.lib.rp_server_submit(self.handle, ctypes.byref(jd), ctypes.byref(jid)), "rp_server_submit")
        return jid.value

    def set_step_groups(self, groups, min_chunk):
        """Bounds a step's work: a mixed job's generation of more than
        `groups` 128-ray groups is traced over several steps (at least
        `min_chunk` groups each); results do not depend on it."""
        _native.check(self.lib.rp_server_set_step_groups(self.handle, int(groups), int(min_chunk)),
                      "rp_server_set_step_groups")

    def stats(self) -> dict:
        """The step loop's counters since creation: steps, jobs summed over
        the steps, the steps' device time, host time inside the steps and
        host time between steps while jobs were in flight (ms)."""
        st = _native.ServerStats()
        _native.check(self.lib.rp_server_get_stats(self.handle, ctypes.byref(st)), "rp_server_get_stats")
        return {k: getattr(st, k) for k, _ in _native.ServerStats._fields_}

    def wait(self, job_id, n_faces=0):
        r = _native.JobResult()
        counts = np.zeros(max(n_faces, 1), dtype=np.uint32)
        _native.check(self.lib.rp_server_wait(self.handle, job_id, ctypes.byref(r), counts.ctypes.data, n_faces),
                      "rp_server_wait")
        out = {k: getattr(r, k) for k, _ in _native.JobResult._fields_}
        out["face_counts"] = counts[:n_faces].copy()
        return out

    def close(self):
        if getattr(self, "handle", None):
            self.lib.rp_server_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def run_stream(server: Server, systems, jobs, flags=1, recursion_limit=8, e2_terminate=1e-6, time_scale=1.0,
               max_length=1000.0):
    """Submits `jobs` at their arrival times (seconds, scaled by time_scale) and
    waits for all of them.  Returns (results in job order, wall seconds)."""
    ids = [None] * len(jobs)
    results = [None] * len(jobs)
    submitted = threading.Semaphore(0)

    def waiter():
        for k in range(len(jobs)):
            submitted.acquire()
            results[k] = server.wait(ids[k], systems[jobs[k]["system"]].n_faces)

    th = threading.Thread(target=waiter, daemon=True)
    th.start()
    t0 = time.perf_counter()
    for k, j in enumerate(jobs):
        delay = t0 + j["t"] * time_scale - time.perf_counter()
        if delay > 0:
            time.sleep(delay)
        src = source_desc(j["source"], j["n_rays"], j["seed"])
        ids[k] = server.submit(systems[j["system"]], src, j["wavelengths"], recursion_limit=recursion_limit,
                               max_length=max_length, flags=flags, e2_terminate=e2_terminate)
        submitted.release()
    th.join()
    return results, time.perf_counter() - t0


def latency_summary(results):
    lat = np.array([r["t_done_ms"] - r["t_submit_ms"] for r in results])
    queue = np.array([r["t_start_ms"] - r["t_submit_ms"] for r in results])
    span = max(r["t_done_ms"] for r in results) - min(r["t_submit_ms"] for r in results)
    segs = float(sum(r["segments"] for r in results))
    return {"jobs": len(results), "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
            "mean_ms": float(lat.mean()), "max_ms": float(lat.max()), "queue_p50_ms": float(np.percentile(queue, 50)),
            "queue_p99_ms": float(np.percentile(queue, 99)), "jobs_per_s": len(results) / (span / 1000.0),
            "segments_per_s": segs / (span / 1000.0), "segments": segs,
            "failed": int(sum(1 for r in results if r["status"] != 0))}
