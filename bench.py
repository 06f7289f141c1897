"""Benchmark of the non-sequential tracing hot path on GB300.

Workload (default): the 1,048,576-ray, 10-face polarised doublet/asphere
system with per-ray Sellmeier dispersion and Fresnel splitting, 8
generations, |E|^2 < 1e-6 termination (raypier_optics_gb300.workloads.config2).
One step = one full trace_rays of that workload.

  value  ray-segments/s of the mixed FP32 / float-float path with the input
         rays already resident in HBM (rp_trace_rays on a device buffer; scene
         uploaded once); `plain_fp64` holds the all-FP64 path on the same
         workload and `precision_vs_plain_fp64` the mixed path's error
         against it (--flags plain makes the FP64 path the headline)
  e2e    the same metric through the C-ABI host-buffer call
         rp_trace_rays_host: pinned host input records -> device -> all
         generations back into pinned host memory, copies inside the timing
  roofline  the generation kernel's algorithmic HBM bytes / its measured time
  cpu_baseline  the reference's Cython tracer (or the C port when the reference
         cannot be built) on the host cores, on a bounded sample

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
       [--workload config2|config1|config3] [--flags plain|mixed]
Under torchrun (N > 1) every rank traces its own 1,048,576-ray shard (weak
scaling: independent rays, no data-path collective); rank 0 prints the line.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)
sys.path.insert(0, os.path.join(REPO, "oracle"))

METRIC = "ray-segments/s at 1M rays, mixed vs plain FP64 on 1 GB300; p50/p99 job latency"
UNIT = "ray-segments/s"
# Algorithmic bytes of the generation kernels (structure of arrays; a
# "gathered" ray is one of generation > 0, read through the gather map from
# its parents' child slots and written to its final record by the kernel that
# traces it):
#   plain generation kernel: per traced ray 168 B (origin, direction,
#     E_vector 72; n, E1, E2 48; OPL, phase 16; wavelength_idx, type, ident
#     12; the ray's wavelength 8; length and end face written 12), per
#     gathered ray 208 B more (map entry 4, normal and parent 28, the other
#     176 B of its record written), per child 188 B written
#   mixed search kernel: per traced ray 72 B (origin, direction 48 read;
#     length, end face 12 and the hand-over's ray parameter and face 12
#     written), per gathered ray 308 B more (map entry 4, the other 100 B of
#     its fields and 28 B of pass-through read, the other 176 B of its record
#     written)
#   mixed material kernel: per ray 4 B (the hand-over's face), per hit 160 B
#     (its 148 B of fields and 12 B of hand-over; the hits on absorbing faces
#     are counted too, so this is an upper bound), per child 188 B written
BYTES = {"plain": {"segment": 168, "gathered": 208, "child": 188},
         "search": {"segment": 72, "gathered": 308},
         "material": {"segment": 4, "hit": 160, "child": 188}}
# FP64 floating-point operations per segment of the plain kernel (ncu: dadd +
# dmul + 2 dfma thread instructions, 859.7 M over the 1,046,875 rays of
# generation 3 of the 262,144-ray configuration-2 trace, this build)
PLAIN_FP64_FLOPS_PER_SEGMENT = 821.2
# DRAM bytes per input ray of a launch, from ncu on generation 3 of the
# 262,144-ray configuration-2 trace (1,046,875 gathered rays), this build:
# dram__bytes_read.sum + dram__bytes_write.sum of each kernel
NCU_TRAFFIC_PER_RAY = {"generation_plain_kernel": 811.6, "mixed_search_kernel": 331.2,
                       "mixed_material_kernel": 425.4}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="config2", choices=["config1", "config2", "config3"])
    ap.add_argument("--flags", default="mixed", choices=["plain", "mixed"])
    ap.add_argument("--rays", type=int, default=0, help="override the ray count")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true", help="skip the host-buffer end-to-end leg")
    ap.add_argument("--e2e-steps", type=int, default=30, help="timed steps of the end-to-end leg (at least --steps)")
    ap.add_argument("--no-mixed", action="store_true", help="skip the second path's leg (plain FP64 when the "
                    "headline is mixed, mixed when it is plain) and the precision sample")
    ap.add_argument("--cpu-sample", type=int, default=0, help="rays in the CPU-baseline sample")
    ap.add_argument("--no-serving", action="store_true", help="skip the job-server stream (configuration 5)")
    ap.add_argument("--serving-jobs", type=int, default=10000, help="jobs in the served stream")
    ap.add_argument("--serving-lanes", type=int, default=64,
                    help="jobs the server holds in flight (each step advances all of them by one generation)")
    ap.add_argument("--serving-isolated", type=float, default=0.03,
                    help="fraction of the stream's jobs, the costliest, also run alone for the isolated service times")
    ap.add_argument("--serving-baseline-jobs", type=int, default=500,
                    help="jobs of the same stream run one at a time through the plain FP64 path")
    ap.add_argument("--no-adjoint", action="store_true", help="skip the differentiable-lens leg (configuration 4)")
    ap.add_argument("--no-clutter", action="store_true",
                    help="skip the clutter-scene leg (configuration 3: mixed at 16.8M rays, plain FP64 at 1M)")
    ap.add_argument("--clutter-rays", type=int, default=1 << 24,
                    help="rays of the clutter-scene leg's mixed path (its plain path takes at most 1M)")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the Gausslet, sequential and E-field legs")
    return ap.parse_args()


def dist_env():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), \
        int(os.environ.get("LOCAL_RANK", "0"))


def workload(name, rays_override=0, rank=0):
    from raypier_optics_gb300 import ctracer
    from raypier_optics_gb300 import workloads as W
    if name == "config1":
        n = rays_override or 4096
        rays, wl = W.config1_rays(ctracer.ray_dtype, n)
        return W.config1_spec(), rays, wl, W.CONFIG1, False
    if name == "config2":
        n = rays_override or (1 << 20)
        rays, wl = W.config2_rays(ctracer.ray_dtype, n, seed=2 + 1000 * rank)
        return W.config2_spec(), rays, wl, W.CONFIG2, True
    n = rays_override or (1 << 20)
    rays, wl = W.config3_rays(ctracer.ray_dtype, n, first_block=rank * ((n + 65535) // 65536))
    return W.config3_spec(), rays, wl, W.CONFIG3, False


class ClockSampler:
    """nvidia-smi clocks / throttle reasons every 200 ms during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device=0):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        for line in self.lines:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for name, v in zip(("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"),
                               f[5:9]):
                if v.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def pipe_peaks(lib, device):
    """FP64 / FP32 fused multiply-add and INT32 multiply-add peaks measured on
    this device by the library (rp_measure_peaks)."""
    a, b, c = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
    if lib.rp_measure_peaks(device, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)) != 0:
        return None
    return {"fp64_tflops": a.value / 1e12, "fp32_tflops": b.value / 1e12, "int32_tops": c.value / 1e12,
            "how": "rp_measure_peaks: 8 independent multiply-add chains per thread, 8 waves of resident blocks, "
                   "best of 3 launches timed with CUDA events"}


def host_link(lib, device):
    """The host link's D2H / H2D copy rates measured on this device by the
    library (rp_measure_host_link), the bound of the e2e leg."""
    a, b = ctypes.c_double(), ctypes.c_double()
    if lib.rp_measure_host_link(device, ctypes.byref(a), ctypes.byref(b)) != 0:
        return None
    return {"d2h_gbs": a.value / 1e9, "h2d_gbs": b.value / 1e9,
            "how": "rp_measure_host_link: one 256 MB cudaMemcpyAsync each way with page-locked host memory, "
                   "best of 3 after a warm-up, CUDA events"}


def e2e_link(h2d_bytes, d2h_bytes, step_ms, peaks):
    """The e2e step's bound by the host link: its input's upload and its
    generations' download at the measured copy rates (the downloads overlap
    the trace, the upload precedes it), against the fastest timed step."""
    link = (peaks or {}).get("host_link")
    if not link or not link["d2h_gbs"] or not link["h2d_gbs"]:
        return None
    bound_ms = h2d_bytes / (link["h2d_gbs"] * 1e6) + d2h_bytes / (link["d2h_gbs"] * 1e6)
    return {"bound_ms": bound_ms, "min_step_ms": step_ms, "frac": bound_ms / step_ms,
            "d2h_gbs": link["d2h_gbs"], "h2d_gbs": link["h2d_gbs"]}


def kernel_rooflines(flags, st, n_first, hbm_peak, hbm_kind, peaks):
    """Achieved HBM bandwidth (algorithmic bytes over the kernel's summed
    launch time) and, for the plain kernel, FP64 throughput, each against its
    measured peak, for the generation kernels of one path over the timed
    steps (st: their rp_stats)."""
    segs, children, hits = float(st.rays_in), float(st.rays_out), float(st.hits)
    gathered = max(segs - n_first, 0.0)
    out = []

    def entry(kernel, ms, nbytes, launches, pipe=None):
        s = ms / 1000.0
        e = {"kernel": kernel, "ms": ms, "hbm": {"achieved_gbs": nbytes / s / 1e9, "peak_gbs": hbm_peak,
                                                  "frac": nbytes / s / 1e9 / hbm_peak, "peak_kind": hbm_kind},
             "algorithmic_bytes": nbytes,
             "traffic_bytes_per_launch": NCU_TRAFFIC_PER_RAY[kernel] * segs / max(launches, 1)}
        e["bound"] = "hbm"
        if pipe:
            e["pipe"] = pipe
            if pipe["frac"] > e["hbm"]["frac"]:
                e["bound"] = pipe["name"]
        out.append(e)

    gens = max(st.generations, 1)
    if flags == 0:
        B = BYTES["plain"]
        nbytes = segs * B["segment"] + gathered * B["gathered"] + children * B["child"]
        pipe = None
        if peaks:
            f = PLAIN_FP64_FLOPS_PER_SEGMENT * segs / (st.kernel_ms / 1000.0) / 1e12
            pipe = {"name": "fp64", "achieved_tflops": f, "peak_tflops": peaks["fp64_tflops"],
                    "frac": f / peaks["fp64_tflops"], "note": "flops per segment from ncu (dadd + dmul + 2 dfma)"}
        entry("generation_plain_kernel", st.kernel_ms, nbytes, gens, pipe)
    else:
        B = BYTES["search"]
        entry("mixed_search_kernel", st.search_ms, segs * B["segment"] + gathered * B["gathered"], gens)
        B = BYTES["material"]
        entry("mixed_material_kernel", st.kernel_ms - st.search_ms,
              segs * B["segment"] + hits * B["hit"] + children * B["child"], gens)
    return out


def measured_peak_hbm():
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def cpu_baseline(name, rays, wl, per_ray, sample):
    import cpu_bench
    n = min(sample, rays.shape[0])
    idx = np.linspace(0, rays.shape[0] - 1, n).astype(np.int64)
    r = cpu_bench.time_cpu(name, rays[idx], wl, per_ray)
    r["sample"] = (f"{n} rays spread over the {rays.shape[0]}-ray workload, all generations, "
                   f"{r['cores']} processes on {cpu_bench.cpu_model()}")
    return r


def run_reference_arm(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    spec, rays, wl, P, per_ray = workload(args.workload, args.rays)
    import cpu_bench
    sample = args.cpu_sample or 16384
    n = min(sample, rays.shape[0])
    idx = np.linspace(0, rays.shape[0] - 1, n).astype(np.int64)
    for _ in range(args.warmup):
        cpu_bench.time_cpu(args.workload, rays[idx[: max(len(idx) // 8, 64)]], wl, per_ray)
    vals, segs, secs, res = [], 0, 0.0, None
    for _ in range(args.steps):
        res = cpu_bench.time_cpu(args.workload, rays[idx], wl, per_ray)
        segs += res["segments"]
        secs += res["seconds"]
    value = segs / secs
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000.0 * secs / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded, PCG64)",
            "impl": "reference",
            "config": {"workload": f"{args.workload}: {rays.shape[0]} rays, sampled", "rays_per_step": n,
                       "recursion_limit": P["recursion_limit"]},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": res["cores"], "kind": res["kind"],
                             "sample": f"{n} rays of {rays.shape[0]} per step, {res['cores']} processes on "
                                       f"{cpu_bench.cpu_model()}"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference_arm(args)
    rank, world, local = dist_env()
    spec, rays, wl, P, per_ray = workload(args.workload, args.rays, rank)

    # CPU baseline first: its worker processes start before any GPU context exists
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline(args.workload, rays, wl, per_ray, args.cpu_sample or 16384)

    from raypier_optics_gb300 import _native, runtime, scene
    from raypier_optics_gb300 import workloads as W
    from raypier_optics_gb300.ctracer import ray_dtype
    import types
    from raypier_optics_gb300 import cdistortions, cfaces, cmaterials, cshapes, ctracer
    dist = None
    if world > 1:
        import torch
        import torch.distributed as tdist
        tdist.init_process_group("gloo")
        dist = tdist
        device = local
    else:
        device = 0
    ctx = runtime.Context(device)
    lib = ctx.lib
    ns = types.SimpleNamespace(ctracer=ctracer, cfaces=cfaces, cmaterials=cmaterials, cshapes=cshapes,
                               cdistortions=cdistortions)
    lists = W.build_scene(spec, ns)
    faces = [f for fl in lists for f in fl.faces]
    for i, f in enumerate(faces):
        f.idx = i
        f.update()
    tables = scene.compile_scene(lists)
    dscene = runtime.DeviceScene(ctx, tables, wl)
    flags = 1 if args.flags == "mixed" else 0
    e2 = P["e2_terminate"]
    rl = P["recursion_limit"]
    max_len = ctypes.c_float(P["max_length"])
    n = rays.shape[0]
    max_gens = rl + 1

    # ---- device-resident throughput ---------------------------------------------------
    g0 = runtime.DeviceRays(ctx, n)
    g0.upload(np.ascontiguousarray(rays))

    def step(stats, fl):
        gens = (ctypes.c_void_p * max_gens)()
        gens[0] = g0.handle
        ng = ctypes.c_int32(0)
        _native.check(lib.rp_trace_rays(ctx.handle, dscene.handle, gens, max_gens, rl, max_len, fl, e2,
                                        ctypes.byref(ng), ctypes.byref(stats)), "rp_trace_rays")
        for g in range(1, max_gens):
            if gens[g]:
                lib.rp_rays_free(ctypes.c_void_p(gens[g]))
        return ng.value

    def timed(fl, sample_clocks):
        for _ in range(max(args.warmup, 0)):
            step(_native.Stats(), fl)
        ctx.synchronize()
        if dist:
            dist.barrier()
        clocks = ClockSampler(device) if sample_clocks else None
        if clocks:
            clocks.start()
        st = _native.Stats()
        t0 = time.perf_counter()
        ng = 0
        for _ in range(args.steps):
            ng = step(st, fl)
        ctx.synchronize()
        wall = time.perf_counter() - t0
        clk = clocks.stop() if clocks else None
        dev_s = st.device_ms / 1000.0
        segs = float(st.rays_in)
        if dist:
            import torch
            tmax = torch.tensor([dev_s], dtype=torch.float64)
            dist.all_reduce(tmax, op=dist.ReduceOp.MAX)
            tsum = torch.tensor([segs], dtype=torch.float64)
            dist.all_reduce(tsum, op=dist.ReduceOp.SUM)
            dev_s, segs = float(tmax[0]), float(tsum[0])
        return st, dev_s, wall, clk, ng, segs / dev_s

    stats, dev_s, wall, clk, ng, value = timed(flags, True)
    segs = stats.rays_in
    children = stats.rays_out
    seg_per_step = segs / args.steps
    other = None
    if not args.no_mixed:
        ost, odev_s, _, _, _, ovalue = timed(1 - flags, False)
        other = {"value": ovalue, "unit": UNIT, "ms_per_step": 1000.0 * odev_s / args.steps,
                 "kernel": "mixed_search_kernel + mixed_material_kernel" if flags == 0 else "generation_plain_kernel",
                 "kernel_ms_per_step": ost.kernel_ms / args.steps}
        mixed_v, plain_v = (ovalue, value) if flags == 0 else (value, ovalue)
        other["speedup_mixed_vs_plain_fp64"] = mixed_v / plain_v
        other["precision_vs_plain_fp64"] = precision_sample(ctx, spec, rays, wl, P, per_ray)
    # rooflines of the generation kernels
    peak, peak_kind = measured_peak_hbm()
    peaks = pipe_peaks(lib, device)
    if peaks is not None:
        peaks["host_link"] = host_link(lib, device)
    krl = kernel_rooflines(flags, stats, n * args.steps, peak, peak_kind, peaks)
    if other is not None:
        krl += kernel_rooflines(1 - flags, ost, n * args.steps, peak, peak_kind, peaks)

    # ---- end to end through the host-buffer C ABI -----------------------------------------
    e2e_value, d2h, e2e_steps = None, 0, {"steps": 0}
    if not args.no_e2e:
        e2e_value, d2h, e2e_steps = run_e2e(args, ctx, lib, dscene, rays, n, rl, max_len, flags, e2, max_gens,
                                            seg_per_step, dist, world)
    extra = {}
    if rank == 0 and world == 1 and not args.no_adjoint:
        extra["adjoint"] = adjoint_leg(ctx)
    if rank == 0 and world == 1 and not args.no_clutter and args.workload != "config3":
        extra["clutter"] = clutter_leg(ctx, args)
    if rank == 0 and world == 1 and not args.no_serving:
        extra["serving"] = serving_leg(args)
    if rank == 0 and world == 1 and not args.no_extras:
        extra["extras"] = extras_leg(ctx)
    if rank == 0:
        emit(args, world, value, dev_s, wall, ng, n, faces, rl, e2, seg_per_step, e2e_value, d2h, e2e_steps,
             krl, peaks, flags, stats, clk, cpu, other, extra)
    if dist:
        dist.barrier()
        dist.destroy_process_group()
    return 0


def run_e2e(args, ctx, lib, dscene, rays, n, rl, max_len, flags, e2, max_gens, seg_per_step, dist, world):
    """rp_trace_rays_host on pinned host records, --e2e-steps timed calls (at
    least --steps): each step's ~11 GB of generations cross the host link,
    which other work on the machine can hold up for a few hundred ms, so
    more steps keep one such stall from setting the mean."""
    from raypier_optics_gb300 import _native
    # output capacity: the measured segment count of a step plus headroom
    out_cap = int(seg_per_step * 1.05) + n
    pin_in = ctypes.c_void_p()
    pin_out = ctypes.c_void_p()
    _native.check(lib.rp_host_alloc(n * 188, ctypes.byref(pin_in)), "rp_host_alloc")
    _native.check(lib.rp_host_alloc(out_cap * 188, ctypes.byref(pin_out)), "rp_host_alloc")
    ctypes.memmove(pin_in, np.ascontiguousarray(rays).ctypes.data, n * 188)
    offs = (ctypes.c_uint64 * (max_gens + 1))()
    e2e_steps = max(1, args.steps, args.e2e_steps)

    def e2e_step(st):
        ng = ctypes.c_int32(0)
        _native.check(lib.rp_trace_rays_host(ctx.handle, dscene.handle, pin_in, n, rl, max_len, flags, e2, pin_out,
                                             out_cap, offs, max_gens, ctypes.byref(ng), ctypes.byref(st)),
                      "rp_trace_rays_host")
        return offs[ng.value]

    e2e_step(_native.Stats())
    ctx.synchronize()
    if dist:
        dist.barrier()
    est = _native.Stats()
    t0 = time.perf_counter()
    d2h = 0
    step_s = []
    for _ in range(e2e_steps):
        ts = time.perf_counter()
        d2h += e2e_step(est) * 188  # the call returns once its downloads have landed
        step_s.append(time.perf_counter() - ts)
    ctx.synchronize()
    e2e_s = time.perf_counter() - t0
    if dist:
        import torch
        tmax = torch.tensor([e2e_s], dtype=torch.float64)
        dist.all_reduce(tmax, op=dist.ReduceOp.MAX)
        e2e_s = float(tmax[0])
    e2e_value = (est.rays_in * world) / e2e_s
    lib.rp_host_free(pin_in)
    lib.rp_host_free(pin_out)
    step_ms = [1000.0 * t for t in step_s]
    return e2e_value, d2h, {"steps": e2e_steps, "min": min(step_ms), "median": statistics.median(step_ms),
                            "max": max(step_ms), "all": [round(t, 2) for t in step_ms]}


def adjoint_leg(ctx, reps=5):
    """Configuration 4: forward (RMS spot radius) and hand-written adjoint of the
    eight-surface lens on 262,144 rays, host wall time per call (each call
    synchronises)."""
    from raypier_optics_gb300 import lens
    from raypier_optics_gb300 import workloads as W
    L = lens.config4_lens(ctx=ctx)
    p = W.config4_params()
    for _ in range(2):
        L.forward(p)
        L.backward()
    tf = tb = 0.0
    loss = 0.0
    for _ in range(reps):
        t0 = time.perf_counter()
        loss, nv = L.forward(p)
        t1 = time.perf_counter()
        g = L.backward()
        tb += time.perf_counter() - t1
        tf += t1 - t0
    L.close()
    return {"workload": "config4: 262144 rays, 8 even-asphere surfaces, 40 FP64 parameters, loss = RMS spot radius",
            "forward_ms": 1000.0 * tf / reps, "backward_ms": 1000.0 * tb / reps, "loss_mm": loss,
            "rays_reaching_image": int(nv), "grad_norm": float(np.linalg.norm(g)),
            "check": "tests/test_gpu_lens.py: adjoint vs central differences (step 1e-6 rel), all 40 parameters"}


def serving_leg(args):
    """Configuration 5: a Poisson stream of jobs (systems of 2-40 faces from the
    configuration-2 face mix, log-uniform 1e3-4e6 rays, wavelengths 0.4-1.0 um)
    replayed in real time against the job server (mixed path; up to
    --serving-lanes jobs in flight, advanced together one generation per step;
    120 GB budget), with the step loop's counters (device time inside the
    steps, host time around them); then the costliest jobs (by rays x (faces +
    19), which orders their service times) run alone through the same server
    for the 99th percentile of isolated service times, the bound the stream's
    p99 is compared with; the first jobs of the same stream also run one at a
    time through the plain FP64 path."""
    from raypier_optics_gb300 import serve
    from raypier_optics_gb300 import workloads as W
    C = W.CONFIG5
    systems, jobs = W.config5_jobs(args.serving_jobs)
    compiled = [serve.CompiledSystem(s) for s in systems]
    srv = serve.Server(hbm_budget=C["hbm_budget"], lanes=args.serving_lanes)
    res, wall = serve.run_stream(srv, compiled, jobs, flags=1, recursion_limit=C["recursion_limit"],
                                 e2_terminate=C["e2_terminate"])
    st = srv.stats()
    srv.close()
    out = serve.latency_summary(res)
    out.update({"rate_jobs_per_s": C["rate"], "jobs_in_flight_max": args.serving_lanes,
                "hbm_budget_bytes": C["hbm_budget"],
                "path": "mixed", "wall_s": wall, "p99_over_p50": out["p99_ms"] / out["p50_ms"]})
    steps = max(st["steps"], 1)
    out["steps"] = {"count": st["steps"], "jobs_per_step": st["step_jobs"] / steps,
                    "device_ms_mean": st["step_gpu_ms"] / steps, "host_ms_mean": st["step_wall_ms"] / steps,
                    "between_steps_ms_mean": st["idle_wall_ms"] / steps,
                    "device_busy_of_wall": st["step_gpu_ms"] / (wall * 1000.0),
                    "device_busy_of_steps": st["step_gpu_ms"] / max(st["step_wall_ms"] + st["idle_wall_ms"], 1e-9)}
    n_iso = min(len(jobs), max(1, math.ceil(args.serving_isolated * len(jobs))))
    if n_iso > 0 and args.serving_isolated > 0:
        cost = np.array([j["n_rays"] * (compiled[j["system"]].n_faces + 19) for j in jobs], dtype=np.float64)
        top = np.argsort(-cost, kind="stable")[:n_iso]
        srv = serve.Server(hbm_budget=C["hbm_budget"], lanes=args.serving_lanes)
        alone = []
        for k in [top[-1]] + list(top):  # one warm-up job, then each job by itself
            r, _ = serve.run_stream(srv, compiled, [dict(jobs[k], t=0.0)], flags=1,
                                    recursion_limit=C["recursion_limit"], e2_terminate=C["e2_terminate"])
            alone.append(r[0]["t_done_ms"] - r[0]["t_submit_ms"])
        srv.close()
        alone = np.array(alone[1:])
        every = np.full(len(jobs), alone.min())
        every[top] = alone
        iso_p99 = float(np.percentile(every, 99))
        out["isolated"] = {"jobs_run_alone": int(n_iso), "p99_ms": iso_p99, "max_ms": float(alone.max()),
                           "how": f"the {n_iso} costliest jobs by rays x (faces + 19) run one by one through "
                                  "the same server; the others counted at the smallest of their times",
                           "stream_p99_over_isolated_p99": out["p99_ms"] / iso_p99}
    nb = min(args.serving_baseline_jobs, len(jobs))
    if nb > 0:
        srv = serve.Server(hbm_budget=C["hbm_budget"], lanes=1)
        bres, bwall = serve.run_stream(srv, compiled, jobs[:nb], flags=0, recursion_limit=C["recursion_limit"],
                                       e2_terminate=C["e2_terminate"])
        srv.close()
        b = serve.latency_summary(bres)
        b.update({"path": "plain FP64, one job at a time", "wall_s": bwall})
        out["plain_one_at_a_time_fp64"] = b
    return out


def clutter_leg(ctx, args):
    """The 64-face clutter scene (configuration 3: Zernike-distorted planes,
    polynomial faces, prisms, spheres, conic mirrors; 12 generations),
    device-resident: the mixed path on args.clutter_rays rays (the stated
    16,777,216 by default) and the plain FP64 path on the first 1,048,576 of
    them (a full-size plain step takes over a minute; both rates are per
    segment), one warm-up and one timed step each (CUDA events on the library
    stream), their index agreement and errors on a 4096-ray sample, and the
    reference's own CPU code on a 2048-ray sample of the same rays."""
    import types

    import cpu_bench
    from raypier_optics_gb300 import _native, cdistortions, cfaces, cmaterials, cshapes, ctracer, runtime, scene
    from raypier_optics_gb300 import workloads as W
    ns = types.SimpleNamespace(ctracer=ctracer, cfaces=cfaces, cmaterials=cmaterials, cshapes=cshapes,
                               cdistortions=cdistortions)
    lib = ctx.lib
    P = W.CONFIG3
    n = args.clutter_rays
    rays, wl = W.config3_rays(ctracer.ray_dtype, n)
    lists = W.build_scene(W.config3_spec(), ns)
    for i, f in enumerate([f for fl in lists for f in fl.faces]):
        f.idx = i
        f.update()
    ds = runtime.DeviceScene(ctx, scene.compile_scene(lists), wl)
    g0 = runtime.DeviceRays(ctx, n)
    g0.upload(np.ascontiguousarray(rays))
    rl = P["recursion_limit"]
    max_gens = rl + 1
    n_plain = min(n, 1 << 20)
    gp = runtime.DeviceRays(ctx, n_plain)
    gp.upload(np.ascontiguousarray(rays[:n_plain]))

    def step(st, fl):
        gens = (ctypes.c_void_p * max_gens)()
        gens[0] = g0.handle if fl else gp.handle
        ng = ctypes.c_int32(0)
        _native.check(lib.rp_trace_rays(ctx.handle, ds.handle, gens, max_gens, rl, ctypes.c_float(P["max_length"]),
                                        fl, P["e2_terminate"], ctypes.byref(ng), ctypes.byref(st)), "rp_trace_rays")
        for g in range(1, max_gens):
            if gens[g]:
                lib.rp_rays_free(ctypes.c_void_p(gens[g]))

    out = {"workload": f"config3: 64 faces, {rl} generations, |E|^2<{P['e2_terminate']} termination; "
                       f"mixed on {n} rays, plain FP64 on the first {n_plain}",
           "timing": "CUDA events on the library stream, 1 warm-up + 1 timed step per path"}
    for fl, name, rays_n in ((1, "mixed", n), (0, "plain_fp64", n_plain)):
        step(_native.Stats(), fl)
        st = _native.Stats()
        step(st, fl)
        out[name] = {"rays": rays_n, "value": st.rays_in / (st.device_ms / 1000.0), "unit": UNIT,
                     "ms_per_step": st.device_ms, "segments_per_step": st.rays_in}
    out["speedup_mixed_vs_plain_fp64"] = out["mixed"]["value"] / out["plain_fp64"]["value"]
    g0.free()
    gp.free()
    ds.free()
    out["precision_mixed_vs_plain_fp64"] = precision_sample(ctx, W.config3_spec(), rays, wl, P, False, 4096)
    idx = np.linspace(0, n - 1, min(2048, n)).astype(np.int64)
    out["cpu_reference"] = cpu_bench.time_cpu("config3", rays[idx], wl, False)
    out["cpu_reference"]["sample"] = f"{len(idx)} rays spread over the {n}-ray workload, all generations"
    return out


def extras_leg(ctx):
    """The paths beside the headline trace, at bench sizes, each next to the
    reference's own CPU code on a sample of the same inputs: Gausslet tracing
    (configuration-1 lens), sequential tracing (trace_ray_sequence through the
    same lens) and the E-field summation over the traced gausslets' modes.
    Host wall time around each call (every call synchronises)."""
    import types

    import cpu_bench
    from raypier_optics_gb300 import cdistortions, cfaces, cfields, cmaterials, cshapes, ctracer, fields, tracer
    from raypier_optics_gb300 import workloads as W
    ns = types.SimpleNamespace(ctracer=ctracer, cfaces=cfaces, cmaterials=cmaterials, cshapes=cshapes,
                               cdistortions=cdistortions)
    out = {}
    seq = [[0, 0], [0, 1], [1, 0], [1, 1], [2, 0]]

    # Gausslets: 65,536 gausslets (0.05 mm waist) through the config-1 lens, 6 generations, FP64
    n = 65536
    rays, wl = W.config1_rays(ctracer.ray_dtype, n)
    g0 = ctracer.GaussletCollection.from_rays(rays)
    g0.wavelengths = wl
    g0.config_parabasal_rays(wl, 0.05, 0.0)
    garr = g0.copy_as_array()
    best, segs = None, 0
    for _ in range(4):
        gc = ctracer.GaussletCollection.from_array(garr)
        gc.wavelengths = wl
        lists = W.build_scene(W.config1_spec(), ns)
        t0 = time.perf_counter()
        traced, _ = tracer.trace_rays(gc, lists, recursion_limit=6, max_length=1000.0)
        segs = sum(t.n_rays for t in traced)
        dt = time.perf_counter() - t0
        best = dt if best is None else min(best, dt)
    out["gausslets"] = {"workload": f"config-1 lens, {n} gausslets, 6 generations, FP64", "value": segs / best,
                        "unit": "gausslet-segments/s", "segments": segs,
                        "cpu_reference": cpu_bench.time_gausslets_cpu(garr[:: max(n // 4096, 1)], wl)}
    last = traced[-1].copy_as_array()

    # sequential: 1,048,576 rays through the five faces of the config-1 lens in order
    n2 = 1 << 20
    rays2, wl2 = W.config1_rays(ctracer.ray_dtype, n2)
    best, segs = None, 0
    for _ in range(3):
        lists = W.build_scene(W.config1_spec(), ns)
        rc = ctracer.RayCollection.from_array(rays2)
        rc.wavelengths = wl2
        t0 = time.perf_counter()
        traced, _ = tracer.trace_ray_sequence(rc, [(lists[l], f) for l, f in seq], recursion_limit=10,
                                              max_length=1000.0)
        segs = sum(t.n_rays for t in traced)
        dt = time.perf_counter() - t0
        best = dt if best is None else min(best, dt)
    out["sequential"] = {"workload": f"config-1 lens, {n2} rays, 5-face sequence, FP64", "value": segs / best,
                         "unit": "ray-segments/s", "segments": segs,
                         "cpu_reference": cpu_bench.time_sequence_cpu(rays2[:: n2 // 16384], wl2, seq)}

    # E-field: the modes of 16,384 traced gausslets summed at 65,536 points near the focus
    gl = last[: 16384]
    gc = ctracer.GaussletCollection.from_array(gl)
    gc.wavelengths = wl
    summ = fields.EFieldSummation(gc)
    gx, gz = np.meshgrid(np.linspace(-0.5, 0.5, 256), np.linspace(80.0, 120.0, 256))
    pts = np.column_stack([gx.reshape(-1), np.zeros(gx.size), gz.reshape(-1)])
    summ.evaluate(pts[:1024])
    best = None
    for _ in range(3):
        t0 = time.perf_counter()
        summ.evaluate(pts)
        dt = time.perf_counter() - t0
        best = dt if best is None else min(best, dt)
    evals = len(gl) * len(pts)
    out["efield"] = {"workload": f"{len(gl)} gausslet modes x {len(pts)} points, FP64", "value": evals / best,
                     "unit": "mode-evaluations/s",
                     "cpu_reference": cpu_bench.time_field_cpu(summ.base_rays.copy_as_array()[:512],
                                                               summ.modes[:512], wl, pts[:4096])}

    # interaction matrix: modes on a 0.1 mm hexagonal lattice (radius 6.7 mm)
    # against test points every 0.05 mm, pairs within 0.25 mm
    rng = np.random.Generator(np.random.PCG64(5))
    s3 = math.sqrt(3.0)
    ii, jj = np.meshgrid(np.arange(-80, 81), np.arange(-80, 81))
    hx, hy = 0.1 * (ii + 0.5 * jj).reshape(-1), 0.1 * (0.5 * s3 * jj).reshape(-1)
    keep = hx * hx + hy * hy <= 6.7 ** 2
    hx, hy = hx[keep].copy(), hy[keep].copy()
    m = len(hx)
    cur = cfields.calc_mode_curvature(hx, hy, rng.normal(0, 0.02, m), rng.normal(0, 0.02, m), rng.normal(0, 0.5, m),
                                      rng.normal(0, 0.5, m), rng.normal(0, 0.2, m))
    g = np.arange(-6.8, 6.8 + 1e-9, 0.05)
    tx, ty = [v.reshape(-1).copy() for v in np.meshgrid(g, g)]
    im_args = (hx, hy, tx, ty) + tuple(cur) + (0.6, 0.1, 0.25, 1.0, 0.05)
    cfields.build_interaction_matrix(*im_args)
    best, entries = None, 0
    for _ in range(3):
        t0 = time.perf_counter()
        data, _ = cfields.build_interaction_matrix(*im_args)
        dt = time.perf_counter() - t0
        best = dt if best is None else min(best, dt)
        entries = len(data)
    out["interaction_matrix"] = {
        "workload": f"{m} modes x {len(tx)} test points, {entries} pairs within 0.25 mm, FP64, host arrays in and out",
        "value": m * len(tx) / best, "unit": "mode-point pairs/s", "entries": entries,
        "cpu_reference": cpu_bench.time_interaction_cpu(*[a[:256] if k in (0, 1, 4, 5, 6, 7, 8, 9) else a
                                                          for k, a in enumerate(im_args[:10])], *im_args[10:])}
    return out


def precision_sample(ctx, spec, rays, wl, P, per_ray, n_sample=16384):
    """Error of the mixed path against the plain FP64 path on a ray sample."""
    import types
    from raypier_optics_gb300 import cdistortions, cfaces, cmaterials, cshapes, ctracer, precision, tracer
    from raypier_optics_gb300 import workloads as W
    ns = types.SimpleNamespace(ctracer=ctracer, cfaces=cfaces, cmaterials=cmaterials, cshapes=cshapes,
                               cdistortions=cdistortions)
    idx = np.linspace(0, rays.shape[0] - 1, min(n_sample, rays.shape[0])).astype(np.int64)
    sub, swl = W.subsample(rays, wl, idx, per_ray_wavelength=per_ray)
    out = []
    for fl in (tracer.RP_TRACE_PLAIN_FP64, tracer.RP_TRACE_MIXED):
        rc = ctracer.RayCollection.from_array(sub)
        rc.wavelengths = swl
        traced, _ = tracer.trace_rays(rc, W.build_scene(spec, ns), recursion_limit=P["recursion_limit"],
                                      max_length=P["max_length"], flags=fl, e2_terminate=P["e2_terminate"], ctx=ctx)
        out.append([t.copy_as_array() for t in traced])
    st = precision.compare_traces(out[1], out[0])
    st["sample_rays"] = int(len(sub))
    return st


def emit(args, world, value, dev_s, wall, ng, n, faces, rl, e2, seg_per_step, e2e_value, d2h, e2e_steps,
         krl, peaks, flags, stats, clk, cpu, other=None, extra=None):
    head = krl[:1] if flags == 0 else krl[:2]  # the headline path's kernels
    dom = max(head, key=lambda k: k["ms"])     # its dominant kernel
    if True:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000.0 * dev_s / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64" if flags == 0 else "f32+float-float",
            "data": "synthetic (seeded PCG64 rays; no dataset)",
            "config": {"workload": f"{args.workload}: {n} rays, {len(faces)} faces, {rl} generations, "
                                   f"|E|^2<{e2} termination, path={args.flags}",
                       "segments_per_step": seg_per_step, "generations": ng,
                       "l2": "inputs larger than L2 (197 MB of input records, GBs of generations per step)",
                       "timing": "CUDA events on the library stream around each trace call (device time); "
                                 f"host wall {1000.0 * wall / args.steps:.2f} ms/step"},
            "e2e": ({"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": n * 188,
                     "d2h_bytes_per_step": int(d2h / e2e_steps["steps"]), "steps": e2e_steps["steps"],
                     "api": "rp_trace_rays_host (pinned host records in and out)",
                     "step_ms": {k: e2e_steps[k] for k in ("min", "median", "max", "all")},
                     "host_link": e2e_link(n * 188, d2h / e2e_steps["steps"], e2e_steps["min"], peaks)}
                    if e2e_value else None),
            "roofline": {"bound": "hbm", "achieved": dom["hbm"]["achieved_gbs"], "peak": dom["hbm"]["peak_gbs"],
                         "unit": "GB/s", "frac": dom["hbm"]["frac"], "traffic": dom["traffic_bytes_per_launch"],
                         "kernel": dom["kernel"],
                         "note": "the headline path's dominant kernel: algorithmic bytes over its summed launch "
                                 f"time (CUDA events); peak {dom['hbm']['peak_kind']}; traffic = ncu DRAM bytes "
                                 "per input ray x rays per launch (average launch); kernel_rooflines has every "
                                 "generation kernel of both paths with the pipe that bounds it"},
            "kernel_rooflines": krl,
            "measured_peaks": peaks,
            "gpu_launches": int(stats.launches),
            "clocks": clk,
        }
        if other is not None:
            line["mixed" if flags == 0 else "plain_fp64"] = other
        if extra:
            line.update(extra)
        if cpu is not None:
            line["cpu_baseline"] = {"value": cpu["value"], "unit": UNIT, "cores": cpu["cores"], "kind": cpu["kind"],
                                    "sample": cpu["sample"]}
        print(json.dumps(line), flush=True)


if __name__ == "__main__":
    sys.exit(main())
