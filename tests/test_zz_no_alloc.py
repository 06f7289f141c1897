"""rp_trace_segment_noalloc through the C ABI against rp_trace_segment.

The allocation-free entry point runs the same generation, tile-scan and
placement kernels as rp_trace_segment with its scratch taken from a fixed
device array, so its children and the updated input rays must agree with
rp_trace_segment's within the parity tolerance, on two calls in a row, and the
context's device memory must not change across the calls.  This file is
collected last so that it also runs after every other GPU test has used the
same process and context."""
import ctypes
import os
import re

import numpy as np
import pytest

from helpers import assert_records, tables_for
from raypier_optics_gb300 import _native, ctracer, runtime
from raypier_optics_gb300 import workloads as W

pytestmark = pytest.mark.gpu

P = W.CONFIG2
RP_ERR_CAPACITY = -2


def max_rays():
    text = open(os.path.join(_native.INCLUDE, "rp_gb300.h")).read()
    return int(re.search(r"#define\s+RP_NOALLOC_MAX_RAYS\s+(\d+)", text).group(1))


def config2_sample(n):
    """`n` rays spread over the config-2 workload (1M-ray lens-train bundle)."""
    total = 1 << 20
    rays, wl = W.config2_rays(ctracer.ray_dtype, total)
    idx = np.linspace(0, total - 1, n).astype(np.int64)
    return W.subsample(rays, wl, idx, per_ray_wavelength=True)


def call(entry, ctx, scene, recs, flags):
    """One generation through `entry`; returns (children, updated inputs,
    stats, context bytes before, context bytes after)."""
    lib = ctx.lib
    din = runtime.DeviceRays(ctx, len(recs))
    din.upload(recs)
    dout = runtime.DeviceRays(ctx, 2 * len(recs))
    st = _native.Stats()
    before = ctx.memory_in_use()
    rc = getattr(lib, entry)(ctx.handle, scene.handle, din.handle, dout.handle, ctypes.c_float(P["max_length"]),
                             flags, ctypes.c_double(P["e2_terminate"]), ctypes.byref(st))
    after = ctx.memory_in_use()
    _native.check(rc, entry)
    n_out = dout.count()
    out = np.zeros(n_out, dtype=ctracer.ray_dtype)
    dout.download(out, n_out)
    upd = np.zeros(len(recs), dtype=ctracer.ray_dtype)
    din.download(upd, len(recs))
    din.free()
    dout.free()
    return out, upd, st, before, after


@pytest.mark.parametrize("flags", [0, 1], ids=["plain_fp64", "mixed"])
@pytest.mark.parametrize("n", [4096, None], ids=["4096_rays", "max_rays"])
def test_noalloc_matches_trace_segment_twice(flags, n):
    n = n or max_rays()
    recs, wl = config2_sample(n)
    tables, _, _ = tables_for(W.config2_spec())
    ctx = runtime.get_context()
    scene = runtime.DeviceScene(ctx, tables, wl)
    exp, exp_upd, exp_st, _, _ = call("rp_trace_segment", ctx, scene, recs, flags)
    assert len(exp) > 0
    for k in range(2):
        got, upd, st, before, after = call("rp_trace_segment_noalloc", ctx, scene, recs, flags)
        what = f"noalloc call {k + 1}"
        assert_records(got, exp, what=what)
        assert_records(upd, exp_upd, what=what + " inputs")
        assert before == after, f"{what}: context memory {before} -> {after}"
        assert (st.rays_in, st.rays_out, st.hits, st.terminated) == \
            (exp_st.rays_in, exp_st.rays_out, exp_st.hits, exp_st.terminated)
        # generation kernel (the mixed path: search and material kernels), tile scan, placement
        assert st.launches == (4 if flags else 3) and st.generations == 1
    scene.free()


def test_noalloc_rejects_more_rays_than_its_limit():
    n = max_rays() + 1
    recs, wl = config2_sample(n)
    tables, _, _ = tables_for(W.config2_spec())
    ctx = runtime.get_context()
    scene = runtime.DeviceScene(ctx, tables, wl)
    din = runtime.DeviceRays(ctx, n)
    din.upload(recs)
    dout = runtime.DeviceRays(ctx, 2 * n)
    dout.upload(recs[:5])  # a reused output buffer: its old count must not survive the rejection
    assert dout.count() == 5
    lib = ctx.lib
    rc = lib.rp_trace_segment_noalloc(ctx.handle, scene.handle, din.handle, dout.handle,
                                      ctypes.c_float(P["max_length"]), 0, ctypes.c_double(P["e2_terminate"]), None)
    assert rc == RP_ERR_CAPACITY
    assert b"fixed limit" in lib.rp_last_error()
    assert dout.count() == 0
    din.free()
    dout.free()
    scene.free()
