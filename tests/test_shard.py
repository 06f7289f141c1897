"""Ray sharding for N > 1: world_size-2 gloo ranks on the CPU each trace a
contiguous shard (with the oracle standing in for each rank's GPU), gather
their per-generation counts, rebase parent indices, and the merged result
equals the single trace of all rays."""
import os
import socket

import numpy as np
import pytest

import oracle
from helpers import assert_generations, tables_for
from raypier_optics_gb300 import ctracer, shard
from raypier_optics_gb300 import workloads as W


def _rays(n):
    rays, wl = W.config2_rays(ctracer.ray_dtype, 1 << 20)
    return W.subsample(rays, wl, np.arange(0, 1 << 20, (1 << 20) // n)[:n], per_ray_wavelength=True)


@pytest.mark.parametrize("world", [1, 2, 3, 5])
def test_merge_of_shards_equals_single_trace(world):
    rays, wl = _rays(96)
    tables, _, _ = tables_for(W.config2_spec())
    full, _ = oracle.trace_rays(tables, wl, rays, 6, 1000.0, 1e-6)
    per = []
    for r in range(world):
        lo, hi = shard.shard_bounds(len(rays), world, r)
        sub = rays[lo:hi].copy()
        gens, _ = oracle.trace_rays(tables, wl, sub, 6, 1000.0, 1e-6)
        per.append(gens)
    merged = shard.merge_generations(per)
    assert_generations(merged, full, exact=True, what=f"world={world}")


def test_shard_bounds_cover_exactly():
    for n in (0, 1, 7, 100, 1 << 20):
        for world in (1, 2, 3, 8):
            spans = [shard.shard_bounds(n, world, r) for r in range(world)]
            assert spans[0][0] == 0 and spans[-1][1] == n
            assert all(a[1] == b[0] for a, b in zip(spans, spans[1:]))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank_main(rank, world, port, q):
    import sys
    here = os.path.dirname(os.path.abspath(__file__))
    repo = os.path.dirname(here)
    for p in (repo, os.path.join(repo, "oracle"), here):
        sys.path.insert(0, p)
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import oracle as orc
    from helpers import tables_for as tf
    from raypier_optics_gb300 import shard as sh
    from raypier_optics_gb300 import workloads as Wk
    rays, wl = _rays(64)
    tables, _, _ = tf(Wk.config2_spec())
    lo, hi = sh.shard_bounds(len(rays), world, rank)
    gens, _ = orc.trace_rays(tables, wl, rays[lo:hi].copy(), 5, 1000.0, 1e-6)
    counts = sh.gather_counts([len(g) for g in gens], 8)
    rebased, offs = sh.rebase_local(gens, rank, counts)
    q.put((rank, [g.tobytes() for g in rebased], offs.tolist(), counts.tolist()))
    dist.barrier()
    dist.destroy_process_group()


def test_gloo_world2_rebase_matches_single_trace():
    import torch.multiprocessing as tmp
    ctx = tmp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = {}
    for _ in range(2):
        rank, gens, offs, counts = q.get(timeout=120)
        res[rank] = ([np.frombuffer(g, dtype=ctracer.ray_dtype) for g in gens], offs, counts)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    rays, wl = _rays(64)
    tables, _, _ = tables_for(W.config2_spec())
    full, _ = oracle.trace_rays(tables, wl, rays, 5, 1000.0, 1e-6)
    n_gens = len(full)
    for g in range(n_gens):
        parts = [res[r][0][g] for r in range(2) if g < len(res[r][0])]
        merged = np.concatenate(parts)
        np.testing.assert_array_equal(merged['parent_idx'], full[g]['parent_idx'])
        np.testing.assert_array_equal(merged['end_face_idx'], full[g]['end_face_idx'])
        np.testing.assert_array_equal(merged['ray_ident'], full[g]['ray_ident'])
    # both ranks saw the same counts, and offsets are the exclusive scan
    assert res[0][2] == res[1][2]
    assert res[1][1][0] == res[0][2][0][0]
