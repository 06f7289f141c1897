"""Sequential tracing (core/tracer.py:50-99 trace_ray_sequence over
ctracer.pyx:2121-2170 trace_one_face_segment_c) against the reference's own
trace of the configuration-1 lens with every face list visited twice: the
oracle on the CPU, the GPU path through the package's trace_ray_sequence."""
from itertools import chain

import numpy as np
import pytest

import oracle
from helpers import NS, X86, assert_generations, load_case
from raypier_optics_gb300 import scene
from raypier_optics_gb300 import workloads as W

CASE = "seq_config1"


def _chained_lists(c):
    lists = W.build_scene(c["spec"], NS)
    seq = c["params"]["sequence"]
    all_faces = list(chain(*(lists[l].faces for l, _ in seq)))
    for i, f in enumerate(all_faces):   # core/tracer.py:76-81: the last position wins
        f.idx = i
        f.update()
    return lists, seq, all_faces


def test_oracle_sequence_matches_reference():
    c = load_case(CASE)
    lists, seq, _ = _chained_lists(c)
    P = c["params"]
    rays = c["rays"].copy()
    rays["length"] = P["max_length"]
    traced = [rays]
    for count, (l, fi) in enumerate(seq):
        tables = scene.compile_scene([lists[l]])
        mutated, kids, _ = oracle.trace_segment(tables, c["wl"], traced[-1], P["max_length"], one_list=0, one_face=fi)
        traced[-1] = mutated
        if count > P["recursion_limit"] or len(kids) == 0:
            break
        traced.append(kids)
    assert_generations(traced, c["gens"], exact=X86, what=CASE)


@pytest.mark.gpu
def test_gpu_sequence_matches_reference():
    from raypier_optics_gb300 import tracer
    from raypier_optics_gb300.ctracer import RayCollection
    c = load_case(CASE)
    lists = W.build_scene(c["spec"], NS)
    rc = RayCollection.from_array(c["rays"].copy())
    rc.wavelengths = c["wl"]
    P = c["params"]
    traced, all_faces = tracer.trace_ray_sequence(rc, [(lists[l], f) for l, f in P["sequence"]],
                                                  recursion_limit=P["recursion_limit"], max_length=P["max_length"])
    assert_generations([t.copy_as_array() for t in traced], c["gens"], what=CASE)
    assert [f.count for f in all_faces] == c["counts"].tolist()
