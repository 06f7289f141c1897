"""The C-ABI library: it builds for sm_103a, loads, exports every entry point
include/rp_gb300.h declares, and its structs have the layout the Python
mirrors assume.  No compute call is made (these run without a GPU)."""
import ctypes
import os
import re
import subprocess
import tempfile

import numpy as np

from raypier_optics_gb300 import _native
from raypier_optics_gb300.ctracer import ray_dtype

HEADER = os.path.join(_native.INCLUDE, "rp_gb300.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(rp_[a-z0-9_]+)\s*\(", text)))


def test_library_builds_and_loads():
    lib = _native.load()
    assert lib.rp_version() == 1


def test_every_declared_symbol_is_exported():
    lib = _native.load()
    names = declared_functions()
    assert len(names) >= 30
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    # and the ctypes mirror covers the whole header
    assert set(names) == set(_native.EXPORTED)


def test_status_strings():
    lib = _native.load()
    for code in (0, -1, -2, -3, -4, -5, -6, -7):
        assert lib.rp_status_string(code)


def test_null_arguments_are_rejected_without_a_device():
    lib = _native.load()
    assert lib.rp_ctx_create(0, 0, None) == -1
    assert lib.rp_ctx_destroy(None) == -1
    assert lib.rp_rays_free(None) == -1
    assert lib.rp_scene_destroy(None) == -1
    assert lib.rp_trace_segment(None, None, None, None, ctypes.c_float(1.0), 0, 0.0, None) == -1


def test_struct_layouts_match_the_header():
    src = r'''
    #include <stdio.h>
    #include <stddef.h>
    #include "rp_gb300.h"
    int main(void) {
      printf("%zu %zu %zu %zu %zu %zu %zu %zu %zu %zu\n", sizeof(rp_ray), sizeof(rp_transform),
             sizeof(rp_facelist), sizeof(rp_face), sizeof(rp_shape_op), sizeof(rp_distortion),
             sizeof(rp_material), sizeof(rp_dispersion), sizeof(rp_scene_desc), sizeof(rp_stats));
      printf("%zu %zu %zu %zu\n", offsetof(rp_ray, refractive_index), offsetof(rp_ray, length),
             offsetof(rp_ray, wavelength_idx), offsetof(rp_face, p));
      printf("%zu %zu %zu %zu %zu %zu %zu %zu\n", sizeof(rp_lens_desc), sizeof(rp_source_desc), sizeof(rp_job_desc),
             sizeof(rp_job_result), offsetof(rp_job_desc, source), offsetof(rp_job_result, t_submit_ms),
             sizeof(rp_server_stats), offsetof(rp_server_stats, idle_wall_ms));
      return 0; }
    '''
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "t.c")
        open(c, "w").write(src)
        exe = os.path.join(d, "t")
        subprocess.run(["gcc", "-I", _native.INCLUDE, c, "-o", exe], check=True)
        out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split("\n")
    sizes = list(map(int, out[0].split()))
    offs = list(map(int, out[1].split()))
    assert sizes[0] == ray_dtype.itemsize == 188
    assert sizes[1] == _native.TRANSFORM_DT.itemsize
    assert sizes[2] == _native.FACELIST_DT.itemsize
    assert sizes[3] == _native.FACE_DT.itemsize
    assert sizes[4] == _native.SHAPE_OP_DT.itemsize
    assert sizes[5] == _native.DISTORTION_DT.itemsize
    assert sizes[6] == _native.MATERIAL_DT.itemsize
    assert sizes[7] == _native.DISPERSION_DT.itemsize
    assert sizes[8] == ctypes.sizeof(_native.SceneDesc)
    assert sizes[9] == ctypes.sizeof(_native.Stats)
    assert offs[0] == ray_dtype.fields['refractive_index'][1]
    assert offs[1] == ray_dtype.fields['length'][1]
    assert offs[2] == ray_dtype.fields['wavelength_idx'][1]
    assert offs[3] == _native.FACE_DT.fields['p'][1]
    more = list(map(int, out[2].split()))
    assert more[0] == ctypes.sizeof(_native.LensDesc)
    assert more[1] == ctypes.sizeof(_native.SourceDesc)
    assert more[2] == ctypes.sizeof(_native.JobDesc)
    assert more[3] == ctypes.sizeof(_native.JobResult)
    assert more[4] == _native.JobDesc.source.offset
    assert more[5] == _native.JobResult.t_submit_ms.offset
    assert more[6] == ctypes.sizeof(_native.ServerStats)
    assert more[7] == _native.ServerStats.idle_wall_ms.offset
