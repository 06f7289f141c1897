"""Build and load ``librp_gb300.so``, the sm_103a CUDA library behind the C ABI
declared in ``include/rp_gb300.h``, and mirror its table structs as numpy dtypes.

The library is built in-tree with ``nvcc`` (no torch, no CMake): each ``.cu``
file compiles to an object in parallel, then they are linked into one shared
library.  The plain FP64 translation units use ``--fmad=false`` so that every
floating-point operation rounds as the reference's C does.
"""
from __future__ import annotations

import ctypes
import os
import shutil
import subprocess
import threading
from concurrent.futures import ThreadPoolExecutor

import numpy as np

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
REPO_DIR = os.path.dirname(PKG_DIR)
CSRC = os.path.join(PKG_DIR, "csrc")
INCLUDE = os.path.join(REPO_DIR, "include")
LIB_PATH = os.path.join(PKG_DIR, "librp_gb300.so")
BUILD_DIR = os.path.join(PKG_DIR, "_build")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# (source, extra flags): the plain path must not contract FMAs.
SOURCES = [
    ("rp_trace.cu", ["--fmad=false"]),
    ("rp_mixed.cu", ["--fmad=true", "-prec-div=false", "-prec-sqrt=false", "-ftz=true"]),
    ("rp_api.cu", ["--fmad=false"]),
    ("rp_unit.cu", ["--fmad=false"]),
    ("rp_lens.cu", ["--fmad=false"]),
    ("rp_serve.cu", ["--fmad=false"]),
    ("rp_gausslet.cu", ["--fmad=false"]),
    ("rp_capture.cu", ["--fmad=false"]),
    ("rp_fields.cu", ["--fmad=false"]),
    ("rp_peaks.cu", ["--fmad=true"]),
]


class RPError(RuntimeError):
    """Raised when a C-ABI call returns a non-zero status."""

    def __init__(self, status: int, where: str, detail: str = ""):
        self.status = status
        msg = f"{where} failed: status {status}"
        if detail:
            msg += f" ({detail})"
        super().__init__(msg)


def _nvcc() -> str:
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build librp_gb300.so")
    return p


def _headers() -> list[str]:
    hs = [os.path.join(INCLUDE, "rp_gb300.h")]
    hs += [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    return hs


def needs_build() -> bool:
    if not os.path.exists(LIB_PATH):
        return True
    t = os.path.getmtime(LIB_PATH)
    deps = [os.path.join(CSRC, s) for s, _ in SOURCES] + _headers()
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile librp_gb300.so for sm_103a (cross-compiles without a GPU)."""
    if not force and not needs_build():
        return LIB_PATH
    os.makedirs(BUILD_DIR, exist_ok=True)
    nvcc = _nvcc()
    common = ARCH + ["-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-I", INCLUDE]

    def compile_one(item):
        src, flags = item
        obj = os.path.join(BUILD_DIR, src.replace(".cu", ".o"))
        cmd = [nvcc] + common + flags + ["-c", os.path.join(CSRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stderr[-4000:]}")
        if verbose and r.stderr:
            print(r.stderr)
        return obj

    with ThreadPoolExecutor(len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = LIB_PATH + ".tmp"
    cmd = [nvcc] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc link failed:\n{r.stderr[-4000:]}")
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


# ---- struct mirrors (must match include/rp_gb300.h) ---------------------------
TRANSFORM_DT = np.dtype([("m", "<f8", (9,)), ("t", "<f8", (3,))])
FACELIST_DT = np.dtype([("trans", TRANSFORM_DT), ("inv_trans", TRANSFORM_DT),
                        ("first_face", "<i4"), ("n_faces", "<i4")])
FACE_DT = np.dtype([("type", "<i4"), ("idx", "<i4"), ("material", "<i4"), ("invert_normal", "<i4"),
                    ("invert_normals", "<i4"), ("shape", "<i4"), ("aux", "<i4"), ("n_aux0", "<i4"),
                    ("n_aux1", "<i4"), ("base", "<i4"), ("distortion", "<i4"), ("reserved", "<i4"),
                    ("tolerance", "<f8"), ("p", "<f8", (16,))])
SHAPE_OP_DT = np.dtype([("op", "<i4"), ("aux", "<i4"), ("n", "<i4"), ("reserved", "<i4"),
                        ("a", "<f8"), ("b", "<f8"), ("c", "<f8"), ("d", "<f8")])
DISTORTION_DT = np.dtype([("type", "<i4"), ("n_coefs", "<i4"), ("k_max", "<i4"), ("aux", "<i4"),
                          ("unit_radius", "<f8"), ("amplitude", "<f8")])
MATERIAL_DT = np.dtype([("type", "<i4"), ("curve_inside", "<i4"), ("curve_outside", "<i4"),
                        ("reserved", "<i4"), ("n_inside", "<f8", (2,)), ("n_outside", "<f8", (2,)),
                        ("reflection_threshold", "<f8"), ("transmission_threshold", "<f8"),
                        ("p", "<f8", (10,))])
DISPERSION_DT = np.dtype([("formula_id", "<i4"), ("n_coefs", "<i4"), ("aux", "<i4"), ("reserved", "<i4"),
                          ("absorption", "<f8"), ("wavelength_min", "<f8"), ("wavelength_max", "<f8")])
assert TRANSFORM_DT.itemsize == 96 and FACELIST_DT.itemsize == 200
assert FACE_DT.itemsize == 184 and SHAPE_OP_DT.itemsize == 48
assert DISTORTION_DT.itemsize == 32 and MATERIAL_DT.itemsize == 144 and DISPERSION_DT.itemsize == 40


class SceneDesc(ctypes.Structure):
    _fields_ = [("n_lists", ctypes.c_int32), ("n_faces", ctypes.c_int32),
                ("n_face_records", ctypes.c_int32), ("n_materials", ctypes.c_int32),
                ("n_shape_ops", ctypes.c_int32), ("n_distortions", ctypes.c_int32),
                ("n_dispersions", ctypes.c_int32), ("n_aux", ctypes.c_int32),
                ("lists", ctypes.c_void_p), ("faces", ctypes.c_void_p),
                ("materials", ctypes.c_void_p), ("shape_ops", ctypes.c_void_p),
                ("distortions", ctypes.c_void_p), ("dispersions", ctypes.c_void_p),
                ("aux", ctypes.c_void_p)]


class LensDesc(ctypes.Structure):
    _fields_ = [("n_surfaces", ctypes.c_int32), ("reserved", ctypes.c_int32), ("z0", ctypes.c_double),
                ("max_length", ctypes.c_double), ("atol", ctypes.c_double), ("tolerance", ctypes.c_double),
                ("semi_diameter", ctypes.c_void_p), ("n_index", ctypes.c_void_p)]


class SourceDesc(ctypes.Structure):
    _fields_ = [("type", ctypes.c_int32), ("reserved", ctypes.c_int32), ("n_rays", ctypes.c_uint64),
                ("seed", ctypes.c_uint64), ("origin", ctypes.c_double * 3), ("half_angle", ctypes.c_double),
                ("radius", ctypes.c_double)]


class JobDesc(ctypes.Structure):
    _fields_ = [("scene", ctypes.c_void_p), ("wavelengths", ctypes.c_void_p), ("n_wl", ctypes.c_int64),
                ("source", SourceDesc), ("recursion_limit", ctypes.c_int32), ("max_length", ctypes.c_float),
                ("flags", ctypes.c_uint32), ("detector_face", ctypes.c_int32), ("e2_terminate", ctypes.c_double)]


class JobResult(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int32), ("generations", ctypes.c_int32), ("segments", ctypes.c_uint64),
                ("detector_hits", ctypes.c_uint64), ("detector_power", ctypes.c_double),
                ("sum_x", ctypes.c_double), ("sum_y", ctypes.c_double), ("sum_xx", ctypes.c_double),
                ("sum_yy", ctypes.c_double), ("t_submit_ms", ctypes.c_double), ("t_start_ms", ctypes.c_double),
                ("t_done_ms", ctypes.c_double)]


class ServerStats(ctypes.Structure):
    _fields_ = [("steps", ctypes.c_uint64), ("step_jobs", ctypes.c_uint64), ("step_gpu_ms", ctypes.c_double),
                ("step_wall_ms", ctypes.c_double), ("idle_wall_ms", ctypes.c_double)]


class Stats(ctypes.Structure):
    _fields_ = [("rays_in", ctypes.c_uint64), ("rays_out", ctypes.c_uint64),
                ("hits", ctypes.c_uint64), ("terminated", ctypes.c_uint64),
                ("device_ms", ctypes.c_double), ("kernel_ms", ctypes.c_double),
                ("launches", ctypes.c_uint64), ("generations", ctypes.c_uint64), ("search_ms", ctypes.c_double)]


# Every symbol the header declares, with its ctypes signature.
_P = ctypes.c_void_p
_I = ctypes.c_int
_SIGS = {
    "rp_version": (_I, []),
    "rp_status_string": (ctypes.c_char_p, [_I]),
    "rp_last_error": (ctypes.c_char_p, []),
    "rp_ctx_create": (_I, [_I, ctypes.c_uint64, ctypes.POINTER(_P)]),
    "rp_ctx_destroy": (_I, [_P]),
    "rp_ctx_synchronize": (_I, [_P]),
    "rp_ctx_memory": (_I, [_P, ctypes.POINTER(ctypes.c_uint64)]),
    "rp_ctx_trim": (_I, [_P]),
    "rp_host_alloc": (_I, [ctypes.c_uint64, ctypes.POINTER(_P)]),
    "rp_host_free": (_I, [_P]),
    "rp_scene_create": (_I, [_P, ctypes.POINTER(SceneDesc), _P, ctypes.c_int64, ctypes.POINTER(_P)]),
    "rp_scene_destroy": (_I, [_P]),
    "rp_scene_bounds": (_I, [ctypes.POINTER(SceneDesc), _P, ctypes.c_int32]),
    "rp_scene_search_bounds": (_I, [ctypes.POINTER(SceneDesc), _P, ctypes.c_int32]),
    "rp_scene_face_counts": (_I, [_P, _P, ctypes.c_int32, _I]),
    "rp_rays_alloc": (_I, [_P, ctypes.c_uint64, ctypes.POINTER(_P)]),
    "rp_rays_free": (_I, [_P]),
    "rp_rays_count": (_I, [_P, ctypes.POINTER(ctypes.c_uint64)]),
    "rp_rays_capacity": (_I, [_P, ctypes.POINTER(ctypes.c_uint64)]),
    "rp_rays_upload_aos": (_I, [_P, _P, ctypes.c_uint64]),
    "rp_gausslets_alloc": (_I, [_P, ctypes.c_uint64, ctypes.POINTER(_P)]),
    "rp_gausslets_free": (_I, [_P]),
    "rp_gausslets_count": (_I, [_P, ctypes.POINTER(ctypes.c_uint64)]),
    "rp_gausslets_upload": (_I, [_P, _P, ctypes.c_uint64]),
    "rp_gausslets_download": (_I, [_P, _P, ctypes.c_uint64]),
    "rp_field_evaluate_modes": (_I, [_P, _P, _P, _P, _P, ctypes.c_uint64, ctypes.c_int32, ctypes.c_double, _P]),
    "rp_field_create": (_I, [_P, _P, ctypes.c_uint64, _P, _P, ctypes.c_int64, ctypes.POINTER(_P)]),
    "rp_field_destroy": (_I, [_P]),
    "rp_field_mode_curvature": (_I, [_P, _P, _P, _P, _P, _P, ctypes.c_uint64, _P, _P, _P, _P, _P, _P]),
    "rp_field_interaction_matrix": (_I, [_P, _P, _P, ctypes.c_uint64, _P, _P, ctypes.c_uint64, _P, _P, _P, _P, _P,
                                         _P, ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                         ctypes.c_uint64, ctypes.POINTER(ctypes.c_uint64), _P, _P, _P]),
    "rp_field_apply_mode_curvature": (_I, [_P, _P, _P, _P]),
    "rp_field_evaluate": (_I, [_P, _P, ctypes.c_uint64, ctypes.c_double, _P]),
    "rp_field_evaluate_device": (_I, [_P, _P, ctypes.c_uint64, ctypes.c_double, _P]),
    "rp_field_sum_gaussian_modes": (_I, [_P, _P, ctypes.c_uint64, _P, _P, ctypes.c_int64, _P, ctypes.c_uint64,
                                         ctypes.c_double, _P]),
    "rp_field_create_from_gausslets": (_I, [_P, _P, ctypes.c_int64, ctypes.c_double, ctypes.POINTER(_P)]),
    "rp_field_create_from_rays": (_I, [_P, _P, _P, ctypes.c_double, ctypes.c_double, _P, ctypes.c_int64,
                                       ctypes.POINTER(_P)]),
    "rp_field_download": (_I, [_P, ctypes.POINTER(ctypes.c_uint64), _P, _P]),
    "rp_field_gausslet_samples": (_I, [_P, _P, _P, _P, _P]),
    "rp_field_ray_samples": (_I, [_P, _P, _P, _P, _P, _P, _P, ctypes.POINTER(ctypes.c_uint64)]),
    "rp_rays_project_to_sphere": (_I, [_P, _P, ctypes.c_double, _P]),
    "rp_gausslets_config_parabasal": (_I, [_P, _P, ctypes.c_int64, ctypes.c_double, ctypes.c_double]),
    "rp_gausslets_total_power": (_I, [_P, ctypes.POINTER(ctypes.c_double)]),
    "rp_measure_peaks": (_I, [_I, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double),
                              ctypes.POINTER(ctypes.c_double)]),
    "rp_measure_host_link": (_I, [_I, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]),
    "rp_select_intersections": (_I, [_P, _P, ctypes.c_int32, _P, _P, ctypes.c_uint32]),
    "rp_select_gausslet_intersections": (_I, [_P, _P, ctypes.c_int32, _P, _P, ctypes.c_uint32]),
    "rp_trace_gausslet_segment": (_I, [_P, _P, _P, _P, ctypes.c_int32, ctypes.c_int32, ctypes.c_double, _P,
                                       ctypes.POINTER(Stats)]),
    "rp_rays_download_aos": (_I, [_P, _P, ctypes.c_uint64]),
    "rp_rays_field": (_I, [_P, ctypes.c_char_p, ctypes.POINTER(_P)]),
    "rp_trace_segment": (_I, [_P, _P, _P, _P, ctypes.c_float, ctypes.c_uint32, ctypes.c_double,
                              ctypes.POINTER(Stats)]),
    "rp_trace_one_face_segment": (_I, [_P, _P, _P, _P, ctypes.c_int32, ctypes.c_int32, ctypes.c_float,
                                       ctypes.c_uint32, ctypes.c_double, ctypes.POINTER(Stats)]),
    "rp_trace_rays": (_I, [_P, _P, ctypes.POINTER(_P), ctypes.c_int32, ctypes.c_int32, ctypes.c_float,
                           ctypes.c_uint32, ctypes.c_double, ctypes.POINTER(ctypes.c_int32),
                           ctypes.POINTER(Stats)]),
    "rp_trace_rays_host": (_I, [_P, _P, _P, ctypes.c_uint64, ctypes.c_int32, ctypes.c_float,
                                ctypes.c_uint32, ctypes.c_double, _P, ctypes.c_uint64,
                                ctypes.POINTER(ctypes.c_uint64), ctypes.c_int32,
                                ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(Stats)]),
    "rp_trace_segment_noalloc": (_I, [_P, _P, _P, _P, ctypes.c_float, ctypes.c_uint32, ctypes.c_double,
                                      ctypes.POINTER(Stats)]),
    "rp_lens_create": (_I, [_P, _P, ctypes.c_uint64, ctypes.POINTER(_P)]),
    "rp_lens_destroy": (_I, [_P]),
    "rp_lens_forward": (_I, [_P, _P, _P, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_uint64)]),
    "rp_lens_backward": (_I, [_P, _P]),
    "rp_lens_image": (_I, [_P, _P, _P, ctypes.c_uint64]),
    "rp_source_generate": (_I, [_P, ctypes.POINTER(SourceDesc), ctypes.c_uint32, _P]),
    "rp_server_create": (_I, [_I, ctypes.c_uint64, ctypes.c_int32, ctypes.POINTER(_P)]),
    "rp_server_submit": (_I, [_P, ctypes.POINTER(JobDesc), ctypes.POINTER(ctypes.c_uint64)]),
    "rp_server_wait": (_I, [_P, ctypes.c_uint64, ctypes.POINTER(JobResult), _P, ctypes.c_int32]),
    "rp_server_set_step_groups": (_I, [_P, ctypes.c_uint32, ctypes.c_uint32]),
    "rp_server_get_stats": (_I, [_P, ctypes.POINTER(ServerStats)]),
    "rp_server_destroy": (_I, [_P]),
    "rp_face_intersect": (_I, [_P, ctypes.c_int32, _P, _P, ctypes.c_uint64, _I, _P]),
    "rp_face_normal": (_I, [_P, ctypes.c_int32, _P, ctypes.c_uint64, _P]),
    "rp_shape_inside": (_I, [_P, ctypes.c_int32, _P, ctypes.c_uint64, _P]),
    "rp_distortion_eval": (_I, [_P, ctypes.c_int32, _P, ctypes.c_uint64, _P]),
    "rp_material_eval": (_I, [_P, ctypes.c_int32, _P, _P, _P, _P, _P, ctypes.c_uint64, _P, _P]),
    "rp_convert_to_sp": (_I, [_P, _P, _P, ctypes.c_uint64, _P]),
    "rp_dispersion_eval": (_I, [_P, ctypes.c_int32, _P, ctypes.c_uint64, _P]),
}
EXPORTED = tuple(_SIGS)

_lib = None
_lock = threading.Lock()


def load(build_if_needed: bool = True) -> ctypes.CDLL:
    """Load librp_gb300.so (building it first if sources are newer)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if build_if_needed and needs_build():
            build()
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("librp_gb300.so is not built; call raypier_optics_gb300._native.build()")
        lib = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in _SIGS.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


RP_ERR_CAPACITY = -2  # include/rp_gb300.h: an output buffer is too small


def check(status: int, where: str) -> None:
    if status != 0:
        lib = load(build_if_needed=False)
        detail = (lib.rp_last_error() or b"").decode(errors="replace")
        raise RPError(status, where, detail)

