"""Accuracy of a trace against an FP64 trace of the same rays.

Used to report the mixed FP32/FP64 path's error against the plain FP64 path
(and, in the tests, against the FP64 oracle): hit-point position (nm), ray
direction (rad) and accumulated optical path (nm), over the rays whose
generation index, parent, end face and type agree in both traces.
"""
from __future__ import annotations

import numpy as np

MM_TO_NM = 1e6
INDEX_FIELDS = ("parent_idx", "end_face_idx", "ray_ident", "ray_type_id", "wavelength_idx")


def compare_traces(test_gens, ref_gens):
    """Error statistics of `test_gens` against `ref_gens` (lists of ray_dtype
    arrays, one per generation)."""
    pos, ang, opl = [], [], []
    n_total = n_match = 0
    n_gens = min(len(test_gens), len(ref_gens))
    for g in range(n_gens):
        a, b = test_gens[g], ref_gens[g]
        n = min(len(a), len(b))
        n_total += max(len(a), len(b))
        if n == 0:
            continue
        a, b = a[:n], b[:n]
        same = np.ones(n, dtype=bool)
        for f in INDEX_FIELDS:
            same &= a[f] == b[f]
        # once the order diverges every later index is shifted: keep the prefix
        bad = np.flatnonzero(~same)
        if bad.size:
            same[bad[0]:] = False
        n_match += int(same.sum())
        if not same.any():
            continue
        aa, bb = a[same], b[same]
        pos.append(np.max(np.abs(aa["origin"] - bb["origin"]), axis=1))
        da = aa["direction"] / np.linalg.norm(aa["direction"], axis=1)[:, None]
        db = bb["direction"] / np.linalg.norm(bb["direction"], axis=1)[:, None]
        ang.append(np.linalg.norm(da - db, axis=1))
        opl.append(np.abs(aa["accumulated_path"] - bb["accumulated_path"]))
    gens_equal = [len(a) for a in test_gens] == [len(b) for b in ref_gens]

    def stats(parts, scale):
        if not parts:
            return {"max": None, "p99": None, "median": None}
        v = np.concatenate(parts) * scale
        return {"max": float(v.max()), "p99": float(np.percentile(v, 99)), "median": float(np.median(v))}

    return {
        "position_nm": stats(pos, MM_TO_NM),
        "direction_rad": stats(ang, 1.0),
        "opl_nm": stats(opl, MM_TO_NM),
        "rays_compared": n_match,
        "rays_total": n_total,
        "index_agreement": (n_match / n_total) if n_total else 1.0,
        "generation_sizes_equal": bool(gens_equal),
    }
