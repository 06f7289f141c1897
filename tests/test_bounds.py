"""The face boxes that let the nearest-hit search skip faces must contain
every point where the face can report a hit.  Checked on the CPU against the
hit points of the oracle (which tests every face, as the reference does) for
every golden scene and larger samples of the benchmark configurations."""
import ctypes

import numpy as np
import pytest

import oracle
from helpers import load_case, tables_for, trace_case_names
from raypier_optics_gb300 import _native, ctracer
from raypier_optics_gb300 import workloads as W


def boxes(tables):
    lib = _native.load()
    out = np.zeros((tables.n_faces, 8), dtype=np.float32)
    d = tables.desc()
    assert lib.rp_scene_bounds(ctypes.byref(d), out.ctypes.data, tables.n_faces) == 0
    return out


def search_boxes(tables):
    lib = _native.load()
    out = np.zeros((tables.n_faces, 16), dtype=np.float32)
    d = tables.desc()
    assert lib.rp_scene_search_bounds(ctypes.byref(d), out.ctypes.data, tables.n_faces) == 0
    return out


def check_hits_inside_search(tables, gens):
    """Every hit on a face with search boxes lies in one of them (the
    searches enter a face at the nearer of its boxes; flag 3: two)."""
    b = search_boxes(tables)
    idx_of = {int(f["idx"]): k for k, f in enumerate(tables.faces[:tables.n_faces])}
    n_checked = 0
    for g in gens:
        hit = g["end_face_idx"] != 0xFFFFFFFF
        pts = g["origin"][hit] + g["direction"][hit] * g["length"][hit][:, None]
        recs = np.array([idx_of[int(i)] for i in g["end_face_idx"][hit]], dtype=np.int64)
        for k in np.unique(recs):
            if b[k, 6] not in (1, 3):
                continue
            p = pts[recs == k]
            inside = np.all((p >= b[k, 0:3].astype(np.float64)) & (p <= b[k, 3:6].astype(np.float64)), axis=1)
            if b[k, 6] == 3:
                inside |= np.all((p >= b[k, 8:11].astype(np.float64)) & (p <= b[k, 11:14].astype(np.float64)), axis=1)
            assert inside.all(), f"face record {k}: {np.count_nonzero(~inside)} hits outside its search boxes"
            n_checked += len(p)
    return n_checked


def line_misses(b, p1, u):
    """The kernels' distortion-face cull restated: the line p1 + s u (local
    frame) never passes over the rectangle b[0..3] = x0, x1, y0, y1."""
    x0, x1, y0, y1 = (float(v) for v in b[:4])
    ux, uy = u[:, 0], u[:, 1]
    corners = [(x0, y0), (x0, y1), (x1, y0), (x1, y1)]
    s = np.stack([ux * (cy - p1[:, 1]) - uy * (cx - p1[:, 0]) for cx, cy in corners], axis=1)
    along_z = (ux == 0) & (uy == 0)
    outside = (p1[:, 0] < x0) | (p1[:, 0] > x1) | (p1[:, 1] < y0) | (p1[:, 1] > y1)
    return np.where(along_z, outside, np.all(s > 0, axis=1) | np.all(s < 0, axis=1))


def list_of_record(tables, k):
    for L in tables.lists:
        if L["first_face"] <= k < L["first_face"] + L["n_faces"]:
            return L
    raise KeyError(k)


def check_hits_inside(tables, gens):
    b = boxes(tables)
    idx_of = {int(f["idx"]): k for k, f in enumerate(tables.faces[:tables.n_faces])}
    n_checked = 0
    for g in gens:
        hit = g["end_face_idx"] != 0xFFFFFFFF
        pts = g["origin"][hit] + g["direction"][hit] * g["length"][hit][:, None]
        recs = np.array([idx_of[int(i)] for i in g["end_face_idx"][hit]], dtype=np.int64)
        for k in np.unique(recs):
            if b[k, 6] == 0:
                continue
            if b[k, 6] == 2:
                # a distortion face: every ray that hit it must pass the line cull
                L = list_of_record(tables, int(k))
                m = L["inv_trans"]["m"].reshape(3, 3)
                sel = np.flatnonzero(hit)[recs == k]
                p1 = g["origin"][sel] @ m.T + L["inv_trans"]["t"]
                u = g["direction"][sel] @ m.T
                assert not line_misses(b[k], p1, u).any(), f"face record {k}: a hit ray would be culled"
                # and its hit point's local (x, y) lies in the padded rectangle: the
                # searches enter the face at the ray's entry into the prism over it
                q = pts[recs == k] @ m.T + L["inv_trans"]["t"]
                x0, x1, y0, y1 = (float(v) for v in b[k, :4])
                inside = (q[:, 0] >= x0) & (q[:, 0] <= x1) & (q[:, 1] >= y0) & (q[:, 1] <= y1)
                assert inside.all(), f"face record {k}: {np.count_nonzero(~inside)} hits outside its prism"
                n_checked += len(sel)
                continue
            p = pts[recs == k]
            lo, hi = b[k, :3].astype(np.float64), b[k, 3:6].astype(np.float64)
            inside = np.all((p >= lo) & (p <= hi), axis=1)
            assert inside.all(), f"face record {k}: {np.count_nonzero(~inside)} hits outside its box"
            n_checked += len(p)
    return n_checked


@pytest.mark.parametrize("name", trace_case_names())
def test_golden_hits_lie_in_face_boxes(name):
    c = load_case(name)
    tables, _, _ = tables_for(c["spec"])
    check_hits_inside(tables, c["gens"])
    check_hits_inside_search(tables, c["gens"])


@pytest.mark.parametrize("config", ["config1", "config2", "config3"])
def test_benchmark_hits_lie_in_face_boxes(config):
    if config == "config1":
        rays, wl = W.config1_rays(ctracer.ray_dtype)
        spec, P, per = W.config1_spec(), W.CONFIG1, False
    elif config == "config2":
        rays, wl = W.config2_rays(ctracer.ray_dtype, 1 << 20)
        rays, wl = W.subsample(rays, wl, np.arange(0, 1 << 20, 128), per_ray_wavelength=True)
        spec, P = W.config2_spec(), W.CONFIG2
    else:
        rays, wl = W.config3_rays(ctracer.ray_dtype, 2048)
        spec, P = W.config3_spec(), W.CONFIG3
    tables, _, _ = tables_for(spec)
    gens, _ = oracle.trace_rays(tables, wl, rays, P["recursion_limit"], P["max_length"], P["e2_terminate"])
    assert check_hits_inside(tables, gens) > 0
    assert check_hits_inside_search(tables, gens) > 0


def test_boxes_are_tight_for_axis_aligned_faces():
    tables, _, _ = tables_for(W.config2_spec())
    b = boxes(tables)
    # first doublet face: a 50 mm R=100 cap at z in [0, 3.18] (+ padding)
    assert b[0, 6] == 1
    assert np.allclose(b[0, :3], [-25, -25, 0], atol=2e-3) and np.allclose(b[0, 3:6], [25, 25, 3.1755], atol=2e-3)
    # the asphere (z from 60 to 60 + 10.6)
    assert b[6, 6] == 1 and 60 - 0.1 < b[6, 2] < 60 and 70.5 < b[6, 5] < 70.8


@pytest.mark.parametrize("name", ["ellipsoid", "saddle", "saddle_rect", "cylinder", "cylinder_neg", "axicon",
                                  "axicon_neg"])
def test_curved_face_boxes_hold_on_dense_samples(name):
    """4096 seeded rays from both sides, through the face scenes of the golden
    set: every hit the oracle reports lies in its face's box."""
    from helpers import load_face_specs
    spec = load_face_specs()[name]
    rng = np.random.Generator(np.random.PCG64(5))
    n = 4096
    th = rng.uniform(0.0, 0.6, n)
    ph = rng.uniform(0.0, 2 * np.pi, n)
    up = rng.uniform(size=n) < 0.5
    d = np.stack([np.sin(th) * np.cos(ph), np.sin(th) * np.sin(ph), np.where(up, 1.0, -1.0) * np.cos(th)], axis=1)
    o = np.stack([rng.uniform(-16, 16, n), rng.uniform(-16, 16, n), np.where(up, -10.0, 45.0)], axis=1)
    e = np.cross(np.array([0.0, 1.0, 0.0]), d)
    e /= np.linalg.norm(e, axis=1)[:, None]
    rays = W.fill_rays(np.zeros(n, dtype=ctracer.ray_dtype), o, d, e)
    tables, _, _ = tables_for(spec)
    assert boxes(tables)[0, 6] == 1
    gens, _ = oracle.trace_rays(tables, np.array([0.55]), rays, 4, 200.0, 0.0)
    assert check_hits_inside(tables, gens) > 100


def dense_rays(n, seed, spread=16.0, z_below=-10.0, z_above=45.0):
    rng = np.random.Generator(np.random.PCG64(seed))
    th = rng.uniform(0.0, 0.6, n)
    ph = rng.uniform(0.0, 2 * np.pi, n)
    up = rng.uniform(size=n) < 0.5
    d = np.stack([np.sin(th) * np.cos(ph), np.sin(th) * np.sin(ph), np.where(up, 1.0, -1.0) * np.cos(th)], axis=1)
    o = np.stack([rng.uniform(-spread, spread, n), rng.uniform(-spread, spread, n), np.where(up, z_below, z_above)],
                 axis=1)
    e = np.cross(np.array([0.0, 1.0, 0.0]), d)
    e /= np.linalg.norm(e, axis=1)[:, None]
    return W.fill_rays(np.zeros(n, dtype=ctracer.ray_dtype), o, d, e)


@pytest.mark.parametrize("name", ["conic_mirror", "conic_inv"])
def test_conic_sheet_boxes_hold_on_dense_samples(name):
    """A conic face's two sheet boxes: 4096 seeded rays from both sides and
    from between the sheets; every hit the oracle reports lies in one of the
    face's boxes, and the boxes are split (each far thinner than their union)."""
    from helpers import load_face_specs
    spec = load_face_specs()[name]
    tables, _, _ = tables_for(spec)
    mb, ub = search_boxes(tables), boxes(tables)
    assert mb[0, 6] == 3
    union_dz = ub[0, 5] - ub[0, 2]
    assert mb[0, 5] - mb[0, 2] < 0.5 * union_dz and mb[0, 13] - mb[0, 10] < 0.5 * union_dz
    n_checked = 0
    for seed, zb, za in ((5, -10.0, 45.0), (6, float(ub[0, 2]) - 5.0, float(ub[0, 5]) + 5.0),
                         (7, 0.5 * float(ub[0, 2] + ub[0, 5]), 0.5 * float(ub[0, 2] + ub[0, 5]))):
        rays = dense_rays(4096, seed, z_below=zb, z_above=za)
        gens, _ = oracle.trace_rays(tables, np.array([0.55]), rays, 4, 5000.0, 0.0)
        n_checked += check_hits_inside_search(tables, gens)
    assert n_checked > 100


def test_conic_sheet_ranges_cover_the_quadric():
    """The sheet ranges of conic faces of the served mix and the clutter scene
    (k in [-2, 0.5], |R| 20-400 mm): every point of the quadric over the
    aperture, sampled densely on both roots, lies in its sheet's box."""
    rng = np.random.Generator(np.random.PCG64(11))
    n_split = 0
    for _ in range(64):
        R = float(rng.uniform(20.0, 400.0)) * (1.0 if rng.uniform() < 0.5 else -1.0)
        k = float(rng.uniform(-2.0, 0.5))
        spec = {"materials": {"m": {"type": "PECMaterial"}},
                "lists": [{"faces": [{"type": "ConicRevolutionFace",
                                      "kw": {"curvature": R, "z_height": 0.0, "conic_const": k},
                                      "shape": {"type": "CircleShape", "kw": {"radius": 12.5}},
                                      "material": "m"}]}]}
        tables, _, _ = tables_for(spec)
        mb = search_boxes(tables)[0]
        if mb[6] != 3:
            continue
        n_split += 1
        beta, Rq = 1.0 + k, -R  # the face's quadric: beta z^2 - 2 Rq z + r^2 = 0 (rp_bounds.h)
        r = np.linspace(0.0, 12.5, 2001)
        disc = Rq * Rq - beta * r * r
        ok = disc >= 0
        for sign in (1.0, -1.0):
            z = (Rq + sign * np.sqrt(disc[ok])) / beta
            in_a = (z >= mb[2]) & (z <= mb[5])
            in_b = (z >= mb[10]) & (z <= mb[13])
            assert np.all(in_a | in_b), (R, k, sign)
    assert n_split > 48
