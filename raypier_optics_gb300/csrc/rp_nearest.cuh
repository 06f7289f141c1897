// rp_nearest.cuh -- the FP64 nearest-hit search over all faces of a scene,
// shared by the plain ray generation (rp_trace.cu) and the Gausslet
// generation (rp_gausslet.cu), and the record copy of the placement kernels.
#pragma once
#include "rp_gen_common.cuh"

namespace rp {

// Entry distance of the ray (FP32, unit direction) into a padded world box
// (lo xyz, hi xyz), +inf for a miss.
__device__ __forceinline__ float slab_enter(const float *b, float ox, float oy, float oz, float ix, float iy,
                                            float iz) {
    float t1 = (b[0] - ox) * ix, t2 = (b[3] - ox) * ix;
    float tmin = fminf(t1, t2), tmax = fmaxf(t1, t2);
    t1 = (b[1] - oy) * iy;
    t2 = (b[4] - oy) * iy;
    tmin = fmaxf(tmin, fminf(t1, t2));
    tmax = fminf(tmax, fmaxf(t1, t2));
    t1 = (b[2] - oz) * iz;
    t2 = (b[5] - oz) * iz;
    tmin = fmaxf(tmin, fminf(t1, t2));
    tmax = fminf(tmax, fmaxf(t1, t2));
    if (!(tmax >= tmin) || tmax < 0.0f) return __int_as_float(0x7f800000);
    return fmaxf(tmin, 0.0f);
}

// Entry distance of the ray (unit direction u, its inverse i) into face f's
// boxes (rp_bounds.h face_world_boxes): flag 1, its box; 3, the nearer of
// its box and its second box (a conic face's two sheets); 2, a distortion
// face's prism (prism_enter); 0 for faces that are always tested.
__device__ __forceinline__ float box_enter(const DevScene &S, int f, float ox, float oy, float oz, float ix, float iy,
                                           float iz, float ux, float uy, float uz) {
    const float *b = S.bounds + 16 * f;
    if (b[6] != 1.0f) {
        if (b[6] == 3.0f)
            return fminf(slab_enter(b, ox, oy, oz, ix, iy, iz), slab_enter(b + 8, ox, oy, oz, ix, iy, iz));
        if (b[6] == 2.0f) return prism_enter(b, ox, oy, oz, ux, uy, uz);
        return 0.0f;
    }
    return slab_enter(b, ox, oy, oz, ix, iy, iz);
}

__device__ __forceinline__ float inv_dir(float v) {
    if (fabsf(v) < 1e-30f) v = copysignf(1e-30f, v);
    return 1.0f / v;
}

// Nearest hit over all faces (trace_segment_c's loops over face lists and
// faces, ctracer.pyx:2092-2105, with FaceList.intersect_c 1882-1904).  The
// reference tests every face in list order and keeps a strictly nearer
// distance, so the result is the smallest distance in (tolerance, max_length)
// and, among equal distances, the earliest face.  Here faces are tested in
// order of their box entry distance and a face whose box the ray cannot reach
// before the current nearest hit is skipped; the exact FP64 test of every
// face that is tested is the reference's, and ties go to the lower record,
// so the outcome is the same.
__device__ __forceinline__ void nearest_hit(const DevScene &S, v3 o, v3 d, v3 pend, double max_len, double &len,
                                            int &best, int &best_list, unsigned *err) {
    float ox = (float)o.x, oy = (float)o.y, oz = (float)o.z;
    float dx = (float)d.x, dy = (float)d.y, dz = (float)d.z;
    float il = 1.0f / sqrtf(dx * dx + dy * dy + dz * dz);
    float ix = inv_dir(dx * il), iy = inv_dir(dy * il), iz = inv_dir(dz * il);
    const float ux = dx * il, uy = dy * il, uz = dz * il;
    // distances along the ray are Euclidean in the reference (h * |p2 - p1|)
    const int nf = S.n_faces;
    const int nmask = nf < 64 ? nf : 64;
    const float lim0 = (float)max_len * 1.000001f + 1e-4f;
    unsigned long long cand = 0;
    for (int f = 0; f < nmask; f++)
        if (box_enter(S, f, ox, oy, oz, ix, iy, iz, ux, uy, uz) <= lim0) cand |= 1ull << f;
    int cur_list = -1;
    v3 p1 = o, p2 = pend;
    while (cand) {
        float tsel = __int_as_float(0x7f800000);
        int sel = -1;
        for (unsigned long long m = cand; m; m &= m - 1) {
            int f = __ffsll((long long)m) - 1;
            float t = box_enter(S, f, ox, oy, oz, ix, iy, iz, ux, uy, uz);
            if (t < tsel) {
                tsel = t;
                sel = f;
            }
        }
        if (sel < 0 || tsel > (float)len * 1.000001f + 1e-4f) break;
        cand &= ~(1ull << sel);
        int l = S.face_list[sel];
        if (l < 0 || l >= S.n_lists) {  // cannot happen for a validated scene
            atomicOr(err, ERR_SHAPE_STACK);
            break;
        }
        if (l != cur_list) {
            const rp_facelist &L = S.lists[l];
            p1 = xform(L.inv_trans.m, L.inv_trans.t, o);
            p2 = xform(L.inv_trans.m, L.inv_trans.t, pend);
            cur_list = l;
        }
        const rp_face &F = S.faces[sel];
        if (distortion_line_misses(S.bounds + 16 * sel, p1, p2)) continue;
        double dist = face_isect(S, F, p1, p2, err);
        if (F.tolerance < dist && (dist < len || (dist == len && best >= 0 && sel < best))) {
            len = dist;
            best = sel;
            best_list = l;
        }
    }
    // faces beyond the first 64 records: list order with the same skip test
    for (int f = nmask; f < nf; f++) {
        if (box_enter(S, f, ox, oy, oz, ix, iy, iz, ux, uy, uz) > (float)len * 1.000001f + 1e-4f) continue;
        int l = S.face_list[f];
        if (l < 0 || l >= S.n_lists) {
            atomicOr(err, ERR_SHAPE_STACK);
            break;
        }
        if (l != cur_list) {
            const rp_facelist &L = S.lists[l];
            p1 = xform(L.inv_trans.m, L.inv_trans.t, o);
            p2 = xform(L.inv_trans.m, L.inv_trans.t, pend);
            cur_list = l;
        }
        const rp_face &F = S.faces[f];
        if (distortion_line_misses(S.bounds + 16 * f, p1, p2)) continue;
        double dist = face_isect(S, F, p1, p2, err);
        if (F.tolerance < dist && (dist < len || (dist == len && best >= 0 && f < best))) {
            len = dist;
            best = f;
            best_list = l;
        }
    }
}

// Copies one ray record between structure-of-arrays buffers.  All 23 loads
// are issued before the first store: the compiler cannot tell the two
// buffers apart, so an interleaved load/store sequence would wait for each
// load in turn.
__device__ __forceinline__ void copy_ray(const RaySoA &s, unsigned long long src, const RaySoA &o,
                                         unsigned long long dst) {
    const double ox = s.ox[src], oy = s.oy[src], oz = s.oz[src];
    const double dx = s.dx[src], dy = s.dy[src], dz = s.dz[src];
    const double nx = s.nx[src], ny = s.ny[src], nz = s.nz[src];
    const double ex = s.ex[src], ey = s.ey[src], ez = s.ez[src];
    const double2 n = s.n[src], e1 = s.e1[src], e2 = s.e2[src];
    const double len = s.len[src], phase = s.phase[src], opl = s.opl[src];
    const unsigned wl = s.wl[src], parent = s.parent[src], endf = s.endf[src], ident = s.ident[src],
                   type = s.type[src];
    o.ox[dst] = ox; o.oy[dst] = oy; o.oz[dst] = oz;
    o.dx[dst] = dx; o.dy[dst] = dy; o.dz[dst] = dz;
    o.nx[dst] = nx; o.ny[dst] = ny; o.nz[dst] = nz;
    o.ex[dst] = ex; o.ey[dst] = ey; o.ez[dst] = ez;
    o.n[dst] = n; o.e1[dst] = e1; o.e2[dst] = e2;
    o.len[dst] = len; o.phase[dst] = phase; o.opl[dst] = opl;
    o.wl[dst] = wl; o.parent[dst] = parent; o.endf[dst] = endf; o.ident[dst] = ident; o.type[dst] = type;
}

// Writes ray `src` of `s` to `dst` of `o` with the given length and end face
// (a generation's input record once its segment is traced).
__device__ __forceinline__ void pass_ray(const RaySoA &s, unsigned long long src, const RaySoA &o,
                                         unsigned long long dst, double len, unsigned endf) {
    const double ox = s.ox[src], oy = s.oy[src], oz = s.oz[src];
    const double dx = s.dx[src], dy = s.dy[src], dz = s.dz[src];
    const double nx = s.nx[src], ny = s.ny[src], nz = s.nz[src];
    const double ex = s.ex[src], ey = s.ey[src], ez = s.ez[src];
    const double2 n = s.n[src], e1 = s.e1[src], e2 = s.e2[src];
    const double phase = s.phase[src], opl = s.opl[src];
    const unsigned wl = s.wl[src], parent = s.parent[src], ident = s.ident[src], type = s.type[src];
    o.ox[dst] = ox; o.oy[dst] = oy; o.oz[dst] = oz;
    o.dx[dst] = dx; o.dy[dst] = dy; o.dz[dst] = dz;
    o.nx[dst] = nx; o.ny[dst] = ny; o.nz[dst] = nz;
    o.ex[dst] = ex; o.ey[dst] = ey; o.ez[dst] = ez;
    o.n[dst] = n; o.e1[dst] = e1; o.e2[dst] = e2;
    o.len[dst] = len; o.phase[dst] = phase; o.opl[dst] = opl;
    o.wl[dst] = wl; o.parent[dst] = parent; o.endf[dst] = endf; o.ident[dst] = ident; o.type[dst] = type;
}

}  // namespace rp
