// rp_gen_common.cuh -- the parts of a generation kernel that do not depend on
// the arithmetic path: shared-memory staging of the scene tables, the
// block-wide scan of per-ray child counts and the stores of children.
//
// Ordering contract (the reference's RayCollection.add_ray_c append order,
// raypier/core/ctracer.pyx:1004-1012 driven by trace_segment_c 2083-2117):
// children are stored in ascending parent index, and a parent's children in
// emission order (reflected before transmitted).  A sub-tile of 32 rays (one
// warp) writes its children, in that order, to its own slot range of a
// scratch arena and publishes their count; a scan of the counts then gives
// every sub-tile its final offset, and the children are copied to their
// place or read from the slots through a gather map by the next generation
// (rp_trace.cu).  Warps never wait for one another, so a warp with slow rays
// does not hold up the others.
#pragma once
#include "rp_kernels.cuh"

namespace rp {

// Stages lists / faces / materials in shared memory; returns the scene view.
// The staged copies may be read only after the caller's next __syncthreads().
__device__ __forceinline__ DevScene stage_tables(const GenArgs &A, unsigned char *smem, unsigned **s_counts) {
    DevScene S = A.S;
    size_t nl = (size_t)S.n_lists * sizeof(rp_facelist) / 8;
    size_t nf = (size_t)S.n_recs * sizeof(rp_face) / 8;
    size_t nm = (size_t)S.n_mats * sizeof(rp_material) / 8;
    double *dst = reinterpret_cast<double *>(smem);
    if (A.smem_tables) {
        const double *src = reinterpret_cast<const double *>(A.S.lists);
        for (size_t k = threadIdx.x; k < nl; k += blockDim.x) dst[k] = src[k];
        src = reinterpret_cast<const double *>(A.S.faces);
        for (size_t k = threadIdx.x; k < nf; k += blockDim.x) dst[nl + k] = src[k];
        src = reinterpret_cast<const double *>(A.S.mats);
        for (size_t k = threadIdx.x; k < nm; k += blockDim.x) dst[nl + nf + k] = src[k];
        S.lists = reinterpret_cast<const rp_facelist *>(dst);
        S.faces = reinterpret_cast<const rp_face *>(dst + nl);
        S.mats = reinterpret_cast<const rp_material *>(dst + nl + nf);
    }
    double *tail = A.smem_tables ? dst + nl + nf + nm : dst;
    // per-face world boxes (16 floats each), then the face -> list map, then hit counters
    float *bnd = reinterpret_cast<float *>(tail);
    for (int k = threadIdx.x; k < S.n_faces * 16; k += blockDim.x) bnd[k] = A.S.bounds[k];
    short *fl = reinterpret_cast<short *>(bnd + S.n_faces * 16);
    // the list ranges are read from global memory: the shared copy above is
    // not complete until the block's next barrier
    for (int l = 0; l < S.n_lists; l++) {
        int f0 = A.S.lists[l].first_face, n = A.S.lists[l].n_faces;
        for (int k = threadIdx.x; k < n; k += blockDim.x)
            if (f0 + k < S.n_faces) fl[f0 + k] = (short)l;
    }
    unsigned *cnt = reinterpret_cast<unsigned *>(tail + (S.n_faces * 16 * 4 + S.n_faces * 2 + 7) / 8);
    for (int k = threadIdx.x; k < S.n_faces; k += blockDim.x) cnt[k] = 0;
    S.bounds = bnd;
    S.face_list = fl;
    *s_counts = cnt;
    return S;
}

// A distortion face's cull (box flag 2, rp_bounds.h): true when the line
// through the local points p1, p2 never passes over the shape's rectangle
// b[0..3] = x0, x1, y0, y1, i.e. all four corners lie strictly on one side of
// the line's (x, y) projection (for a line along z: its (x, y) lies outside).
__device__ __forceinline__ bool distortion_line_misses(const float *b, v3 p1, v3 p2) {
    if (b[6] != 2.0f) return false;
    const double ux = p2.x - p1.x, uy = p2.y - p1.y;
    const double x0 = b[0], x1 = b[1], y0 = b[2], y1 = b[3];
    if (ux == 0.0 && uy == 0.0) return p1.x < x0 || p1.x > x1 || p1.y < y0 || p1.y > y1;
    const double s00 = ux * (y0 - p1.y) - uy * (x0 - p1.x), s01 = ux * (y1 - p1.y) - uy * (x0 - p1.x);
    const double s10 = ux * (y0 - p1.y) - uy * (x1 - p1.x), s11 = ux * (y1 - p1.y) - uy * (x1 - p1.x);
    return (s00 > 0.0 && s01 > 0.0 && s10 > 0.0 && s11 > 0.0) || (s00 < 0.0 && s01 < 0.0 && s10 < 0.0 && s11 < 0.0);
}

// A DistortionFace's entry distance for the searches' culling (its box record
// b, flag 2: b[0..3] its shape's padded rectangle x0, x1, y0, y1 in the face
// list's frame, b[8..15] the x and y rows of the world-to-list map).  The
// reference accepts only a point of the ray's line whose local (x, y) lies
// inside the shape (cfaces.pyx:2402), converged or not, so no hit lies before
// the ray enters the prism over that rectangle.  The ray (world origin o, unit
// direction u) goes to the list's frame in FP32, with a margin above that
// rounding; the parameter along the ray is its world distance in both
// frames.  Infinity when the prism lies behind the ray or the line misses it.
static __device__ __noinline__ float prism_enter(const float *b, float ox, float oy, float oz, float ux, float uy,
                                                 float uz) {
    const float *r0 = b + 8, *r1 = b + 12;
    const float qx = fmaf(r0[0], ox, fmaf(r0[1], oy, fmaf(r0[2], oz, r0[3])));
    const float qy = fmaf(r1[0], ox, fmaf(r1[1], oy, fmaf(r1[2], oz, r1[3])));
    const float vx = fmaf(r0[0], ux, fmaf(r0[1], uy, r0[2] * uz));
    const float vy = fmaf(r1[0], ux, fmaf(r1[1], uy, r1[2] * uz));
    // FP32 rounding of the map: a few units of 6e-8 of the terms' magnitudes
    const float m = 1e-6f * (fabsf(ox) + fabsf(oy) + fabsf(oz) + fabsf(r0[3]) + fabsf(r1[3]) + 1.0f);
    const float INF = __int_as_float(0x7f800000);
    float t0 = 0.0f, t1 = INF;
    const float lo[2] = {b[0] - m, b[2] - m}, hi[2] = {b[1] + m, b[3] + m}, q[2] = {qx, qy}, v[2] = {vx, vy};
#pragma unroll
    for (int k = 0; k < 2; k++) {
        if (fabsf(v[k]) < 1e-20f) {
            if (q[k] < lo[k] || q[k] > hi[k]) return INF;
        } else {
            const float iv = 1.0f / v[k];
            const float a = (lo[k] - q[k]) * iv, c = (hi[k] - q[k]) * iv;
            t0 = fmaxf(t0, fminf(a, c));
            t1 = fminf(t1, fmaxf(a, c));
        }
    }
    // (the padded bounds cover the position's rounding; the relative margin
    // the direction's)
    if (!(t1 + 1e-4f * fabsf(t1) + m >= t0)) return INF;
    return fmaxf(t0 - 1e-4f * fabsf(t0) - m, 0.0f);
}

// Exclusive scan of `c` over the block; *total_out gets the block total.
// Must be called by all threads of the block.
__device__ __forceinline__ unsigned block_scan(unsigned c, unsigned *total_out) {
    __shared__ unsigned s_warp[RP_BLOCK / 32];
    const unsigned lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned v = c;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        unsigned t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= (unsigned)o) v += t;
    }
    if (lane == 31) s_warp[warp] = v;
    __syncthreads();
    if (warp == 0) {
        unsigned w = (lane < RP_BLOCK / 32) ? s_warp[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            unsigned t = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= (unsigned)o) w += t;
        }
        if (lane < RP_BLOCK / 32) s_warp[lane] = w;  // inclusive warp prefixes
    }
    __syncthreads();
    unsigned before = (warp > 0) ? s_warp[warp - 1] : 0u;
    *total_out = s_warp[RP_BLOCK / 32 - 1];
    return before + (v - c);
}

// Exclusive scan of `c` over the warp; *total_out gets the warp total.  Must
// be called by all 32 lanes.
__device__ __forceinline__ unsigned warp_scan(unsigned c, unsigned *total_out) {
    const unsigned lane = threadIdx.x & 31;
    unsigned v = c;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        unsigned t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= (unsigned)o) v += t;
    }
    *total_out = __shfl_sync(0xffffffffu, v, 31);
    return v - c;
}

// Sub-tile (warp) index and its first slot for a kernel that runs one thread
// per ray with blockIdx.x * RP_BLOCK + threadIdx.x as the ray index.
__device__ __forceinline__ unsigned long long sub_tile_of_thread() {
    return ((unsigned long long)blockIdx.x * RP_BLOCK + threadIdx.x) / RP_SUB;
}

// Writes one child record at slot k of `out`.
__device__ __forceinline__ void store_child(const RaySoA &out, unsigned long long k, const ChildCommon &cc,
                                            const Child &ch, double phase, unsigned wl, unsigned parent,
                                            unsigned endf, unsigned ident) {
    out.ox[k] = cc.origin.x;
    out.oy[k] = cc.origin.y;
    out.oz[k] = cc.origin.z;
    out.dx[k] = ch.d.x;
    out.dy[k] = ch.d.y;
    out.dz[k] = ch.d.z;
    out.nx[k] = cc.normal.x;
    out.ny[k] = cc.normal.y;
    out.nz[k] = cc.normal.z;
    out.ex[k] = cc.E.x;
    out.ey[k] = cc.E.y;
    out.ez[k] = cc.E.z;
    out.n[k] = ch.n;
    out.e1[k] = ch.e1;
    out.e2[k] = ch.e2;
    out.len[k] = ch.len;
    out.phase[k] = phase + cc.dphase;
    out.opl[k] = cc.opl;
    out.wl[k] = wl;
    out.parent[k] = parent;
    out.endf[k] = endf;
    out.ident[k] = ident;
    out.type[k] = ch.type;
}

// |E1|^2 + |E2|^2 in the order the oracle uses for the termination rule.
__device__ __forceinline__ double child_e2(const Child &c) {
    return c.e1.x * c.e1.x + c.e1.y * c.e1.y + c.e2.x * c.e2.x + c.e2.y * c.e2.y;
}

// Flushes shared-memory hit counters and block statistics.
__device__ __forceinline__ void flush_counts(const GenArgs &A, const DevScene &S, unsigned *s_counts) {
    __syncthreads();
    for (int k = threadIdx.x; k < S.n_faces; k += blockDim.x) {
        unsigned c = s_counts[k];
        if (c) atomicAdd(&A.face_counts[k], c);
    }
}

}  // namespace rp
