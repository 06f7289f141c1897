// rp_capture.cu -- post-trace ray capture: select_ray_intersections /
// select_gausslet_intersections (raypier/core/ctracer.pyx:1981-2058).
// Compiled with --fmad=false: the face tests round as the reference's C.
//
// One thread takes one ray (or gausslet base ray) of a traced generation,
// copies it, and intersects the copy with every face of one face list from
// its origin to origin + direction * length, keeping the nearest hit
// (FaceList.intersect_c, ctracer.pyx:1882-1904).  Rays that meet a face are
// written, in input order, with that face's distance as length and its index
// as end_face_idx, and wavelength_idx shifted by the collection's offset into
// the concatenated wavelength list.  Placement is the generation's: warp
// scan into sub-tile slots, sub-tile scan, coalesced copy.
#include "rp_nearest.cuh"

namespace rp {

__global__ void __launch_bounds__(RP_BLOCK) capture_kernel(GaussArgs G, unsigned wl_offset, int with_para) {
    const GenArgs &A = G.g;
    extern __shared__ __align__(16) unsigned char smem[];
    unsigned *s_counts;
    DevScene S = stage_tables(A, smem, &s_counts);
    __syncthreads();
    const unsigned tile = blockIdx.x;
    const unsigned long long i = (unsigned long long)tile * RP_BLOCK + threadIdx.x;
    int best = -1;
    double len = 0.0;
    if (i < A.n_in) {
        v3 o = mkv(A.in.ox[i], A.in.oy[i], A.in.oz[i]);
        v3 d = mkv(A.in.dx[i], A.in.dy[i], A.in.dz[i]);
        len = A.in.len[i];
        v3 pend = addv(o, mulvs(d, len));
        const rp_facelist &L = S.lists[A.one_list];
        v3 p1 = xform(L.inv_trans.m, L.inv_trans.t, o);
        v3 p2 = xform(L.inv_trans.m, L.inv_trans.t, pend);
        for (int k = 0; k < L.n_faces; k++) {
            const int f = L.first_face + k;
            const rp_face &F = S.faces[f];
            double dist = face_isect(S, F, p1, p2, A.err);
            if (F.tolerance < dist && dist < len) {
                len = dist;
                best = f;
            }
        }
    }
    const unsigned nc = best >= 0 ? 1u : 0u;
    unsigned sub_n;
    const unsigned excl = warp_scan(nc, &sub_n);
    const unsigned long long qs = sub_tile_of_thread();
    if (nc) {
        const unsigned long long q = qs * RP_SUB_SLOTS + excl;
        copy_ray(A.in, i, A.scratch, q);
        A.scratch.len[q] = len;
        A.scratch.endf[q] = (unsigned)S.faces[best].idx;
        A.scratch.wl[q] = A.in.wl[i] + wl_offset;
        if (with_para)
            for (int f = 0; f < RP_PARA_ARRAYS; f++)
                G.pscratch[(unsigned long long)f * G.pscratch_cap + q] = G.pin[(unsigned long long)f * G.pin_cap + i];
    }
    if ((threadIdx.x & 31) == 0 && qs < rp_n_sub(A.n_in)) A.tile_counts[qs] = sub_n;
}

static cudaError_t prepare_capture(size_t smem) {
    if (smem <= 48 * 1024) return cudaSuccess;
    return cudaFuncSetAttribute(capture_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
}

cudaError_t launch_capture(const GaussArgs &a, unsigned wl_offset, int with_para, size_t smem, cudaStream_t st) {
    if (a.g.n_in == 0) return cudaSuccess;
    unsigned grid = (unsigned)((a.g.n_in + RP_BLOCK - 1) / RP_BLOCK);
    cudaError_t e = prepare_capture(smem);
    if (e != cudaSuccess) return e;
    capture_kernel<<<grid, RP_BLOCK, smem, st>>>(a, wl_offset, with_para);
    return cudaGetLastError();
}

}  // namespace rp
