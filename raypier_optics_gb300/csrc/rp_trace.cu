// rp_trace.cu -- plain FP64 generation kernel (one launch per generation) and
// the layout kernels.  Compiled with --fmad=false: every FP64 operation of the
// nearest-hit search and of the materials rounds as the reference's C does.
//
// One thread traces one ray of the generation (trace_segment_c,
// raypier/core/ctracer.pyx:2062-2118):
//   1. length = (double)(float)max_length, end_face_idx = -1, far point;
//   2. for every face list: origin and far point to local coordinates, test
//      each face, keep the nearest with tolerance < dist < length (strict, so
//      the earlier face wins a tie: FaceList.intersect_c 1882-1904);
//   3. on a hit: count it, hit point, orientation (compute_orientation_c
//      1939-1953), material evaluation into 0..2 children;
//   4. children go to the warp's sub-tile slots of the child arena (warp scan
//      of the per-ray counts); a scan of the sub-tile counts then either
//      copies them to their final place or, inside trace_rays, gives the next
//      generation a gather map through which it reads them.
#include <cstdint>
#include <map>
#include <mutex>

#include "rp_nearest.cuh"

namespace rp {

__global__ void __launch_bounds__(RP_BLOCK) generation_plain_kernel(GenArgs A) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ unsigned s_hits, s_term;
    unsigned *s_counts;
    DevScene S = stage_tables(A, smem, &s_counts);
    if (threadIdx.x == 0) {
        s_hits = 0;
        s_term = 0;
    }
    __syncthreads();
    const unsigned tile = blockIdx.x;
    const unsigned long long i = (unsigned long long)tile * RP_BLOCK + threadIdx.x;
    const bool active = i < A.n_in;
    // the ray's record in `in`: gathered through the map, or in place
    const unsigned long long src = active && A.in_map ? (unsigned long long)A.in_map[i] : i;

    int best = -1, best_list = -1;
    double len = A.max_len;
    v3 o = mkv(0, 0, 0), d = mkv(0, 0, 0);
    if (active) {
        o = mkv(A.in.ox[src], A.in.oy[src], A.in.oz[src]);
        d = mkv(A.in.dx[src], A.in.dy[src], A.in.dz[src]);
        v3 pend = addv(o, mulvs(d, A.max_len));
        if (A.one_list >= 0) {
            // sequential trace: one face of one list (FaceList.intersect_one_face_c, ctracer.pyx:1861-1879)
            const rp_facelist &L = S.lists[A.one_list];
            v3 p1 = xform(L.inv_trans.m, L.inv_trans.t, o);
            v3 p2 = xform(L.inv_trans.m, L.inv_trans.t, pend);
            int f = L.first_face + A.one_face;
            const rp_face &F = S.faces[f];
            double dist = face_isect(S, F, p1, p2, A.err);
            if (F.tolerance < dist && dist < len) {
                len = dist;
                best = f;
                best_list = A.one_list;
            }
        } else {
            nearest_hit(S, o, d, pend, A.max_len, len, best, best_list, A.err);
        }
        const unsigned endf = best >= 0 ? (unsigned)S.faces[best].idx : 0xFFFFFFFFu;
        if (A.in_map) {
            pass_ray(A.in, src, A.wb, i, len, endf);
        } else {
            A.in.len[i] = len;
            A.in.endf[i] = endf;
        }
        if (best >= 0) {
            atomicAdd(&s_counts[best], 1u);
            atomicAdd(&s_hits, 1u);
        }
    }

    if (!A.emit) {
        flush_counts(A, S, s_counts);
        if (threadIdx.x == 0) atomicAdd(&A.stats[0], (unsigned long long)s_hits);
        return;
    }

    // material evaluation
    Child ch[2];
    ChildCommon cc;
    int nc = 0;
    if (active && best >= 0) {
        const rp_facelist &L = S.lists[best_list];
        const rp_face &F = S.faces[best];
        v3 point = addv(o, mulvs(d, len));
        v3 lp = xform(L.inv_trans.m, L.inv_trans.t, point);
        v3 nrm = face_normal(S, F, lp, A.err);
        v3 tng = face_tangent(F);
        if (F.invert_normal) {
            nrm = negv(nrm);
            tng = negv(tng);
        }
        nrm = rotv(L.trans.m, nrm);
        tng = rotv(L.trans.m, tng);
        if (F.material >= 0) {
            RayState r;
            r.o = o;
            r.d = d;
            r.E = mkv(A.in.ex[src], A.in.ey[src], A.in.ez[src]);
            r.n = A.in.n[src];
            r.e1 = A.in.e1[src];
            r.e2 = A.in.e2[src];
            r.len = len;
            r.opl = A.in.opl[src];
            r.type = A.in.type[src];
            r.wl = A.in.wl[src];
            nc = eval_children(S, S.mats[F.material], r, point, nrm, tng, cc, ch, A.err);
            if (A.e2_term > 0.0 && nc > 0) {
                int w = 0;
                for (int k = 0; k < nc; k++) {
                    if (!(child_e2(ch[k]) < A.e2_term)) {
                        if (w != k) ch[w] = ch[k];
                        w++;
                    }
                }
                if (w < nc) atomicAdd(&s_term, (unsigned)(nc - w));
                nc = w;
            }
        }
    }

    // children go to the warp's slot range in parent order: the exclusive
    // warp scan of the per-ray counts is each ray's first slot
    unsigned sub_children;
    const unsigned excl = warp_scan((unsigned)nc, &sub_children);
    const unsigned long long q = sub_tile_of_thread();
    if (nc > 0) {
        double phase = A.in.phase[src];
        unsigned wl = A.in.wl[src], ident = A.in.ident[src];
        unsigned endf = (unsigned)S.faces[best].idx;
        const unsigned long long slot = q * RP_SUB_SLOTS + excl;
        for (int k = 0; k < nc; k++) store_child(A.scratch, slot + k, cc, ch[k], phase, wl, (unsigned)i, endf, ident);
    }
    if ((threadIdx.x & 31) == 0 && q < rp_n_sub(A.n_in)) A.tile_counts[q] = sub_children;
    flush_counts(A, S, s_counts);
    if (threadIdx.x == 0) {
        atomicAdd(&A.stats[0], (unsigned long long)s_hits);
        if (s_term) atomicAdd(&A.stats[1], (unsigned long long)s_term);
    }
}

size_t generation_smem_bytes(int n_lists, int n_recs, int n_mats, int n_faces) {
    // tables (when staged) + boxes + face->list map (padded to 8 bytes) + hit counters
    size_t tail = ((size_t)n_faces * 16 * 4 + (size_t)n_faces * 2 + 7) / 8 * 8 + (size_t)n_faces * sizeof(unsigned);
    return (size_t)n_lists * sizeof(rp_facelist) + (size_t)n_recs * sizeof(rp_face) +
           (size_t)n_mats * sizeof(rp_material) + tail;
}

cudaError_t launch_generation_plain(const GenArgs &a, size_t smem, cudaStream_t st) {
    if (a.n_in == 0) return cudaSuccess;
    unsigned grid = (unsigned)((a.n_in + RP_BLOCK - 1) / RP_BLOCK);
    cudaError_t e = prepare_generation_plain(a, smem);
    if (e != cudaSuccess) return e;
    generation_plain_kernel<<<grid, RP_BLOCK, smem, st>>>(a);
    return cudaGetLastError();
}

// Raises the kernel's dynamic shared-memory limit once per device to the
// largest size seen (under a lock: several host threads launch).
cudaError_t prepare_generation_plain(const GenArgs &a, size_t smem) {
    (void)a;
    if (smem <= 48 * 1024) return cudaSuccess;
    static std::mutex mu;
    static std::map<int, size_t> configured;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lock(mu);
    if (configured[dev] >= smem) return cudaSuccess;
    e = cudaFuncSetAttribute(generation_plain_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e == cudaSuccess) configured[dev] = smem;
    return e;
}

// ---- child placement ------------------------------------------------------
// One block scans the per-sub-tile child counts (exclusive prefix + total).
// Warp w owns a contiguous chunk of the counts (a multiple of 128 long): it
// sums the chunk with 16-byte loads, one block-wide scan of the 32 chunk sums
// gives each chunk its start, and the warp then scans its chunk 128 counts at
// a time with a running carry, writing the offsets with 16-byte stores.
#define RP_SCAN_SLICE 128  // counts per warp step: 4 per lane
__device__ __forceinline__ void scan_counts(const unsigned *counts, unsigned long long n, unsigned long long *offsets,
                                            unsigned long long *total) {
    __shared__ unsigned long long s_warp[32];
    const unsigned lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const bool vec = ((reinterpret_cast<uintptr_t>(counts) | reinterpret_cast<uintptr_t>(offsets)) & 15) == 0;
    const unsigned long long per = (n + 32ull * RP_SCAN_SLICE - 1) / (32ull * RP_SCAN_SLICE) * RP_SCAN_SLICE;
    const unsigned long long c0 = per * warp < n ? per * warp : n;
    const unsigned long long c1 = c0 + per < n ? c0 + per : n;
    // the four counts of this lane in the slice at `base` (zeros past the chunk)
    auto load4 = [&](unsigned long long base, unsigned &v0, unsigned &v1, unsigned &v2, unsigned &v3) {
        const unsigned long long k = base + 4ull * lane;
        if (vec && k + 3 < c1) {
            const uint4 v = *reinterpret_cast<const uint4 *>(counts + k);
            v0 = v.x; v1 = v.y; v2 = v.z; v3 = v.w;
        } else {
            v0 = k < c1 ? counts[k] : 0u;
            v1 = k + 1 < c1 ? counts[k + 1] : 0u;
            v2 = k + 2 < c1 ? counts[k + 2] : 0u;
            v3 = k + 3 < c1 ? counts[k + 3] : 0u;
        }
    };
    unsigned long long sum = 0;
#pragma unroll 4
    for (unsigned long long base = c0; base < c1; base += RP_SCAN_SLICE) {
        unsigned v0, v1, v2, v3;
        load4(base, v0, v1, v2, v3);
        sum += (unsigned long long)v0 + v1 + v2 + v3;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
    if (lane == 0) s_warp[warp] = sum;
    __syncthreads();
    if (warp == 0) {
        unsigned long long w = s_warp[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            unsigned long long t = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= (unsigned)o) w += t;
        }
        s_warp[lane] = w;  // inclusive prefixes of the chunk sums
    }
    __syncthreads();
    unsigned long long carry = warp ? s_warp[warp - 1] : 0ull;
    for (unsigned long long base = c0; base < c1; base += RP_SCAN_SLICE) {
        unsigned v0, v1, v2, v3;
        load4(base, v0, v1, v2, v3);
        const unsigned ls = v0 + v1 + v2 + v3;
        unsigned x = ls;  // inclusive warp scan of the lane sums
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            unsigned t = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= (unsigned)o) x += t;
        }
        const unsigned long long e0 = carry + (x - ls), e1 = e0 + v0, e2 = e1 + v1, e3 = e2 + v2;
        const unsigned long long k = base + 4ull * lane;
        if (vec && k + 3 < c1) {
            reinterpret_cast<ulonglong2 *>(offsets + k)[0] = make_ulonglong2(e0, e1);
            reinterpret_cast<ulonglong2 *>(offsets + k)[1] = make_ulonglong2(e2, e3);
        } else {
            if (k < c1) offsets[k] = e0;
            if (k + 1 < c1) offsets[k + 1] = e1;
            if (k + 2 < c1) offsets[k + 2] = e2;
            if (k + 3 < c1) offsets[k + 3] = e3;
        }
        carry += __shfl_sync(0xffffffffu, x, 31);
    }
    if (threadIdx.x == 0) *total = s_warp[31];
}

__global__ void __launch_bounds__(1024) tile_scan_kernel(const unsigned *counts, unsigned long long n,
                                                         unsigned long long *offsets, unsigned long long *total) {
    scan_counts(counts, n, offsets, total);
}

// The same with the count read from device memory (a batch step's unit count
// is known only on the device when its graph is launched).
__global__ void __launch_bounds__(1024) tile_scan_dev_kernel(const unsigned *counts, const unsigned *n_dev,
                                                             unsigned long long *offsets, unsigned long long *total) {
    scan_counts(counts, (unsigned long long)*n_dev, offsets, total);
}

cudaError_t launch_tile_scan_dev(const unsigned *counts, const unsigned *n_dev, unsigned long long *offsets,
                                 unsigned long long *total, cudaStream_t st) {
    tile_scan_dev_kernel<<<1, 1024, 0, st>>>(counts, n_dev, offsets, total);
    return cudaGetLastError();
}

cudaError_t launch_count_scan(const unsigned *counts, unsigned long long n, unsigned long long *offsets,
                              unsigned long long *total, cudaStream_t st) {
    tile_scan_kernel<<<1, 1024, 0, st>>>(counts, n, offsets, total);
    return cudaGetLastError();
}

cudaError_t launch_tile_scan(const GenArgs &a, cudaStream_t st) {
    tile_scan_kernel<<<1, 1024, 0, st>>>(a.tile_counts, rp_n_units(a.n_in, a.unit_rays), a.tile_offsets, a.out_count);
    return cudaGetLastError();
}

// Slots of one child-slot unit (two per ray of the unit).
__host__ __device__ __forceinline__ unsigned unit_slots(int unit_rays) {
    return 2u * (unit_rays > 0 ? (unsigned)unit_rays : (unsigned)RP_SUB);
}

// Moves each unit's children from the front of its slot range to their
// final place: one warp per unit, a straight coalesced copy of
// tile_counts[q] records to tile_offsets[q].
__global__ void __launch_bounds__(RP_BLOCK) place_children_kernel(GenArgs A, unsigned long long n_units) {
    const unsigned long long q = sub_tile_of_thread();  // one warp per unit
    if (q >= n_units) return;
    const unsigned lane = threadIdx.x & 31;
    const unsigned us = unit_slots(A.unit_rays);
    const unsigned count = A.tile_counts[q];
    const unsigned long long base = A.tile_offsets[q];
    if (count > us || base + count > A.out_cap) {
        if (lane == 0) atomicOr(A.err, ERR_OVERFLOW);
        return;
    }
    const unsigned long long src = q * us;
    for (unsigned j = lane; j < count; j += RP_SUB) copy_ray(A.scratch, src + j, A.out, base + j);
}

cudaError_t launch_place_children(const GenArgs &a, cudaStream_t st) {
    const unsigned long long n_units = rp_n_units(a.n_in, a.unit_rays);
    if (n_units == 0) return cudaSuccess;
    const unsigned grid = (unsigned)((n_units + RP_SUB_PER_BLOCK - 1) / RP_SUB_PER_BLOCK);
    place_children_kernel<<<grid, RP_BLOCK, 0, st>>>(a, n_units);
    return cudaGetLastError();
}

// The children's gather map instead of their copy: child j of unit q is
// ray tile_offsets[q] + j of the next generation and lives at arena slot
// q * (slots per unit) + j.  4 bytes per child instead of a 188-byte record
// read and written: the next generation's kernel reads each record through
// the map and writes it to its final place while tracing it.
__global__ void __launch_bounds__(RP_BLOCK) child_map_kernel(const unsigned *counts,
                                                             const unsigned long long *offsets,
                                                             unsigned long long n_units, unsigned us, unsigned *map,
                                                             unsigned long long map_cap, unsigned *err) {
    const unsigned long long q = sub_tile_of_thread();  // one warp per unit
    if (q >= n_units) return;
    const unsigned lane = threadIdx.x & 31;
    const unsigned count = counts[q];
    const unsigned long long base = offsets[q];
    if (count > us || base + count > map_cap) {
        if (lane == 0) atomicOr(err, ERR_OVERFLOW);
        return;
    }
    for (unsigned j = lane; j < count; j += RP_SUB) map[base + j] = (unsigned)(q * us + j);
}

cudaError_t launch_child_map(const GenArgs &a, unsigned *map, unsigned long long map_cap, cudaStream_t st) {
    const unsigned long long n_units = rp_n_units(a.n_in, a.unit_rays);
    if (n_units == 0) return cudaSuccess;
    const unsigned grid = (unsigned)((n_units + RP_SUB_PER_BLOCK - 1) / RP_SUB_PER_BLOCK);
    child_map_kernel<<<grid, RP_BLOCK, 0, st>>>(a.tile_counts, a.tile_offsets, n_units, unit_slots(a.unit_rays), map,
                                                map_cap, a.err);
    return cudaGetLastError();
}

// ---- small copies without a copy engine ----------------------------------------
// A generation's counters go to the host by SM stores into mapped page-locked
// memory, and the counter block is cleared by a kernel: copies and fills on
// the stream would queue on a copy engine behind the bulk downloads of
// earlier generations and hold the trace up.
__global__ void copy_words_kernel(const unsigned long long *src, unsigned long long *dst, int n) {
    if ((int)threadIdx.x < n) dst[threadIdx.x] = src[threadIdx.x];
    __threadfence_system();
}
__global__ void zero_words_kernel(unsigned long long *dst, int n) {
    if ((int)threadIdx.x < n) dst[threadIdx.x] = 0ull;
}

cudaError_t launch_copy_words(const unsigned long long *src, unsigned long long *dst, int n, cudaStream_t st) {
    copy_words_kernel<<<1, 32, 0, st>>>(src, dst, n);
    return cudaGetLastError();
}
cudaError_t launch_zero_words(unsigned long long *dst, int n, cudaStream_t st) {
    zero_words_kernel<<<1, 32, 0, st>>>(dst, n);
    return cudaGetLastError();
}

// ---- AoS <-> SoA ----------------------------------------------------------
// The packed 188-byte record (include/rp_gb300.h rp_ray) is not 16-byte
// aligned per ray, but 128 consecutive records (24,064 bytes) are when the
// first one is, so a block moves its 128 records through shared memory with
// 16-byte accesses and each thread then (de)assembles its own record from
// 4-byte words.  The packed side may be device memory or mapped pinned host
// memory (written or read across the host link directly); a packed buffer
// that does not start on a 16-byte boundary is moved in 4-byte words.
#define RP_AOS_WORDS (RP_RAY_BYTES / 4)

__device__ __forceinline__ double w2d(const unsigned *w, int k) {
    return __hiloint2double((int)w[k + 1], (int)w[k]);
}
__device__ __forceinline__ void d2w(unsigned *w, int k, double v) {
    w[k] = (unsigned)__double2loint(v);
    w[k + 1] = (unsigned)__double2hiint(v);
}

__global__ void __launch_bounds__(RP_BLOCK) aos_to_soa_kernel(const unsigned char *aos, RaySoA soa,
                                                                unsigned long long n) {
    __shared__ __align__(16) unsigned sw[RP_BLOCK * RP_AOS_WORDS];
    unsigned long long r0 = (unsigned long long)blockIdx.x * RP_BLOCK;
    unsigned long long nr = n - r0 < RP_BLOCK ? n - r0 : RP_BLOCK;
    const unsigned *src = reinterpret_cast<const unsigned *>(aos + r0 * RP_RAY_BYTES);
    unsigned nwords = (unsigned)(nr * RP_AOS_WORDS);
    if (nr == RP_BLOCK && ((uintptr_t)aos & 15) == 0) {
        const uint4 *s4 = reinterpret_cast<const uint4 *>(src);
        uint4 *d4 = reinterpret_cast<uint4 *>(sw);
        for (unsigned k = threadIdx.x; k < nwords / 4; k += RP_BLOCK) d4[k] = s4[k];
    } else {
        for (unsigned k = threadIdx.x; k < nwords; k += RP_BLOCK) sw[k] = src[k];
    }
    __syncthreads();
    if (threadIdx.x < nr) {
        const unsigned *w = sw + threadIdx.x * RP_AOS_WORDS;
        unsigned long long i = r0 + threadIdx.x;
        soa.ox[i] = w2d(w, 0);  soa.oy[i] = w2d(w, 2);  soa.oz[i] = w2d(w, 4);
        soa.dx[i] = w2d(w, 6);  soa.dy[i] = w2d(w, 8);  soa.dz[i] = w2d(w, 10);
        soa.nx[i] = w2d(w, 12); soa.ny[i] = w2d(w, 14); soa.nz[i] = w2d(w, 16);
        soa.ex[i] = w2d(w, 18); soa.ey[i] = w2d(w, 20); soa.ez[i] = w2d(w, 22);
        soa.n[i] = make_double2(w2d(w, 24), w2d(w, 26));
        soa.e1[i] = make_double2(w2d(w, 28), w2d(w, 30));
        soa.e2[i] = make_double2(w2d(w, 32), w2d(w, 34));
        soa.len[i] = w2d(w, 36);
        soa.phase[i] = w2d(w, 38);
        soa.opl[i] = w2d(w, 40);
        soa.wl[i] = w[42];
        soa.parent[i] = w[43];
        soa.endf[i] = w[44];
        soa.ident[i] = w[45];
        soa.type[i] = w[46];
    }
}

__global__ void __launch_bounds__(RP_BLOCK) soa_to_aos_kernel(RaySoA soa, unsigned char *aos,
                                                                unsigned long long n) {
    __shared__ __align__(16) unsigned sw[RP_BLOCK * RP_AOS_WORDS];
    unsigned long long r0 = (unsigned long long)blockIdx.x * RP_BLOCK;
    unsigned long long nr = n - r0 < RP_BLOCK ? n - r0 : RP_BLOCK;
    if (threadIdx.x < nr) {
        unsigned *w = sw + threadIdx.x * RP_AOS_WORDS;
        unsigned long long i = r0 + threadIdx.x;
        d2w(w, 0, soa.ox[i]);  d2w(w, 2, soa.oy[i]);  d2w(w, 4, soa.oz[i]);
        d2w(w, 6, soa.dx[i]);  d2w(w, 8, soa.dy[i]);  d2w(w, 10, soa.dz[i]);
        d2w(w, 12, soa.nx[i]); d2w(w, 14, soa.ny[i]); d2w(w, 16, soa.nz[i]);
        d2w(w, 18, soa.ex[i]); d2w(w, 20, soa.ey[i]); d2w(w, 22, soa.ez[i]);
        double2 c = soa.n[i];
        d2w(w, 24, c.x); d2w(w, 26, c.y);
        c = soa.e1[i];
        d2w(w, 28, c.x); d2w(w, 30, c.y);
        c = soa.e2[i];
        d2w(w, 32, c.x); d2w(w, 34, c.y);
        d2w(w, 36, soa.len[i]);
        d2w(w, 38, soa.phase[i]);
        d2w(w, 40, soa.opl[i]);
        w[42] = soa.wl[i];
        w[43] = soa.parent[i];
        w[44] = soa.endf[i];
        w[45] = soa.ident[i];
        w[46] = soa.type[i];
    }
    __syncthreads();
    unsigned *dst = reinterpret_cast<unsigned *>(aos + r0 * RP_RAY_BYTES);
    unsigned nwords = (unsigned)(nr * RP_AOS_WORDS);
    if (nr == RP_BLOCK && ((uintptr_t)aos & 15) == 0) {
        uint4 *d4 = reinterpret_cast<uint4 *>(dst);
        const uint4 *s4 = reinterpret_cast<const uint4 *>(sw);
        for (unsigned k = threadIdx.x; k < nwords / 4; k += RP_BLOCK) d4[k] = s4[k];
    } else {
        for (unsigned k = threadIdx.x; k < nwords; k += RP_BLOCK) dst[k] = sw[k];
    }
}

cudaError_t launch_aos_to_soa(const void *aos, RaySoA soa, unsigned long long n, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    unsigned grid = (unsigned)((n + RP_BLOCK - 1) / RP_BLOCK);
    aos_to_soa_kernel<<<grid, RP_BLOCK, 0, st>>>(reinterpret_cast<const unsigned char *>(aos), soa, n);
    return cudaGetLastError();
}

cudaError_t launch_soa_to_aos(RaySoA soa, void *aos, unsigned long long n, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    unsigned grid = (unsigned)((n + RP_BLOCK - 1) / RP_BLOCK);
    soa_to_aos_kernel<<<grid, RP_BLOCK, 0, st>>>(soa, reinterpret_cast<unsigned char *>(aos), n);
    return cudaGetLastError();
}

// ---- dispersion tables: BaseDispersionCurve.c_evaluate_n (cmaterials.pyx:206-228)
static __device__ double curve_n(const rp_dispersion &c, const double *coefs, double wavelen) {
    switch (c.formula_id) {
        case 0: return coefs[0];  // nondispersive_0, 107-108
        case 1: {                 // sellmeier_1, 110-119
            double n2 = 1.0, wl2 = wavelen * wavelen;
            n2 += coefs[0];
            for (int i = 0; i < (c.n_coefs - 1) / 2; i++) {
                double b = coefs[2 * i + 2];
                n2 += coefs[2 * i + 1] * wl2 / (wl2 - b * b);
            }
            return sqrt(n2);
        }
        case 2: {  // sellmeier_2, 121-130
            double n2 = 1.0, wl2 = wavelen * wavelen;
            n2 += coefs[0];
            for (int i = 0; i < (c.n_coefs - 1) / 2; i++) n2 += coefs[2 * i + 1] * wl2 / (wl2 - coefs[2 * i + 2]);
            return sqrt(n2);
        }
        case 3: {  // sellmeier_3, 133-140
            double n2 = coefs[0];
            for (int i = 1; i < c.n_coefs - 1; i += 2) n2 += coefs[i] * (pow(wavelen, coefs[i + 1]));
            return sqrt(n2);
        }
        default: return nan_d();
    }
}

__global__ void dispersion_table_kernel(const rp_dispersion *curves, int n_curves, const double *aux,
                                        const double *wl, long long n_wl, double2 *ntab) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)n_curves * n_wl) return;
    int c = (int)(t / n_wl);
    long long i = t - (long long)c * n_wl;
    rp_dispersion cv = curves[c];
    double n_imag = 0.0001 * cv.absorption / (4 * 3.14159265358979323846);
    ntab[t] = make_double2(curve_n(cv, aux + cv.aux, wl[i]), n_imag * wl[i]);
}

cudaError_t launch_dispersion_table(const rp_dispersion *curves, int n_curves, const double *aux,
                                    const double *wl, long long n_wl, double2 *ntab, cudaStream_t st) {
    long long n = (long long)n_curves * n_wl;
    if (n == 0) return cudaSuccess;
    dispersion_table_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(curves, n_curves, aux, wl, n_wl, ntab);
    return cudaGetLastError();
}

}  // namespace rp
