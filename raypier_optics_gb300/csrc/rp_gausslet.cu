// rp_gausslet.cu -- Gausslet generation (trace_gausslet_c /
// trace_one_face_gausslet_c with trace_parabasal_rays,
// raypier/core/ctracer.pyx:2214-2385) and the Gausslet record layout kernels.
// Compiled with --fmad=false, like the plain ray path: the base ray's face
// search, its material and the parabasal arithmetic round as the reference's C.
//
// One thread traces one gausslet:
//   1. the base ray finds the nearest face exactly as a ray of a plain
//      generation does (or tests the one face of a sequential step), from its
//      current length (the reference resets lengths at the end of the
//      previous generation, not here);
//   2. on a hit the material evaluates the base ray's children; a
//      decomposition material (ResampleGaussletMaterial) records the gausslet
//      instead;
//   3. the six parabasal rays are tested, in order, against that face alone
//      with is_base_ray = 0; the first one that misses ends the gausslet
//      without children (trace_parabasal_rays returns early);
//   4. otherwise each child of the base ray becomes a child gausslet: its
//      parabasal rays start at their hit points and leave in the direction
//      the material's eval_parabasal_ray_c gives for that child's type.
// Children are placed as in a ray generation: warp scan into the sub-tile's
// child slots, sub-tile scan, coalesced placement (base rays and parabasal
// rays).
#include <map>
#include <mutex>

#include "rp_nearest.cuh"

namespace rp {

__device__ __forceinline__ double &para_at(double *base, unsigned long long cap, int j, int f,
                                           unsigned long long i) {
    return base[((unsigned long long)(j * RP_PARA_FIELDS + f)) * cap + i];
}

// Orientation of face F of list L at world point `point` (compute_orientation_c,
// ctracer.pyx:1939-1953).
__device__ __forceinline__ void orientation(const DevScene &S, const rp_facelist &L, const rp_face &F, v3 point,
                                            v3 &nrm, v3 &tng, unsigned *err) {
    v3 lp = xform(L.inv_trans.m, L.inv_trans.t, point);
    nrm = face_normal(S, F, lp, err);
    tng = face_tangent(F);
    if (F.invert_normal) {
        nrm = negv(nrm);
        tng = negv(tng);
    }
    nrm = rotv(L.trans.m, nrm);
    tng = rotv(L.trans.m, tng);
}

__global__ void __launch_bounds__(RP_BLOCK) gausslet_generation_kernel(GaussArgs G) {
    const GenArgs &A = G.g;
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ unsigned s_hits;
    unsigned *s_counts;
    DevScene S = stage_tables(A, smem, &s_counts);
    if (threadIdx.x == 0) s_hits = 0;
    __syncthreads();
    const unsigned tile = blockIdx.x;
    const unsigned long long i = (unsigned long long)tile * RP_BLOCK + threadIdx.x;
    const bool active = i < A.n_in;

    int best = -1, best_list = -1;
    double len = 0.0;
    v3 o = mkv(0, 0, 0), d = mkv(0, 0, 0);
    if (active) {
        o = mkv(A.in.ox[i], A.in.oy[i], A.in.oz[i]);
        d = mkv(A.in.dx[i], A.in.dy[i], A.in.dz[i]);
        len = A.in.len[i];
        v3 pend = addv(o, mulvs(d, A.max_len));
        if (A.one_list >= 0) {
            // FaceList.intersect_one_face_c, ctracer.pyx:1861-1879
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
            // every accepted distance is below the starting length, which
            // therefore bounds the boxes worth testing
            nearest_hit(S, o, d, pend, len, len, best, best_list, A.err);
        }
        A.in.len[i] = len;
        A.in.endf[i] = best >= 0 ? (unsigned)S.faces[best].idx : 0xFFFFFFFFu;
        if (best >= 0) {
            atomicAdd(&s_counts[best], 1u);
            atomicAdd(&s_hits, 1u);
        }
    }

    Child ch[2];
    ChildCommon cc;
    int nc = 0;
    if (active && best >= 0) {
        const rp_facelist &L = S.lists[best_list];
        const rp_face &F = S.faces[best];
        v3 point = addv(o, mulvs(d, len));
        v3 nrm, tng;
        orientation(S, L, F, point, nrm, tng, A.err);
        if (F.material >= 0) {
            const rp_material &M = S.mats[F.material];
            if (M.type == RP_MAT_RESAMPLE_GAUSSLET) {
                // ResampleGaussletMaterial.eval_child_ray_c, cmaterials.pyx:1806-1818
                if ((A.in.type[i] & RP_GAUSSLET_RAY) && G.captured) G.captured[i] = F.material + 1;
            } else {
                RayState r;
                r.o = o;
                r.d = d;
                r.E = mkv(A.in.ex[i], A.in.ey[i], A.in.ez[i]);
                r.n = A.in.n[i];
                r.e1 = A.in.e1[i];
                r.e2 = A.in.e2[i];
                r.len = len;
                r.opl = A.in.opl[i];
                r.type = A.in.type[i];
                r.wl = A.in.wl[i];
                nc = eval_children(S, M, r, point, nrm, tng, cc, ch, A.err);
            }
        }
        // the parabasal rays against the same face (trace_parabasal_rays,
        // ctracer.pyx:2365-2374; FaceList.intersect_para_c 1914-1926)
        for (int j = 0; j < 6; j++) {
            v3 po = mkv(para_at(G.pin, G.pin_cap, j, 0, i), para_at(G.pin, G.pin_cap, j, 1, i),
                        para_at(G.pin, G.pin_cap, j, 2, i));
            v3 pd = mkv(para_at(G.pin, G.pin_cap, j, 3, i), para_at(G.pin, G.pin_cap, j, 4, i),
                        para_at(G.pin, G.pin_cap, j, 5, i));
            double plen = para_at(G.pin, G.pin_cap, j, 9, i);
            v3 pe = addv(po, mulvs(pd, A.max_len));
            v3 p1 = xform(L.inv_trans.m, L.inv_trans.t, po);
            v3 p2 = xform(L.inv_trans.m, L.inv_trans.t, pe);
            double dist = face_isect_para(S, F, p1, p2, A.err);
            if (F.tolerance < dist && dist < plen) {
                para_at(G.pin, G.pin_cap, j, 9, i) = dist;
            } else {
                nc = 0;
                break;
            }
        }
    }

    unsigned sub_children;
    const unsigned excl = warp_scan((unsigned)nc, &sub_children);
    const unsigned long long q = sub_tile_of_thread();
    if (nc > 0) {
        const rp_facelist &L = S.lists[best_list];
        const rp_face &F = S.faces[best];
        const rp_material &M = S.mats[F.material];
        double phase = A.in.phase[i];
        unsigned wl = A.in.wl[i], ident = A.in.ident[i];
        unsigned endf = (unsigned)F.idx;
        const unsigned long long slot = q * RP_SUB_SLOTS + excl;
        for (int k = 0; k < nc; k++) {
            Child c = ch[k];
            c.len = A.max_len;  // reset_length_c
            store_child(A.scratch, slot + k, cc, c, phase, wl, (unsigned)i, endf, ident);
        }
        for (int j = 0; j < 6; j++) {
            v3 po = mkv(para_at(G.pin, G.pin_cap, j, 0, i), para_at(G.pin, G.pin_cap, j, 1, i),
                        para_at(G.pin, G.pin_cap, j, 2, i));
            v3 pd = mkv(para_at(G.pin, G.pin_cap, j, 3, i), para_at(G.pin, G.pin_cap, j, 4, i),
                        para_at(G.pin, G.pin_cap, j, 5, i));
            double plen = para_at(G.pin, G.pin_cap, j, 9, i);
            v3 pt = addv(po, mulvs(pd, plen));
            v3 nrm, tng;
            orientation(S, L, F, pt, nrm, tng, A.err);
            for (int k = 0; k < nc; k++) {
                v3 dir, pn;
                eval_parabasal(S, M, ch[k].n, wl, ch[k].type, pd, nrm, tng, dir, pn, A.err);
                const unsigned long long sk = slot + k;
                double *P = G.pscratch;
                const unsigned long long C = G.pscratch_cap;
                para_at(P, C, j, 0, sk) = pt.x;
                para_at(P, C, j, 1, sk) = pt.y;
                para_at(P, C, j, 2, sk) = pt.z;
                para_at(P, C, j, 3, sk) = dir.x;
                para_at(P, C, j, 4, sk) = dir.y;
                para_at(P, C, j, 5, sk) = dir.z;
                para_at(P, C, j, 6, sk) = pn.x;
                para_at(P, C, j, 7, sk) = pn.y;
                para_at(P, C, j, 8, sk) = pn.z;
                para_at(P, C, j, 9, sk) = A.max_len;  // reset_length_c
            }
        }
    }
    if ((threadIdx.x & 31) == 0 && q < rp_n_sub(A.n_in)) A.tile_counts[q] = sub_children;
    flush_counts(A, S, s_counts);
    if (threadIdx.x == 0) atomicAdd(&A.stats[0], (unsigned long long)s_hits);
}

static cudaError_t prepare_gausslet(size_t smem) {
    if (smem <= 48 * 1024) return cudaSuccess;
    static std::mutex mu;
    static std::map<int, size_t> configured;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lock(mu);
    if (configured[dev] >= smem) return cudaSuccess;
    e = cudaFuncSetAttribute(gausslet_generation_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e == cudaSuccess) configured[dev] = smem;
    return e;
}

cudaError_t launch_gausslet_generation(const GaussArgs &a, size_t smem, cudaStream_t st) {
    if (a.g.n_in == 0) return cudaSuccess;
    unsigned grid = (unsigned)((a.g.n_in + RP_BLOCK - 1) / RP_BLOCK);
    cudaError_t e = prepare_gausslet(smem);
    if (e != cudaSuccess) return e;
    gausslet_generation_kernel<<<grid, RP_BLOCK, smem, st>>>(a);
    return cudaGetLastError();
}

// Moves each sub-tile's child gausslets (base ray and parabasal rays) to
// their final place, as place_children_kernel does for rays.
__global__ void __launch_bounds__(RP_BLOCK) gausslet_place_kernel(GaussArgs G, unsigned long long n_sub) {
    const GenArgs &A = G.g;
    const unsigned long long q = sub_tile_of_thread();
    if (q >= n_sub) return;
    const unsigned lane = threadIdx.x & 31;
    const unsigned count = A.tile_counts[q];
    const unsigned long long base = A.tile_offsets[q];
    if (count > RP_SUB_SLOTS || base + count > A.out_cap || base + count > G.pout_cap) {
        if (lane == 0) atomicOr(A.err, ERR_OVERFLOW);
        return;
    }
    const unsigned long long src = q * RP_SUB_SLOTS;
    for (unsigned j = lane; j < count; j += RP_SUB) {
        copy_ray(A.scratch, src + j, A.out, base + j);
        for (int pj = 0; pj < 6; pj++) {  // one parabasal ray's ten fields: loads first, then stores
            double v[RP_PARA_FIELDS];
#pragma unroll
            for (int f = 0; f < RP_PARA_FIELDS; f++) v[f] = para_at(G.pscratch, G.pscratch_cap, pj, f, src + j);
#pragma unroll
            for (int f = 0; f < RP_PARA_FIELDS; f++) para_at(G.pout, G.pout_cap, pj, f, base + j) = v[f];
        }
    }
}

cudaError_t launch_gausslet_place(const GaussArgs &a, unsigned long long n_sub, cudaStream_t st) {
    if (n_sub == 0) return cudaSuccess;
    const unsigned grid = (unsigned)((n_sub + RP_SUB_PER_BLOCK - 1) / RP_SUB_PER_BLOCK);
    gausslet_place_kernel<<<grid, RP_BLOCK, 0, st>>>(a, n_sub);
    return cudaGetLastError();
}

// ---- packed records <-> device layout ---------------------------------------
// A 668-byte record is 4-byte aligned; 64 consecutive records (42,752 bytes)
// are 16-byte aligned, so a block of 64 threads moves its records through
// shared memory with 16-byte accesses and each thread (de)assembles one.
#define RP_G_BLOCK 64
#define RP_G_WORDS (RP_GAUSSLET_BYTES / 4)
#define RP_RAY_WORDS (RP_RAY_BYTES / 4)

__device__ __forceinline__ double gw2d(const unsigned *w, int k) {
    return __hiloint2double((int)w[k + 1], (int)w[k]);
}
__device__ __forceinline__ void gd2w(unsigned *w, int k, double v) {
    w[k] = (unsigned)__double2loint(v);
    w[k + 1] = (unsigned)__double2hiint(v);
}

__global__ void __launch_bounds__(RP_G_BLOCK) gausslet_aos_to_soa_kernel(const unsigned char *aos, RaySoA soa,
                                                                           double *para, unsigned long long cap,
                                                                           unsigned long long n) {
    __shared__ __align__(16) unsigned sw[RP_G_BLOCK * RP_G_WORDS];
    unsigned long long r0 = (unsigned long long)blockIdx.x * RP_G_BLOCK;
    unsigned long long nr = n - r0 < RP_G_BLOCK ? n - r0 : RP_G_BLOCK;
    const unsigned *src = reinterpret_cast<const unsigned *>(aos + r0 * RP_GAUSSLET_BYTES);
    unsigned nwords = (unsigned)(nr * RP_G_WORDS);
    if (nr == RP_G_BLOCK) {
        const uint4 *s4 = reinterpret_cast<const uint4 *>(src);
        uint4 *d4 = reinterpret_cast<uint4 *>(sw);
        for (unsigned k = threadIdx.x; k < nwords / 4; k += RP_G_BLOCK) d4[k] = s4[k];
    } else {
        for (unsigned k = threadIdx.x; k < nwords; k += RP_G_BLOCK) sw[k] = src[k];
    }
    __syncthreads();
    if (threadIdx.x < nr) {
        const unsigned *w = sw + threadIdx.x * RP_G_WORDS;
        unsigned long long i = r0 + threadIdx.x;
        soa.ox[i] = gw2d(w, 0);  soa.oy[i] = gw2d(w, 2);  soa.oz[i] = gw2d(w, 4);
        soa.dx[i] = gw2d(w, 6);  soa.dy[i] = gw2d(w, 8);  soa.dz[i] = gw2d(w, 10);
        soa.nx[i] = gw2d(w, 12); soa.ny[i] = gw2d(w, 14); soa.nz[i] = gw2d(w, 16);
        soa.ex[i] = gw2d(w, 18); soa.ey[i] = gw2d(w, 20); soa.ez[i] = gw2d(w, 22);
        soa.n[i] = make_double2(gw2d(w, 24), gw2d(w, 26));
        soa.e1[i] = make_double2(gw2d(w, 28), gw2d(w, 30));
        soa.e2[i] = make_double2(gw2d(w, 32), gw2d(w, 34));
        soa.len[i] = gw2d(w, 36);
        soa.phase[i] = gw2d(w, 38);
        soa.opl[i] = gw2d(w, 40);
        soa.wl[i] = w[42];
        soa.parent[i] = w[43];
        soa.endf[i] = w[44];
        soa.ident[i] = w[45];
        soa.type[i] = w[46];
        for (int j = 0; j < 6; j++)
            for (int f = 0; f < RP_PARA_FIELDS; f++)
                para_at(para, cap, j, f, i) = gw2d(w, RP_RAY_WORDS + 2 * (j * RP_PARA_FIELDS + f));
    }
}

__global__ void __launch_bounds__(RP_G_BLOCK) gausslet_soa_to_aos_kernel(RaySoA soa, const double *para,
                                                                           unsigned long long cap, unsigned char *aos,
                                                                           unsigned long long n) {
    __shared__ __align__(16) unsigned sw[RP_G_BLOCK * RP_G_WORDS];
    unsigned long long r0 = (unsigned long long)blockIdx.x * RP_G_BLOCK;
    unsigned long long nr = n - r0 < RP_G_BLOCK ? n - r0 : RP_G_BLOCK;
    if (threadIdx.x < nr) {
        unsigned *w = sw + threadIdx.x * RP_G_WORDS;
        unsigned long long i = r0 + threadIdx.x;
        gd2w(w, 0, soa.ox[i]);  gd2w(w, 2, soa.oy[i]);  gd2w(w, 4, soa.oz[i]);
        gd2w(w, 6, soa.dx[i]);  gd2w(w, 8, soa.dy[i]);  gd2w(w, 10, soa.dz[i]);
        gd2w(w, 12, soa.nx[i]); gd2w(w, 14, soa.ny[i]); gd2w(w, 16, soa.nz[i]);
        gd2w(w, 18, soa.ex[i]); gd2w(w, 20, soa.ey[i]); gd2w(w, 22, soa.ez[i]);
        double2 c = soa.n[i];
        gd2w(w, 24, c.x); gd2w(w, 26, c.y);
        c = soa.e1[i];
        gd2w(w, 28, c.x); gd2w(w, 30, c.y);
        c = soa.e2[i];
        gd2w(w, 32, c.x); gd2w(w, 34, c.y);
        gd2w(w, 36, soa.len[i]);
        gd2w(w, 38, soa.phase[i]);
        gd2w(w, 40, soa.opl[i]);
        w[42] = soa.wl[i];
        w[43] = soa.parent[i];
        w[44] = soa.endf[i];
        w[45] = soa.ident[i];
        w[46] = soa.type[i];
        for (int j = 0; j < 6; j++)
            for (int f = 0; f < RP_PARA_FIELDS; f++)
                gd2w(w, RP_RAY_WORDS + 2 * (j * RP_PARA_FIELDS + f), para[((unsigned long long)(j * RP_PARA_FIELDS + f)) * cap + i]);
    }
    __syncthreads();
    unsigned *dst = reinterpret_cast<unsigned *>(aos + r0 * RP_GAUSSLET_BYTES);
    unsigned nwords = (unsigned)(nr * RP_G_WORDS);
    if (nr == RP_G_BLOCK) {
        uint4 *d4 = reinterpret_cast<uint4 *>(dst);
        const uint4 *s4 = reinterpret_cast<const uint4 *>(sw);
        for (unsigned k = threadIdx.x; k < nwords / 4; k += RP_G_BLOCK) d4[k] = s4[k];
    } else {
        for (unsigned k = threadIdx.x; k < nwords; k += RP_G_BLOCK) dst[k] = sw[k];
    }
}

cudaError_t launch_gausslet_aos_to_soa(const void *aos, RaySoA soa, double *para, unsigned long long cap,
                                       unsigned long long n, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    unsigned grid = (unsigned)((n + RP_G_BLOCK - 1) / RP_G_BLOCK);
    gausslet_aos_to_soa_kernel<<<grid, RP_G_BLOCK, 0, st>>>(reinterpret_cast<const unsigned char *>(aos), soa, para,
                                                             cap, n);
    return cudaGetLastError();
}

cudaError_t launch_gausslet_soa_to_aos(RaySoA soa, const double *para, unsigned long long cap, void *aos,
                                       unsigned long long n, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    unsigned grid = (unsigned)((n + RP_G_BLOCK - 1) / RP_G_BLOCK);
    gausslet_soa_to_aos_kernel<<<grid, RP_G_BLOCK, 0, st>>>(soa, para, cap, reinterpret_cast<unsigned char *>(aos),
                                                             n);
    return cudaGetLastError();
}

// ---- parabasal rays of a circular Gaussian mode ---------------------------------
// GaussletCollection.config_parabasal_rays (ctracer.pyx:1430-1476), one
// gausslet per thread.  The base direction b (normalised) and two unit
// vectors across it, d1 = |b x o| and d2 = |b x d1| (o the y axis when
// b_x > b_y, else the x axis), carry three pairs of parabasal rays at the
// angles 2 pi k / 3: both start on a circle of the waist radius about the
// waist point (the base origin moved `wd` along b) and lean by
// +-theta0 = lambda / (pi w) towards the tangent of that circle; each is then
// moved back by `wd` along its own direction.  P.rc/rs hold radius x cos / sin
// and P.c/s the cos / sin of the three angles, taken from the host C library
// so that the device reproduces the reference's values; theta0's divisor
// (pi radius 1000, lambda in um) is P.kt.  Normal and length are the base ray's.
__device__ __forceinline__ v3 unit_of(v3 a) {
    const double m = sqrt(((a.x * a.x) + (a.y * a.y)) + (a.z * a.z));
    return mkv(a.x / m, a.y / m, a.z / m);
}
__device__ __forceinline__ v3 cross_of(v3 a, v3 b) {
    return mkv((a.y * b.z) - (a.z * b.y), (a.z * b.x) - (a.x * b.z), (a.x * b.y) - (a.y * b.x));
}

__global__ void parabasal_config_kernel(RaySoA b, double *para, unsigned long long cap, unsigned long long n,
                                        const double *wl, long long n_wl, ParabasalConfig P, unsigned *err) {
    const unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const v3 bd = unit_of(mkv(b.dx[i], b.dy[i], b.dz[i]));
    const v3 o = bd.x > bd.y ? mkv(0.0, 1.0, 0.0) : mkv(1.0, 0.0, 0.0);
    const v3 d1 = unit_of(cross_of(bd, o));
    const v3 d2 = unit_of(cross_of(bd, d1));
    const unsigned w = b.wl[i];
    if ((long long)w >= n_wl) {
        atomicOr(err, 1u);
        return;
    }
    const double theta0 = wl[w] / P.kt;
    const v3 org = mkv(b.ox[i], b.oy[i], b.oz[i]);
    const double nx = b.nx[i], ny = b.ny[i], nz = b.nz[i], len = b.len[i];
    for (int k = 0; k < 3; k++) {
        v3 c = mkv((d1.x * P.rc[k]) + (d2.x * P.rs[k]), (d1.y * P.rc[k]) + (d2.y * P.rs[k]),
                   (d1.z * P.rc[k]) + (d2.z * P.rs[k]));
        c = mkv(c.x + org.x, c.y + org.y, c.z + org.z);
        c = mkv(c.x + (bd.x * P.wd), c.y + (bd.y * P.wd), c.z + (bd.z * P.wd));
        const double ts = (-theta0) * P.s[k], tc = theta0 * P.c[k];
        const v3 t = mkv((d1.x * ts) + (d2.x * tc), (d1.y * ts) + (d2.y * tc), (d1.z * ts) + (d2.z * tc));
        const v3 dir[2] = {mkv(bd.x + t.x, bd.y + t.y, bd.z + t.z), mkv(bd.x - t.x, bd.y - t.y, bd.z - t.z)};
        for (int h = 0; h < 2; h++) {
            const v3 u = unit_of(dir[h]);
            const int j = 2 * k + h;
            para_at(para, cap, j, 0, i) = c.x - (dir[h].x * P.wd);
            para_at(para, cap, j, 1, i) = c.y - (dir[h].y * P.wd);
            para_at(para, cap, j, 2, i) = c.z - (dir[h].z * P.wd);
            para_at(para, cap, j, 3, i) = u.x;
            para_at(para, cap, j, 4, i) = u.y;
            para_at(para, cap, j, 5, i) = u.z;
            para_at(para, cap, j, 6, i) = nx;
            para_at(para, cap, j, 7, i) = ny;
            para_at(para, cap, j, 8, i) = nz;
            para_at(para, cap, j, 9, i) = len;
        }
    }
}

cudaError_t launch_parabasal_config(RaySoA base, double *para, unsigned long long cap, unsigned long long n,
                                    const double *wl, long long n_wl, const ParabasalConfig &P, unsigned *err,
                                    cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    parabasal_config_kernel<<<(unsigned)((n + 127) / 128), 128, 0, st>>>(base, para, cap, n, wl, n_wl, P, err);
    return cudaGetLastError();
}

// GaussletCollection.total_power (ctracer.pyx:1482-1496): the sum over the
// base rays of (|E1|^2 + |E2|^2) n.  Each block of RP_POWER_BLOCK threads adds
// its gausslets' terms in a fixed tree order into partial[blockIdx.x]; the
// host adds the partials in block order, so the result does not depend on
// scheduling.
__global__ void __launch_bounds__(RP_POWER_BLOCK) power_partials_kernel(RaySoA b, unsigned long long n,
                                                                        double *partial) {
    __shared__ double s[RP_POWER_BLOCK];
    const unsigned long long i = (unsigned long long)blockIdx.x * RP_POWER_BLOCK + threadIdx.x;
    double v = 0.0;
    if (i < n) {
        const double nr = b.n[i].x;
        const double2 e1 = b.e1[i], e2 = b.e2[i];
        v = ((((e1.x * e1.x) * nr) + ((e1.y * e1.y) * nr)) + ((e2.x * e2.x) * nr)) + ((e2.y * e2.y) * nr);
    }
    s[threadIdx.x] = v;
    __syncthreads();
    for (int h = RP_POWER_BLOCK / 2; h > 0; h >>= 1) {
        if ((int)threadIdx.x < h) s[threadIdx.x] = s[threadIdx.x] + s[threadIdx.x + h];
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[blockIdx.x] = s[0];
}

cudaError_t launch_power_partials(RaySoA base, unsigned long long n, double *partial, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    power_partials_kernel<<<(unsigned)((n + RP_POWER_BLOCK - 1) / RP_POWER_BLOCK), RP_POWER_BLOCK, 0, st>>>(base, n,
                                                                                                         partial);
    return cudaGetLastError();
}

}  // namespace rp
