// rp_api.cu -- the C ABI (include/rp_gb300.h): contexts, scenes, device ray
// buffers and the trace entry points.  No C++ exception crosses the boundary;
// every entry point returns an rp status code.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>
#include <vector>

#include "../../include/rp_gb300.h"
#include "rp_bounds.h"
#include "rp_internal.h"
#include "rp_zkprog.h"

static thread_local char g_last_error[256] = "";

static int cuda_fail(cudaError_t e, const char *what) {
    snprintf(g_last_error, sizeof g_last_error, "%s: %s", what, cudaGetErrorString(e));
    return RP_ERR_CUDA;
}
#define CK(call)                                          \
    do {                                                  \
        cudaError_t _e = (call);                          \
        if (_e != cudaSuccess) return cuda_fail(_e, #call); \
    } while (0)

// ---- memory: a per-context caching allocator ----------------------------------
// Freed blocks are kept and handed out again to requests of up to the same
// size (best fit, at most 2x larger), so a steady tracing loop allocates no
// device memory after its first iteration.  Blocks are released to CUDA when
// the budget would otherwise be exceeded, by rp_ctx_trim, and at destroy.
// The pool is guarded by pool_mu: the job server frees a job's buffers from
// the thread that finishes it, whichever context made them.
static void pool_release_all(rp_ctx *ctx) {  // pool_mu held
    for (auto &b : ctx->pool) cudaFree(b.p);
    ctx->pool.clear();
    ctx->pooled = 0;
}

// Best fit among the pooled blocks at most twice the request.  (Blocks kept
// to exact size classes made the job server's lanes allocate and trim far
// more often: p50 latency 4.9 instead of 3.2 ms.)
static int ctx_alloc(rp_ctx *ctx, void **p, size_t bytes, size_t *got) {
    std::lock_guard<std::mutex> lk(ctx->pool_mu);
    bytes = bytes ? bytes : 16;
    *got = bytes;
    int best = -1;
    for (size_t k = 0; k < ctx->pool.size(); k++) {
        size_t b = ctx->pool[k].bytes;
        if (b >= bytes && b <= 2 * bytes && (best < 0 || b < ctx->pool[best].bytes)) best = (int)k;
    }
    if (best >= 0) {
        *p = ctx->pool[best].p;
        size_t b = ctx->pool[best].bytes;
        *got = b;
        ctx->pool.erase(ctx->pool.begin() + best);
        ctx->pooled -= b;
        ctx->in_use += b;
        return RP_OK;
    }
    if (ctx->budget && ctx->in_use + ctx->pooled + bytes > ctx->budget) pool_release_all(ctx);
    if (ctx->budget && ctx->in_use + bytes > ctx->budget) {
        snprintf(g_last_error, sizeof g_last_error, "device budget of %llu bytes exceeded",
                 (unsigned long long)ctx->budget);
        return RP_ERR_BUDGET;
    }
    cudaError_t e = cudaMalloc(p, bytes);
    if (e == cudaErrorMemoryAllocation && !ctx->pool.empty()) {
        cudaGetLastError();
        pool_release_all(ctx);
        e = cudaMalloc(p, bytes);
    }
    if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc");
    ctx->in_use += bytes;
    return RP_OK;
}

// Returns the block to the pool; `bytes` must be the size it was allocated
// with (pool blocks keep their own size).
static void ctx_free(rp_ctx *ctx, void *p, size_t bytes) {
    if (!p) return;
    std::lock_guard<std::mutex> lk(ctx->pool_mu);
    bytes = bytes ? bytes : 16;
    ctx->in_use -= bytes;
    ctx->pool.push_back(PoolBlock{p, bytes});
    ctx->pooled += bytes;
}

int rp__ctx_alloc(rp_ctx *ctx, void **p, size_t bytes, size_t *got) { return ctx_alloc(ctx, p, bytes, got); }
void rp__ctx_free(rp_ctx *ctx, void *p, size_t bytes) { ctx_free(ctx, p, bytes); }
int rp__cuda_fail(cudaError_t e, const char *what) { return cuda_fail(e, what); }
void rp__set_error(const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_last_error, sizeof g_last_error, fmt, ap);
    va_end(ap);
}

extern "C" {

// rp_trace_segment_noalloc's cached scratch address of a device (defined
// with it below); a new context looks it up again.
static void noalloc_forget(int device);

int rp_version(void) { return RP_ABI_VERSION; }

const char *rp_status_string(int s) {
    switch (s) {
        case RP_OK: return "ok";
        case RP_ERR_INVALID: return "invalid argument";
        case RP_ERR_CAPACITY: return "output capacity exceeded";
        case RP_ERR_BUDGET: return "device memory budget exceeded";
        case RP_ERR_TIMEOUT: return "bounded device wait timed out";
        case RP_ERR_CUDA: return "CUDA error";
        case RP_ERR_UNSUPPORTED: return "unsupported face/material type";
        case RP_ERR_NOMEM: return "host allocation failed";
        default: return "unknown status";
    }
}

const char *rp_last_error(void) { return g_last_error; }

int rp_ctx_create(int device, uint64_t hbm_budget, rp_ctx **out) {
    if (!out) return RP_ERR_INVALID;
    *out = nullptr;
    int ndev = 0;
    CK(cudaGetDeviceCount(&ndev));
    if (device < 0 || device >= ndev) return RP_ERR_INVALID;
    CK(cudaSetDevice(device));
    rp_ctx *c = new (std::nothrow) rp_ctx();
    if (!c) return RP_ERR_NOMEM;
    c->device = device;
    c->budget = hbm_budget;
    cudaError_t e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaHostAlloc((void **)&c->h_pinned, 8 * sizeof(unsigned long long), cudaHostAllocMapped);
    if (e == cudaSuccess) e = cudaHostGetDevicePointer((void **)&c->d_pinned, c->h_pinned, 0);
    if (e == cudaSuccess) e = cudaEventCreate(&c->ev0);
    if (e == cudaSuccess) e = cudaEventCreate(&c->ev1);
    if (e != cudaSuccess) {
        delete c;
        return cuda_fail(e, "rp_ctx_create");
    }
    noalloc_forget(device);
    *out = c;
    return RP_OK;
}

int rp_ctx_destroy(rp_ctx *c) {
    if (!c) return RP_ERR_INVALID;
    cudaSetDevice(c->device);
    cudaStreamSynchronize(c->stream);
    if (c->arena) rp_rays_free(c->arena);
    if (c->arena2) rp_rays_free(c->arena2);
    for (int k = 0; k < 2; k++)
        if (c->child_map[k]) ctx_free(c, c->child_map[k], c->child_map_bytes[k]);
    {
        std::lock_guard<std::mutex> lk(c->pool_mu);
        pool_release_all(c);
    }
    for (auto ev : c->gen_ev) cudaEventDestroy(ev);
    if (c->scratch) cudaFree(c->scratch);
    if (c->h_pinned) cudaFreeHost(c->h_pinned);
    cudaEventDestroy(c->ev0);
    cudaEventDestroy(c->ev1);
    if (c->copy_stream) cudaStreamDestroy(c->copy_stream);
    cudaStreamDestroy(c->stream);
    delete c;
    return RP_OK;
}

int rp_ctx_synchronize(rp_ctx *c) {
    if (!c) return RP_ERR_INVALID;
    CK(cudaStreamSynchronize(c->stream));
    return RP_OK;
}

int rp_ctx_memory(rp_ctx *c, uint64_t *bytes) {
    if (!c || !bytes) return RP_ERR_INVALID;
    *bytes = c->in_use + c->pooled + c->scratch_bytes;
    return RP_OK;
}

int rp_ctx_trim(rp_ctx *c) {
    if (!c) return RP_ERR_INVALID;
    CK(cudaSetDevice(c->device));
    CK(cudaStreamSynchronize(c->stream));
    std::lock_guard<std::mutex> lk(c->pool_mu);
    pool_release_all(c);
    return RP_OK;
}

int rp_host_alloc(uint64_t bytes, void **ptr) {
    if (!ptr) return RP_ERR_INVALID;
    CK(cudaMallocHost(ptr, bytes ? bytes : 16));
    return RP_OK;
}

int rp_host_free(void *ptr) {
    if (!ptr) return RP_OK;
    CK(cudaFreeHost(ptr));
    return RP_OK;
}

// ---- scenes -------------------------------------------------------------------
static size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

static int validate_scene(const rp_scene_desc *d) {
    if (!d || d->n_lists < 0 || d->n_faces < 0 || d->n_face_records < d->n_faces || d->n_materials < 0 ||
        d->n_shape_ops < 0 || d->n_distortions < 0 || d->n_dispersions < 0 || d->n_aux < 0)
        return RP_ERR_INVALID;
    int expect = 0;
    for (int l = 0; l < d->n_lists; l++) {
        const rp_facelist &L = d->lists[l];
        if (L.first_face != expect || L.n_faces < 0) return RP_ERR_INVALID;
        expect += L.n_faces;
    }
    if (expect != d->n_faces) return RP_ERR_INVALID;
    auto aux_ok = [&](long long off, long long count) { return off >= 0 && count >= 0 && off + count <= d->n_aux; };
    for (int k = 0; k < d->n_shape_ops; k++) {
        const rp_shape_op &op = d->shape_ops[k];
        if (op.op < RP_SHAPE_END || op.op > RP_SHAPE_NOT) return RP_ERR_UNSUPPORTED;
        if (op.op == RP_SHAPE_POLYGON && !aux_ok(op.aux, 2LL * op.n)) return RP_ERR_INVALID;
    }
    for (int f = 0; f < d->n_face_records; f++) {
        const rp_face &F = d->faces[f];
        if (F.type < RP_FACE_NONE || F.type > RP_FACE_AXICON) return RP_ERR_UNSUPPORTED;
        if (F.type == RP_FACE_ELLIPSOIDAL && !aux_ok(F.aux, 24)) return RP_ERR_INVALID;
        if (f < d->n_faces && (F.material < 0 || F.material >= d->n_materials)) return RP_ERR_INVALID;
        if (F.shape < -1 || F.shape >= d->n_shape_ops) return RP_ERR_INVALID;
        if (F.type == RP_FACE_EXTPOLY) {
            if (F.n_aux0 < 1 || F.n_aux0 > 8 || F.n_aux1 < 1 || F.n_aux1 > 8) return RP_ERR_UNSUPPORTED;
            if (!aux_ok(F.aux, (long long)F.n_aux0 * F.n_aux1)) return RP_ERR_INVALID;
        }
        if ((F.type == RP_FACE_ORIENTED_POLYGON || F.type == RP_FACE_POLYGON) && !aux_ok(F.aux, 2LL * F.n_aux0))
            return RP_ERR_INVALID;
        if (F.type == RP_FACE_DISTORTION) {
            if (F.base < d->n_faces || F.base >= d->n_face_records) return RP_ERR_INVALID;
            if (d->faces[F.base].type == RP_FACE_DISTORTION) return RP_ERR_UNSUPPORTED;
            if (F.distortion < 0 || F.distortion >= d->n_distortions) return RP_ERR_INVALID;
        }
    }
    for (int m = 0; m < d->n_materials; m++) {
        const rp_material &M = d->materials[m];
        if (M.type < RP_MAT_NONE || M.type > RP_MAT_RESAMPLE_GAUSSLET) return RP_ERR_UNSUPPORTED;
        if ((M.type == RP_MAT_FULL_DIELECTRIC_DISPERSIVE || M.type == RP_MAT_COATED_DISPERSIVE) &&
            (M.curve_inside < 0 || M.curve_inside >= d->n_dispersions || M.curve_outside < 0 ||
             M.curve_outside >= d->n_dispersions))
            return RP_ERR_INVALID;
        if (M.type == RP_MAT_COATED_DISPERSIVE &&
            !(M.p[0] >= 0.0 && M.p[0] < (double)d->n_dispersions && M.p[0] == (double)(int)M.p[0]))
            return RP_ERR_INVALID;
    }
    for (int c = 0; c < d->n_dispersions; c++) {
        int fid = d->dispersions[c].formula_id;
        if (fid < 0 || fid > 3) return RP_ERR_UNSUPPORTED;
    }
    for (int k = 0; k < d->n_distortions; k++) {
        const rp_distortion &D = d->distortions[k];
        if (D.type != RP_DIST_ZERNIKE && D.type != RP_DIST_SIMPLE_J7) return RP_ERR_UNSUPPORTED;
        if (D.type == RP_DIST_ZERNIKE) {
            if (D.k_max < 0 || D.k_max > 48) return RP_ERR_UNSUPPORTED;
            if (!aux_ok(D.aux, 5LL * D.n_coefs)) return RP_ERR_INVALID;
            for (int i = 0; i < D.n_coefs; i++) {
                double n = d->aux[D.aux + 5 * i + 1], m = d->aux[D.aux + 5 * i + 2], kk = d->aux[D.aux + 5 * i + 3];
                if (n < 0 || n > 8 || m < -n || m > n || kk < 0 || kk >= 48) return RP_ERR_UNSUPPORTED;
            }
        }
    }
    for (int c = 0; c < d->n_dispersions; c++)
        if (!aux_ok(d->dispersions[c].aux, d->dispersions[c].n_coefs)) return RP_ERR_INVALID;
    return RP_OK;
}

int rp_scene_create(rp_ctx *ctx, const rp_scene_desc *d, const double *wavelengths, int64_t n_wl, rp_scene **out) {
    if (!ctx || !out) return RP_ERR_INVALID;
    *out = nullptr;
    int v = validate_scene(d);
    if (v != RP_OK) {
        snprintf(g_last_error, sizeof g_last_error, "malformed or unsupported scene");
        return v;
    }
    if (n_wl < 0 || (n_wl > 0 && !wavelengths)) return RP_ERR_INVALID;
    // wavelength range check: BaseDispersionCurve.c_evaluate_n raises ValueError (cmaterials.pyx:220-224)
    for (int c = 0; c < d->n_dispersions; c++) {
        const rp_dispersion &D = d->dispersions[c];
        for (int64_t i = 0; i < n_wl; i++) {
            if (wavelengths[i] < D.wavelength_min || wavelengths[i] > D.wavelength_max) {
                snprintf(g_last_error, sizeof g_last_error,
                         "Wavelength (%f) outside range of dispersion curve (%f -> %f)", wavelengths[i],
                         D.wavelength_min, D.wavelength_max);
                return RP_ERR_INVALID;
            }
        }
    }
    CK(cudaSetDevice(ctx->device));
    rp_scene *s = new (std::nothrow) rp_scene();
    if (!s) return RP_ERR_NOMEM;
    s->ctx = ctx;
    s->n_faces = d->n_faces;
    s->host_faces.assign(d->faces, d->faces + d->n_face_records);
    s->host_lists.assign(d->lists, d->lists + d->n_lists);
    s->mixed_fallback = 0;
    for (int f = 0; f < d->n_faces; f++) {
        int t = d->faces[f].type;
        if (t != RP_FACE_CIRCULAR && t != RP_FACE_RECTANGULAR && t != RP_FACE_SHAPED_PLANAR &&
            t != RP_FACE_SPHERICAL && t != RP_FACE_SHAPED_SPHERICAL && t != RP_FACE_CONIC && t != RP_FACE_ASPHERIC)
            s->mixed_fallback = 1;  // (DistortionFace and ExtendedPolynomialFace run in that form's FP32 code)
    }
    for (int m = 0; m < d->n_materials; m++) {
        int t = d->materials[m].type;
        if (t != RP_MAT_NONE && t != RP_MAT_OPAQUE && t != RP_MAT_PEC && t != RP_MAT_DIELECTRIC &&
            t != RP_MAT_FULL_DIELECTRIC && t != RP_MAT_FULL_DIELECTRIC_DISPERSIVE && t != RP_MAT_TRANSPARENT)
            s->mixed_fallback = 1;
    }
    size_t o_lists = 0;
    size_t o_faces = o_lists + align256(sizeof(rp_facelist) * d->n_lists);
    size_t o_mats = o_faces + align256(sizeof(rp_face) * d->n_face_records);
    size_t o_shapes = o_mats + align256(sizeof(rp_material) * d->n_materials);
    size_t o_dists = o_shapes + align256(sizeof(rp_shape_op) * d->n_shape_ops);
    size_t o_disp = o_dists + align256(sizeof(rp_distortion) * d->n_distortions);
    size_t o_aux = o_disp + align256(sizeof(rp_dispersion) * d->n_dispersions);
    size_t o_wl = o_aux + align256(sizeof(double) * d->n_aux);
    size_t o_ntab = o_wl + align256(sizeof(double) * (size_t)n_wl);
    size_t o_cnt = o_ntab + align256(sizeof(double2) * (size_t)n_wl * d->n_dispersions);
    size_t o_bnd = o_cnt + align256(sizeof(unsigned) * (d->n_face_records + 1));
    // compiled Zernike programs: per distortion the z and the z-gradient one
    std::vector<int> zk_off((size_t)2 * d->n_distortions + 2, -1);
    std::vector<short> zk_prog;
    for (int q = 0; q < d->n_distortions; q++) {
        const rp_distortion &dq = d->distortions[q];
        if (dq.type != RP_DIST_ZERNIKE || dq.aux < 0 || (int64_t)dq.aux + 5 * (int64_t)dq.n_coefs > d->n_aux) continue;
        for (int g = 0; g < 2; g++) {
            std::vector<short> prog;
            if (zk_compile(dq.n_coefs, dq.k_max, d->aux + dq.aux, g == 1, prog)) {
                zk_off[2 * q + g] = (int)zk_prog.size();
                zk_prog.insert(zk_prog.end(), prog.begin(), prog.end());
            }
        }
    }
    // the mixed path's FP32 tables of the distortions whose programs replay
    // on polynomials (rp_zkprog.h)
    std::vector<int> zk32_off((size_t)d->n_distortions + 1, -1);
    std::vector<double> zk64;
    std::vector<zkp::Table> ztab((size_t)d->n_distortions);
    for (int q = 0; q < d->n_distortions; q++) {
        const rp_distortion &dq = d->distortions[q];
        if (zk_off[2 * q] < 0 || zk_off[2 * q + 1] < 0) continue;
        const short *pz = zk_prog.data() + zk_off[2 * q], *pg = zk_prog.data() + zk_off[2 * q + 1];
        const std::vector<short> vz(pz, pz + 3 + pz[0] * RP_ZKOP_WORDS + pz[2]);
        const std::vector<short> vg(pg, pg + 3 + pg[0] * RP_ZKOP_WORDS + pg[2]);
        if (!zkp::build(dq.n_coefs, dq.unit_radius, d->aux + dq.aux, vz, vg, ztab[(size_t)q])) continue;
        zk32_off[(size_t)q] = (int)zk64.size();
        zkp::pack(ztab[(size_t)q], zk64);
    }
    const std::vector<float> zk32(zk64.begin(), zk64.end());
    // FP32 copies of the ExtendedPolynomialFace coefficient matrices
    std::vector<int> ep32_off((size_t)d->n_face_records + 1, -1);
    std::vector<float> ep32;
    for (int r = 0; r < d->n_face_records; r++) {
        const rp_face &F = d->faces[r];
        if (F.type != RP_FACE_EXTPOLY) continue;
        ep32_off[(size_t)r] = (int)ep32.size();
        ep32.push_back((float)F.n_aux0);
        ep32.push_back((float)F.n_aux1);
        for (int k = 0; k < F.n_aux0 * F.n_aux1; k++) ep32.push_back((float)d->aux[F.aux + k]);
    }
    size_t o_zkoff = o_bnd + align256(sizeof(float) * 16 * (size_t)(d->n_faces + 1));
    size_t o_zkprog = o_zkoff + align256(sizeof(int) * zk_off.size());
    size_t o_fl = o_zkprog + align256(sizeof(short) * (zk_prog.size() + 1));
    size_t o_zk32off = o_fl + align256(sizeof(short) * (size_t)(d->n_faces + 1));
    size_t o_zk32 = o_zk32off + align256(sizeof(int) * zk32_off.size());
    size_t o_zk64 = o_zk32 + align256(sizeof(float) * (zk32.size() + 1));
    size_t o_ep32off = o_zk64 + align256(sizeof(double) * (zk64.size() + 1));
    size_t o_ep32 = o_ep32off + align256(sizeof(int) * ep32_off.size());
    size_t total = o_ep32 + align256(sizeof(float) * (ep32.size() + 1));
    // owning list of each traced face (kernels that read the tables from global memory)
    std::vector<short> face_list((size_t)d->n_faces + 1, (short)-1);
    for (int l = 0; l < d->n_lists; l++)
        for (int k = 0; k < d->lists[l].n_faces; k++) {
            const int f = d->lists[l].first_face + k;
            if (f >= 0 && f < d->n_faces) face_list[f] = (short)l;
        }
    int rc = ctx_alloc(ctx, &s->dev_block, total, &s->dev_bytes);
    if (rc) {
        delete s;
        return rc;
    }
    unsigned char *b = (unsigned char *)s->dev_block;
    cudaStream_t st = ctx->stream;
    cudaError_t e = cudaSuccess;
#define UP(off, ptr, bytes) \
    if (e == cudaSuccess && (bytes) > 0) e = cudaMemcpyAsync(b + (off), (ptr), (bytes), cudaMemcpyHostToDevice, st)
    UP(o_lists, d->lists, sizeof(rp_facelist) * d->n_lists);
    UP(o_faces, d->faces, sizeof(rp_face) * d->n_face_records);
    UP(o_mats, d->materials, sizeof(rp_material) * d->n_materials);
    UP(o_shapes, d->shape_ops, sizeof(rp_shape_op) * d->n_shape_ops);
    UP(o_dists, d->distortions, sizeof(rp_distortion) * d->n_distortions);
    UP(o_disp, d->dispersions, sizeof(rp_dispersion) * d->n_dispersions);
    UP(o_aux, d->aux, sizeof(double) * d->n_aux);
    UP(o_wl, wavelengths, sizeof(double) * (size_t)n_wl);
    // the searches' boxes: a face's box, or a conic face's two sheet boxes (rp_bounds.h)
    std::vector<float> bounds((size_t)d->n_faces * 16 + 16, 0.0f);
    for (int l = 0; l < d->n_lists; l++)
        for (int k = 0; k < d->lists[l].n_faces; k++) {
            int f = d->lists[l].first_face + k;
            face_world_boxes(d, d->lists[l], d->faces[f], &bounds[(size_t)f * 16]);
        }
    UP(o_bnd, bounds.data(), sizeof(float) * 16 * (size_t)d->n_faces);
    UP(o_zk32off, zk32_off.data(), sizeof(int) * zk32_off.size());
    UP(o_zk32, zk32.data(), sizeof(float) * zk32.size());
    UP(o_zk64, zk64.data(), sizeof(double) * zk64.size());
    UP(o_ep32off, ep32_off.data(), sizeof(int) * ep32_off.size());
    UP(o_ep32, ep32.data(), sizeof(float) * ep32.size());
    UP(o_zkoff, zk_off.data(), sizeof(int) * zk_off.size());
    UP(o_zkprog, zk_prog.data(), sizeof(short) * zk_prog.size());
    UP(o_fl, face_list.data(), sizeof(short) * (size_t)d->n_faces);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);  // the host vectors are pageable and about to go out of scope
#undef UP
    if (e == cudaSuccess) e = cudaMemsetAsync(b + o_cnt, 0, sizeof(unsigned) * (d->n_face_records + 1), st);
    DevScene &S = s->S;
    S.lists = (const rp_facelist *)(b + o_lists);
    S.faces = (const rp_face *)(b + o_faces);
    S.mats = (const rp_material *)(b + o_mats);
    S.shapes = (const rp_shape_op *)(b + o_shapes);
    S.dists = (const rp_distortion *)(b + o_dists);
    S.aux = (const double *)(b + o_aux);
    S.ntab = (const double2 *)(b + o_ntab);
    S.bounds = (const float *)(b + o_bnd);
    S.face_list = (const short *)(b + o_fl);
    S.zk_off = (const int *)(b + o_zkoff);
    S.zk_prog = (const short *)(b + o_zkprog);
    S.zk32_off = (const int *)(b + o_zk32off);
    S.zk32 = (const float *)(b + o_zk32);
    S.zk64 = (const double *)(b + o_zk64);
    S.ep32_off = (const int *)(b + o_ep32off);
    S.ep32 = (const float *)(b + o_ep32);
    S.n_wl = n_wl;
    S.wl = (const double *)(b + o_wl);
    S.n_lists = d->n_lists;
    S.n_faces = d->n_faces;
    S.n_recs = d->n_face_records;
    S.n_mats = d->n_materials;
    S.n_shapes = d->n_shape_ops;
    S.n_dists = d->n_distortions;
    s->face_counts = (unsigned *)(b + o_cnt);
    s->disp = (const rp_dispersion *)(b + o_disp);
    s->n_disp = d->n_dispersions;
    if (e == cudaSuccess)
        e = launch_dispersion_table((const rp_dispersion *)(b + o_disp), d->n_dispersions, (const double *)(b + o_aux),
                                    (const double *)(b + o_wl), n_wl, (double2 *)(b + o_ntab), st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        ctx_free(ctx, s->dev_block, s->dev_bytes);
        delete s;
        return cuda_fail(e, "rp_scene_create");
    }
    s->smem = generation_smem_bytes(d->n_lists, d->n_face_records, d->n_materials, d->n_faces);
    s->smem_tables = 1;
    if (s->smem > 160 * 1024) {  // tables too large to stage: read them from global memory
        s->smem_tables = 0;
        s->smem = generation_smem_bytes(0, 0, 0, d->n_faces);
    }
    if (s->smem > 200 * 1024) {
        ctx_free(ctx, s->dev_block, s->dev_bytes);
        delete s;
        snprintf(g_last_error, sizeof g_last_error, "scene has too many faces (%d)", d->n_faces);
        return RP_ERR_UNSUPPORTED;
    }
    *out = s;
    return RP_OK;
}

int rp_scene_bounds(const rp_scene_desc *d, float *out, int32_t n_faces) {
    if (!d || !out || n_faces != d->n_faces) return RP_ERR_INVALID;
    int v = validate_scene(d);
    if (v != RP_OK) return v;
    for (int l = 0; l < d->n_lists; l++)
        for (int k = 0; k < d->lists[l].n_faces; k++) {
            int f = d->lists[l].first_face + k;
            face_world_box(d, d->lists[l], d->faces[f], out + (size_t)f * 8);
        }
    return RP_OK;
}

int rp_scene_search_bounds(const rp_scene_desc *d, float *out, int32_t n_faces) {
    if (!d || !out || n_faces != d->n_faces) return RP_ERR_INVALID;
    int v = validate_scene(d);
    if (v != RP_OK) return v;
    for (int l = 0; l < d->n_lists; l++)
        for (int k = 0; k < d->lists[l].n_faces; k++) {
            int f = d->lists[l].first_face + k;
            face_world_boxes(d, d->lists[l], d->faces[f], out + (size_t)f * 16);
        }
    return RP_OK;
}

int rp_scene_destroy(rp_scene *s) {
    if (!s) return RP_ERR_INVALID;
    cudaSetDevice(s->ctx->device);
    cudaStreamSynchronize(s->ctx->stream);
    ctx_free(s->ctx, s->dev_block, s->dev_bytes);
    delete s;
    return RP_OK;
}

int rp_scene_face_counts(rp_scene *s, uint32_t *counts, int32_t n_faces, int reset) {
    if (!s || !counts || n_faces != s->n_faces) return RP_ERR_INVALID;
    CK(cudaSetDevice(s->ctx->device));
    CK(cudaMemcpyAsync(counts, s->face_counts, sizeof(unsigned) * n_faces, cudaMemcpyDeviceToHost, s->ctx->stream));
    if (reset) CK(cudaMemsetAsync(s->face_counts, 0, sizeof(unsigned) * n_faces, s->ctx->stream));
    CK(cudaStreamSynchronize(s->ctx->stream));
    return RP_OK;
}

// ---- rays ---------------------------------------------------------------------
static void soa_carve(rp_rays *r) {
    unsigned char *b = (unsigned char *)r->block;
    size_t c = r->cap, off = 0;
    auto take = [&](size_t elem) {
        unsigned char *p = b + off;
        off += align256(elem * c);
        return p;
    };
    RaySoA &s = r->soa;
    s.ox = (double *)take(8); s.oy = (double *)take(8); s.oz = (double *)take(8);
    s.dx = (double *)take(8); s.dy = (double *)take(8); s.dz = (double *)take(8);
    s.nx = (double *)take(8); s.ny = (double *)take(8); s.nz = (double *)take(8);
    s.ex = (double *)take(8); s.ey = (double *)take(8); s.ez = (double *)take(8);
    s.n = (double2 *)take(16); s.e1 = (double2 *)take(16); s.e2 = (double2 *)take(16);
    s.len = (double *)take(8); s.phase = (double *)take(8); s.opl = (double *)take(8);
    s.wl = (unsigned *)take(4); s.parent = (unsigned *)take(4); s.endf = (unsigned *)take(4);
    s.ident = (unsigned *)take(4); s.type = (unsigned *)take(4);
}

static size_t soa_bytes(uint64_t cap) {
    size_t c = cap ? cap : 1, t = 0;
    const size_t sizes[] = {8, 8, 8, 8, 8, 8, 8, 8, 8, 8, 8, 8, 16, 16, 16, 8, 8, 8, 4, 4, 4, 4, 4};
    for (size_t e : sizes) t += align256(e * c);
    return t;
}

int rp_rays_alloc(rp_ctx *ctx, uint64_t cap, rp_rays **out) {
    if (!ctx || !out) return RP_ERR_INVALID;
    *out = nullptr;
    CK(cudaSetDevice(ctx->device));
    rp_rays *r = new (std::nothrow) rp_rays();
    if (!r) return RP_ERR_NOMEM;
    r->ctx = ctx;
    r->cap = cap ? cap : 1;
    r->n = 0;
    int rc = ctx_alloc(ctx, &r->block, soa_bytes(r->cap), &r->bytes);
    if (rc) {
        delete r;
        return rc;
    }
    soa_carve(r);
    *out = r;
    return RP_OK;
}

int rp_rays_free(rp_rays *r) {
    if (!r) return RP_ERR_INVALID;
    cudaSetDevice(r->ctx->device);
    cudaStreamSynchronize(r->ctx->stream);
    ctx_free(r->ctx, r->block, r->bytes);
    delete r;
    return RP_OK;
}

int rp_rays_count(const rp_rays *r, uint64_t *n) {
    if (!r || !n) return RP_ERR_INVALID;
    *n = r->n;
    return RP_OK;
}

int rp_rays_capacity(const rp_rays *r, uint64_t *cap) {
    if (!r || !cap) return RP_ERR_INVALID;
    *cap = r->cap;
    return RP_OK;
}

// Host AoS <-> device SoA: when the host buffer is page-locked (and so mapped
// into the device's address space) the layout kernel reads or writes it
// directly across the host link; otherwise the records go through a device
// staging buffer and one cudaMemcpyAsync.
static int with_staging(rp_ctx *ctx, size_t bytes, void **p, size_t *got) { return ctx_alloc(ctx, p, bytes, got); }

// The device address of page-locked host memory at `p`, or null.
static void *mapped_host_ptr(const void *p) {
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return at.type == cudaMemoryTypeHost ? at.devicePointer : nullptr;
}

int rp_rays_upload_aos(rp_rays *r, const void *records, uint64_t n) {
    if (!r || (n && !records)) return RP_ERR_INVALID;
    if (n > r->cap) return RP_ERR_CAPACITY;
    rp_ctx *ctx = r->ctx;
    CK(cudaSetDevice(ctx->device));
    void *stage = nullptr;
    size_t bytes = (size_t)n * RP_RAY_BYTES, got = 0;
    if (void *mapped = n ? mapped_host_ptr(records) : nullptr) {
        cudaError_t e = launch_aos_to_soa(mapped, r->soa, n, ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) return cuda_fail(e, "rp_rays_upload_aos");
        r->n = n;
        return RP_OK;
    }
    if (n) {
        int rc = with_staging(ctx, bytes, &stage, &got);
        if (rc) return rc;
        cudaError_t e = cudaMemcpyAsync(stage, records, bytes, cudaMemcpyHostToDevice, ctx->stream);
        if (e == cudaSuccess) e = launch_aos_to_soa(stage, r->soa, n, ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        ctx_free(ctx, stage, got);
        if (e != cudaSuccess) return cuda_fail(e, "rp_rays_upload_aos");
    }
    r->n = n;
    return RP_OK;
}

int rp_rays_download_aos(const rp_rays *r, void *records, uint64_t n) {
    if (!r || (n && !records)) return RP_ERR_INVALID;
    if (n > r->n) return RP_ERR_CAPACITY;
    rp_ctx *ctx = r->ctx;
    CK(cudaSetDevice(ctx->device));
    if (!n) return RP_OK;
    if (void *mapped = mapped_host_ptr(records)) {
        cudaError_t e = launch_soa_to_aos(r->soa, mapped, n, ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) return cuda_fail(e, "rp_rays_download_aos");
        return RP_OK;
    }
    void *stage = nullptr;
    size_t bytes = (size_t)n * RP_RAY_BYTES, got = 0;
    int rc = with_staging(ctx, bytes, &stage, &got);
    if (rc) return rc;
    cudaError_t e = launch_soa_to_aos(r->soa, stage, n, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(records, stage, bytes, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    ctx_free(ctx, stage, got);
    if (e != cudaSuccess) return cuda_fail(e, "rp_rays_download_aos");
    return RP_OK;
}

int rp_rays_field(const rp_rays *r, const char *name, void **p) {
    if (!r || !name || !p) return RP_ERR_INVALID;
    const RaySoA &s = r->soa;
    struct {
        const char *n;
        void *p;
    } t[] = {{"origin_x", s.ox}, {"origin_y", s.oy}, {"origin_z", s.oz}, {"direction_x", s.dx},
             {"direction_y", s.dy}, {"direction_z", s.dz}, {"normal_x", s.nx}, {"normal_y", s.ny},
             {"normal_z", s.nz}, {"E_vector_x", s.ex}, {"E_vector_y", s.ey}, {"E_vector_z", s.ez},
             {"refractive_index", s.n}, {"E1_amp", s.e1}, {"E2_amp", s.e2}, {"length", s.len},
             {"phase", s.phase}, {"accumulated_path", s.opl}, {"wavelength_idx", s.wl},
             {"parent_idx", s.parent}, {"end_face_idx", s.endf}, {"ray_ident", s.ident},
             {"ray_type_id", s.type}};
    for (auto &e : t)
        if (!strcmp(e.n, name)) {
            *p = e.p;
            return RP_OK;
        }
    return RP_ERR_INVALID;
}

// ---- tracing ------------------------------------------------------------------
#define SCRATCH_HDR 64

// Per-generation scratch: [out_count | err | pad | stats[2] | tile counter |
// group counter | pad], then the per-unit child counts and offsets, then the
// mixed path's per-ray hit hand-over (rp_hit_bytes).
static size_t scratch_bytes_for(uint64_t n_sub) {
    return SCRATCH_HDR + align256(n_sub * sizeof(unsigned)) + align256(n_sub * sizeof(unsigned long long)) +
           rp_hit_bytes(n_sub * RP_SUB);
}

// Scratch for a generation of n_sub sub-tiles (rp_n_sub of its ray count).
static int ensure_scratch(rp_ctx *ctx, uint64_t n_sub) {
    size_t need = scratch_bytes_for(n_sub);
    if (need <= ctx->scratch_bytes) return RP_OK;
    if (ctx->scratch) {
        cudaStreamSynchronize(ctx->stream);
        cudaFree(ctx->scratch);
        ctx->scratch = nullptr;
        ctx->scratch_bytes = 0;
    }
    size_t bytes = need * 2;
    if (ctx->budget && ctx->in_use + bytes > ctx->budget) return RP_ERR_BUDGET;
    CK(cudaMalloc((void **)&ctx->scratch, bytes));
    ctx->scratch_bytes = bytes;
    return RP_OK;
}

// A child-slot arena: two ray slots per ray of the largest generation traced
// so far (kept by the context and reused).
static int ensure_arena_slot(rp_ctx *ctx, rp_rays **slot, uint64_t n_tiles) {
    uint64_t need = n_tiles * RP_TILE_SLOTS;
    if (*slot && (*slot)->cap >= need) return RP_OK;
    if (*slot) {
        rp_rays_free(*slot);
        *slot = nullptr;
    }
    return rp_rays_alloc(ctx, need + need / 4, slot);
}
static int ensure_arena(rp_ctx *ctx, uint64_t n_tiles) { return ensure_arena_slot(ctx, &ctx->arena, n_tiles); }

// Gather map k of trace_rays, for the children of a generation of n_in rays
// (at most two each).  The map it replaces was last read by a kernel the host
// has already waited for.
static int ensure_child_map(rp_ctx *ctx, int k, uint64_t n_in) {
    const uint64_t need = 2 * n_in;
    if (ctx->child_map[k] && ctx->child_map_cap[k] >= need) return RP_OK;
    if (ctx->child_map[k]) {
        ctx_free(ctx, ctx->child_map[k], ctx->child_map_bytes[k]);
        ctx->child_map[k] = nullptr;
        ctx->child_map_cap[k] = 0;
    }
    const uint64_t cap = need + need / 4;
    int rc = ctx_alloc(ctx, (void **)&ctx->child_map[k], cap * sizeof(unsigned), &ctx->child_map_bytes[k]);
    if (rc) return rc;
    ctx->child_map_cap[k] = cap;
    return RP_OK;
}

// Where trace_rays keeps a generation: its records in an arena read through a
// gather map (src, in_map), and the arena and map its children go to.
struct GenLinks {
    rp_rays *src = nullptr;           // null: the generation's records are in place
    const unsigned *in_map = nullptr;
    rp_rays **arena = nullptr;        // null: the context's arena
    unsigned *map_out = nullptr;      // null: the children are copied to their place afterwards
    uint64_t map_cap = 0;
};

// The mixed path's child-slot unit and per-ray hand-over, carved from a
// generation scratch of n_sub sub-tiles laid out as scratch_bytes_for; the
// plain path keeps the sub-tile unit.
void rp__set_mixed_handover(GenArgs &a, uint32_t flags, unsigned char *sc, uint64_t n_sub) {
    a.group_next = (unsigned *)(sc + 44);
    if (!(flags & RP_TRACE_MIXED)) {
        a.unit_rays = RP_SUB;
        return;
    }
    a.unit_rays = RP_GROUP;
    unsigned char *h = sc + SCRATCH_HDR + align256(n_sub * sizeof(unsigned)) + align256(n_sub * sizeof(unsigned long long));
    a.hit_t = (float2 *)h;
    a.hit_face = (int *)(h + align256(n_sub * RP_SUB * 8));
}

// Launches the generation kernel (and, when children are kept, the tile scan)
// and queues the read-back of count / error / statistics into h_pinned.
static int launch_gen(rp_ctx *ctx, rp_scene *s, rp_rays *in, float max_length, uint32_t flags, double e2, int emit,
                      int one_list, int one_face, GenArgs &a, const GenLinks &lk = GenLinks()) {
    uint64_t n_in = in->n;
    uint64_t n_tiles = (n_in + RP_BLOCK - 1) / RP_BLOCK;
    const uint64_t n_sub = rp_n_sub(n_in);
    rp_rays **arena = lk.arena ? lk.arena : &ctx->arena;
    int rc = ensure_scratch(ctx, n_sub);
    if (rc) return rc;
    if (emit) {
        rc = ensure_arena_slot(ctx, arena, n_tiles);
        if (rc) return rc;
    }
    unsigned char *sc = ctx->scratch;
    {
        cudaError_t ez = launch_zero_words((unsigned long long *)sc, SCRATCH_HDR / 8, ctx->stream);
        if (ez != cudaSuccess) return cuda_fail(ez, "counter clear");
    }
    memset(&a, 0, sizeof a);
    a.in = lk.src ? lk.src->soa : in->soa;
    a.in_map = lk.src ? lk.in_map : nullptr;
    a.wb = in->soa;
    a.out = in->soa;
    a.n_in = n_in;
    a.out_cap = 0;
    a.max_len = (double)max_length;
    a.e2_term = e2;
    a.emit = emit;
    a.one_list = one_list;
    a.one_face = one_face;
    a.S = s->S;
    a.smem_tables = s->smem_tables;
    a.mixed_fallback = s->mixed_fallback;
    a.out_count = (unsigned long long *)(sc + 0);
    a.err = (unsigned *)(sc + 8);
    a.stats = (unsigned long long *)(sc + 24);
    a.tile_next = (unsigned *)(sc + 40);
    a.tile_counts = (unsigned *)(sc + SCRATCH_HDR);
    a.tile_offsets = (unsigned long long *)(sc + SCRATCH_HDR + align256(n_sub * sizeof(unsigned)));
    a.scratch = emit ? (*arena)->soa : in->soa;
    a.face_counts = s->face_counts;
    rp__set_mixed_handover(a, flags, sc, n_sub);
    if (ctx->gen_ev.empty()) {
        ctx->gen_ev.resize(3);
        for (auto &ev : ctx->gen_ev) CK(cudaEventCreate(&ev));
    }
    CK(cudaEventRecord(ctx->gen_ev[0], ctx->stream));
    cudaError_t e = (flags & RP_TRACE_MIXED) ? launch_generation_mixed(a, s->smem, ctx->stream, ctx->gen_ev[2])
                                             : launch_generation_plain(a, s->smem, ctx->stream);
    if (e != cudaSuccess) return cuda_fail(e, "generation kernel launch");
    CK(cudaEventRecord(ctx->gen_ev[1], ctx->stream));
    if (emit) {
        e = launch_tile_scan(a, ctx->stream);
        if (e != cudaSuccess) return cuda_fail(e, "tile scan launch");
        if (lk.map_out) {
            e = launch_child_map(a, lk.map_out, lk.map_cap, ctx->stream);
            if (e != cudaSuccess) return cuda_fail(e, "child map launch");
        }
    }
    e = launch_copy_words((const unsigned long long *)sc, ctx->d_pinned, 5, ctx->stream);
    if (e != cudaSuccess) return cuda_fail(e, "counter read-back");
    return RP_OK;
}

// Waits for the generation, turns its error bits into a status and returns
// the number of children in *count.
static int finish_gen(rp_ctx *ctx, int emit, uint32_t flags, rp_stats *st, uint64_t n_in, uint64_t *count) {
    CK(cudaStreamSynchronize(ctx->stream));
    unsigned long long cnt = ctx->h_pinned[0];
    unsigned err = (unsigned)(ctx->h_pinned[1] & 0xffffffffu);
    unsigned long long hits = ctx->h_pinned[3], term = ctx->h_pinned[4];
    if (st) {
        const bool mixed = (flags & RP_TRACE_MIXED) != 0;
        float ms = 0, sms = 0;
        cudaEventElapsedTime(&ms, ctx->gen_ev[0], ctx->gen_ev[1]);
        if (mixed && n_in) cudaEventElapsedTime(&sms, ctx->gen_ev[0], ctx->gen_ev[2]);
        st->rays_in += n_in;
        st->hits += hits;
        st->terminated += term;
        st->kernel_ms += ms;
        st->search_ms += sms;
        // counter clear, generation kernel(s), [tile scan, map or placement,] read-back
        st->launches += (emit ? 5 : 3) + (mixed && emit && n_in ? 1 : 0);
        st->generations += 1;
    }
    *count = emit ? cnt : 0;

    if (err & ERR_WAVELENGTH) {
        snprintf(g_last_error, sizeof g_last_error, "a ray's wavelength_idx is outside the wavelength table");
        return RP_ERR_INVALID;
    }
    if (err & (ERR_ZK_STACK | ERR_SHAPE_STACK)) {
        snprintf(g_last_error, sizeof g_last_error, "device evaluation limit hit (err=0x%x)", err);
        return RP_ERR_INVALID;
    }
    if (err & ERR_OVERFLOW) {
        snprintf(g_last_error, sizeof g_last_error, "child slots overflowed (err=0x%x)", err);
        return RP_ERR_CAPACITY;
    }
    return RP_OK;
}

// Moves the generation's children into `out` (capacity checked by the caller).
static int place_gen(rp_ctx *ctx, GenArgs &a, rp_rays *out, uint64_t count, rp_stats *st) {
    a.out = out->soa;
    a.out_cap = out->cap;
    cudaError_t e = launch_place_children(a, ctx->stream);
    if (e != cudaSuccess) return cuda_fail(e, "child placement launch");
    out->n = count;
    if (st) st->rays_out += count;
    return RP_OK;
}

static int one_generation(rp_ctx *ctx, rp_scene *s, rp_rays *in, rp_rays *out, float max_length, uint32_t flags,
                          double e2, int one_list, int one_face, rp_stats *st) {
    GenArgs a;
    uint64_t count = 0;
    int rc = launch_gen(ctx, s, in, max_length, flags, e2, 1, one_list, one_face, a);
    if (rc == RP_OK) rc = finish_gen(ctx, 1, flags, st, in->n, &count);
    if (rc) return rc;
    if (count > out->cap) {
        snprintf(g_last_error, sizeof g_last_error, "%llu children do not fit the output buffer",
                 (unsigned long long)count);
        return RP_ERR_CAPACITY;
    }
    rc = place_gen(ctx, a, out, count, st);
    if (rc) return rc;
    // the placement kernel reports an overflow in the same error word
    CK(cudaMemcpyAsync(ctx->h_pinned, a.err, sizeof(unsigned), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    if ((unsigned)(ctx->h_pinned[0] & 0xffffffffu) & ERR_OVERFLOW) {
        out->n = 0;
        if (st) st->rays_out -= count;
        snprintf(g_last_error, sizeof g_last_error, "child placement overflowed its slots or the output buffer");
        return RP_ERR_CAPACITY;
    }
    return RP_OK;
}

int rp_trace_segment(rp_ctx *ctx, rp_scene *s, rp_rays *in, rp_rays *out, float max_length, uint32_t flags,
                     double e2, rp_stats *st) {
    if (!ctx || !s || !in || !out || in == out || s->ctx != ctx) return RP_ERR_INVALID;
    CK(cudaSetDevice(ctx->device));
    out->n = 0;
    if (in->n == 0) return RP_OK;
    CK(cudaEventRecord(ctx->ev0, ctx->stream));
    int rc = one_generation(ctx, s, in, out, max_length, flags, e2, -1, -1, st);
    CK(cudaEventRecord(ctx->ev1, ctx->stream));
    CK(cudaEventSynchronize(ctx->ev1));
    if (st) {
        float ms = 0;
        cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
        st->device_ms += ms;
    }
    return rc;
}

int rp_trace_one_face_segment(rp_ctx *ctx, rp_scene *s, rp_rays *in, rp_rays *out, int32_t list_idx,
                              int32_t face_idx, float max_length, uint32_t flags, double e2, rp_stats *st) {
    if (!ctx || !s || !in || !out || in == out || s->ctx != ctx) return RP_ERR_INVALID;
    if (list_idx < 0 || list_idx >= s->S.n_lists) return RP_ERR_INVALID;
    if (face_idx < 0 || face_idx >= s->host_lists[list_idx].n_faces) return RP_ERR_INVALID;
    CK(cudaSetDevice(ctx->device));
    out->n = 0;
    if (in->n == 0) return RP_OK;
    return one_generation(ctx, s, in, out, max_length, flags, e2, list_idx, face_idx, st);
}

// Called once generation g's records are final (its kernel has run and the
// main stream is synchronised); a non-zero return ends the trace.
typedef int (*gen_done_fn)(void *user, int g, rp_rays *rays);

static int trace_rays_impl(rp_ctx *ctx, rp_scene *s, rp_rays **gens, int32_t max_gens, int32_t recursion_limit,
                           float max_length, uint32_t flags, double e2, int32_t *n_gens, rp_stats *st,
                           gen_done_fn done, void *user) {
    CK(cudaSetDevice(ctx->device));
    *n_gens = 0;
    for (int g = 1; g < max_gens; g++) gens[g] = nullptr;
    int count = 0;
    rp_rays *rays = gens[0];
    CK(cudaEventRecord(ctx->ev0, ctx->stream));
    int rc = RP_OK;
    // Generation g > 0 is never copied out of its parents' child arena on its
    // own: the kernel that traces it reads each record through the gather map
    // and writes it, with its length and end face, to gens[g].  The two arenas
    // and maps alternate, one read while the other is written.
    GenLinks lk;
    int par = 0;
    // core/tracer.py:40-45: while rays.n_rays > 0 and count < recursion_limit
    while (rays->n > 0 && count < recursion_limit) {
        int last = (count + 1 == recursion_limit);  // children of this generation are discarded
        if (!last && count + 1 >= max_gens) {
            rc = RP_ERR_CAPACITY;
            break;
        }
        lk.arena = par ? &ctx->arena2 : &ctx->arena;
        lk.map_out = nullptr;
        lk.map_cap = 0;
        if (!last) {
            rc = ensure_child_map(ctx, par, rays->n);
            if (rc) break;
            lk.map_out = ctx->child_map[par];
            lk.map_cap = ctx->child_map_cap[par];
        }
        GenArgs a;
        uint64_t n_child = 0;
        rc = launch_gen(ctx, s, rays, max_length, flags, e2, last ? 0 : 1, -1, -1, a, lk);
        if (rc == RP_OK) rc = finish_gen(ctx, last ? 0 : 1, flags, st, rays->n, &n_child);
        if (rc) break;
        count++;
        if (done && (rc = done(user, count - 1, rays)) != RP_OK) break;
        if (last || n_child == 0) break;
        rp_rays *next = nullptr;
        rc = rp_rays_alloc(ctx, n_child, &next);  // exact size: the count is known
        if (rc) break;
        next->n = n_child;  // its records are written by the kernel that traces it
        if (st) st->rays_out += n_child;
        gens[count] = next;
        rays = next;
        lk.src = *lk.arena;
        lk.in_map = ctx->child_map[par];
        par ^= 1;
    }
    CK(cudaEventRecord(ctx->ev1, ctx->stream));
    CK(cudaEventSynchronize(ctx->ev1));
    if (st) {
        float ms = 0;
        cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
        st->device_ms += ms;
    }
    *n_gens = count;
    return rc;
}

int rp_trace_rays(rp_ctx *ctx, rp_scene *s, rp_rays **gens, int32_t max_gens, int32_t recursion_limit,
                  float max_length, uint32_t flags, double e2, int32_t *n_gens, rp_stats *st) {
    if (!ctx || !s || !gens || !gens[0] || max_gens < 1 || !n_gens || s->ctx != ctx) return RP_ERR_INVALID;
    return trace_rays_impl(ctx, s, gens, max_gens, recursion_limit, max_length, flags, e2, n_gens, st, nullptr,
                           nullptr);
}

// Download of each finished generation into a page-locked output buffer while
// the next generation is traced: the layout kernel packs the generation into
// a device staging buffer on the main stream (a few hundred microseconds at
// device bandwidth), and the copy stream moves it to the host with the copy
// engine, which takes no SMs from the tracing kernels.
struct OverlapDownload {
    rp_ctx *ctx;
    unsigned char *out;  // the caller's page-locked records
    uint64_t cap, off;
    uint64_t *gen_offsets;
    rp_stats *st;
    std::vector<std::pair<void *, size_t>> staging;  // freed once the copy stream is done
    std::vector<cudaEvent_t> events;
};

static int overlap_download(void *user, int g, rp_rays *rays) {
    OverlapDownload *d = static_cast<OverlapDownload *>(user);
    rp_ctx *ctx = d->ctx;
    const uint64_t n = rays->n;
    if (d->off + n > d->cap) {
        snprintf(g_last_error, sizeof g_last_error, "the output buffer holds %llu records",
                 (unsigned long long)d->cap);
        return RP_ERR_CAPACITY;
    }
    d->gen_offsets[g] = d->off;
    if (n) {
        void *stage = nullptr;
        size_t got = 0;
        int rc = with_staging(ctx, (size_t)n * RP_RAY_BYTES, &stage, &got);
        if (rc) return rc;
        d->staging.emplace_back(stage, got);
        cudaEvent_t ev;
        CK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
        d->events.push_back(ev);
        cudaError_t e = launch_soa_to_aos(rays->soa, stage, n, ctx->stream);
        if (e == cudaSuccess) e = cudaEventRecord(ev, ctx->stream);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(ctx->copy_stream, ev, 0);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(d->out + d->off * RP_RAY_BYTES, stage, (size_t)n * RP_RAY_BYTES,
                                cudaMemcpyDeviceToHost, ctx->copy_stream);
        if (e != cudaSuccess) return cuda_fail(e, "generation download");
        if (d->st) d->st->launches += 1;  // layout kernel of the download
    }
    d->off += n;
    d->gen_offsets[g + 1] = d->off;
    return RP_OK;
}

int rp_trace_rays_host(rp_ctx *ctx, rp_scene *s, const void *in_records, uint64_t n, int32_t recursion_limit,
                       float max_length, uint32_t flags, double e2, void *out_records, uint64_t out_cap,
                       uint64_t *gen_offsets, int32_t max_gens, int32_t *n_gens, rp_stats *st) {
    if (!ctx || !s || (n && !in_records) || !gen_offsets || !n_gens || max_gens < 1) return RP_ERR_INVALID;
    std::vector<rp_rays *> gens(max_gens + 1, nullptr);
    int rc = rp_rays_alloc(ctx, n, &gens[0]);
    if (rc) return rc;
    rc = rp_rays_upload_aos(gens[0], in_records, n);
    if (rc == RP_OK && st && n) st->launches += 1;  // layout kernel of the upload
    const bool pinned_out = out_cap && mapped_host_ptr(out_records);
    if (rc == RP_OK && pinned_out) {
        // page-locked output: each generation is downloaded as soon as it is
        // final, overlapping the following generations
        if (!ctx->copy_stream) {
            cudaError_t e = cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking);
            if (e != cudaSuccess) rc = cuda_fail(e, "copy stream");
        }
        if (rc == RP_OK) {
            OverlapDownload d{ctx, (unsigned char *)out_records, out_cap, 0, gen_offsets, st, {}, {}};
            gen_offsets[0] = 0;
            rc = trace_rays_impl(ctx, s, gens.data(), max_gens, recursion_limit, max_length, flags, e2, n_gens, st,
                                 overlap_download, &d);
            cudaError_t e = cudaStreamSynchronize(ctx->stream);
            if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->copy_stream);
            if (rc == RP_OK && e != cudaSuccess) rc = cuda_fail(e, "generation download");
            for (auto &b : d.staging) ctx_free(ctx, b.first, b.second);
            for (auto ev : d.events) cudaEventDestroy(ev);
        }
    } else if (rc == RP_OK) {
        rc = rp_trace_rays(ctx, s, gens.data(), max_gens, recursion_limit, max_length, flags, e2, n_gens, st);
        if (rc == RP_OK) {
            uint64_t off = 0;
            gen_offsets[0] = 0;
            for (int g = 0; g < *n_gens; g++) {
                uint64_t c = gens[g]->n;
                if (off + c > out_cap) {
                    rc = RP_ERR_CAPACITY;
                    break;
                }
                rc = rp_rays_download_aos(gens[g], (unsigned char *)out_records + off * RP_RAY_BYTES, c);
                if (rc) break;
                if (st && c) st->launches += 1;  // layout kernel of the download
                off += c;
                gen_offsets[g + 1] = off;
            }
        }
    }
    for (auto *g : gens)
        if (g) rp_rays_free(g);
    return rc;
}

// ---- Gausslets ------------------------------------------------------------------

int rp_gausslets_alloc(rp_ctx *ctx, uint64_t cap, rp_gausslets **out) {
    if (!ctx || !out) return RP_ERR_INVALID;
    *out = nullptr;
    rp_gausslets *g = new (std::nothrow) rp_gausslets();
    if (!g) return RP_ERR_NOMEM;
    g->ctx = ctx;
    g->cap = cap ? cap : 1;
    int rc = rp_rays_alloc(ctx, g->cap, &g->base);
    if (rc == RP_OK) rc = ctx_alloc(ctx, (void **)&g->para, (size_t)RP_PARA_ARRAYS * g->cap * sizeof(double),
                                    &g->para_bytes);
    if (rc) {
        if (g->base) rp_rays_free(g->base);
        delete g;
        return rc;
    }
    *out = g;
    return RP_OK;
}

int rp_gausslets_free(rp_gausslets *g) {
    if (!g) return RP_ERR_INVALID;
    rp_rays_free(g->base);  // synchronises the stream
    ctx_free(g->ctx, g->para, g->para_bytes);
    delete g;
    return RP_OK;
}

int rp_gausslets_count(const rp_gausslets *g, uint64_t *n) {
    if (!g || !n) return RP_ERR_INVALID;
    *n = g->base->n;
    return RP_OK;
}

int rp_gausslets_upload(rp_gausslets *g, const void *records, uint64_t n) {
    if (!g || (n && !records)) return RP_ERR_INVALID;
    if (n > g->cap) return RP_ERR_CAPACITY;
    rp_ctx *ctx = g->ctx;
    CK(cudaSetDevice(ctx->device));
    if (n) {
        void *stage = nullptr;
        size_t bytes = (size_t)n * RP_GAUSSLET_BYTES, got = 0;
        int rc = with_staging(ctx, bytes, &stage, &got);
        if (rc) return rc;
        cudaError_t e = cudaMemcpyAsync(stage, records, bytes, cudaMemcpyHostToDevice, ctx->stream);
        if (e == cudaSuccess) e = launch_gausslet_aos_to_soa(stage, g->base->soa, g->para, g->cap, n, ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        ctx_free(ctx, stage, got);
        if (e != cudaSuccess) return cuda_fail(e, "rp_gausslets_upload");
    }
    g->base->n = n;
    return RP_OK;
}

int rp_gausslets_download(const rp_gausslets *g, void *records, uint64_t n) {
    if (!g || (n && !records)) return RP_ERR_INVALID;
    if (n > g->base->n) return RP_ERR_CAPACITY;
    rp_ctx *ctx = g->ctx;
    CK(cudaSetDevice(ctx->device));
    if (!n) return RP_OK;
    void *stage = nullptr;
    size_t bytes = (size_t)n * RP_GAUSSLET_BYTES, got = 0;
    int rc = with_staging(ctx, bytes, &stage, &got);
    if (rc) return rc;
    cudaError_t e = launch_gausslet_soa_to_aos(g->base->soa, g->para, g->cap, stage, n, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(records, stage, bytes, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    ctx_free(ctx, stage, got);
    if (e != cudaSuccess) return cuda_fail(e, "rp_gausslets_download");
    return RP_OK;
}

int rp_gausslets_config_parabasal(rp_gausslets *g, const double *wavelengths, int64_t n_wl, double radius,
                                  double working_dist) {
    if (!g || n_wl < 0 || (n_wl && !wavelengths)) return RP_ERR_INVALID;
    rp_ctx *ctx = g->ctx;
    CK(cudaSetDevice(ctx->device));
    const uint64_t n = g->base->n;
    if (n == 0) return RP_OK;
    ParabasalConfig P;
    for (int k = 0; k < 3; k++) {
        // the angle as the reference forms it, (j * 2) * pi / 6 for j = 2k; the
        // C library's cos / sin at run time (not a compile-time folding)
        volatile double angle = ((double)(4 * k) * 3.141592653589793) / 6.0;
        const double a = angle;
        P.c[k] = cos(a);
        P.s[k] = sin(a);
        P.rc[k] = radius * P.c[k];
        P.rs[k] = radius * P.s[k];
    }
    P.kt = (3.141592653589793 * radius) * 1000.0;
    P.wd = working_dist;
    const size_t wl_b = ((size_t)(n_wl ? n_wl : 1) * sizeof(double) + 255) & ~(size_t)255;
    unsigned char *blk = nullptr;
    size_t got = 0;
    int rc = ctx_alloc(ctx, (void **)&blk, wl_b + 256, &got);
    if (rc) return rc;
    double *dwl = (double *)blk;
    unsigned *err = (unsigned *)(blk + wl_b);
    cudaError_t e = cudaMemsetAsync(err, 0, sizeof(unsigned), ctx->stream);
    if (e == cudaSuccess && n_wl)
        e = cudaMemcpyAsync(dwl, wavelengths, (size_t)n_wl * sizeof(double), cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = launch_parabasal_config(g->base->soa, g->para, g->cap, n, dwl, n_wl, P, err, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(ctx->h_pinned, err, sizeof(unsigned), cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    const unsigned ferr = (unsigned)(ctx->h_pinned[0] & 0xffffffffu);
    ctx_free(ctx, blk, got);
    if (e != cudaSuccess) return cuda_fail(e, "rp_gausslets_config_parabasal");
    if (ferr) {
        snprintf(g_last_error, sizeof g_last_error, "a gausslet's wavelength_idx is outside the wavelength list");
        return RP_ERR_INVALID;
    }
    return RP_OK;
}

int rp_gausslets_total_power(const rp_gausslets *g, double *power) {
    if (!g || !power) return RP_ERR_INVALID;
    *power = 0.0;
    rp_ctx *ctx = g->ctx;
    CK(cudaSetDevice(ctx->device));
    const uint64_t n = g->base->n;
    if (n == 0) return RP_OK;
    const uint64_t nb = (n + RP_POWER_BLOCK - 1) / RP_POWER_BLOCK;
    double *part = nullptr;
    size_t got = 0;
    int rc = ctx_alloc(ctx, (void **)&part, nb * sizeof(double), &got);
    if (rc) return rc;
    std::vector<double> h(nb);
    cudaError_t e = launch_power_partials(g->base->soa, n, part, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(h.data(), part, nb * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    ctx_free(ctx, part, got);
    if (e != cudaSuccess) return cuda_fail(e, "rp_gausslets_total_power");
    double s = 0.0;
    for (uint64_t b = 0; b < nb; b++) s += h[b];
    *power = s;
    return RP_OK;
}

int rp_trace_gausslet_segment(rp_ctx *ctx, rp_scene *s, rp_gausslets *in, rp_gausslets *out, int32_t list_idx,
                              int32_t face_idx, double max_length, int32_t *captured, rp_stats *st) {
    if (!ctx || !s || !in || !out || in == out || s->ctx != ctx || in->ctx != ctx || out->ctx != ctx)
        return RP_ERR_INVALID;
    if (list_idx >= 0) {
        if (list_idx >= s->S.n_lists) return RP_ERR_INVALID;
        if (face_idx < 0 || face_idx >= s->host_lists[list_idx].n_faces) return RP_ERR_INVALID;
    }
    CK(cudaSetDevice(ctx->device));
    out->base->n = 0;
    const uint64_t n_in = in->base->n;
    if (captured)
        for (uint64_t i = 0; i < n_in; i++) captured[i] = 0;
    if (n_in == 0) return RP_OK;
    const uint64_t n_tiles = (n_in + RP_BLOCK - 1) / RP_BLOCK;
    const uint64_t n_sub = rp_n_sub(n_in);
    int rc = ensure_scratch(ctx, n_sub);
    if (rc == RP_OK) rc = ensure_arena(ctx, n_tiles);
    if (rc) return rc;
    const uint64_t slots = n_tiles * RP_TILE_SLOTS;
    double *pscratch = nullptr;
    int *dcap = nullptr;
    size_t pbytes = 0, cbytes = 0;
    rc = ctx_alloc(ctx, (void **)&pscratch, (size_t)RP_PARA_ARRAYS * slots * sizeof(double), &pbytes);
    if (rc) return rc;
    if (captured) {
        rc = ctx_alloc(ctx, (void **)&dcap, n_in * sizeof(int), &cbytes);
        if (rc) {
            ctx_free(ctx, pscratch, pbytes);
            return rc;
        }
    }
    auto release = [&]() {
        cudaStreamSynchronize(ctx->stream);
        ctx_free(ctx, pscratch, pbytes);
        if (dcap) ctx_free(ctx, dcap, cbytes);
    };
    unsigned char *sc = ctx->scratch;
    GaussArgs ga;
    memset(&ga, 0, sizeof ga);
    GenArgs &a = ga.g;
    a.in = in->base->soa;
    a.out = out->base->soa;
    a.n_in = n_in;
    a.out_cap = out->cap;
    a.max_len = max_length;
    a.emit = 1;
    a.one_list = list_idx >= 0 ? list_idx : -1;
    a.one_face = list_idx >= 0 ? face_idx : -1;
    a.S = s->S;
    a.smem_tables = s->smem_tables;
    a.out_count = (unsigned long long *)(sc + 0);
    a.err = (unsigned *)(sc + 8);
    a.stats = (unsigned long long *)(sc + 24);
    a.tile_next = (unsigned *)(sc + 40);
    a.tile_counts = (unsigned *)(sc + SCRATCH_HDR);
    a.tile_offsets = (unsigned long long *)(sc + SCRATCH_HDR + align256(n_sub * sizeof(unsigned)));
    a.scratch = ctx->arena->soa;
    a.face_counts = s->face_counts;
    ga.pin = in->para;
    ga.pin_cap = in->cap;
    ga.pscratch = pscratch;
    ga.pscratch_cap = slots;
    ga.pout = out->para;
    ga.pout_cap = out->cap;
    ga.captured = dcap;
    cudaError_t e = cudaMemsetAsync(sc, 0, SCRATCH_HDR, ctx->stream);
    if (e == cudaSuccess && dcap) e = cudaMemsetAsync(dcap, 0, n_in * sizeof(int), ctx->stream);
    if (e == cudaSuccess) e = cudaEventRecord(ctx->ev0, ctx->stream);
    if (e == cudaSuccess) e = launch_gausslet_generation(ga, s->smem, ctx->stream);
    if (e == cudaSuccess) e = cudaEventRecord(ctx->ev1, ctx->stream);
    if (e == cudaSuccess) e = launch_tile_scan(a, ctx->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(ctx->h_pinned, sc, 5 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) {
        release();
        return cuda_fail(e, "gausslet generation");
    }
    const unsigned long long count = ctx->h_pinned[0];
    const unsigned err = (unsigned)(ctx->h_pinned[1] & 0xffffffffu);
    if (st) {
        float ms = 0;
        cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
        st->rays_in += n_in;
        st->hits += ctx->h_pinned[3];
        st->kernel_ms += ms;
        st->device_ms += ms;
        st->launches += 3;  // generation, tile scan, placement
        st->generations += 1;
    }
    if (err & ERR_WAVELENGTH) {
        release();
        snprintf(g_last_error, sizeof g_last_error, "a ray's wavelength_idx is outside the wavelength table");
        return RP_ERR_INVALID;
    }
    if (err & (ERR_ZK_STACK | ERR_SHAPE_STACK)) {
        release();
        snprintf(g_last_error, sizeof g_last_error, "device evaluation limit hit (err=0x%x)", err);
        return RP_ERR_INVALID;
    }
    if (count > out->cap) {
        release();
        snprintf(g_last_error, sizeof g_last_error, "%llu child gausslets do not fit the output buffer", count);
        return RP_ERR_CAPACITY;
    }
    e = launch_gausslet_place(ga, n_sub, ctx->stream);
    if (e == cudaSuccess && dcap)
        e = cudaMemcpyAsync(captured, dcap, n_in * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    release();
    if (e != cudaSuccess) return cuda_fail(e, "gausslet placement");
    out->base->n = count;
    if (st) st->rays_out += count;
    return RP_OK;
}

// ---- post-trace capture ---------------------------------------------------------
// Shared by rp_select_intersections and rp_select_gausslet_intersections: the
// capture kernel writes each hit ray (and its parabasal rays) to its tile's
// slots, then the tile scan and the placement kernel compact them.
static int capture_common(rp_ctx *ctx, rp_scene *s, int32_t list_idx, rp_rays *in_base, const double *pin,
                          uint64_t pin_cap, rp_rays *out_base, double *pout, uint64_t pout_cap, uint32_t wl_offset,
                          uint64_t *n_out) {
    if (list_idx < 0 || list_idx >= s->S.n_lists) return RP_ERR_INVALID;
    CK(cudaSetDevice(ctx->device));
    *n_out = 0;
    out_base->n = 0;
    const uint64_t n_in = in_base->n;
    if (n_in == 0) return RP_OK;
    const uint64_t n_tiles = (n_in + RP_BLOCK - 1) / RP_BLOCK;
    const uint64_t n_sub = rp_n_sub(n_in);
    int rc = ensure_scratch(ctx, n_sub);
    if (rc == RP_OK) rc = ensure_arena(ctx, n_tiles);
    if (rc) return rc;
    const int with_para = pin != nullptr;
    const uint64_t slots = n_tiles * RP_TILE_SLOTS;
    double *pscratch = nullptr;
    size_t pbytes = 0;
    if (with_para) {
        rc = ctx_alloc(ctx, (void **)&pscratch, (size_t)RP_PARA_ARRAYS * slots * sizeof(double), &pbytes);
        if (rc) return rc;
    }
    unsigned char *sc = ctx->scratch;
    GaussArgs ga;
    memset(&ga, 0, sizeof ga);
    GenArgs &a = ga.g;
    a.in = in_base->soa;
    a.out = out_base->soa;
    a.n_in = n_in;
    a.out_cap = out_base->cap;
    a.one_list = list_idx;
    a.one_face = -1;
    a.S = s->S;
    a.smem_tables = s->smem_tables;
    a.out_count = (unsigned long long *)(sc + 0);
    a.err = (unsigned *)(sc + 8);
    a.stats = (unsigned long long *)(sc + 24);
    a.tile_next = (unsigned *)(sc + 40);
    a.tile_counts = (unsigned *)(sc + SCRATCH_HDR);
    a.tile_offsets = (unsigned long long *)(sc + SCRATCH_HDR + align256(n_sub * sizeof(unsigned)));
    a.scratch = ctx->arena->soa;
    a.face_counts = s->face_counts;
    ga.pin = const_cast<double *>(pin);
    ga.pin_cap = pin_cap;
    ga.pscratch = pscratch;
    ga.pscratch_cap = slots;
    ga.pout = pout;
    ga.pout_cap = pout_cap;
    cudaError_t e = cudaMemsetAsync(sc, 0, SCRATCH_HDR, ctx->stream);
    if (e == cudaSuccess) e = launch_capture(ga, wl_offset, with_para, s->smem, ctx->stream);
    if (e == cudaSuccess) e = launch_tile_scan(a, ctx->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(ctx->h_pinned, sc, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) {
        if (pscratch) ctx_free(ctx, pscratch, pbytes);
        return cuda_fail(e, "capture kernel");
    }
    const unsigned long long count = ctx->h_pinned[0];
    const unsigned err = (unsigned)(ctx->h_pinned[1] & 0xffffffffu);
    if (err & (ERR_ZK_STACK | ERR_SHAPE_STACK)) {
        if (pscratch) ctx_free(ctx, pscratch, pbytes);
        snprintf(g_last_error, sizeof g_last_error, "device evaluation limit hit (err=0x%x)", err);
        return RP_ERR_INVALID;
    }
    if (count > out_base->cap || (with_para && count > pout_cap)) {
        if (pscratch) ctx_free(ctx, pscratch, pbytes);
        snprintf(g_last_error, sizeof g_last_error, "%llu captured rays do not fit the output buffer", count);
        return RP_ERR_CAPACITY;
    }
    e = with_para ? launch_gausslet_place(ga, n_sub, ctx->stream) : launch_place_children(a, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (pscratch) ctx_free(ctx, pscratch, pbytes);
    if (e != cudaSuccess) return cuda_fail(e, "capture placement");
    out_base->n = count;
    *n_out = count;
    return RP_OK;
}

int rp_select_intersections(rp_ctx *ctx, rp_scene *s, int32_t list_idx, rp_rays *in, rp_rays *out,
                            uint32_t wl_offset) {
    if (!ctx || !s || !in || !out || in == out || s->ctx != ctx) return RP_ERR_INVALID;
    uint64_t n = 0;
    return capture_common(ctx, s, list_idx, in, nullptr, 0, out, nullptr, 0, wl_offset, &n);
}

int rp_select_gausslet_intersections(rp_ctx *ctx, rp_scene *s, int32_t list_idx, rp_gausslets *in,
                                     rp_gausslets *out, uint32_t wl_offset) {
    if (!ctx || !s || !in || !out || in == out || s->ctx != ctx) return RP_ERR_INVALID;
    uint64_t n = 0;
    return capture_common(ctx, s, list_idx, in->base, in->para, in->cap, out->base, out->para, out->cap, wl_offset,
                          &n);
}

// ---- allocation-free single generation -------------------------------------
// rp_trace_segment_noalloc runs the same three kernels as rp_trace_segment
// (generation, tile scan, placement) but takes every scratch byte from one
// fixed device array, laid out for RP_NOALLOC_MAX_RAYS input rays:
//   [0, 64)       counters: child total (u64 @0), error bits (u32 @8),
//                 hits and terminated children (2 x u64 @24), next tile to
//                 trace (u32 @40) -- zeroed per call
//   tile_counts   u32 per 32-ray sub-tile (the mixed path uses one per group)
//   tile_offsets  u64 per sub-tile
//   hand-over     the mixed path's hit ray parameter (8 bytes) and face (4
//                 bytes) per ray, between its search and material kernels
//   child slots   2 per ray, structure of arrays (188 bytes per slot)
#define NA_TILES (RP_NOALLOC_MAX_RAYS / RP_BLOCK)
#define NA_SUBS (RP_NOALLOC_MAX_RAYS / RP_SUB)
#define NA_SLOTS ((size_t)NA_TILES * RP_TILE_SLOTS)
#define NA_OFF_TILE_COUNTS ((size_t)SCRATCH_HDR)
#define NA_OFF_TILE_OFFSETS (NA_OFF_TILE_COUNTS + (((size_t)NA_SUBS * 4 + 255) & ~(size_t)255))
#define NA_OFF_HIT ((NA_OFF_TILE_OFFSETS + (size_t)NA_SUBS * 8 + 255) & ~(size_t)255)
#define NA_OFF_SLOTS (NA_OFF_HIT + (size_t)rp_hit_bytes(RP_NOALLOC_MAX_RAYS))
#define NA_SLOT_BYTES ((size_t)RP_RAY_BYTES * NA_SLOTS)
#define NA_TOTAL (NA_OFF_SLOTS + NA_SLOT_BYTES)
#define NA_MAX_DEVICES 64

static_assert(RP_NOALLOC_MAX_RAYS % RP_BLOCK == 0, "the ray limit must be whole tiles");
static_assert(NA_SLOTS % 64 == 0, "each SoA field of the slot arena must be a multiple of 256 bytes");

static __device__ __align__(256) unsigned char g_noalloc_scratch[NA_TOTAL];

static unsigned char *g_noalloc_base[NA_MAX_DEVICES];
static std::mutex g_noalloc_mu;

// One-time set-up per device, with that device current: the device address
// of g_noalloc_scratch (resolving it loads this file's device code there).
// The scratch address is cached per device; a context created after a reset
// of the device's primary context (which reloads the module, and may move
// the array) must not use the old one, so rp_ctx_create forgets it.
static void noalloc_forget(int device) {
    if (device < 0 || device >= NA_MAX_DEVICES) return;
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    g_noalloc_base[device] = nullptr;
}

static int noalloc_scratch(int device, unsigned char **base) {
    if (device < 0 || device >= NA_MAX_DEVICES) {
        snprintf(g_last_error, sizeof g_last_error, "rp_trace_segment_noalloc: device %d beyond its table of %d",
                 device, NA_MAX_DEVICES);
        return RP_ERR_INVALID;
    }
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_base[device]) {
        if (soa_bytes(NA_SLOTS) != NA_SLOT_BYTES) {
            snprintf(g_last_error, sizeof g_last_error, "rp_trace_segment_noalloc: slot arena layout mismatch");
            return RP_ERR_INVALID;
        }
        void *p = nullptr;
        CK(cudaGetSymbolAddress(&p, g_noalloc_scratch));
        if (!p || ((uintptr_t)p & 255)) {
            snprintf(g_last_error, sizeof g_last_error, "rp_trace_segment_noalloc: bad scratch address");
            return RP_ERR_CUDA;
        }
        g_noalloc_base[device] = (unsigned char *)p;
    }
    *base = g_noalloc_base[device];
    return RP_OK;
}

int rp_trace_segment_noalloc(rp_ctx *ctx, rp_scene *s, rp_rays *in, rp_rays *out, float max_length, uint32_t flags,
                             double e2, rp_stats *st) {
    if (!ctx || !s || !in || !out || in == out || s->ctx != ctx) return RP_ERR_INVALID;
    out->n = 0;  // a rejected call leaves no stale count in a reused output buffer
    if (in->n > RP_NOALLOC_MAX_RAYS) {
        snprintf(g_last_error, sizeof g_last_error,
                 "rp_trace_segment_noalloc: %llu input rays exceed its fixed limit of %d (use rp_trace_segment)",
                 (unsigned long long)in->n, RP_NOALLOC_MAX_RAYS);
        return RP_ERR_CAPACITY;
    }
    CK(cudaSetDevice(ctx->device));
    unsigned char *sc = nullptr;
    int rc = noalloc_scratch(ctx->device, &sc);
    if (rc) return rc;
    if (in->n == 0) return RP_OK;
    const uint64_t n_sub = rp_n_sub(in->n);

    rp_rays slots;  // a view of the slot arena; owns nothing
    memset(&slots, 0, sizeof slots);
    slots.block = sc + NA_OFF_SLOTS;
    slots.cap = NA_SLOTS;
    soa_carve(&slots);

    GenArgs a;
    memset(&a, 0, sizeof a);
    a.in = in->soa;
    a.out = in->soa;
    a.n_in = in->n;
    a.max_len = (double)max_length;
    a.e2_term = e2;
    a.emit = 1;
    a.one_list = -1;
    a.one_face = -1;
    a.S = s->S;
    a.smem_tables = s->smem_tables;
    a.mixed_fallback = s->mixed_fallback;
    a.out_count = (unsigned long long *)(sc + 0);
    a.err = (unsigned *)(sc + 8);
    a.stats = (unsigned long long *)(sc + 24);
    a.tile_next = (unsigned *)(sc + 40);
    a.tile_counts = (unsigned *)(sc + NA_OFF_TILE_COUNTS);
    a.tile_offsets = (unsigned long long *)(sc + NA_OFF_TILE_OFFSETS);
    a.scratch = slots.soa;
    a.face_counts = s->face_counts;
    rp__set_mixed_handover(a, flags, sc, NA_SUBS);  // the hand-over at NA_OFF_HIT

    CK(cudaMemsetAsync(sc, 0, SCRATCH_HDR, ctx->stream));
    CK(cudaEventRecord(ctx->ev0, ctx->stream));
    cudaError_t e = (flags & RP_TRACE_MIXED) ? launch_generation_mixed(a, s->smem, ctx->stream)
                                             : launch_generation_plain(a, s->smem, ctx->stream);
    if (e != cudaSuccess) return cuda_fail(e, "generation kernel launch");
    CK(cudaEventRecord(ctx->ev1, ctx->stream));
    e = launch_tile_scan(a, ctx->stream);
    if (e != cudaSuccess) return cuda_fail(e, "tile scan launch");
    CK(cudaMemcpyAsync(ctx->h_pinned, sc, 5 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));

    const unsigned long long count = ctx->h_pinned[0];
    const unsigned err = (unsigned)(ctx->h_pinned[1] & 0xffffffffu);
    if (st) {
        float ms = 0;
        cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
        st->rays_in += in->n;
        st->hits += ctx->h_pinned[3];
        st->terminated += ctx->h_pinned[4];
        st->kernel_ms += ms;
        st->device_ms += ms;
        st->launches += (flags & RP_TRACE_MIXED) ? 4 : 3;  // generation kernel(s), tile scan, placement
        st->generations += 1;
    }
    if (err & ERR_WAVELENGTH) {
        snprintf(g_last_error, sizeof g_last_error, "a ray's wavelength_idx is outside the wavelength table");
        return RP_ERR_INVALID;
    }
    if (err & (ERR_ZK_STACK | ERR_SHAPE_STACK)) {
        snprintf(g_last_error, sizeof g_last_error, "device evaluation limit hit (err=0x%x)", err);
        return RP_ERR_INVALID;
    }
    if (count > out->cap) {
        snprintf(g_last_error, sizeof g_last_error, "%llu children do not fit the output buffer", count);
        return RP_ERR_CAPACITY;
    }
    a.out = out->soa;
    a.out_cap = out->cap;
    e = launch_place_children(a, ctx->stream);
    if (e != cudaSuccess) return cuda_fail(e, "child placement launch");
    CK(cudaMemcpyAsync(ctx->h_pinned, a.err, sizeof(unsigned), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    if ((unsigned)(ctx->h_pinned[0] & 0xffffffffu) & ERR_OVERFLOW) {
        snprintf(g_last_error, sizeof g_last_error, "child placement overflowed its slots or the output buffer");
        return RP_ERR_CAPACITY;
    }
    out->n = count;
    if (st) st->rays_out += count;
    return RP_OK;
}

// ---- differentiable sequential lens --------------------------------------------
struct rp_lens {
    rp_ctx *ctx;
    int n_surf;
    double z0, max_len, atol, tol;
    std::vector<double> semi, nidx;
    uint64_t cap;
    void *block;
    size_t bytes;
    LensArgs a;                   // device pointers; rays / counts of the last forward
    unsigned blocks_cap;
    std::vector<double> params;   // of the last forward
    double n_valid, loss;
    int have_forward;
};

static size_t lens_layout(int n_surf, uint64_t cap, size_t off[8]) {
    const unsigned nb = lens_block_count(cap ? cap : 1);
    size_t o = 0;
    off[0] = o; o += align256(sizeof(rp_face) * (n_surf + 1));                   // faces
    off[1] = o; o += align256(sizeof(double) * (n_surf + 1));                    // indices
    off[2] = o; o += align256(sizeof(rp_shape_op) * 2 * n_surf);                 // apertures
    off[3] = o;                                                                   // (no per-surface states)
    off[4] = o; o += align256(sizeof(double) * 2 * (cap ? cap : 1));             // image points
    off[5] = o; o += align256(cap ? cap : 1);                                    // valid flags
    off[6] = o; o += align256(sizeof(double) * 3 * nb);                          // partial sums
    off[7] = o; o += align256(sizeof(double) * (5 * n_surf + 1) * nb + 64);      // gradient sums, error word
    return o;
}

// Face records of the lens for `params` (AsphericFace packing as the Python
// face classes do; the image plane is a CircularFace).
static void lens_tables(const rp_lens *L, const double *prm, std::vector<rp_face> &faces,
                        std::vector<rp_shape_op> &shapes) {
    const int n = L->n_surf;
    faces.assign(n + 1, rp_face());
    shapes.assign(2 * n, rp_shape_op());
    double z = L->z0;
    for (int k = 0; k < n; k++) {
        rp_face &F = faces[k];
        memset(&F, 0, sizeof F);
        F.type = RP_FACE_ASPHERIC;
        F.idx = k;
        F.material = -1;
        F.shape = 2 * k;
        F.base = -1;
        F.distortion = -1;
        F.tolerance = L->tol;
        const double c = prm[k], A4 = prm[2 * n + k], A6 = prm[3 * n + k];
        F.p[0] = c;
        F.p[1] = z;
        F.p[2] = prm[n + k];
        F.p[3] = A4;
        F.p[4] = A6;
        F.p[10] = L->atol;
        F.p[11] = A6 != 0.0 ? 3.0 : 2.0;
        F.p[12] = pow(-c, 3.0);
        rp_shape_op &S = shapes[2 * k];
        S.op = RP_SHAPE_CIRCLE;
        S.c = L->semi[k];
        shapes[2 * k + 1].op = RP_SHAPE_END;
        z += prm[4 * n + k];
    }
    rp_face &I = faces[n];
    memset(&I, 0, sizeof I);
    I.type = RP_FACE_CIRCULAR;
    I.idx = n;
    I.material = -1;
    I.shape = -1;
    I.base = -1;
    I.distortion = -1;
    I.tolerance = L->tol;
    I.p[0] = 1.0e9;  // diameter: the image plane catches every ray
    I.p[2] = z;
}

int rp_lens_create(rp_ctx *ctx, const rp_lens_desc *d, uint64_t max_rays, rp_lens **out) {
    if (!ctx || !d || !out || d->n_surfaces < 1 || d->n_surfaces > 64 || !d->semi_diameter || !d->n_index)
        return RP_ERR_INVALID;
    *out = nullptr;
    CK(cudaSetDevice(ctx->device));
    rp_lens *L = new (std::nothrow) rp_lens();
    if (!L) return RP_ERR_NOMEM;
    L->ctx = ctx;
    L->n_surf = d->n_surfaces;
    L->z0 = d->z0;
    L->max_len = d->max_length;
    L->atol = d->atol;
    L->tol = d->tolerance;
    L->semi.assign(d->semi_diameter, d->semi_diameter + d->n_surfaces);
    L->nidx.assign(d->n_index, d->n_index + d->n_surfaces + 1);
    L->cap = max_rays;
    size_t off[8];
    size_t total = lens_layout(L->n_surf, max_rays, off);
    int rc = ctx_alloc(ctx, &L->block, total, &L->bytes);
    if (rc) {
        delete L;
        return rc;
    }
    unsigned char *b = (unsigned char *)L->block;
    memset(&L->a, 0, sizeof L->a);
    L->a.n_surf = L->n_surf;
    L->a.faces = (const rp_face *)(b + off[0]);
    L->a.nidx = (const double *)(b + off[1]);
    L->a.S.shapes = (const rp_shape_op *)(b + off[2]);
    L->a.S.n_shapes = 2 * L->n_surf;
    L->a.max_len = L->max_len;
    L->a.img = (double *)(b + off[4]);
    L->a.valid = b + off[5];
    L->a.part = (double *)(b + off[6]);
    L->a.gpart = (double *)(b + off[7]);
    L->blocks_cap = lens_block_count(max_rays ? max_rays : 1);
    L->a.err = (unsigned *)(b + off[7] + sizeof(double) * (5 * L->n_surf + 1) * L->blocks_cap);
    CK(cudaMemcpyAsync((void *)L->a.nidx, L->nidx.data(), sizeof(double) * (L->n_surf + 1), cudaMemcpyHostToDevice,
                       ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    *out = L;
    return RP_OK;
}

int rp_lens_destroy(rp_lens *L) {
    if (!L) return RP_ERR_INVALID;
    cudaSetDevice(L->ctx->device);
    cudaStreamSynchronize(L->ctx->stream);
    ctx_free(L->ctx, L->block, L->bytes);
    delete L;
    return RP_OK;
}

int rp_lens_forward(rp_lens *L, const double *params, const rp_rays *rays, double *loss, uint64_t *n_valid) {
    if (!L || !params || !rays || !loss || rays->ctx != L->ctx) return RP_ERR_INVALID;
    if (rays->n > L->cap) {
        snprintf(g_last_error, sizeof g_last_error, "%llu rays exceed the lens capacity of %llu",
                 (unsigned long long)rays->n, (unsigned long long)L->cap);
        return RP_ERR_CAPACITY;
    }
    rp_ctx *ctx = L->ctx;
    CK(cudaSetDevice(ctx->device));
    const int n = L->n_surf;
    for (int k = 0; k < n; k++) {
        const double R = -params[k], beta = 1.0 + params[n + k];
        if (!(R != 0.0) || !(beta * L->semi[k] * L->semi[k] < R * R) || !(params[4 * n + k] == params[4 * n + k])) {
            snprintf(g_last_error, sizeof g_last_error,
                     "lens surface %d: the aperture reaches the conic's rim (1 - beta r^2 / R^2 <= 0)", k);
            return RP_ERR_INVALID;
        }
    }
    std::vector<rp_face> faces;
    std::vector<rp_shape_op> shapes;
    lens_tables(L, params, faces, shapes);
    CK(cudaMemcpyAsync((void *)L->a.faces, faces.data(), sizeof(rp_face) * faces.size(), cudaMemcpyHostToDevice,
                       ctx->stream));
    CK(cudaMemcpyAsync((void *)L->a.S.shapes, shapes.data(), sizeof(rp_shape_op) * shapes.size(),
                       cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemsetAsync(L->a.err, 0, sizeof(unsigned), ctx->stream));
    L->a.in = rays->soa;
    L->a.n = rays->n;
    const unsigned nb = lens_block_count(rays->n);
    cudaError_t e = launch_lens_forward(L->a, ctx->stream);
    if (e != cudaSuccess) return cuda_fail(e, "lens forward launch");
    std::vector<double> part(3 * (size_t)nb);
    if (rays->n) CK(cudaMemcpyAsync(part.data(), L->a.part, sizeof(double) * part.size(), cudaMemcpyDeviceToHost,
                                    ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    double cnt = 0.0, sx = 0.0, sy = 0.0;
    for (unsigned b = 0; b < nb; b++) {
        cnt += part[3 * b];
        sx += part[3 * b + 1];
        sy += part[3 * b + 2];
    }
    L->a.xm = cnt > 0 ? sx / cnt : 0.0;
    L->a.ym = cnt > 0 ? sy / cnt : 0.0;
    double s2 = 0.0;
    if (cnt > 0) {
        e = launch_lens_spread(L->a, ctx->stream);
        if (e != cudaSuccess) return cuda_fail(e, "lens spread launch");
        CK(cudaMemcpyAsync(part.data(), L->a.part, sizeof(double) * nb, cudaMemcpyDeviceToHost, ctx->stream));
        CK(cudaStreamSynchronize(ctx->stream));
        for (unsigned b = 0; b < nb; b++) s2 += part[b];
    }
    L->n_valid = cnt;
    L->loss = cnt > 0 ? sqrt(s2 / cnt) : 0.0;
    L->params.assign(params, params + 5 * n);
    L->have_forward = 1;
    *loss = L->loss;
    if (n_valid) *n_valid = (uint64_t)cnt;
    return RP_OK;
}

int rp_lens_backward(rp_lens *L, double *grad) {
    if (!L || !grad) return RP_ERR_INVALID;
    if (!L->have_forward) {
        snprintf(g_last_error, sizeof g_last_error, "rp_lens_backward needs a forward first");
        return RP_ERR_INVALID;
    }
    rp_ctx *ctx = L->ctx;
    CK(cudaSetDevice(ctx->device));
    const int n = L->n_surf, np = 5 * n + 1;
    for (int j = 0; j < 5 * n; j++) grad[j] = 0.0;
    if (!(L->n_valid > 0) || !(L->loss > 0)) return RP_OK;
    L->a.scale = 1.0 / (L->n_valid * L->loss);
    const unsigned nb = lens_block_count(L->a.n);
    cudaError_t e = launch_lens_backward(L->a, ctx->stream);
    if (e != cudaSuccess) return cuda_fail(e, "lens backward launch");
    std::vector<double> gp((size_t)np * nb);
    CK(cudaMemcpyAsync(gp.data(), L->a.gpart, sizeof(double) * gp.size(), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    std::vector<double> g(np, 0.0);
    for (unsigned b = 0; b < nb; b++)
        for (int j = 0; j < np; j++) g[j] += gp[(size_t)b * np + j];
    // per surface (dR, dbeta, dA4, dA6, dz_k) and dz_image -> the parameter vector
    double zacc = g[5 * n];  // d/dz_image
    for (int k = n - 1; k >= 0; k--) {
        grad[k] = -g[5 * k];             // curvature = -R
        grad[n + k] = g[5 * k + 1];      // conic: beta = 1 + conic
        grad[2 * n + k] = g[5 * k + 2];  // A4
        grad[3 * n + k] = g[5 * k + 3];  // A6
        grad[4 * n + k] = zacc;          // thickness k moves every vertex after k and the image plane
        zacc += g[5 * k + 4];
    }
    return RP_OK;
}

int rp_lens_image(const rp_lens *L, double *xy, uint8_t *valid, uint64_t n) {
    if (!L || !xy || !valid || n > L->a.n) return RP_ERR_INVALID;
    CK(cudaSetDevice(L->ctx->device));
    if (n) {
        CK(cudaMemcpyAsync(xy, L->a.img, sizeof(double) * 2 * n, cudaMemcpyDeviceToHost, L->ctx->stream));
        CK(cudaMemcpyAsync(valid, L->a.valid, n, cudaMemcpyDeviceToHost, L->ctx->stream));
    }
    CK(cudaStreamSynchronize(L->ctx->stream));
    return RP_OK;
}

// internal accessors for rp_unit.cu (not part of the public header)
int rp__scene_view(rp_scene *s, DevScene *out, cudaStream_t *st, int *device) {
    if (!s) return RP_ERR_INVALID;
    *out = s->S;
    *st = s->ctx->stream;
    *device = s->ctx->device;
    return RP_OK;
}

int rp__ctx_stream(rp_ctx *c, cudaStream_t *st, int *device) {
    if (!c) return RP_ERR_INVALID;
    *st = c->stream;
    *device = c->device;
    return RP_OK;
}

int rp__scene_curve(rp_scene *s, const rp_dispersion **dcurve, int *n_curves) {
    if (!s) return RP_ERR_INVALID;
    *dcurve = s->disp;
    *n_curves = s->n_disp;
    return RP_OK;
}

}  // extern "C"
