// rp_serve.cu -- the trace-job server: continuous batching of whole traces.
//
// Jobs (a scene, a ray source, trace parameters) are submitted from any host
// thread.  A fixed set of lanes, each a host thread with its own context
// (CUDA stream and caching allocator), takes jobs from one FIFO queue as soon
// as the lane is free and the HBM budget admits the job's estimated footprint;
// jobs on different lanes run on the device at the same time, so a job that
// arrives while others are tracing starts as soon as a lane and memory free
// up.  A lane runs its job generation by generation like rp_trace_rays
// (core/tracer.py:40-45): the source rays are generated on the device, and
// each generation is one CUDA graph (generation kernel, tile scan, child
// placement, detector tally, read-back of the counters) whose launch
// parameters are updated in the instantiated graph for the next generation.
// State stays on the device: a job returns its counters and the tallies of
// the rays that ended on its detector face, reduced on the device in a fixed
// order, so a job's result does not depend on what else is running.
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <new>
#include <thread>

#include "rp_internal.h"

namespace rp {

// ---- device side ---------------------------------------------------------------
struct SourceArgs {
    RaySoA out;
    unsigned long long n, seed;
    int type;
    double ox, oy, oz, half_angle, radius;
    unsigned n_wl;
};

// splitmix64 (Steele, Lea & Flood, "Fast splittable pseudorandom number
// generators", OOPSLA 2014): counter-based, so ray i of a job is the same
// whatever else runs.
__device__ __forceinline__ unsigned long long mix64(unsigned long long z) {
    z += 0x9e3779b97f4a7c15ULL;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
}
__device__ __forceinline__ double unit_of(unsigned long long z) { return (double)(z >> 11) * 0x1.0p-53; }

__global__ void source_kernel(SourceArgs A) {
    const unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= A.n) return;
    const unsigned long long base = mix64(A.seed ^ (i * 0xd1342543de82ef95ULL));
    const double u1 = unit_of(mix64(base + 1)), u2 = unit_of(mix64(base + 2)), u3 = unit_of(mix64(base + 3)),
                 u4 = unit_of(mix64(base + 4));
    const double two_pi = 6.283185307179586;
    double ox = A.ox, oy = A.oy, dx = 0.0, dy = 0.0, dz = 1.0;
    if (A.type == RP_SOURCE_POINT_CONE) {
        const double ct = 1.0 - u1 * (1.0 - cos(A.half_angle));
        const double st = sqrt(fmax(0.0, 1.0 - ct * ct));
        double sp, cp;
        sincos(two_pi * u2, &sp, &cp);
        dx = st * cp;
        dy = st * sp;
        dz = ct;
    } else {  // collimated disc
        const double r = A.radius * sqrt(u1);
        double sp, cp;
        sincos(two_pi * u2, &sp, &cp);
        ox += r * cp;
        oy += r * sp;
    }
    // linear polarisation at angle pi u3 in the plane perpendicular to d:
    // e1 = normalise(y x d), e2 = d x e1
    double ex = dz, ez = -dx;
    const double inv = 1.0 / sqrt(ex * ex + ez * ez);
    ex *= inv;
    ez *= inv;
    const double fx = dy * ez, fy = dz * ex - dx * ez, fz = -dy * ex;
    double sps, cps;
    sincos(3.141592653589793 * u3, &sps, &cps);
    const RaySoA &o = A.out;
    o.ox[i] = ox;
    o.oy[i] = oy;
    o.oz[i] = A.oz;
    o.dx[i] = dx;
    o.dy[i] = dy;
    o.dz[i] = dz;
    o.nx[i] = 0.0;
    o.ny[i] = 0.0;
    o.nz[i] = 1.0;
    o.ex[i] = cps * ex + sps * fx;
    o.ey[i] = sps * fy;
    o.ez[i] = cps * ez + sps * fz;
    o.n[i] = make_double2(1.0, 0.0);
    o.e1[i] = make_double2(1.0, 0.0);
    o.e2[i] = make_double2(0.0, 0.0);
    o.len[i] = 0.0;
    o.phase[i] = 0.0;
    o.opl[i] = 0.0;
    unsigned w = (unsigned)(u4 * (double)A.n_wl);
    o.wl[i] = w < A.n_wl ? w : A.n_wl - 1;
    o.parent[i] = 0;
    o.endf[i] = 0;
    o.ident[i] = (unsigned)i;
    o.type[i] = 0;
}

#define RP_TALLY_BLOCK 256
#define RP_TALLY_N 6  // hits, power, sum x, sum y, sum x^2, sum y^2

// Per block: the tallies of the generation's rays that ended on the detector
// face (hit point origin + direction * length; power (|E1|^2 + |E2|^2) Re n,
// ctracer.pyx:1971-1978).
__global__ void __launch_bounds__(RP_TALLY_BLOCK) tally_kernel(RaySoA in, unsigned long long n, unsigned detector,
                                                                double *partials) {
    __shared__ double s[RP_TALLY_N][RP_TALLY_BLOCK / 32];
    const unsigned long long i = (unsigned long long)blockIdx.x * RP_TALLY_BLOCK + threadIdx.x;
    double v[RP_TALLY_N] = {0, 0, 0, 0, 0, 0};
    if (i < n && in.endf[i] == detector) {
        const double L = in.len[i];
        const double x = in.ox[i] + in.dx[i] * L, y = in.oy[i] + in.dy[i] * L;
        const double2 a = in.e1[i], b = in.e2[i];
        v[0] = 1.0;
        v[1] = (a.x * a.x + a.y * a.y + b.x * b.x + b.y * b.y) * in.n[i].x;
        v[2] = x;
        v[3] = y;
        v[4] = x * x;
        v[5] = y * y;
    }
    for (int k = 0; k < RP_TALLY_N; k++) {
        double t = v[k];
        for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
        if ((threadIdx.x & 31) == 0) s[k][threadIdx.x >> 5] = t;
    }
    __syncthreads();
    if (threadIdx.x < RP_TALLY_N) {
        double t = 0.0;
        for (int w = 0; w < RP_TALLY_BLOCK / 32; w++) t += s[threadIdx.x][w];
        partials[(size_t)blockIdx.x * RP_TALLY_N + threadIdx.x] = t;
    }
}

// Adds the block partials, in block order, to the job's accumulators.
__global__ void tally_finish_kernel(const double *partials, unsigned nb, double *acc) {
    if (threadIdx.x >= RP_TALLY_N) return;
    double t = 0.0;
    for (unsigned b = 0; b < nb; b++) t += partials[(size_t)b * RP_TALLY_N + threadIdx.x];
    acc[threadIdx.x] += t;
}

}  // namespace rp

// ---- host side -------------------------------------------------------------------
namespace {

using Clock = std::chrono::steady_clock;

struct Job {
    uint64_t id = 0;
    std::vector<rp_facelist> lists;
    std::vector<rp_face> faces;
    std::vector<rp_material> mats;
    std::vector<rp_shape_op> shapes;
    std::vector<rp_distortion> dists;
    std::vector<rp_dispersion> disps;
    std::vector<double> aux, wl;
    rp_scene_desc desc;
    rp_source_desc source;
    int32_t recursion_limit = 0, detector = -1;
    float max_length = 0.0f;
    uint32_t flags = 0;
    double e2 = 0.0;
    uint64_t est_bytes = 0;
    rp_job_result res;
    std::vector<uint32_t> face_counts;
    bool done = false;
};

struct Lane {
    int index = 0;
    rp_ctx *ctx = nullptr;
    std::thread th;
    uint64_t reserved = 0;
    cudaGraphExec_t exec[2] = {nullptr, nullptr};  // [emit]
    unsigned char *scratch = nullptr;               // header | tile counts | tile offsets | tally partials
    size_t scratch_bytes = 0;
    rp_rays *arena = nullptr;
    double *acc = nullptr;                          // device tally accumulators
    unsigned long long *h_hdr = nullptr;            // pinned read-back of the header
    double *h_acc = nullptr;                        // pinned read-back of the tallies
};

}  // namespace

struct rp_server {
    int device = 0;
    uint64_t budget = 0;
    std::vector<Lane *> lanes;
    std::mutex mu;
    std::condition_variable cv_pending, cv_done;
    std::deque<Job *> pending;
    std::map<uint64_t, Job *> jobs;
    uint64_t next_id = 1;
    uint64_t reserved_total = 0;
    int busy = 0;
    bool stop = false;
    Clock::time_point t0;
};

namespace {

double ms_since(const rp_server *s) {
    return std::chrono::duration<double, std::milli>(Clock::now() - s->t0).count();
}

size_t align256s(size_t x) { return (x + 255) & ~(size_t)255; }

// Device bytes a job is expected to hold: the generation in flight (n), its
// child buffer (2n), the child-slot arena (2n plus a quarter) and the scene.
uint64_t job_estimate(const Job *j) {
    const uint64_t n = j->source.n_rays;
    return n * (uint64_t)RP_RAY_BYTES * 6 + (uint64_t)(j->faces.size() + j->lists.size() + j->mats.size()) * 512 +
           (uint64_t)j->wl.size() * 64 + (1u << 20);
}

int lane_scratch(Lane *L, uint64_t n_tiles) {
    const size_t nb_tally = (size_t)((n_tiles * RP_BLOCK + RP_TALLY_BLOCK - 1) / RP_TALLY_BLOCK);
    const uint64_t n_sub = n_tiles * RP_SUB_PER_BLOCK;  // count entries are per 32-ray sub-tile
    const size_t need = 64 + align256s(n_sub * 4) + align256s(n_sub * 8) + rp_hit_bytes(n_sub * RP_SUB) +
                        align256s(nb_tally * RP_TALLY_N * 8);
    if (need <= L->scratch_bytes) return RP_OK;
    if (L->scratch) {
        cudaStreamSynchronize(L->ctx->stream);
        cudaFree(L->scratch);
        L->scratch = nullptr;
        L->scratch_bytes = 0;
    }
    cudaError_t e = cudaMalloc((void **)&L->scratch, need * 2);
    if (e != cudaSuccess) return rp__cuda_fail(e, "server scratch");
    L->scratch_bytes = need * 2;
    return RP_OK;
}

int lane_arena(Lane *L, uint64_t n_tiles) {
    const uint64_t need = n_tiles * RP_TILE_SLOTS;
    uint64_t cap = 0;
    if (L->arena) rp_rays_capacity(L->arena, &cap);
    if (L->arena && cap >= need) return RP_OK;
    if (L->arena) {
        rp_rays_free(L->arena);
        L->arena = nullptr;
    }
    return rp_rays_alloc(L->ctx, need + need / 4, &L->arena);
}

// Captures one generation into a graph and launches it through the lane's
// instantiated graph for that shape, updating its parameters in place.
int run_generation(Lane *L, rp_scene *sc, rp_rays *in, rp_rays *out, const Job *j, int emit) {
    rp_ctx *ctx = L->ctx;
    const uint64_t n = in->n, n_tiles = (n + RP_BLOCK - 1) / RP_BLOCK;
    int rc = lane_scratch(L, n_tiles);
    if (rc == RP_OK && emit) rc = lane_arena(L, n_tiles);
    if (rc) return rc;
    unsigned char *sc0 = L->scratch;
    GenArgs a;
    memset(&a, 0, sizeof a);
    a.in = in->soa;
    a.out = emit ? out->soa : in->soa;
    a.n_in = n;
    a.out_cap = emit ? out->cap : 0;
    a.max_len = (double)j->max_length;
    a.e2_term = j->e2;
    a.emit = emit;
    a.one_list = -1;
    a.one_face = -1;
    a.S = sc->S;
    a.smem_tables = sc->smem_tables;
    a.mixed_fallback = sc->mixed_fallback;
    a.out_count = (unsigned long long *)(sc0 + 0);
    a.err = (unsigned *)(sc0 + 8);
    a.stats = (unsigned long long *)(sc0 + 24);
    a.tile_next = (unsigned *)(sc0 + 40);
    const uint64_t n_sub = n_tiles * RP_SUB_PER_BLOCK;
    a.tile_counts = (unsigned *)(sc0 + 64);
    a.tile_offsets = (unsigned long long *)(sc0 + 64 + align256s(n_sub * 4));
    double *partials = (double *)(sc0 + 64 + align256s(n_sub * 4) + align256s(n_sub * 8) + rp_hit_bytes(n_sub * RP_SUB));
    a.scratch = emit ? L->arena->soa : in->soa;
    a.face_counts = sc->face_counts;
    const bool mixed = (j->flags & RP_TRACE_MIXED) != 0;
    rp__set_mixed_handover(a, j->flags, sc0, n_sub);
    cudaError_t e = mixed ? prepare_generation_mixed(a, sc->smem) : prepare_generation_plain(a, sc->smem);
    if (e != cudaSuccess) return rp__cuda_fail(e, "generation set-up");
    const unsigned nb_tally = (unsigned)((n + RP_TALLY_BLOCK - 1) / RP_TALLY_BLOCK);

    cudaStream_t st = ctx->stream;
    cudaGraph_t graph = nullptr;
    e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return rp__cuda_fail(e, "cudaStreamBeginCapture");
    cudaError_t ce = cudaMemsetAsync(sc0, 0, 64, st);
    if (ce == cudaSuccess) ce = mixed ? launch_generation_mixed(a, sc->smem, st) : launch_generation_plain(a, sc->smem, st);
    if (ce == cudaSuccess && emit) ce = launch_tile_scan(a, st);
    if (ce == cudaSuccess && emit) ce = launch_place_children(a, st);
    if (ce == cudaSuccess && j->detector >= 0) {
        tally_kernel<<<nb_tally, RP_TALLY_BLOCK, 0, st>>>(in->soa, n, (unsigned)j->detector, partials);
        tally_finish_kernel<<<1, 32, 0, st>>>(partials, nb_tally, L->acc);
        ce = cudaGetLastError();
    }
    if (ce == cudaSuccess)
        ce = cudaMemcpyAsync(L->h_hdr, sc0, 5 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, st);
    e = cudaStreamEndCapture(st, &graph);
    if (ce != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        return rp__cuda_fail(ce, "generation capture");
    }
    if (e != cudaSuccess) return rp__cuda_fail(e, "cudaStreamEndCapture");
    cudaGraphExec_t &ex = L->exec[emit ? 1 : 0];
    bool fresh = ex == nullptr;
    if (!fresh) {
        cudaGraphExecUpdateResultInfo info;
        if (cudaGraphExecUpdate(ex, graph, &info) != cudaSuccess) {
            cudaGetLastError();
            cudaGraphExecDestroy(ex);
            ex = nullptr;
            fresh = true;
        }
    }
    if (fresh) {
        e = cudaGraphInstantiate(&ex, graph, 0);
        if (e != cudaSuccess) {
            cudaGraphDestroy(graph);
            ex = nullptr;
            return rp__cuda_fail(e, "cudaGraphInstantiate");
        }
    }
    cudaGraphDestroy(graph);
    e = cudaGraphLaunch(ex, st);
    if (e != cudaSuccess) return rp__cuda_fail(e, "cudaGraphLaunch");
    e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return rp__cuda_fail(e, "generation");
    const unsigned err = (unsigned)(L->h_hdr[1] & 0xffffffffu);
    if (err & (ERR_WAVELENGTH | ERR_ZK_STACK | ERR_SHAPE_STACK | ERR_OVERFLOW)) {
        rp__set_error("generation error bits 0x%x", err);
        return RP_ERR_INVALID;
    }
    return RP_OK;
}

void run_job(rp_server *srv, Lane *L, Job *j) {
    rp_ctx *ctx = L->ctx;
    j->res.t_start_ms = ms_since(srv);
    rp_scene *sc = nullptr;
    rp_rays *g = nullptr;
    int rc = rp_scene_create(ctx, &j->desc, j->wl.empty() ? nullptr : j->wl.data(), (int64_t)j->wl.size(), &sc);
    const uint64_t n0 = j->source.n_rays;
    if (rc == RP_OK) rc = rp_rays_alloc(ctx, n0 ? n0 : 1, &g);
    if (rc == RP_OK && cudaMemsetAsync(L->acc, 0, RP_TALLY_N * sizeof(double), ctx->stream) != cudaSuccess)
        rc = RP_ERR_CUDA;
    if (rc == RP_OK && n0) {
        SourceArgs A;
        A.out = g->soa;
        A.n = n0;
        A.seed = j->source.seed;
        A.type = j->source.type;
        A.ox = j->source.origin[0];
        A.oy = j->source.origin[1];
        A.oz = j->source.origin[2];
        A.half_angle = j->source.half_angle;
        A.radius = j->source.radius;
        A.n_wl = (unsigned)(j->wl.empty() ? 1 : j->wl.size());
        source_kernel<<<(unsigned)((n0 + 255) / 256), 256, 0, ctx->stream>>>(A);
        if (cudaGetLastError() != cudaSuccess) rc = RP_ERR_CUDA;
        g->n = n0;
    }
    uint64_t segments = 0;
    int count = 0;
    while (rc == RP_OK && g && g->n > 0 && count < j->recursion_limit) {
        const int last = (count + 1 == j->recursion_limit);
        rp_rays *out = nullptr;
        if (!last) rc = rp_rays_alloc(ctx, 2 * g->n, &out);
        if (rc) break;
        rc = run_generation(L, sc, g, out, j, last ? 0 : 1);
        if (rc) {
            if (out) rp_rays_free(out);
            break;
        }
        segments += g->n;
        count++;
        const uint64_t n_child = last ? 0 : L->h_hdr[0];
        rp_rays_free(g);
        g = out;
        if (g) g->n = n_child;
        if (last || n_child == 0) break;
    }
    if (g) rp_rays_free(g);
    j->res.status = rc;
    j->res.generations = count;
    j->res.segments = segments;
    if (sc) {
        j->face_counts.assign(j->desc.n_faces, 0u);
        if (rc == RP_OK && j->desc.n_faces)
            rc = rp_scene_face_counts(sc, j->face_counts.data(), j->desc.n_faces, 0);
        rp_scene_destroy(sc);
    }
    if (rc == RP_OK) {
        if (cudaMemcpy(L->h_acc, L->acc, RP_TALLY_N * sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess)
            rc = RP_ERR_CUDA;
    }
    j->res.status = rc;
    j->res.detector_hits = rc == RP_OK ? (uint64_t)L->h_acc[0] : 0;
    j->res.detector_power = rc == RP_OK ? L->h_acc[1] : 0.0;
    j->res.sum_x = rc == RP_OK ? L->h_acc[2] : 0.0;
    j->res.sum_y = rc == RP_OK ? L->h_acc[3] : 0.0;
    j->res.sum_xx = rc == RP_OK ? L->h_acc[4] : 0.0;
    j->res.sum_yy = rc == RP_OK ? L->h_acc[5] : 0.0;
    j->res.t_done_ms = ms_since(srv);
}

uint64_t lane_memory(Lane *L) {
    uint64_t b = 0;
    rp_ctx_memory(L->ctx, &b);
    return b + L->scratch_bytes;
}

void lane_main(rp_server *srv, Lane *L) {
    cudaSetDevice(srv->device);
    for (;;) {
        Job *j = nullptr;
        {
            std::unique_lock<std::mutex> lk(srv->mu);
            for (;;) {
                if (srv->stop && srv->pending.empty()) return;
                if (!srv->pending.empty()) {
                    Job *h = srv->pending.front();
                    const uint64_t mine = lane_memory(L);
                    const uint64_t need = mine > h->est_bytes ? mine : h->est_bytes;
                    const uint64_t others = srv->reserved_total - L->reserved;
                    if (others + need <= srv->budget || srv->busy == 0) {
                        srv->pending.pop_front();
                        srv->reserved_total = others + need;
                        L->reserved = need;
                        srv->busy++;
                        j = h;
                        break;
                    }
                    if (mine > 0 && L->reserved == mine) {
                        // memory pressure: give this idle lane's cached blocks back
                        lk.unlock();
                        rp_ctx_trim(L->ctx);
                        lk.lock();
                        srv->reserved_total -= L->reserved;
                        L->reserved = lane_memory(L);
                        srv->reserved_total += L->reserved;
                        continue;
                    }
                }
                srv->cv_pending.wait(lk);
            }
        }
        run_job(srv, L, j);
        {
            std::lock_guard<std::mutex> lk(srv->mu);
            const uint64_t now = lane_memory(L);
            srv->reserved_total = srv->reserved_total - L->reserved + now;
            L->reserved = now;
            srv->busy--;
            j->done = true;
        }
        srv->cv_done.notify_all();
        srv->cv_pending.notify_all();
    }
}

template <class T>
void copy_table(std::vector<T> &dst, const T *src, int32_t n) {
    dst.assign(src && n > 0 ? src : nullptr, src && n > 0 ? src + n : nullptr);
}

void destroy_lane(Lane *L) {
    if (!L) return;
    cudaSetDevice(L->ctx ? L->ctx->device : 0);
    for (auto &e : L->exec)
        if (e) cudaGraphExecDestroy(e);
    if (L->arena) rp_rays_free(L->arena);
    if (L->scratch) cudaFree(L->scratch);
    if (L->acc) cudaFree(L->acc);
    if (L->h_hdr) cudaFreeHost(L->h_hdr);
    if (L->h_acc) cudaFreeHost(L->h_acc);
    if (L->ctx) rp_ctx_destroy(L->ctx);
    delete L;
}

}  // namespace

extern "C" {

int rp_source_generate(rp_ctx *ctx, const rp_source_desc *src, uint32_t n_wl, rp_rays *out) {
    if (!ctx || !src || !out || src->n_rays > out->cap || n_wl < 1) return RP_ERR_INVALID;
    if (src->type != RP_SOURCE_POINT_CONE && src->type != RP_SOURCE_COLLIMATED_DISC) return RP_ERR_INVALID;
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e != cudaSuccess) return rp__cuda_fail(e, "cudaSetDevice");
    out->n = src->n_rays;
    if (!src->n_rays) return RP_OK;
    SourceArgs A;
    A.out = out->soa;
    A.n = src->n_rays;
    A.seed = src->seed;
    A.type = src->type;
    A.ox = src->origin[0];
    A.oy = src->origin[1];
    A.oz = src->origin[2];
    A.half_angle = src->half_angle;
    A.radius = src->radius;
    A.n_wl = n_wl;
    source_kernel<<<(unsigned)((src->n_rays + 255) / 256), 256, 0, ctx->stream>>>(A);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    return e == cudaSuccess ? RP_OK : rp__cuda_fail(e, "source kernel");
}

int rp_server_create(int device, uint64_t hbm_budget, int32_t lanes, rp_server **out) {
    if (!out || lanes < 1 || lanes > 64) return RP_ERR_INVALID;
    *out = nullptr;
    rp_server *s = new (std::nothrow) rp_server();
    if (!s) return RP_ERR_NOMEM;
    s->device = device;
    s->budget = hbm_budget ? hbm_budget : ~(uint64_t)0;
    s->t0 = Clock::now();
    for (int k = 0; k < lanes; k++) {
        Lane *L = new (std::nothrow) Lane();
        if (!L) {
            rp_server_destroy(s);
            return RP_ERR_NOMEM;
        }
        L->index = k;
        int rc = rp_ctx_create(device, 0, &L->ctx);
        if (rc == RP_OK && cudaMalloc((void **)&L->acc, RP_TALLY_N * sizeof(double)) != cudaSuccess) rc = RP_ERR_CUDA;
        if (rc == RP_OK && cudaMallocHost((void **)&L->h_hdr, 8 * sizeof(unsigned long long)) != cudaSuccess)
            rc = RP_ERR_CUDA;
        if (rc == RP_OK && cudaMallocHost((void **)&L->h_acc, RP_TALLY_N * sizeof(double)) != cudaSuccess)
            rc = RP_ERR_CUDA;
        if (rc) {
            destroy_lane(L);
            rp_server_destroy(s);
            return rc;
        }
        s->lanes.push_back(L);
    }
    for (Lane *L : s->lanes) L->th = std::thread(lane_main, s, L);
    *out = s;
    return RP_OK;
}

int rp_server_submit(rp_server *s, const rp_job_desc *jd, uint64_t *job_id) {
    if (!s || !jd || !jd->scene || !job_id) return RP_ERR_INVALID;
    const rp_scene_desc *d = jd->scene;
    if (jd->source.type != RP_SOURCE_POINT_CONE && jd->source.type != RP_SOURCE_COLLIMATED_DISC) return RP_ERR_INVALID;
    if (jd->recursion_limit < 0 || jd->n_wl < 0 || (jd->n_wl > 0 && !jd->wavelengths)) return RP_ERR_INVALID;
    Job *j = new (std::nothrow) Job();
    if (!j) return RP_ERR_NOMEM;
    copy_table(j->lists, d->lists, d->n_lists);
    copy_table(j->faces, d->faces, d->n_face_records);
    copy_table(j->mats, d->materials, d->n_materials);
    copy_table(j->shapes, d->shape_ops, d->n_shape_ops);
    copy_table(j->dists, d->distortions, d->n_distortions);
    copy_table(j->disps, d->dispersions, d->n_dispersions);
    copy_table(j->aux, d->aux, d->n_aux);
    j->wl.assign(jd->wavelengths, jd->wavelengths + jd->n_wl);
    j->desc = *d;
    j->desc.lists = j->lists.data();
    j->desc.faces = j->faces.data();
    j->desc.materials = j->mats.data();
    j->desc.shape_ops = j->shapes.data();
    j->desc.distortions = j->dists.data();
    j->desc.dispersions = j->disps.data();
    j->desc.aux = j->aux.data();
    j->source = jd->source;
    j->recursion_limit = jd->recursion_limit;
    j->max_length = jd->max_length;
    j->flags = jd->flags;
    j->detector = jd->detector_face;
    j->e2 = jd->e2_terminate;
    j->est_bytes = job_estimate(j);
    memset(&j->res, 0, sizeof j->res);
    {
        std::lock_guard<std::mutex> lk(s->mu);
        if (s->stop) {
            delete j;
            return RP_ERR_INVALID;
        }
        j->id = s->next_id++;
        j->res.t_submit_ms = ms_since(s);
        s->jobs[j->id] = j;
        s->pending.push_back(j);
        *job_id = j->id;
    }
    s->cv_pending.notify_all();
    return RP_OK;
}

int rp_server_wait(rp_server *s, uint64_t job_id, rp_job_result *res, uint32_t *face_counts, int32_t n_faces) {
    if (!s || !res) return RP_ERR_INVALID;
    Job *j = nullptr;
    {
        std::unique_lock<std::mutex> lk(s->mu);
        auto it = s->jobs.find(job_id);
        if (it == s->jobs.end()) return RP_ERR_INVALID;
        j = it->second;
        s->cv_done.wait(lk, [&] { return j->done; });
        s->jobs.erase(it);
    }
    *res = j->res;
    if (face_counts)
        for (int32_t k = 0; k < n_faces && k < (int32_t)j->face_counts.size(); k++) face_counts[k] = j->face_counts[k];
    delete j;
    return RP_OK;
}

int rp_server_destroy(rp_server *s) {
    if (!s) return RP_ERR_INVALID;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
    }
    s->cv_pending.notify_all();
    for (Lane *L : s->lanes)
        if (L->th.joinable()) L->th.join();
    for (Lane *L : s->lanes) destroy_lane(L);
    for (auto &kv : s->jobs) delete kv.second;
    delete s;
    return RP_OK;
}

}  // extern "C"
