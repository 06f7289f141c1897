// rp_serve.cu -- the trace-job server: continuous batching of generations.
//
// Jobs (a scene, a ray source, trace parameters) are submitted from any host
// thread and wait in one FIFO queue.  One step loop drives the device: each
// step first admits waiting jobs while a slot is free and the HBM budget
// holds their estimated footprint (their scenes and tables are uploaded and
// their source rays generated on the device), then advances EVERY admitted
// job by one generation (core/tracer.py:40-45, per job) in one batch: the
// jobs' rays are numbered in 128-ray groups across the batch, and one launch
// of the mixed path's search kernel and one of its material kernel drain the
// batch's (job, group) work items from device counters, so rays of all jobs
// share each launch.  One scan of the per-group child counts, one placement
// and one detector tally serve the whole batch; the step is one CUDA graph,
// captured once and replayed with its parameters in device memory (the
// batch table is copied in by the graph itself), followed by one read-back
// of every job's child count and tallies.  A job's rays stay in its own
// buffers and are reduced in a fixed order within the job, so its result
// does not depend on what else is in the batch.  Jobs on the plain FP64 path
// run their own generation kernels inside the same step.
#include <algorithm>
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
#include "rp_nearest.cuh"

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

#define RP_SERVE_WARPS_PER_BLOCK 8
#define RP_TALLY_N 6  // hits, power, sum x, sum y, sum x^2, sum y^2

// Per batch step, written by batch_finish_kernel into mapped host memory.
struct StepOut {
    unsigned long long count[RP_BATCH_MAX_JOBS];  // children of each slot's generation
    double acc[RP_BATCH_MAX_JOBS][RP_TALLY_N];     // each slot's detector tallies so far
    unsigned err;
    unsigned pad;
};

// One warp per global group: the mixed jobs' children move from their slot
// range to their final place in the job's next generation, at the group's
// offset within its job.
__global__ void batch_place_kernel(const BatchDev *B, const unsigned long long *offsets, unsigned *err) {
    const unsigned lane = threadIdx.x & 31;
    const unsigned long long warps = (unsigned long long)gridDim.x * (blockDim.x >> 5);
    for (unsigned long long u = (unsigned long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
         u < B->total_units; u += warps) {
        const int j = batch_job_of(B, (unsigned)u);
        const BatchJob &J = B->jobs[j];
        if (!J.mixed || !J.a.emit) continue;
        const unsigned lu = (unsigned)(u - B->unit_start[j]);
        const unsigned count = J.a.tile_counts[lu];
        const unsigned long long base = offsets[u] - offsets[B->unit_start[j]];
        if (count > RP_TILE_SLOTS || base + count > J.a.out_cap) {
            if (lane == 0) atomicOr(err, ERR_OVERFLOW);
            continue;
        }
        const unsigned long long src = (unsigned long long)lu * RP_TILE_SLOTS;
        for (unsigned k = lane; k < count; k += 32) copy_ray(J.a.scratch, src + k, J.a.out, base + k);
    }
}

// One warp per global group: the tallies of the group's rays that ended on
// their job's detector face (hit point origin + direction * length; power
// (|E1|^2 + |E2|^2) Re n, ctracer.pyx:1971-1978), each lane over its four
// rays in order, then a fixed tree across the warp.
__global__ void batch_tally_kernel(const BatchDev *B) {
    const unsigned lane = threadIdx.x & 31;
    const unsigned long long warps = (unsigned long long)gridDim.x * (blockDim.x >> 5);
    for (unsigned long long u = (unsigned long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
         u < B->total_units; u += warps) {
        const int j = batch_job_of(B, (unsigned)u);
        const BatchJob &J = B->jobs[j];
        const RaySoA &in = J.a.in;
        const unsigned long long g0 = (u - B->unit_start[j]) * (unsigned long long)RP_GROUP;
        double v[RP_TALLY_N] = {0, 0, 0, 0, 0, 0};
        for (int c = 0; c < RP_GROUP / 32; c++) {
            const unsigned long long i = g0 + 32 * c + lane;
            if (i < J.a.n_in && J.detector >= 0 && in.endf[i] == (unsigned)J.detector) {
                const double L = in.len[i];
                const double x = in.ox[i] + in.dx[i] * L, y = in.oy[i] + in.dy[i] * L;
                const double2 a = in.e1[i], b = in.e2[i];
                v[0] += 1.0;
                v[1] += (a.x * a.x + a.y * a.y + b.x * b.x + b.y * b.y) * in.n[i].x;
                v[2] += x;
                v[3] += y;
                v[4] += x * x;
                v[5] += y * y;
            }
        }
        for (int k = 0; k < RP_TALLY_N; k++) {
            double t = v[k];
            for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
            if (lane == 0) J.part[(u - B->unit_start[j]) * RP_TALLY_N + k] = t;
        }
    }
}

// One block per job of the batch: when this step completes the job's
// generation, its groups' tally partials are summed in a fixed order that
// depends only on the generation (thread t adds groups t, t + 256, ... in
// turn, then a fixed tree over the threads) and added to its slot's
// accumulators; and the step's child count (from the batch scan, or a
// plain-path job's own scan) -- written to mapped host memory.
#define RP_FINISH_THREADS 256
__global__ void __launch_bounds__(RP_FINISH_THREADS)
    batch_finish_kernel(const BatchDev *B, const unsigned long long *offsets, const unsigned long long *total,
                        double *acc, const unsigned *ctr, StepOut *out) {
    __shared__ double red[RP_TALLY_N][RP_FINISH_THREADS];
    const int j = blockIdx.x;
    if (j >= B->n_jobs) return;
    const BatchJob &J = B->jobs[j];
    const unsigned u0 = B->unit_start[j], u1 = B->unit_start[j + 1];
    double v[RP_TALLY_N] = {0, 0, 0, 0, 0, 0};
    if (J.gen_done)
        for (unsigned long long u = threadIdx.x; u < J.gen_units; u += RP_FINISH_THREADS)
            for (int k = 0; k < RP_TALLY_N; k++) v[k] += J.part_gen[u * RP_TALLY_N + k];
    for (int k = 0; k < RP_TALLY_N; k++) red[k][threadIdx.x] = v[k];
    __syncthreads();
    for (int h = RP_FINISH_THREADS / 2; h > 0; h >>= 1) {
        if ((int)threadIdx.x < h)
            for (int k = 0; k < RP_TALLY_N; k++) red[k][threadIdx.x] += red[k][threadIdx.x + h];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        double *a = acc + (size_t)J.slot * RP_TALLY_N;
        for (int k = 0; k < RP_TALLY_N; k++) {
            if (J.gen_done)
                a[k] = J.first ? red[k][0] : a[k] + red[k][0];
            else if (J.first)
                a[k] = 0.0;  // (the slot's previous job left its sums)
            out->acc[J.slot][k] = a[k];
        }
        unsigned long long c = 0;
        if (J.mixed)
            c = J.a.emit ? ((j + 1 < B->n_jobs ? offsets[u1] : *total) - offsets[u0]) : 0ull;
        else
            c = J.own_count ? *J.own_count : 0ull;  // set only when the plain job keeps children
        out->count[J.slot] = c;
        if (j == 0) out->err = ctr[2] | ctr[3];
        __threadfence_system();
    }
}

}  // namespace rp

// ---- host side -------------------------------------------------------------------
namespace {

using Clock = std::chrono::steady_clock;

size_t align256s(size_t x) { return (x + 255) & ~(size_t)255; }

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
    // while admitted
    int slot = -1;
    int gen = 0;
    uint64_t segments = 0;
    bool mixed = true;
    rp_scene *sc = nullptr;
    void *mx = nullptr;           // float / float-float tables (mixed)
    size_t mx_bytes = 0;
    rp_rays *cur = nullptr, *next = nullptr, *spare = nullptr, *arena = nullptr;  // spare: cur's ping-pong partner
    unsigned char *hand = nullptr;  // hit hand-over (mixed) or own scan scratch (plain)
    size_t hand_bytes = 0, hand_cap = 0;
    bool active = false;            // admitted and taking part in the steps
    // a generation traced in chunks (mixed): units done, children placed so far
    uint64_t done_units = 0, next_n = 0;
    uint64_t chunk = 0;             // units of the current step
    double *part = nullptr;         // per-unit detector tallies of the generation
    size_t part_bytes = 0, part_cap = 0;
};

}  // namespace

struct rp_server {
    int device = 0;
    uint64_t budget = 0;
    int max_jobs = 0;
    rp_ctx *ctx = nullptr;   // the steps' stream and buffers
    rp_ctx *actx = nullptr;  // admission: scenes, tables and source rays, on its own stream
    std::thread loop, admit_th;
    std::mutex mu;
    std::condition_variable cv_pending, cv_step, cv_done;
    std::deque<Job *> pending;
    std::deque<Job *> ready;  // admitted, joining at the next step
    int admitting = 0;        // jobs in admission
    uint64_t step_groups = 0, min_chunk = 0;  // a step's group budget and smallest chunk (set at creation)
    std::map<uint64_t, Job *> jobs;
    std::vector<Job *> slots;  // admitted jobs by slot
    uint64_t next_id = 1;
    uint64_t reserved = 0;
    bool stop = false;
    Clock::time_point t0;
    // batch step buffers (device unless noted)
    BatchDev *h_batch = nullptr, *d_batch = nullptr;  // h_batch: pinned
    unsigned *d_ctr = nullptr;
    unsigned *d_counts = nullptr;
    unsigned long long *d_offsets = nullptr, *d_total = nullptr, *d_dummy = nullptr;
    double *d_acc = nullptr;
    StepOut *h_out = nullptr, *d_out = nullptr;  // mapped pinned
    size_t unit_cap = 0;
    cudaGraphExec_t step_exec = nullptr;
    cudaEvent_t ev_start = nullptr, ev_end = nullptr;  // around each step's device work
    rp_server_stats stats{};                           // under mu
};

namespace {

double ms_since(const rp_server *s) {
    return std::chrono::duration<double, std::milli>(Clock::now() - s->t0).count();
}

// Device bytes a job is expected to hold: the generation in flight (n), its
// child buffer (2n), the child-slot arena (2n plus a quarter) and the scene.
uint64_t job_estimate(const Job *j) {
    const uint64_t n = j->source.n_rays;
    return n * (uint64_t)RP_RAY_BYTES * 6 + (uint64_t)(j->faces.size() + j->lists.size() + j->mats.size()) * 512 +
           (uint64_t)j->wl.size() * 64 + (1u << 20);
}

void free_unit_arrays(rp_server *s) {
    if (s->d_counts) cudaFree(s->d_counts);
    if (s->d_offsets) cudaFree(s->d_offsets);
    s->d_counts = nullptr;
    s->d_offsets = nullptr;
    s->unit_cap = 0;
}

// The step graph: the batch table's upload, the counters' clear, the mixed
// jobs' search and material kernels, the scan of every group's child count,
// the placement, the tallies and the per-job results.  Its pointers are
// fixed for a unit capacity; a larger batch re-allocates and re-captures it.
int capture_step(rp_server *s) {
    rp_ctx *ctx = s->ctx;
    cudaStream_t st = ctx->stream;
    if (s->step_exec) {
        cudaGraphExecDestroy(s->step_exec);
        s->step_exec = nullptr;
    }
    // kernel attributes are set before the capture (set-up calls are not captured)
    size_t ss = 0, ms = 0;
    int sb = 0, mb = 0;
    cudaError_t e = prepare_batch_mixed(&ss, &ms, &sb, &mb);
    if (e != cudaSuccess) return rp__cuda_fail(e, "batch kernel set-up");
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, s->device);
    const unsigned small_grid = (unsigned)(sms > 0 ? 4 * sms : 512);
    cudaGraph_t g = nullptr;
    e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return rp__cuda_fail(e, "cudaStreamBeginCapture");
    cudaError_t ce = cudaMemcpyAsync(s->d_batch, s->h_batch, sizeof(BatchDev), cudaMemcpyHostToDevice, st);
    if (ce == cudaSuccess) ce = cudaMemsetAsync(s->d_ctr, 0, 3 * sizeof(unsigned), st);  // [3]: the plain jobs' errors
    if (ce == cudaSuccess) ce = launch_batch_mixed(s->d_batch, s->d_ctr, st);
    if (ce == cudaSuccess) ce = launch_tile_scan_dev(s->d_counts, &s->d_batch->total_units, s->d_offsets, s->d_total, st);
    if (ce == cudaSuccess) {
        batch_place_kernel<<<small_grid, 32 * RP_SERVE_WARPS_PER_BLOCK, 0, st>>>(s->d_batch, s->d_offsets, s->d_ctr + 2);
        batch_tally_kernel<<<small_grid, 32 * RP_SERVE_WARPS_PER_BLOCK, 0, st>>>(s->d_batch);
        batch_finish_kernel<<<RP_BATCH_MAX_JOBS, RP_FINISH_THREADS, 0, st>>>(s->d_batch, s->d_offsets, s->d_total,
                                                                            s->d_acc, s->d_ctr, s->d_out);
        ce = cudaGetLastError();
    }
    e = cudaStreamEndCapture(st, &g);
    if (ce != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        return rp__cuda_fail(ce, "step capture");
    }
    if (e != cudaSuccess) return rp__cuda_fail(e, "cudaStreamEndCapture");
    e = cudaGraphInstantiate(&s->step_exec, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        s->step_exec = nullptr;
        return rp__cuda_fail(e, "cudaGraphInstantiate");
    }
    return RP_OK;
}

int ensure_units(rp_server *s, size_t units) {
    if (units <= s->unit_cap && s->step_exec) return RP_OK;
    size_t cap = s->unit_cap ? s->unit_cap : 4096;
    while (cap < units) cap *= 2;
    cudaStreamSynchronize(s->ctx->stream);
    free_unit_arrays(s);
    cudaError_t e = cudaMalloc((void **)&s->d_counts, (cap + 1) * sizeof(unsigned));
    if (e == cudaSuccess) e = cudaMalloc((void **)&s->d_offsets, (cap + 1) * sizeof(unsigned long long));
    if (e != cudaSuccess) {
        free_unit_arrays(s);
        return rp__cuda_fail(e, "batch unit arrays");
    }
    s->unit_cap = cap;
    return capture_step(s);
}

// (Ray buffers return to the pool of the context that made them; the
// hand-over was made by the steps' context, the tables by admission's.)
void release_job_buffers(rp_server *s, Job *j) {
    if (j->cur) rp_rays_free(j->cur);
    if (j->next) rp_rays_free(j->next);
    if (j->spare) rp_rays_free(j->spare);
    if (j->arena) rp_rays_free(j->arena);
    j->cur = j->next = j->spare = j->arena = nullptr;
    if (j->hand) rp__ctx_free(s->ctx, j->hand, j->hand_bytes);
    if (j->part) rp__ctx_free(s->ctx, j->part, j->part_bytes);
    if (j->mx) rp__ctx_free(s->actx, j->mx, j->mx_bytes);
    j->part = nullptr;
    j->part_cap = 0;
    j->hand = nullptr;
    j->mx = nullptr;
    j->hand_cap = 0;
}

// Admission, on the admission context's stream while the steps run: the
// job's scene and tables on the device and its source rays generated into
// its first generation; done when the stream has finished them.
int admit(rp_server *s, Job *j) {
    rp_ctx *ctx = s->actx;
    j->res.t_start_ms = ms_since(s);
    j->mixed = (j->flags & RP_TRACE_MIXED) != 0;
    int rc = rp_scene_create(ctx, &j->desc, j->wl.empty() ? nullptr : j->wl.data(), (int64_t)j->wl.size(), &j->sc);
    if (rc) return rc;
    if (j->mixed && j->sc->mixed_fallback) {
        rp__set_error("the batched mixed path serves scenes of specialised faces and materials only");
        return RP_ERR_UNSUPPORTED;
    }
    const uint64_t n0 = j->source.n_rays;
    rc = rp_rays_alloc(ctx, n0 ? n0 : 1, &j->cur);
    if (rc) return rc;
    if (j->mixed) {
        j->mx_bytes = batch_tables_bytes(j->sc->S.n_lists, j->sc->S.n_faces);
        rc = rp__ctx_alloc(ctx, &j->mx, j->mx_bytes, &j->mx_bytes);
        if (rc) return rc;
        GenArgs a;
        memset(&a, 0, sizeof a);
        a.S = j->sc->S;
        a.max_len = (double)j->max_length;
        cudaError_t e = launch_batch_tables(a, j->mx, ctx->stream);
        if (e != cudaSuccess) return rp__cuda_fail(e, "batch tables");
    }
    if (n0) {
        SourceArgs A;
        A.out = j->cur->soa;
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
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return rp__cuda_fail(e, "source kernel");
    }
    j->cur->n = n0;
    j->gen = 0;
    j->segments = 0;
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return rp__cuda_fail(e, "admission");
    return RP_OK;
}

void finish_job(rp_server *s, Job *j, int status) {
    j->res.status = status;
    j->res.generations = j->gen;
    j->res.segments = j->segments;
    if (j->sc) {
        j->face_counts.assign(j->desc.n_faces, 0u);
        if (j->desc.n_faces) {
            int rc = rp_scene_face_counts(j->sc, j->face_counts.data(), j->desc.n_faces, 0);
            if (rc && j->res.status == RP_OK) j->res.status = rc;
        }
    }
    if (j->res.status == RP_OK && j->slot >= 0 && j->gen > 0) {
        const double *a = s->h_out->acc[j->slot];
        j->res.detector_hits = (uint64_t)a[0];
        j->res.detector_power = a[1];
        j->res.sum_x = a[2];
        j->res.sum_y = a[3];
        j->res.sum_xx = a[4];
        j->res.sum_yy = a[5];
    }
    release_job_buffers(s, j);
    if (j->sc) {
        rp_scene_destroy(j->sc);
        j->sc = nullptr;
    }
    j->res.t_done_ms = ms_since(s);
    {
        std::lock_guard<std::mutex> lk(s->mu);
        if (j->slot >= 0) s->slots[j->slot] = nullptr;
        s->reserved -= j->est_bytes;
        j->done = true;
    }
    s->cv_done.notify_all();
    s->cv_pending.notify_all();  // a slot and budget are free for admission
}

// Buffer `b` with room for `need` records: kept when it has it, else replaced
// by one with a quarter more room (a job's generations grow by splitting, so
// its buffers are re-allocated only a few times in its life).
int ensure_rays(rp_ctx *ctx, rp_rays **b, uint64_t need) {
    uint64_t cap = 0;
    if (*b) rp_rays_capacity(*b, &cap);
    if (*b && cap >= need) return RP_OK;
    if (*b) rp_rays_free(*b);
    *b = nullptr;
    return rp_rays_alloc(ctx, need + need / 4, b);
}

// A ray buffer's fields from record k on.
RaySoA soa_at(const RaySoA &r, uint64_t k) {
    RaySoA o = r;
    o.ox += k; o.oy += k; o.oz += k; o.dx += k; o.dy += k; o.dz += k;
    o.nx += k; o.ny += k; o.nz += k; o.ex += k; o.ey += k; o.ez += k;
    o.n += k; o.e1 += k; o.e2 += k;
    o.len += k; o.phase += k; o.opl += k;
    o.wl += k; o.parent += k; o.endf += k; o.ident += k; o.type += k;
    return o;
}

// Grows a device block of the steps' context to at least `need` bytes.
int ensure_block(rp_ctx *ctx, void **p, size_t &bytes, size_t &cap, size_t need) {
    if (need <= cap && *p) return RP_OK;
    if (*p) rp__ctx_free(ctx, *p, bytes);
    *p = nullptr;
    cap = 0;
    const size_t want = need + need / 4;
    const int rc = rp__ctx_alloc(ctx, p, want, &bytes);
    if (rc) return rc;
    cap = want;
    return RP_OK;
}

// A job's arguments for this step, with buffers grown as needed.  A mixed
// job's generation is traced in chunks of whole 128-ray groups: this step
// takes j->chunk groups from j->done_units on; the arguments are views of
// the generation's buffers from that point (its rays, hand-over, the next
// generation after the children placed so far), and the children's parent
// index starts at the chunk's first ray.  The next generation (two children
// per ray at most), the hand-over and the per-group tallies are sized for
// the whole generation when it starts; the child-slot arena for the chunk.
// A plain-path job takes its whole generation (its own scan scratch).
int prepare_job(rp_server *s, Job *j, GenArgs &a) {
    rp_ctx *ctx = s->ctx;
    const uint64_t n = j->cur->n;
    const uint64_t units = (n + RP_GROUP - 1) / RP_GROUP;
    const int emit = j->gen + 1 < j->recursion_limit;
    if (!j->mixed) j->chunk = units;
    int rc = RP_OK;
    if (j->done_units == 0) {
        if (emit) {
            rc = ensure_rays(ctx, &j->spare, 2 * n);
            if (rc) return rc;
            j->next = j->spare;
            j->spare = nullptr;
        }
        // mixed: hit hand-over for n rays; plain: counters, sub-tile counts and offsets
        const uint64_t n_sub = rp_n_sub(n);
        const size_t need = j->mixed ? (size_t)rp_hit_bytes(n ? n : 1)
                                     : 64 + align256s(n_sub * 4) + align256s(n_sub * 8) + 256;
        void *h = j->hand;
        rc = ensure_block(ctx, &h, j->hand_bytes, j->hand_cap, need);
        j->hand = (unsigned char *)h;
        if (rc) return rc;
        void *pp = j->part;
        rc = ensure_block(ctx, &pp, j->part_bytes, j->part_cap, (size_t)(units ? units : 1) * RP_TALLY_N * 8);
        j->part = (double *)pp;
        if (rc) return rc;
    }
    if (emit) {
        rc = ensure_rays(ctx, &j->arena, j->chunk * RP_TILE_SLOTS);
        if (rc) return rc;
    }
    const uint64_t r0 = j->done_units * RP_GROUP;
    const uint64_t nc = n - r0 < j->chunk * RP_GROUP ? n - r0 : j->chunk * RP_GROUP;
    memset(&a, 0, sizeof a);
    a.in = soa_at(j->cur->soa, r0);
    a.wb = a.in;
    a.out = emit ? soa_at(j->next->soa, j->next_n) : a.in;
    a.out_cap = emit ? j->next->cap - j->next_n : 0;
    a.n_in = nc;
    a.parent_base = r0;
    a.max_len = (double)j->max_length;
    a.e2_term = j->e2;
    a.emit = emit;
    a.one_list = -1;
    a.one_face = -1;
    a.S = j->sc->S;
    a.smem_tables = j->sc->smem_tables;
    a.mixed_fallback = j->sc->mixed_fallback;
    a.scratch = emit ? j->arena->soa : a.in;
    a.face_counts = j->sc->face_counts;
    a.stats = s->d_dummy;
    if (j->mixed) {
        a.err = s->d_ctr + 2;
        a.unit_rays = RP_GROUP;
        a.hit_t = (float2 *)j->hand + r0;
        a.hit_face = (int *)(j->hand + align256s((size_t)(n ? n : 1) * 8)) + r0;
    } else {
        const uint64_t n_sub = rp_n_sub(n);
        unsigned char *sc = j->hand;
        a.out_count = (unsigned long long *)sc;
        a.err = s->d_ctr + 3;
        a.tile_next = (unsigned *)(sc + 40);
        a.unit_rays = RP_SUB;
        a.tile_counts = (unsigned *)(sc + 64);
        a.tile_offsets = (unsigned long long *)(sc + 64 + align256s(n_sub * 4));
    }
    return RP_OK;
}

// Groups a step traces (4M rays: a few milliseconds of the mixed kernels)
// and the smallest chunk: a step takes every generation that fits in the budget,
// smallest first, then the rest of the budget goes to the earliest-submitted
// of the remaining jobs and at least the minimum chunk to each other one, so
// that a small job's steps are not as long as a large job's generation and
// the large jobs are served in arrival order.
#define RP_STEP_UNITS 32768  // (served stream, 4,000 jobs: p99 50 / 43 / 37 / 35 / 48 ms at 4,096 / 8,192 /
                             //  16,384 / 32,768 groups / unbounded)
#define RP_MIN_CHUNK 1024

// One step: every active job advances one generation.
void run_step(rp_server *s, std::vector<Job *> act) {
    const Clock::time_point t_enter = Clock::now();
    rp_ctx *ctx = s->ctx;
    cudaStream_t st = ctx->stream;
    BatchDev &B = *s->h_batch;
    std::vector<GenArgs> plain_args;
    std::vector<Job *> failed;
    unsigned units = 0;
    int nj = 0;
    {
        // this step's chunks: the mixed jobs by the groups left in their
        // generations, fewest first (then by arrival)
        std::vector<Job *> order;
        for (Job *j : act)
            if (j->mixed) order.push_back(j);
        auto left = [](const Job *j) { return (j->cur->n + RP_GROUP - 1) / RP_GROUP - j->done_units; };
        std::sort(order.begin(), order.end(), [&](const Job *x, const Job *y) {
            return left(x) < left(y) || (left(x) == left(y) && x->id < y->id);
        });
        uint64_t budget, mc;
        {
            std::lock_guard<std::mutex> lk(s->mu);
            budget = s->step_groups;
            mc = s->min_chunk;
        }
        // whole generations that fit, fewest groups first; then the rest of
        // the budget to the earliest-submitted remaining job and at least
        // min_chunk groups to each other one
        std::vector<Job *> big;
        for (Job *j : order) {
            const uint64_t l = left(j);
            if (l <= budget) {
                j->chunk = l;
                budget -= l;
            } else {
                big.push_back(j);
            }
        }
        std::sort(big.begin(), big.end(), [](const Job *x, const Job *y) { return x->id < y->id; });
        for (Job *j : big) {
            const uint64_t l = left(j), c = budget > mc ? budget : mc;
            j->chunk = l < c ? l : c;
            budget = budget > j->chunk ? budget - j->chunk : 0;
        }
    }
    for (Job *j : act) {
        GenArgs a;
        int rc = prepare_job(s, j, a);
        if (rc) {
            failed.push_back(j);
            j->res.status = rc;
            continue;
        }
        BatchJob &J = B.jobs[nj];
        J.a = a;
        J.mx_lists = j->mx;
        // the face table follows the list table (batch_tables_bytes of the lists alone)
        J.mx_faces = j->mx ? static_cast<const unsigned char *>(j->mx) + batch_tables_bytes(j->sc->S.n_lists, 0)
                           : nullptr;
        J.own_count = (!j->mixed && a.emit) ? a.out_count : nullptr;
        J.detector = j->detector;
        J.mixed = j->mixed ? 1 : 0;
        J.slot = j->slot;
        J.first = j->gen == 0;
        const uint64_t gen_units = (j->cur->n + RP_GROUP - 1) / RP_GROUP;
        J.part = j->part + j->done_units * RP_TALLY_N;
        J.part_gen = j->part;
        J.gen_units = gen_units;
        J.gen_done = j->done_units + j->chunk >= gen_units;
        B.unit_start[nj] = units;
        const unsigned ju = (unsigned)((a.n_in + RP_GROUP - 1) / RP_GROUP);
        J.a.tile_counts = nullptr;  // set below, once the unit arrays exist
        if (!j->mixed) {
            plain_args.push_back(a);
            J.a.emit = 0;  // the batch kernels leave a plain job's rays alone
        }
        units += ju;
        nj++;
        act[nj - 1] = j;
    }
    act.resize(nj);
    for (Job *j : failed) finish_job(s, j, j->res.status);
    if (nj == 0) return;
    B.n_jobs = nj;
    B.total_units = units;
    B.unit_start[nj] = units;
    int rc = ensure_units(s, units);
    if (rc) {
        for (Job *j : act) finish_job(s, j, rc);
        return;
    }
    for (int k = 0; k < nj; k++) {
        B.jobs[k].a.tile_counts = s->d_counts + B.unit_start[k];
        B.jobs[k].a.tile_offsets = s->d_offsets + B.unit_start[k];
    }
    // plain-path jobs: their own generation, scan and placement, queued first
    cudaError_t e = cudaEventRecord(s->ev_start, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(s->d_ctr + 3, 0, sizeof(unsigned), st);
    for (size_t p = 0, k = 0; k < (size_t)nj && e == cudaSuccess; k++) {
        if (B.jobs[k].mixed) continue;
        GenArgs &a = plain_args[p++];
        e = cudaMemsetAsync(a.out_count, 0, 64, st);
        if (e == cudaSuccess) e = launch_generation_plain(a, act[k]->sc->smem, st);
        if (e == cudaSuccess && a.emit) e = launch_tile_scan(a, st);
        if (e == cudaSuccess && a.emit) e = launch_place_children(a, st);
    }
    if (e == cudaSuccess) e = cudaGraphLaunch(s->step_exec, st);
    if (e == cudaSuccess) e = cudaEventRecord(s->ev_end, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    float gpu_ms = 0.0f;
    if (e == cudaSuccess) cudaEventElapsedTime(&gpu_ms, s->ev_start, s->ev_end);
    const unsigned err = e == cudaSuccess ? s->h_out->err : 0u;
    for (int k = 0; k < nj; k++) {
        Job *j = act[k];
        const uint64_t n = j->cur->n;
        if (e != cudaSuccess) {
            finish_job(s, j, rp__cuda_fail(e, "batch step"));
            continue;
        }
        if (err & (ERR_WAVELENGTH | ERR_ZK_STACK | ERR_SHAPE_STACK | ERR_OVERFLOW)) {
            rp__set_error("batch step error bits 0x%x", err);
            finish_job(s, j, RP_ERR_INVALID);
            continue;
        }
        const uint64_t r0 = j->done_units * RP_GROUP;
        j->segments += n - r0 < j->chunk * RP_GROUP ? n - r0 : j->chunk * RP_GROUP;
        uint64_t count = s->h_out->count[j->slot];
        if (j->mixed) {
            j->next_n += count;
            j->done_units += j->chunk;
            if (j->done_units < (n + RP_GROUP - 1) / RP_GROUP) continue;  // the generation goes on next step
            count = j->next_n;
            j->done_units = 0;
            j->next_n = 0;
        }
        j->gen++;
        if (j->next && count > 0) {
            j->spare = j->cur;  // reused for the generation after next
            j->cur = j->next;
            j->cur->n = count;
            j->next = nullptr;
        } else {
            finish_job(s, j, RP_OK);
        }
    }
    const double wall = std::chrono::duration<double, std::milli>(Clock::now() - t_enter).count();
    std::lock_guard<std::mutex> lk(s->mu);
    s->stats.steps++;
    s->stats.step_jobs += (uint64_t)nj;
    s->stats.step_gpu_ms += gpu_ms;
    s->stats.step_wall_ms += wall;
}

// The steps: the jobs admitted since the last step join, then every active
// job advances one generation; waits while none is active.
void step_loop(rp_server *s) {
    cudaSetDevice(s->device);
    Clock::time_point t_last = Clock::now();
    bool after_step = false;  // the previous pass ran a step
    for (;;) {
        std::vector<Job *> act;
        {
            std::unique_lock<std::mutex> lk(s->mu);
            // time between the previous step and this one, unless the loop waited for jobs
            if (after_step)
                s->stats.idle_wall_ms += std::chrono::duration<double, std::milli>(Clock::now() - t_last).count();
            for (;;) {
                for (Job *j : s->ready) j->active = true;
                s->ready.clear();
                for (Job *j : s->slots)
                    if (j && j->active) act.push_back(j);
                if (!act.empty()) break;
                if (s->stop && s->pending.empty() && s->admitting == 0) return;
                s->cv_step.wait(lk);
            }
        }
        run_step(s, act);
        t_last = Clock::now();
        after_step = true;
    }
}

// Admission: FIFO, while a slot is free and the budget holds (one job is
// always admitted when none is in flight), each job prepared on the
// admission stream and handed to the steps when ready.
void admit_loop(rp_server *s) {
    cudaSetDevice(s->device);
    for (;;) {
        Job *h = nullptr;
        {
            std::unique_lock<std::mutex> lk(s->mu);
            for (;;) {
                if (!s->pending.empty()) {
                    int free_slot = -1, busy = 0;
                    for (int k = 0; k < s->max_jobs; k++) {
                        if (!s->slots[k] && free_slot < 0) free_slot = k;
                        if (s->slots[k]) busy++;
                    }
                    Job *p = s->pending.front();
                    if (free_slot >= 0 && (busy == 0 || s->reserved + p->est_bytes <= s->budget)) {
                        s->pending.pop_front();
                        p->slot = free_slot;
                        s->slots[free_slot] = p;
                        s->reserved += p->est_bytes;
                        s->admitting++;
                        h = p;
                        break;
                    }
                }
                if (s->stop && s->pending.empty()) return;
                s->cv_pending.wait(lk);
            }
        }
        const int rc = admit(s, h);
        const bool done = rc != RP_OK || h->source.n_rays == 0 || h->recursion_limit <= 0;
        if (done) finish_job(s, h, rc);
        {
            std::lock_guard<std::mutex> lk(s->mu);
            s->admitting--;
            if (!done) s->ready.push_back(h);
        }
        s->cv_step.notify_all();
    }
}

template <class T>
void copy_table(std::vector<T> &dst, const T *src, int32_t n) {
    dst.assign(src && n > 0 ? src : nullptr, src && n > 0 ? src + n : nullptr);
}

void destroy_buffers(rp_server *s) {
    if (s->step_exec) cudaGraphExecDestroy(s->step_exec);
    if (s->ev_start) cudaEventDestroy(s->ev_start);
    if (s->ev_end) cudaEventDestroy(s->ev_end);
    free_unit_arrays(s);
    if (s->d_batch) cudaFree(s->d_batch);
    if (s->d_ctr) cudaFree(s->d_ctr);
    if (s->d_total) cudaFree(s->d_total);
    if (s->d_acc) cudaFree(s->d_acc);
    if (s->h_batch) cudaFreeHost(s->h_batch);
    if (s->h_out) cudaFreeHost(s->h_out);
    if (s->ctx) rp_ctx_destroy(s->ctx);
    if (s->actx) rp_ctx_destroy(s->actx);
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
    if (!out || lanes < 1) return RP_ERR_INVALID;
    *out = nullptr;
    rp_server *s = new (std::nothrow) rp_server();
    if (!s) return RP_ERR_NOMEM;
    s->device = device;
    s->budget = hbm_budget ? hbm_budget : ~(uint64_t)0;
    s->max_jobs = lanes < RP_BATCH_MAX_JOBS ? lanes : RP_BATCH_MAX_JOBS;
    s->step_groups = RP_STEP_UNITS;
    s->min_chunk = RP_MIN_CHUNK;
    s->slots.assign(s->max_jobs, nullptr);
    s->t0 = Clock::now();
    int rc = rp_ctx_create(device, 0, &s->ctx);
    if (rc == RP_OK) rc = rp_ctx_create(device, 0, &s->actx);
    cudaError_t e = cudaSuccess;
    if (rc == RP_OK) {
        e = cudaMallocHost((void **)&s->h_batch, sizeof(BatchDev));
        if (e == cudaSuccess) e = cudaHostAlloc((void **)&s->h_out, sizeof(StepOut), cudaHostAllocMapped);
        if (e == cudaSuccess) e = cudaHostGetDevicePointer((void **)&s->d_out, s->h_out, 0);
        if (e == cudaSuccess) e = cudaMalloc((void **)&s->d_batch, sizeof(BatchDev));
        if (e == cudaSuccess) e = cudaMalloc((void **)&s->d_ctr, RP_BATCH_WORDS * sizeof(unsigned));
        if (e == cudaSuccess) e = cudaMalloc((void **)&s->d_total, 4 * sizeof(unsigned long long));
        if (e == cudaSuccess) e = cudaMalloc((void **)&s->d_acc, RP_BATCH_MAX_JOBS * RP_TALLY_N * sizeof(double));
        if (e == cudaSuccess) e = cudaEventCreate(&s->ev_start);
        if (e == cudaSuccess) e = cudaEventCreate(&s->ev_end);
        if (e != cudaSuccess) rc = rp__cuda_fail(e, "server buffers");
    }
    if (rc == RP_OK) {
        memset(s->h_batch, 0, sizeof(BatchDev));
        memset(s->h_out, 0, sizeof(StepOut));
        s->d_dummy = s->d_total + 2;
        rc = ensure_units(s, 4096);
    }
    if (rc) {
        destroy_buffers(s);
        delete s;
        return rc;
    }
    s->loop = std::thread(step_loop, s);
    s->admit_th = std::thread(admit_loop, s);
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

int rp_server_set_step_groups(rp_server *s, uint32_t groups, uint32_t min_chunk) {
    if (!s || groups < 1 || min_chunk < 1) return RP_ERR_INVALID;
    std::lock_guard<std::mutex> lk(s->mu);
    s->step_groups = groups;
    s->min_chunk = min_chunk;
    return RP_OK;
}

int rp_server_get_stats(rp_server *s, rp_server_stats *out) {
    if (!s || !out) return RP_ERR_INVALID;
    std::lock_guard<std::mutex> lk(s->mu);
    *out = s->stats;
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
    if (s->admit_th.joinable()) s->admit_th.join();
    s->cv_step.notify_all();
    if (s->loop.joinable()) s->loop.join();
    for (auto &kv : s->jobs) delete kv.second;
    destroy_buffers(s);
    delete s;
    return RP_OK;
}

}  // extern "C"
