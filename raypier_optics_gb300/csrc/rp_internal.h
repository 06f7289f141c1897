// rp_internal.h -- definitions shared by the C-ABI translation units
// (rp_api.cu: contexts, scenes, rays, tracing; rp_serve.cu: the job server).
// Not part of the public header.
#pragma once
#include <cuda_runtime.h>

#include <cstdarg>
#include <mutex>
#include <vector>

#include "../../include/rp_gb300.h"
#include "rp_kernels.cuh"

using namespace rp;

struct PoolBlock {
    void *p;
    size_t bytes;
};

struct rp_ctx {
    int device;
    cudaStream_t stream;
    uint64_t budget;
    uint64_t in_use;                 // bytes of live allocations
    std::vector<PoolBlock> pool;     // freed blocks kept for reuse
    uint64_t pooled;                 // bytes in `pool`
    std::mutex pool_mu;              // the pool and the byte counts (a buffer may be freed from another thread)
    std::vector<cudaEvent_t> gen_ev; // per-generation kernel events (pairs)
    struct rp_rays *arena;           // child slots of the generation being traced
    struct rp_rays *arena2;          // trace_rays: the other arena (one is read while the other is written)
    unsigned *child_map[2];          // trace_rays: gather maps of the next generation (alternating)
    uint64_t child_map_cap[2];
    size_t child_map_bytes[2];
    // per-generation scratch: [out_count | err | pad | stats[2] | tile counter | pad | tile counts, offsets]
    unsigned char *scratch;
    size_t scratch_bytes;
    unsigned long long *h_pinned;  // 8 words of pinned host memory for small read-backs
    unsigned long long *d_pinned;  // h_pinned's device address (kernels store to it directly)
    cudaEvent_t ev0, ev1;
    cudaStream_t copy_stream;      // downloads that overlap the next generation (created on first use)
};

struct rp_scene {
    rp_ctx *ctx;
    DevScene S;               // device pointers
    void *dev_block;          // one allocation holding every table
    size_t dev_bytes;
    unsigned *face_counts;    // per face record
    int n_faces;
    size_t smem;              // bytes of tables staged per block
    int smem_tables;
    int mixed_fallback;       // faces or materials the mixed kernel leaves to its FP64 code
    const rp_dispersion *disp;  // device copy of the dispersion curve table
    int n_disp;
    std::vector<rp_face> host_faces;
    std::vector<rp_facelist> host_lists;
};

// A device gausslet collection: base rays plus the parabasal rays' fields,
// field f of parabasal ray j of gausslet i at para[(j * RP_PARA_FIELDS + f) * cap + i].
struct rp_gausslets {
    rp_ctx *ctx;
    struct rp_rays *base;  // base rays; base->n is the gausslet count
    double *para;          // RP_PARA_ARRAYS arrays of cap doubles
    size_t para_bytes;
    uint64_t cap;
};

struct rp_rays {
    rp_ctx *ctx;
    uint64_t cap, n;
    void *block;
    size_t bytes;
    RaySoA soa;
};


// helpers implemented in rp_api.cu
int rp__ctx_alloc(rp_ctx *ctx, void **p, size_t bytes, size_t *got);
void rp__ctx_free(rp_ctx *ctx, void *p, size_t bytes);
int rp__cuda_fail(cudaError_t e, const char *what);
void rp__set_error(const char *fmt, ...);
// The mixed path's child-slot unit and per-ray hand-over (search -> material
// kernel) carved from a generation scratch block laid out as [64-byte
// counters | n_sub u32 counts | n_sub u64 offsets | rp_hit_bytes(n_sub * 32)],
// each part 256-byte aligned; the plain path keeps the sub-tile unit.
extern "C" void rp__set_mixed_handover(GenArgs &a, uint32_t flags, unsigned char *sc, uint64_t n_sub);
