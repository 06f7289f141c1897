// rp_kernels.cuh -- kernel-side data layout and launch interface shared by the
// plain and mixed generation kernels and the host API.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "rp_device.cuh"

namespace rp {

// Structure-of-arrays ray storage: one array per scalar field of ray_t
// (raypier/core/ctracer.pxd:40-48); complex fields are double2 (re, im).
struct RaySoA {
    double *ox, *oy, *oz, *dx, *dy, *dz, *nx, *ny, *nz, *ex, *ey, *ez;
    double2 *n, *e1, *e2;
    double *len, *phase, *opl;
    unsigned *wl, *parent, *endf, *ident, *type;
};

// Child placement works on sub-tiles of RP_SUB rays (one warp): sub-tile q
// owns RP_SUB_SLOTS consecutive slots of a scratch ray arena (two per ray).
// The generation kernel writes the sub-tile's children to the front of that
// range in parent order (warp scan of the per-ray counts) and their number to
// tile_counts[q]; once every sub-tile's total is known (tile scan) the
// placement kernel copies each sub-tile's children to their final, contiguous
// place, or (the generation loop of trace_rays) the child-map kernel records
// each child's slot so that the next generation reads it from there (see
// GenArgs::in_map).  No ray, warp or block waits for another.  Blocks are RP_BLOCK
// threads, so a block covers RP_BLOCK / RP_SUB sub-tiles (RP_TILE_SLOTS slots).
#define RP_BLOCK 128
#define RP_TILE_SLOTS (2 * RP_BLOCK)
#define RP_SUB 32
#define RP_SUB_SLOTS (2 * RP_SUB)
#define RP_SUB_PER_BLOCK (RP_BLOCK / RP_SUB)
__host__ __device__ inline unsigned long long rp_n_sub(unsigned long long n_rays) { return (n_rays + RP_SUB - 1) / RP_SUB; }
// The mixed path places children by groups of RP_GROUP rays (RP_TILE_SLOTS
// slots each): its material kernel compacts the rays of a group that produce
// children into full warps.  The plain path's unit is the sub-tile.
#define RP_GROUP RP_BLOCK
__host__ __device__ inline unsigned long long rp_n_units(unsigned long long n_rays, int unit_rays) {
    const unsigned long long u = unit_rays > 0 ? (unsigned long long)unit_rays : RP_SUB;
    return (n_rays + u - 1) / u;
}

struct GenArgs {
    RaySoA in, out;
    unsigned long long n_in;      // rays [0, n_in) of `in` are traced
    unsigned long long out_cap;   // children go to out[0, out_cap)
    double max_len;               // (double)(float)max_length
    double e2_term;               // drop children with |E1|^2+|E2|^2 < e2_term (if > 0)
    int emit;                     // 0: count hits only (last generation of trace_rays)
    int one_list, one_face;       // >= 0: sequential trace of one face of one list
    DevScene S;                   // global-memory tables
    int smem_tables;              // 1: lists/faces/materials staged in shared memory
    int mixed_fallback;           // mixed kernel: the scene has faces / materials only its FP64 code handles
    RaySoA scratch;                 // child slots: RP_SUB_SLOTS per sub-tile
    unsigned *tile_counts;          // [n_sub] children of each sub-tile
    unsigned long long *tile_offsets;  // [n_sub] exclusive prefix (scan kernel)
    unsigned long long *out_count;  // total children (scan kernel)
    unsigned *err;                  // error bits
    unsigned *face_counts;          // per face record hit counters
    unsigned long long *stats;      // [0] hits, [1] terminated children
    unsigned *tile_next;            // next sub-tile to trace (kernels that loop over them; zeroed per launch)
    // Gathered input (the generation loop of trace_rays): when in_map is set,
    // ray g of the generation is slot in_map[g] of `in` (the previous
    // generation's child arena), and the kernel writes its complete record,
    // with length and end face, to wb[g]; the children's parent index is g.
    // Otherwise `in` holds the rays at [0, n_in) and length and end face are
    // written there.
    const unsigned *in_map;
    RaySoA wb;
    // Child-slot unit: 0 or RP_SUB (a sub-tile of one warp, 2 * RP_SUB slots)
    // or RP_GROUP (the mixed path: RP_TILE_SLOTS slots); tile_counts and
    // tile_offsets then hold one entry per unit.
    int unit_rays;
    // The mixed path's hand-over from its search kernel to its material
    // kernel, per ray: the ray parameter of the hit (float-float hi, lo) and
    // the hit face record (-1: none); and the material kernel's group counter.
    float2 *hit_t;
    int *hit_face;
    unsigned *group_next;
    // Added to the children's parent index: the first ray of the part of a
    // generation these arguments cover (the job server traces a large
    // generation in chunks); 0 otherwise.
    unsigned long long parent_base;
};
// ---- batches of trace jobs (the job server, rp_serve.cu) ----
// One generation of every job of a batch runs in one launch of each mixed
// kernel: the jobs' 128-ray groups are numbered consecutively across the
// batch (job j owns global units [unit_start[j], unit_start[j + 1])), warps
// take global sub-tiles or groups from the batch's counters, and each item
// runs with its job's generation arguments and tables, read from global
// memory.  A job's rays stay in place in its own buffers (no gather map).
#define RP_BATCH_MAX_JOBS 64
struct BatchJob {
    GenArgs a;            // the job's generation: in place (in = wb); its arena, hand-over and count views
    const void *mx_lists; // its float / float-float list and face tables (mixed kernels)
    const void *mx_faces;
    const unsigned long long *own_count;  // plain-path job keeping children: the count of its own tile scan
    int detector;         // Face.idx whose hits are tallied, -1 for none
    int mixed;            // 1: traced by the batch kernels; 0: by its own plain-path launches
    int slot;             // the job's server slot (tally accumulators, results)
    int first;            // 1 on the job's first generation (its accumulators start from zero)
    // Detector tallies: per unit of the job's whole generation (part_gen,
    // gen_units units); `part` is the entry of the step's first unit.  The
    // step that completes the generation (gen_done) sums them in a fixed
    // order, however the generation was split into steps.
    double *part;
    const double *part_gen;
    unsigned long long gen_units;
    int gen_done;
};
struct BatchDev {
    int n_jobs;
    unsigned total_units;
    unsigned unit_start[RP_BATCH_MAX_JOBS + 1];
    BatchJob jobs[RP_BATCH_MAX_JOBS];
};
// counters of a batch step, zeroed before it: [0] next sub-tile, [1] next group, [2] error bits
#define RP_BATCH_WORDS 8
// The batch's job owning global unit u (the last job whose first unit is <= u).
__device__ __forceinline__ int batch_job_of(const BatchDev *B, unsigned u) {
    int lo = 0, hi = B->n_jobs - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (B->unit_start[mid] <= u)
            lo = mid;
        else
            hi = mid - 1;
    }
    return lo;
}
// mixed-path kernels over a batch (rp_mixed.cu); the jobs' scenes use only
// faces and materials the mixed kernels specialise, and the tables of each job
// are filled once by launch_batch_tables
cudaError_t prepare_batch_mixed(size_t *search_smem, size_t *mat_smem, int *search_blocks, int *mat_blocks);
cudaError_t launch_batch_mixed(const BatchDev *batch, unsigned *ctr, cudaStream_t st);
size_t batch_tables_bytes(int n_lists, int n_faces);
cudaError_t launch_batch_tables(const GenArgs &a, void *tables, cudaStream_t st);
// the unit count scan with the unit count read from device memory
cudaError_t launch_tile_scan_dev(const unsigned *counts, const unsigned *n_dev, unsigned long long *offsets,
                                 unsigned long long *total, cudaStream_t st);

// Bytes of per-ray hand-over storage (hit_t, hit_face) the mixed path needs
// for n rays, each array on a 256-byte boundary.
__host__ __device__ constexpr unsigned long long rp_hit_bytes(unsigned long long n) {
    return ((n * 8 + 255) & ~255ull) + ((n * 4 + 255) & ~255ull);
}

// launchers (rp_trace.cu / rp_mixed.cu); return cudaError_t
cudaError_t launch_generation_plain(const GenArgs &a, size_t smem, cudaStream_t st);
// (the mixed path: the search kernel, then, when children are kept, the
// material kernel; `mid`, if given, is recorded between the two)
cudaError_t launch_generation_mixed(const GenArgs &a, size_t smem, cudaStream_t st, cudaEvent_t mid = nullptr);
// one-time per-configuration set-up (attributes, occupancy), so that a following
// launch of the same configuration can be stream-captured
cudaError_t prepare_generation_plain(const GenArgs &a, size_t smem);
cudaError_t prepare_generation_mixed(const GenArgs &a, size_t smem);
// unit count scan (one block) and the scatter of children to their final
// slots (one warp per unit); the unit count is rp_n_units(a.n_in, a.unit_rays)
cudaError_t launch_tile_scan(const GenArgs &a, cudaStream_t st);
cudaError_t launch_place_children(const GenArgs &a, cudaStream_t st);
// exclusive prefix of n unsigned counts (one block) and their total
cudaError_t launch_count_scan(const unsigned *counts, unsigned long long n, unsigned long long *offsets,
                              unsigned long long *total, cudaStream_t st);
// the gather map of the children instead of their copy: map[offset + j] = the
// arena slot of the sub-tile's child j (the next generation reads through it)
cudaError_t launch_child_map(const GenArgs &a, unsigned *map, unsigned long long map_cap, cudaStream_t st);
// at most 32 words: a copy by SM stores (dst may be mapped host memory) and a clear
cudaError_t launch_copy_words(const unsigned long long *src, unsigned long long *dst, int n, cudaStream_t st);
cudaError_t launch_zero_words(unsigned long long *dst, int n, cudaStream_t st);
cudaError_t launch_aos_to_soa(const void *aos, RaySoA soa, unsigned long long n, cudaStream_t st);
cudaError_t launch_soa_to_aos(RaySoA soa, void *aos, unsigned long long n, cudaStream_t st);
cudaError_t launch_dispersion_table(const rp_dispersion *curves, int n_curves, const double *aux,
                                    const double *wl, long long n_wl, double2 *ntab, cudaStream_t st);
size_t generation_smem_bytes(int n_lists, int n_recs, int n_mats, int n_faces);

// ---- Gausslets (rp_gausslet.cu) ----
// Parabasal ray j's field f (0-2 origin, 3-5 direction, 6-8 normal, 9 length)
// of gausslet i lives at para[(j * RP_PARA_FIELDS + f) * cap + i].
#define RP_PARA_FIELDS 10
#define RP_PARA_ARRAYS (6 * RP_PARA_FIELDS)
struct GaussArgs {
    GenArgs g;                       // base rays: in, child slots, output, as for a ray generation
    double *pin;                     // parabasal rays of the input (lengths of those tested are updated)
    unsigned long long pin_cap;
    double *pscratch;                // parabasal rays of the child slots
    unsigned long long pscratch_cap;
    double *pout;                    // parabasal rays of the output
    unsigned long long pout_cap;
    int *captured;                   // [n_in] 1 + material of a decomposition material that captured it (or null)
};
cudaError_t launch_gausslet_generation(const GaussArgs &a, size_t smem, cudaStream_t st);
cudaError_t launch_gausslet_place(const GaussArgs &a, unsigned long long n_sub, cudaStream_t st);
cudaError_t launch_capture(const GaussArgs &a, unsigned wl_offset, int with_para, size_t smem, cudaStream_t st);
cudaError_t launch_gausslet_aos_to_soa(const void *aos, RaySoA soa, double *para, unsigned long long cap,
                                       unsigned long long n, cudaStream_t st);
cudaError_t launch_gausslet_soa_to_aos(RaySoA soa, const double *para, unsigned long long cap, void *aos,
                                       unsigned long long n, cudaStream_t st);
// config_parabasal_rays: host-evaluated constants of the three ray pairs
struct ParabasalConfig {
    double rc[3], rs[3];  // radius * cos, radius * sin of the angle 2 pi k / 3
    double c[3], s[3];    // cos, sin of that angle
    double kt;            // pi * radius * 1000 (theta0 = wavelength / kt)
    double wd;            // working distance
};
cudaError_t launch_parabasal_config(RaySoA base, double *para, unsigned long long cap, unsigned long long n,
                                    const double *wl, long long n_wl, const ParabasalConfig &P, unsigned *err,
                                    cudaStream_t st);
#define RP_POWER_BLOCK 256
cudaError_t launch_power_partials(RaySoA base, unsigned long long n, double *partial, cudaStream_t st);

// ---- differentiable sequential lens (rp_lens.cu) ----
struct LensArgs {
    int n_surf;                 // aspheric surfaces; faces[n_surf] is the image plane
    const rp_face *faces;       // [n_surf + 1]
    const double *nidx;         // [n_surf + 1] index before surface 0 and after each surface
    DevScene S;                 // shape table (apertures) for the face functions
    double max_len;             // segment length of the intersection tests
    RaySoA in;                  // input rays (origin, direction)
    unsigned long long n;
    double *img;                // [2 n] image-plane x, y
    unsigned char *valid;       // [n] ray reached the image
    double *part;               // per-block partial sums
    double *gpart;              // [blocks][5 n_surf + 1] per-block gradient sums
    double xm, ym, scale;       // centroid and 1 / (N * loss) for the adjoint
    unsigned *err;
};
cudaError_t launch_lens_forward(const LensArgs &L, cudaStream_t st);
cudaError_t launch_lens_spread(const LensArgs &L, cudaStream_t st);
cudaError_t launch_lens_backward(const LensArgs &L, cudaStream_t st);
unsigned lens_block_count(unsigned long long n);

}  // namespace rp
