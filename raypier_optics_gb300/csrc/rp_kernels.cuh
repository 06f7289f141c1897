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

// Tile status words of the decoupled look-back scan: flag in the top 2 bits.
#define RP_TILE_AGG (1ull << 62)
#define RP_TILE_PREFIX (2ull << 62)
#define RP_TILE_VALUE_MASK ((1ull << 62) - 1)

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
    unsigned *tile_counter;       // ticket counter (zeroed before launch)
    unsigned long long *tile_state;
    unsigned long long *out_count;  // total children (written by the last tile)
    unsigned *err;                  // error bits
    unsigned *face_counts;          // per face record hit counters
    unsigned long long *stats;      // [0] hits, [1] terminated children
};

#define RP_BLOCK 128

// launchers (rp_trace.cu / rp_mixed.cu); return cudaError_t
cudaError_t launch_generation_plain(const GenArgs &a, size_t smem, cudaStream_t st);
cudaError_t launch_generation_mixed(const GenArgs &a, size_t smem, cudaStream_t st);
cudaError_t launch_aos_to_soa(const void *aos, RaySoA soa, unsigned long long n, cudaStream_t st);
cudaError_t launch_soa_to_aos(RaySoA soa, void *aos, unsigned long long n, cudaStream_t st);
cudaError_t launch_dispersion_table(const rp_dispersion *curves, int n_curves, const double *aux,
                                    const double *wl, long long n_wl, double2 *ntab, cudaStream_t st);
size_t generation_smem_bytes(int n_lists, int n_recs, int n_mats, int n_faces);

}  // namespace rp
