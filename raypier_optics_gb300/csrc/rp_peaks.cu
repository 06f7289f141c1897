// rp_peaks.cu -- measured arithmetic peaks of the device, the denominators of
// the pipe rooflines the benchmark reports next to the HBM one: FP64 and FP32
// fused multiply-add throughput and 32-bit integer multiply-add throughput.
//
// Each thread runs RP_PEAK_CHAINS independent multiply-add chains (enough to
// cover the pipes' latency) for a fixed number of iterations, on a grid of
// several waves of resident blocks; the kernel time comes from CUDA events on
// the launching stream after a warm-up launch, and the best of a few launches
// is kept.  The chains' final values are folded into one store per thread so
// the compiler cannot drop the work.  Compiled without FMA contraction
// changes: the operations are written as explicit fma / integer mad.
#include <cuda_runtime.h>

#include <cstdint>

#include "rp_internal.h"

namespace rp {

#define RP_PEAK_CHAINS 8
#define RP_PEAK_BLOCK 256

template <typename T>
__device__ __forceinline__ T peak_mad(T a, T b, T c);
template <>
__device__ __forceinline__ double peak_mad<double>(double a, double b, double c) { return fma(a, b, c); }
template <>
__device__ __forceinline__ float peak_mad<float>(float a, float b, float c) { return fmaf(a, b, c); }
template <>
__device__ __forceinline__ unsigned peak_mad<unsigned>(unsigned a, unsigned b, unsigned c) { return a * b + c; }

// acc_k <- acc_k * m + a for iters iterations; m and a come from arguments so
// the chains cannot be folded at compile time.
template <typename T>
__global__ void __launch_bounds__(RP_PEAK_BLOCK) peak_kernel(T m, T a, int iters, T *out) {
    T acc[RP_PEAK_CHAINS];
#pragma unroll
    for (int k = 0; k < RP_PEAK_CHAINS; k++) acc[k] = (T)(threadIdx.x + k);
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int k = 0; k < RP_PEAK_CHAINS; k++) acc[k] = peak_mad<T>(acc[k], m, a);
    }
    T s = acc[0];
#pragma unroll
    for (int k = 1; k < RP_PEAK_CHAINS; k++) s = s + acc[k];
    out[(size_t)blockIdx.x * RP_PEAK_BLOCK + threadIdx.x] = s;
}

// Multiply-adds per second of peak_kernel<T> on the current device.
template <typename T>
static int measure(cudaStream_t st, int blocks, int iters, T m, T a, double *rate) {
    T *out = nullptr;
    cudaError_t e = cudaMalloc((void **)&out, (size_t)blocks * RP_PEAK_BLOCK * sizeof(T));
    if (e != cudaSuccess) return rp__cuda_fail(e, "peak buffer");
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    float best = 0.0f;
    for (int rep = 0; rep < 4 && e == cudaSuccess; rep++) {  // the first launch is the warm-up
        e = cudaEventRecord(e0, st);
        if (e == cudaSuccess) {
            peak_kernel<T><<<blocks, RP_PEAK_BLOCK, 0, st>>>(m, a, iters, out);
            e = cudaGetLastError();
        }
        if (e == cudaSuccess) e = cudaEventRecord(e1, st);
        if (e == cudaSuccess) e = cudaEventSynchronize(e1);
        float ms = 0.0f;
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
        if (e == cudaSuccess && rep > 0 && (best == 0.0f || ms < best)) best = ms;
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaFree(out);
    if (e != cudaSuccess) return rp__cuda_fail(e, "peak kernel");
    const double mads = (double)blocks * RP_PEAK_BLOCK * RP_PEAK_CHAINS * (double)iters;
    *rate = best > 0.0f ? mads / (best * 1e-3) : 0.0;
    return RP_OK;
}

}  // namespace rp

extern "C" int rp_measure_peaks(int device, double *fp64_flops, double *fp32_flops, double *int32_ops) {
    if (!fp64_flops || !fp32_flops || !int32_ops) return RP_ERR_INVALID;
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) return rp__cuda_fail(e, "cudaSetDevice");
    int sms = 0, per_sm = 0;
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    if (e == cudaSuccess)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, rp::peak_kernel<double>, RP_PEAK_BLOCK, 0);
    if (e != cudaSuccess) return rp__cuda_fail(e, "device attributes");
    const int blocks = 8 * sms * (per_sm > 0 ? per_sm : 1);  // eight waves of resident blocks
    cudaStream_t st = nullptr;
    e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
    if (e != cudaSuccess) return rp__cuda_fail(e, "stream");
    double r64 = 0, r32 = 0, ri = 0;
    // FP64 runs at a small fraction of the FP32 rate: fewer iterations keep each launch near a few milliseconds
    int rc = rp::measure<double>(st, blocks, 256, 0.999999, 1e-7, &r64);
    if (rc == RP_OK) rc = rp::measure<float>(st, blocks, 8192, 0.9999f, 1e-4f, &r32);
    if (rc == RP_OK) rc = rp::measure<unsigned>(st, blocks, 4096, 1664525u, 1013904223u, &ri);
    cudaStreamDestroy(st);
    if (rc) return rc;
    *fp64_flops = 2.0 * r64;  // a fused multiply-add is two floating-point operations
    *fp32_flops = 2.0 * r32;
    *int32_ops = ri;
    return RP_OK;
}

// Host-link copy rates: one cudaMemcpyAsync of RP_LINK_BYTES between device
// memory and page-locked host memory each way, best of three after a warm-up,
// timed with CUDA events.  The end-to-end entry points move every generation
// over this link, so its rate bounds them.
#define RP_LINK_BYTES ((size_t)256 << 20)

extern "C" int rp_measure_host_link(int device, double *d2h_bytes_per_s, double *h2d_bytes_per_s) {
    if (!d2h_bytes_per_s || !h2d_bytes_per_s) return RP_ERR_INVALID;
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) return rp__cuda_fail(e, "cudaSetDevice");
    void *d = nullptr, *h = nullptr;
    cudaStream_t st = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    e = cudaMalloc(&d, RP_LINK_BYTES);
    if (e == cudaSuccess) e = cudaHostAlloc(&h, RP_LINK_BYTES, cudaHostAllocDefault);
    if (e == cudaSuccess) e = cudaMemset(d, 0, RP_LINK_BYTES);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    float best[2] = {0.0f, 0.0f};
    for (int dir = 0; dir < 2 && e == cudaSuccess; dir++) {
        for (int rep = 0; rep < 4 && e == cudaSuccess; rep++) {  // the first copy is the warm-up
            e = cudaEventRecord(e0, st);
            if (e == cudaSuccess)
                e = dir == 0 ? cudaMemcpyAsync(h, d, RP_LINK_BYTES, cudaMemcpyDeviceToHost, st)
                             : cudaMemcpyAsync(d, h, RP_LINK_BYTES, cudaMemcpyHostToDevice, st);
            if (e == cudaSuccess) e = cudaEventRecord(e1, st);
            if (e == cudaSuccess) e = cudaEventSynchronize(e1);
            float ms = 0.0f;
            if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
            if (e == cudaSuccess && rep > 0 && (best[dir] == 0.0f || ms < best[dir])) best[dir] = ms;
        }
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (st) cudaStreamDestroy(st);
    if (h) cudaFreeHost(h);
    if (d) cudaFree(d);
    if (e != cudaSuccess) return rp__cuda_fail(e, "host link copies");
    *d2h_bytes_per_s = best[0] > 0.0f ? RP_LINK_BYTES / (best[0] * 1e-3) : 0.0;
    *h2d_bytes_per_s = best[1] > 0.0f ? RP_LINK_BYTES / (best[1] * 1e-3) : 0.0;
    return RP_OK;
}
