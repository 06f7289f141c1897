// rp_mixed.cu -- mixed FP32/FP64 generation kernel (placeholder until built).
#include "rp_kernels.cuh"

namespace rp {
cudaError_t launch_generation_mixed(const GenArgs &a, size_t smem, cudaStream_t st) {
    (void)a; (void)smem; (void)st;
    return cudaErrorNotSupported;
}
}  // namespace rp
