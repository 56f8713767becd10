// Placeholder for the FFT-based paths until the radix kernels land.
#include "fbp_internal.cuh"
namespace fbp {
fbp_status launch_log_fft(fbp_context*, const float*, float*, uint32_t, uint32_t, uint32_t, float, cudaStream_t) {
    return set_error(FBP_ERR_UNSUPPORTED, "LoG-FFT filter not built");
}
}  // namespace fbp
