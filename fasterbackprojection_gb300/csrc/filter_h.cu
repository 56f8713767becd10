// Temporal band-pass filter of every scan point's histogram.
//
// Replaces Laser::filter_H_cuda (Laser.cu:128-240), padIntensity (:80-126)
// and multiplyHK (fourier.cuh:17-31).  The reference pads each histogram by
// t6sigma - 1 bins on both sides, runs a batched complex FFT of length
// n = T + 2(t6sigma - 1), multiplies by the FFT of an ifft-shifted complex
// Gaussian-windowed wave K, inverse-transforms without the 1/n factor and
// keeps the real part of the unpadded bins.  For a real input that equals
//     out[t] = n * sum_u h_ext[u] * Re(K_shift[(t - u) mod n])
// with h_ext the padded signal, so the filter here is a direct real
// correlation with n * Re(K_shift) taps, truncated where the taps fall below
// 1e-12 of the largest (the Gaussian envelope makes the rest negligible).
// No FFT, no host round trip, the filter runs in place on device data.
#include "fbp_internal.cuh"

#include <cmath>
#include <vector>

namespace fbp {

constexpr int kMaxTaps = 2048;
__constant__ float c_filter_taps[kMaxTaps];

// One CTA filters one series at a time (grid-stride over series).  Shared
// memory holds the padded period P[k] = h_ext[k - pad], k < n, extended
// circularly by R on both sides: S[i] = P[(i - R) mod n], i < n + 2R, so
//     out[t] = sum_{j=0}^{2R} taps[j] * S[t + pad + 2R - j]
// is the circular correlation the padded FFTs compute.
__global__ void filter_h_kernel(float* __restrict__ data, uint64_t nseries, uint32_t T, int n, int R, int pad,
                                int edge) {
    extern __shared__ float sh[];  // n + 2R floats
    const int E = n + 2 * R;
    for (uint64_t s = blockIdx.x; s < nseries; s += gridDim.x) {
        float* h = data + s * T;
        const float first = h[0], last = h[T - 1];
        for (int i = threadIdx.x; i < E; i += blockDim.x) {
            int k = (i - R) % n;
            if (k < 0) k += n;
            const int u = k - pad;  // signal index
            float v;
            if (u >= 0 && u < (int)T) v = h[u];
            else if (edge) v = u < 0 ? first : last;
            else v = 0.f;
            sh[i] = v;
        }
        __syncthreads();
        for (int t = threadIdx.x; t < (int)T; t += blockDim.x) {
            float acc = 0.f;
            const float* hp = sh + t + pad + 2 * R;
            for (int j = 0; j <= 2 * R; ++j) acc = fmaf(hp[-j], c_filter_taps[j], acc);
            h[t] = acc;
        }
        __syncthreads();
    }
}

// Host: the taps of filter_H (Laser.cu:131-172) in double precision.
// Returns R (taps cover lags -R..R), the padding, and n.
fbp_status filter_h_taps(uint32_t nt, float delta_t, float wl_mean, float wl_sigma, std::vector<float>& taps, int& R,
                         int& pad, int& n_out) {
    // Laser.cu:131-139, in float like the reference.
    float sig_f = wl_sigma;
    if (std::fabs(wl_sigma - 0.0f) < 1.19209290e-07f) sig_f = wl_mean / std::sqrt(2.0f);
    const double sigma = sig_f;
    int t6 = (int)std::round(6.0f * sig_f / delta_t);
    if (t6 % 2 == 1) t6 += 1;
    if (t6 < 1) return set_error(FBP_ERR_INVALID_ARG, "filter_H: wavelength too short for the bin width");
    const int n = (int)nt + 2 * (t6 - 1);
    pad = t6 - 1;
    n_out = n;
    const double dt = delta_t;
    const double tmax = dt * (n - 1);
    std::vector<double> env(n);
    double envsum = 0.0;
    for (int i = 0; i < n; ++i) {
        const double v = (i * dt - tmax * 0.5) / sigma;
        env[i] = std::exp(-(v * v) * 0.5);
        envsum += env[i];
    }
    // Re(K_shift[m]) = Re(K[(m + n/2) % n]); lag delta uses index delta mod n.
    auto kr = [&](long m) {
        const long idx = (m % n + n) % n;
        const long src = (idx + n / 2) % n;
        const double phase = 2.0 * M_PI * (src * dt) / (double)wl_mean;
        return env[src] * std::cos(phase) / envsum;
    };
    // Lags are circular over the padded period: |lag| <= n/2 covers them all.
    double kmax = 0.0;
    for (int m = -n / 2; m <= n / 2; ++m) kmax = std::max(kmax, std::fabs(kr(m)));
    int r = 0;
    for (int m = 1; m <= n / 2; ++m)
        if (std::fabs(kr(m)) > 1e-12 * kmax || std::fabs(kr(-m)) > 1e-12 * kmax) r = m;
    if (2 * r + 1 > kMaxTaps) return set_error(FBP_ERR_UNSUPPORTED, "filter_H: filter longer than 2047 taps");
    R = r;
    taps.assign(2 * r + 1, 0.f);
    for (int j = 0; j <= 2 * r; ++j) taps[j] = (float)((double)n * kr(j - r));
    return FBP_OK;
}

fbp_status filter_h_device(fbp_context* ctx, float* data, uint64_t nseries, uint32_t T, float delta_t, float wl_mean,
                           float wl_sigma, int border, cudaStream_t stream) {
    std::vector<float> taps;
    int R = 0, pad = 0, n = 0;
    FBP_TRY(filter_h_taps(T, delta_t, wl_mean, wl_sigma, taps, R, pad, n));
    FBP_TRY_CUDA(cudaMemcpyToSymbolAsync(c_filter_taps, taps.data(), taps.size() * sizeof(float), 0,
                                         cudaMemcpyHostToDevice, stream));
    const size_t smem = (size_t)(n + 2 * R) * sizeof(float);
    if (smem > (size_t)ctx->smem_optin) return set_error(FBP_ERR_UNSUPPORTED, "filter_H: series too long for one CTA");
    FBP_TRY_CUDA(cudaFuncSetAttribute(filter_h_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const unsigned blocks = (unsigned)std::min<uint64_t>(nseries, (uint64_t)ctx->sm_count * 8);
    filter_h_kernel<<<blocks, 256, smem, stream>>>(data, nseries, T, n, R, pad, border == FBP_BORDER_EDGE);
    FBP_CHECK_LAUNCH(ctx, "filter_h_kernel");
    return FBP_OK;
}

}  // namespace fbp

using namespace fbp;

extern "C" fbp_status fbp_filter_h(fbp_context* ctx, float* data, uint64_t num_series, uint32_t num_bins, float delta_t,
                                   float wl_mean, float wl_sigma, int border, void* stream) {
    clear_error();
    FBP_TRY(check_ctx(ctx));
    if (!data || num_series == 0 || num_bins == 0) return set_error(FBP_ERR_INVALID_ARG, "fbp_filter_h: empty input");
    if (!(delta_t > 0.f) || !(wl_mean > 0.f)) return set_error(FBP_ERR_INVALID_ARG, "fbp_filter_h: delta_t and wl_mean must be > 0");
    if (border != FBP_BORDER_ZERO && border != FBP_BORDER_EDGE)
        return set_error(FBP_ERR_INVALID_ARG, "fbp_filter_h: unknown border mode");
    return filter_h_device(ctx, data, num_series, num_bins, delta_t, wl_mean, wl_sigma, border, (cudaStream_t)stream);
}
