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
// Taps by value (kernel parameters): concurrent calls share no state.
struct FilterTaps {
    float w[kMaxTaps];
};

// One CTA filters one series at a time (grid-stride over series).  Shared
// memory holds the padded period P[k] = h_ext[k - pad], k < n, extended
// circularly by R on both sides: S[i] = P[(i - R) mod n], i < n + 2R, so
//     out[t] = sum_{j=0}^{2R} taps[j] * S[t + pad + 2R - j]
// is the circular correlation the padded FFTs compute.
// Every thread produces Q = 8 consecutive outputs.  It keeps two windows of
// Q values of S in registers (ping-pong: the window that served the high half
// of one block of Q taps serves the low half of the next) and adds tap J + s
// to output q from window slot Q + q - s: one 32-byte row of S per Q taps for
// Q * Q FMAs.  Each output still sums its taps in order j = 0..2R; the taps
// are zero-padded to a multiple of 2Q (zero terms), and S is preceded by F
// zero slots (3Q <= F < 4Q, making S-index + F of every window start a
// multiple of Q) so the last, unused window loads stay in bounds.
// Rows of S are 8 floats; the two 16-byte halves of row k trade places when
// bit 2 of k is set, so the 16-byte loads of 8 consecutive threads (8
// consecutive rows) fall in 8 different bank groups.
constexpr int kFilterQ = 8;

// 8k + 4 (half ^ bit 2 of k): bit 2 of 8k is clear, so OR and XOR compose.
__device__ __forceinline__ int srow_addr(int k, int half) { return ((k << 3) | (k & 4)) ^ (half << 2); }

__device__ __forceinline__ void srow_load(const float* sh, int k, float (&v)[kFilterQ]) {
    const float4 a = *reinterpret_cast<const float4*>(sh + srow_addr(k, 0));
    const float4 b = *reinterpret_cast<const float4*>(sh + srow_addr(k, 1));
    v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
    v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
}

// acc[q] += t[st] * window slot (Q + q - st), slots [0, Q) in lo, [Q, 2Q) in hi.
__device__ __forceinline__ void filter_block(const float* t, const float (&lo)[kFilterQ], const float (&hi)[kFilterQ],
                                             float (&acc)[kFilterQ]) {
    constexpr int Q = kFilterQ;
#pragma unroll
    for (int st = 0; st < Q; ++st)
#pragma unroll
        for (int q = 0; q < Q; ++q) {
            const int m = Q + q - st;
            acc[q] = fmaf(m < Q ? lo[m] : hi[m - Q], t[st], acc[q]);
        }
}

// Taps J .. J + Q - 1 from the shared copy (two 16-byte loads).
__device__ __forceinline__ void filter_block_shared(const float* s_taps, int J, const float (&lo)[kFilterQ],
                                                    const float (&hi)[kFilterQ], float (&acc)[kFilterQ]) {
    const float4 ta = *reinterpret_cast<const float4*>(s_taps + J);
    const float4 tb = *reinterpret_cast<const float4*>(s_taps + J + 4);
    const float t[kFilterQ] = {ta.x, ta.y, ta.z, ta.w, tb.x, tb.y, tb.z, tb.w};
    filter_block(t, lo, hi, acc);
}

// NJ > 0: exactly NJ blocks of 2Q taps, unrolled, each FMA reading its tap
// from the kernel parameters (constant bank; zero past the last tap).
// NJ == 0: any tap count, taps from the shared copy.
template <int NJ>
__global__ void __launch_bounds__(128) filter_h_kernel(float* __restrict__ data, uint64_t nseries, uint32_t T, int n,
                                                       int R, int pad, int edge, int F, int ntp, int rows,
                                                       const __grid_constant__ FilterTaps taps) {
    constexpr int Q = kFilterQ;
    extern __shared__ __align__(16) float sh[];  // taps (ntp, zero-padded), then `rows` rows of S
    const int E = n + 2 * R;
    const int ntaps = 2 * R + 1;
    float* s_taps = sh;
    float* sser = sh + ntp;
    for (int j = threadIdx.x; j < ntp; j += blockDim.x) s_taps[j] = j < ntaps ? taps.w[j] : 0.f;
    for (uint64_t s = blockIdx.x; s < nseries; s += gridDim.x) {
        float* h = data + s * T;
        // Fill one 16-byte half row (four consecutive slots) per thread and
        // step.  Slots before S[0] and past S[E - 1] are zero; a slot whose
        // signal index falls outside [0, T) takes the clamped border sample
        // (edge) or zero, so every load is in bounds and unconditional.
        for (int g = threadIdx.x; g < 2 * rows; g += blockDim.x) {
            float v[4];
#pragma unroll
            for (int b = 0; b < 4; ++b) {
                const int i = 4 * g + b - F;  // S index
                int k = i - R;                // circular index: -R <= k < n + R for i in [0, E), R < n
                k += k < 0 ? n : 0;
                k -= k >= n ? n : 0;
                const int u = k - pad;  // signal index
                const float x = h[min(max(u, 0), (int)T - 1)];
                const bool keep = i >= 0 && i < E && (edge || (u >= 0 && u < (int)T));
                v[b] = keep ? x : 0.f;
            }
            *reinterpret_cast<float4*>(sser + srow_addr(g >> 1, g & 1)) = make_float4(v[0], v[1], v[2], v[3]);
        }
        __syncthreads();
        for (int t0 = threadIdx.x * Q; t0 < (int)T; t0 += blockDim.x * Q) {
            // out[t0 + q] = sum_j taps[j] * S[b0 - j + q], b0 = t0 + pad + 2R; in slots
            // b = b0 + F (a multiple of Q), window of block J: slots b - J - Q .. b - J + Q.
            const int kb = (t0 + pad + 2 * R + F) >> 3;  // row of slot b
            float A[Q], B[Q], acc[Q];
            srow_load(sser, kb - 1, A);
            srow_load(sser, kb, B);
#pragma unroll
            for (int q = 0; q < Q; ++q) acc[q] = 0.f;
            if constexpr (NJ > 0) {
#pragma unroll
                for (int jj = 0; jj < NJ; ++jj) {
                    const int k = kb - 2 * jj;  // kb - J / Q with J = 2Q jj
                    filter_block(taps.w + 2 * Q * jj, A, B, acc);
                    srow_load(sser, k - 2, B);  // low window of block J + Q
                    filter_block(taps.w + 2 * Q * jj + Q, B, A, acc);
                    srow_load(sser, k - 3, A);  // low window of block J + 2Q
                }
            } else {
                for (int J = 0; J < ntp; J += 2 * Q) {
                    const int k = kb - (J >> 3);
                    filter_block_shared(s_taps, J, A, B, acc);
                    srow_load(sser, k - 2, B);  // low window of block J + Q
                    filter_block_shared(s_taps, J + Q, B, A, acc);
                    srow_load(sser, k - 3, A);  // low window of block J + 2Q
                }
            }
#pragma unroll
            for (int q = 0; q < Q; ++q)
                if (t0 + q < (int)T) h[t0 + q] = acc[q];
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
    FilterTaps tp{};
    for (size_t j = 0; j < taps.size(); ++j) tp.w[j] = taps[j];
    constexpr int Q = kFilterQ;
    const int ntp = (2 * R + 1 + 2 * Q - 1) / (2 * Q) * (2 * Q);
    if (ntp > kMaxTaps) return set_error(FBP_ERR_UNSUPPORTED, "filter_H: filter longer than the tap table");
    // F zero slots before S: 3Q <= F < 4Q with (pad + 2R + F) % Q == 0.
    const int F = 3 * Q + (Q - (pad + 2 * R + 3 * Q) % Q) % Q;
    // Highest slot read: t0 + pad + 2R + F + Q - 1 with t0 <= T - 1 (< E + F + Q).
    const int rows = (n + 2 * R + F + Q) / Q + 1;
    const size_t smem = ((size_t)ntp + (size_t)Q * rows) * sizeof(float);
    if (smem > (size_t)ctx->smem_optin) return set_error(FBP_ERR_UNSUPPORTED, "filter_H: series too long for one CTA");
    const unsigned blocks = (unsigned)std::min<uint64_t>(nseries, (uint64_t)ctx->sm_count * 16);
    auto go = [&](auto kernel) -> fbp_status {
        FBP_TRY_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        kernel<<<blocks, 128, smem, stream>>>(data, nseries, T, n, R, pad, border == FBP_BORDER_EDGE, F, ntp, rows, tp);
        FBP_CHECK_LAUNCH(ctx, "filter_h_kernel");
        return FBP_OK;
    };
    // Unrolled forms for 2 .. 12 blocks of 16 taps (wavelengths of about 2
    // to 20 bins; 10 bins, the reference's default, gives 107 taps = 7 blocks).
    switch (ntp / (2 * Q)) {
        case 2: return go(filter_h_kernel<2>);
        case 3: return go(filter_h_kernel<3>);
        case 4: return go(filter_h_kernel<4>);
        case 5: return go(filter_h_kernel<5>);
        case 6: return go(filter_h_kernel<6>);
        case 7: return go(filter_h_kernel<7>);
        case 8: return go(filter_h_kernel<8>);
        case 9: return go(filter_h_kernel<9>);
        case 10: return go(filter_h_kernel<10>);
        case 11: return go(filter_h_kernel<11>);
        case 12: return go(filter_h_kernel<12>);
        default: return go(filter_h_kernel<0>);
    }
}

}  // namespace fbp

using namespace fbp;

extern "C" fbp_status fbp_filter_h(fbp_context* ctx, float* data, uint64_t num_series, uint32_t num_bins, float delta_t,
                                   float wl_mean, float wl_sigma, int border, void* stream) {
    return guarded("fbp_filter_h", [&]() -> fbp_status {
        clear_error();
        FBP_TRY(check_ctx(ctx));
        if (!data || num_series == 0 || num_bins == 0) return set_error(FBP_ERR_INVALID_ARG, "fbp_filter_h: empty input");
        if (!(delta_t > 0.f) || !(wl_mean > 0.f)) return set_error(FBP_ERR_INVALID_ARG, "fbp_filter_h: delta_t and wl_mean must be > 0");
        if (border != FBP_BORDER_ZERO && border != FBP_BORDER_EDGE)
            return set_error(FBP_ERR_INVALID_ARG, "fbp_filter_h: unknown border mode");
        return filter_h_device(ctx, data, num_series, num_bins, delta_t, wl_mean, wl_sigma, border, (cudaStream_t)stream);
    });
}
