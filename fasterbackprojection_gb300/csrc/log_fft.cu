// LoG-FFT filter (LoGFFT::compute, PostprocessingFilters.cu:36-77) on the
// half spectrum of the real volume, with the compile-time Stockham passes of
// fft_lean.cuh.  out = unnormalised inverse FFT of FFT(in) * LoG(k) with the
// response of buildLoGKernel3D (transient_postprocessing.cuh:116-148), real
// and even, so the volume's spectrum keeps its Hermitian symmetry and only
// kx = 0 .. nx/2 is stored (the reference's R2C / C2R layout).  Five passes:
//   1. x, real to complex: rows y and y + 1 of a plane are the real and
//      imaginary parts of one complex FFT; the two half spectra are split
//      from it by symmetry (X_a = (Z + conj Z*) / 2, X_b = (Z - conj Z*) / 2i).
//   2. y forward, 3. z forward * LoG * z inverse, 4. y inverse: strided
//      columns, C adjacent kx per CTA.
//   5. x, complex to real: each row pair's full spectrum is rebuilt from the
//      half (conjugate symmetry) as Z = X_a + i X_b, one inverse FFT gives
//      both rows (real and imaginary parts).
// Every axis a power of two in [32, 1024]; other sizes use the full-complex
// line passes of fft.cu.
#include "fft.cuh"
#include "fft_lean.cuh"

#include <algorithm>

namespace fbp {
namespace {

constexpr int kLogNT = 256;
constexpr int log_lines(int log2n) { return std::min(16, 8192 >> log2n); }

template <int LOG2N>
constexpr size_t log_smem() {
    return ((size_t)log_lines(LOG2N) * line_stride(1 << LOG2N) + stage_table_size(LOG2N)) * sizeof(float2);
}

struct LogFftParams {
    const float* in;
    float* out;
    float2* spec;  // [nz][ny][nx/2 + 1]
    const float2* tw;
    int nx, ny, nz, hn;  // hn = nx/2 + 1
    float sigma;
};

template <int LOG2N>
__device__ __forceinline__ float2* log_stage_table(float2* sm, const float2* tw) {
    constexpr int N = 1 << LOG2N, C = log_lines(LOG2N), LS = line_stride(N), TWN = stage_table_size(LOG2N);
    float2* t = sm + C * LS;
    for (int i = threadIdx.x; i < TWN; i += kLogNT) t[i] = tw[i];
    return t;
}

// Pass 1: row pairs (2 pr, 2 pr + 1) of plane z -> half spectra.
template <int LOG2N>
__global__ void __launch_bounds__(kLogNT) log_x_r2c_kernel(LogFftParams p) {
    constexpr int N = 1 << LOG2N, C = log_lines(LOG2N), LS = line_stride(N), PL = C * N / kLogNT;
    extern __shared__ __align__(16) float2 sm[];
    float2* lines = sm;
    float2* tw = log_stage_table<LOG2N>(sm, p.tw);
    const int z = blockIdx.y, pr0 = blockIdx.x * C, npairs = p.ny / 2;
    const float* plane = p.in + (size_t)z * p.ny * N;
    {
        float2 v[PL];
#pragma unroll
        for (int u = 0; u < PL; ++u) {
            const int e = threadIdx.x + u * kLogNT, i = e / N, j = e % N, pr = pr0 + i;
            v[u] = pr < npairs ? make_float2(plane[(size_t)(2 * pr) * N + j], plane[(size_t)(2 * pr + 1) * N + j])
                               : make_float2(0.f, 0.f);
        }
#pragma unroll
        for (int u = 0; u < PL; ++u) {
            const int e = threadIdx.x + u * kLogNT;
            lines[(e / N) * LS + pidx(e % N)] = v[u];
        }
    }
    __syncthreads();
    lean_fft<LOG2N, 0, C, kLogNT, false, false>(lines, tw, LS);
    float2* sp = p.spec + (size_t)z * p.ny * p.hn;
    for (int e = threadIdx.x; e < C * p.hn; e += kLogNT) {
        const int i = e / p.hn, k = e % p.hn, pr = pr0 + i;
        if (pr >= npairs) continue;
        const float2 a = lines[i * LS + pidx(k)], b = lines[i * LS + pidx((N - k) & (N - 1))];
        // Z = A + iB with A, B the rows' spectra; conj(Z[-k]) = A - iB at k.
        const float2 xa = make_float2(0.5f * (a.x + b.x), 0.5f * (a.y - b.y));
        const float2 xb = make_float2(0.5f * (a.y + b.y), 0.5f * (b.x - a.x));
        sp[(size_t)(2 * pr) * p.hn + k] = xa;
        sp[(size_t)(2 * pr + 1) * p.hn + k] = xb;
    }
}

// Passes 2-4: lines of N points with element stride `es`, C adjacent kx per
// CTA, line outer index blockIdx.y (z for the y lines, y for the z lines).
// MODE 0 forward, 1 inverse, 2 forward * LoG * inverse (z lines).
template <int LOG2N, int MODE>
__global__ void __launch_bounds__(kLogNT) log_strided_kernel(LogFftParams p, long long es, long long outer) {
    constexpr int N = 1 << LOG2N, C = log_lines(LOG2N), LS = line_stride(N), PL = C * N / kLogNT;
    extern __shared__ __align__(16) float2 sm[];
    float2* lines = sm;
    float2* tw = log_stage_table<LOG2N>(sm, p.tw);
    const int kx0 = blockIdx.x * C, o = blockIdx.y;
    float2* base = p.spec + (size_t)o * outer;
    {
        float2 v[PL];
#pragma unroll
        for (int u = 0; u < PL; ++u) {
            const int e = threadIdx.x + u * kLogNT, i = e % C, j = e / C;
            v[u] = kx0 + i < p.hn ? base[j * es + kx0 + i] : make_float2(0.f, 0.f);
        }
#pragma unroll
        for (int u = 0; u < PL; ++u) {
            const int e = threadIdx.x + u * kLogNT;
            lines[(e % C) * LS + pidx(e / C)] = v[u];
        }
    }
    __syncthreads();
    lean_fft<LOG2N, 0, C, kLogNT, MODE == 1, false>(lines, tw, LS);
    if (MODE == 2) {
        for (int e = threadIdx.x; e < C * N; e += kLogNT) {
            const int i = e / N, kz = e % N;
            const float r = log_response(kx0 + i, o, kz, p.nx, p.ny, p.nz, p.sigma);
            float2& c = lines[i * LS + pidx(kz)];
            c = make_float2(c.x * r, c.y * r);
        }
        __syncthreads();
        lean_fft<LOG2N, 0, C, kLogNT, true, false>(lines, tw, LS);
    }
    for (int e = threadIdx.x; e < C * N; e += kLogNT) {
        const int i = e % C, j = e / C;
        if (kx0 + i < p.hn) base[j * es + kx0 + i] = lines[i * LS + pidx(j)];
    }
}

// Pass 5: half spectra of row pairs -> the real rows.
template <int LOG2N>
__global__ void __launch_bounds__(kLogNT) log_x_c2r_kernel(LogFftParams p) {
    constexpr int N = 1 << LOG2N, C = log_lines(LOG2N), LS = line_stride(N);
    extern __shared__ __align__(16) float2 sm[];
    float2* lines = sm;
    float2* tw = log_stage_table<LOG2N>(sm, p.tw);
    const int z = blockIdx.y, pr0 = blockIdx.x * C, npairs = p.ny / 2;
    const float2* sp = p.spec + (size_t)z * p.ny * p.hn;
    for (int e = threadIdx.x; e < C * N; e += kLogNT) {
        const int i = e / N, k = e % N, pr = pr0 + i;
        float2 zk = make_float2(0.f, 0.f);
        if (pr < npairs) {
            const int kk = k <= N / 2 ? k : N - k;
            const float2 xa = sp[(size_t)(2 * pr) * p.hn + kk], xb = sp[(size_t)(2 * pr + 1) * p.hn + kk];
            // Z = X_a + i X_b, with X[k] = conj(X[N - k]) above N/2.
            zk = k <= N / 2 ? make_float2(xa.x - xb.y, xa.y + xb.x) : make_float2(xa.x + xb.y, xb.x - xa.y);
        }
        lines[i * LS + pidx(k)] = zk;
    }
    __syncthreads();
    lean_fft<LOG2N, 0, C, kLogNT, true, false>(lines, tw, LS);
    float* plane = p.out + (size_t)z * p.ny * N;
    for (int e = threadIdx.x; e < C * N; e += kLogNT) {
        const int i = e / N, j = e % N, pr = pr0 + i;
        if (pr >= npairs) continue;
        const float2 v = lines[i * LS + pidx(j)];
        plane[(size_t)(2 * pr) * N + j] = v.x;
        plane[(size_t)(2 * pr + 1) * N + j] = v.y;
    }
}

// One pass of the given kind for axis length 2^log2n.
// kind 0: x r2c, 1: y forward, 2: z forward * LoG * inverse, 3: y inverse, 4: x c2r.
template <int LOG2N>
fbp_status log_pass(fbp_context* ctx, int kind, LogFftParams p, cudaStream_t s) {
    constexpr int C = log_lines(LOG2N);
    constexpr size_t smem = log_smem<LOG2N>();
    FBP_TRY(stage_twiddles(ctx, LOG2N, s, &p.tw));
    const unsigned xg = cdiv(p.ny / 2, C), cg = cdiv(p.hn, C);
    switch (kind) {
        case 0: {
            auto k = log_x_r2c_kernel<LOG2N>;
            FBP_TRY_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
            k<<<dim3(xg, p.nz), kLogNT, smem, s>>>(p);
            FBP_CHECK_LAUNCH(ctx, "log_x_r2c_kernel");
            return FBP_OK;
        }
        case 4: {
            auto k = log_x_c2r_kernel<LOG2N>;
            FBP_TRY_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
            k<<<dim3(xg, p.nz), kLogNT, smem, s>>>(p);
            FBP_CHECK_LAUNCH(ctx, "log_x_c2r_kernel");
            return FBP_OK;
        }
        case 1:
        case 3: {
            auto k = kind == 1 ? log_strided_kernel<LOG2N, 0> : log_strided_kernel<LOG2N, 1>;
            FBP_TRY_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
            k<<<dim3(cg, p.nz), kLogNT, smem, s>>>(p, (long long)p.hn, (long long)p.ny * p.hn);
            FBP_CHECK_LAUNCH(ctx, "log_strided_kernel");
            return FBP_OK;
        }
        default: {
            auto k = log_strided_kernel<LOG2N, 2>;
            FBP_TRY_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
            k<<<dim3(cg, p.ny), kLogNT, smem, s>>>(p, (long long)p.ny * p.hn, (long long)p.hn);
            FBP_CHECK_LAUNCH(ctx, "log_strided_kernel");
            return FBP_OK;
        }
    }
}

int ilog2_pow2(uint32_t v) {
    if (v == 0 || (v & (v - 1))) return -1;
    int l = 0;
    while ((1u << l) < v) ++l;
    return l;
}

fbp_status dispatch(fbp_context* ctx, int log2n, int kind, const LogFftParams& p, cudaStream_t s) {
    switch (log2n) {
        case 5: return log_pass<5>(ctx, kind, p, s);
        case 6: return log_pass<6>(ctx, kind, p, s);
        case 7: return log_pass<7>(ctx, kind, p, s);
        case 8: return log_pass<8>(ctx, kind, p, s);
        case 9: return log_pass<9>(ctx, kind, p, s);
        case 10: return log_pass<10>(ctx, kind, p, s);
        default: return set_error(FBP_ERR_UNSUPPORTED, "LoG-FFT: axis length outside the half-spectrum path");
    }
}

}  // namespace

bool log_fft_half_supported(uint32_t nx, uint32_t ny, uint32_t nz) {
    for (uint32_t n : {nx, ny, nz}) {
        const int l = ilog2_pow2(n);
        if (l < 5 || l > 10) return false;
    }
    return true;
}

fbp_status launch_log_fft_half(fbp_context* ctx, const float* in, float* out, uint32_t nx, uint32_t ny, uint32_t nz,
                               float sigma, cudaStream_t s) {
    LogFftParams p{};
    p.in = in;
    p.out = out;
    p.nx = (int)nx;
    p.ny = (int)ny;
    p.nz = (int)nz;
    p.hn = (int)nx / 2 + 1;
    p.sigma = sigma;
    void* buf = nullptr;
    FBP_TRY(workspace(ctx, WS_FFT_A, (size_t)nz * ny * p.hn * sizeof(float2), s, &buf));
    p.spec = static_cast<float2*>(buf);
    const int lx = ilog2_pow2(nx), ly = ilog2_pow2(ny), lz = ilog2_pow2(nz);
    FBP_TRY(dispatch(ctx, lx, 0, p, s));
    FBP_TRY(dispatch(ctx, ly, 1, p, s));
    FBP_TRY(dispatch(ctx, lz, 2, p, s));
    FBP_TRY(dispatch(ctx, ly, 3, p, s));
    FBP_TRY(dispatch(ctx, lx, 4, p, s));
    return FBP_OK;
}

}  // namespace fbp
