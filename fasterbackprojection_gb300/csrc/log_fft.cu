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

// ---------------------------------------------- 256-point lines in registers
// A 256-point line as 16 x 16 (the four-step factorisation, n = n1 + 16 n2,
// k = k1 + 16 k2): the line's 16 threads each hold v[n2] = x[n1 + 16 n2], take
// a 16-point DFT over n2 in registers, multiply by w256^(n1 k1), trade values
// through shared memory once (a transposition), and take a 16-point DFT over
// n1; the thread then holds v[k2] = X[n1 + 16 k2].  The same holds for the
// inverse, so a forward and an inverse transform chain without reordering.
// Shared-memory traffic is one write and one read per element per transform,
// against one per element per Stockham pass plus the staging of the lines.
constexpr int kFsRow = 17;                  // a scratch row: 16 values + 1 pad
constexpr int kFsLine = 16 * kFsRow + 1;    // a line's scratch (odd: conflict-free across lines)
constexpr int kFsTw = 16 + 256;             // the stage tables of n = 256 (radix 16, 16)

template <bool INV>
__device__ __forceinline__ void fs256(float2 (&v)[16], float2* s, int n1, const float2* tw) {
    dft16<INV>(v);
#pragma unroll
    for (int k1 = 1; k1 < 16; ++k1) {
        float2 w = tw[16 + k1 * 16 + n1];  // second stage table: entry jm * 16 + k = w256^(jm k)
        if (INV) w.y = -w.y;
        v[k1] = cmul(v[k1], w);
    }
#pragma unroll
    for (int k1 = 0; k1 < 16; ++k1) s[k1 * kFsRow + n1] = v[k1];
    __syncthreads();
#pragma unroll
    for (int m = 0; m < 16; ++m) v[m] = s[n1 * kFsRow + m];
    __syncthreads();  // the scratch is free again
    dft16<INV>(v);
}

// Pass 1 for nx = 256: thread (line i = row pair, n1); loads straight from
// the rows, the half spectra split after one more exchange.
__global__ void __launch_bounds__(kLogNT) log_x_r2c256_kernel(LogFftParams p) {
    __shared__ float2 tw[kFsTw];
    __shared__ float2 scratch[16 * kFsLine];
    for (int e = threadIdx.x; e < kFsTw; e += kLogNT) tw[e] = p.tw[e];
    const int n1 = threadIdx.x & 15, i = threadIdx.x >> 4;
    const int z = blockIdx.y, pr = blockIdx.x * 16 + i;
    const bool ok = pr < p.ny / 2;
    const float* ra = p.in + ((size_t)z * p.ny + 2 * (size_t)pr) * 256;
    float2 v[16];
#pragma unroll
    for (int n2 = 0; n2 < 16; ++n2)
        v[n2] = ok ? make_float2(ra[n1 + 16 * n2], ra[256 + n1 + 16 * n2]) : make_float2(0.f, 0.f);
    __syncthreads();  // tw
    float2* s = scratch + i * kFsLine;
    fs256<false>(v, s, n1, tw);
#pragma unroll
    for (int k2 = 0; k2 < 16; ++k2) s[k2 * kFsRow + n1] = v[k2];
    __syncthreads();
    if (!ok) return;
    float2* sp = p.spec + ((size_t)z * p.ny + 2 * (size_t)pr) * p.hn;
#pragma unroll
    for (int k2 = 0; k2 <= 8; ++k2) {
        const int k = n1 + 16 * k2, km = (256 - k) & 255;
        if (k > 128) continue;
        const float2 a = v[k2], b = s[(km >> 4) * kFsRow + (km & 15)];
        // Z = A + iB with A, B the rows' spectra; conj(Z[-k]) = A - iB at k.
        sp[k] = make_float2(0.5f * (a.x + b.x), 0.5f * (a.y - b.y));
        sp[p.hn + k] = make_float2(0.5f * (a.y + b.y), 0.5f * (b.x - a.x));
    }
}

// Passes 2-4 for lines of 256: thread (kx offset i, n1), so each load and
// store of a warp covers 16 adjacent kx of two lines.
template <int MODE>
__global__ void __launch_bounds__(kLogNT) log_strided256_kernel(LogFftParams p, long long es, long long outer) {
    __shared__ float2 tw[kFsTw];
    __shared__ float2 scratch[16 * kFsLine];
    for (int e = threadIdx.x; e < kFsTw; e += kLogNT) tw[e] = p.tw[e];
    const int i = threadIdx.x & 15, n1 = threadIdx.x >> 4;
    const int kx0 = blockIdx.x * 16, o = blockIdx.y;
    const bool ok = kx0 + i < p.hn;
    float2* base = p.spec + (size_t)o * outer + kx0 + i;
    float2 v[16];
#pragma unroll
    for (int n2 = 0; n2 < 16; ++n2) v[n2] = ok ? base[(n1 + 16 * n2) * es] : make_float2(0.f, 0.f);
    __syncthreads();  // tw
    float2* s = scratch + i * kFsLine;
    fs256<MODE == 1>(v, s, n1, tw);
    if (MODE == 2) {
#pragma unroll
        for (int k2 = 0; k2 < 16; ++k2) {
            const float r = log_response(kx0 + i, o, n1 + 16 * k2, p.nx, p.ny, p.nz, p.sigma);
            v[k2] = make_float2(v[k2].x * r, v[k2].y * r);
        }
        fs256<true>(v, s, n1, tw);
    }
    if (ok) {
#pragma unroll
        for (int k2 = 0; k2 < 16; ++k2) base[(n1 + 16 * k2) * es] = v[k2];
    }
}

// Pass 5 for nx = 256: each row pair's full spectrum rebuilt from the half
// while loading (Z = X_a + i X_b, conjugate symmetry above N/2).
__global__ void __launch_bounds__(kLogNT) log_x_c2r256_kernel(LogFftParams p) {
    __shared__ float2 tw[kFsTw];
    __shared__ float2 scratch[16 * kFsLine];
    for (int e = threadIdx.x; e < kFsTw; e += kLogNT) tw[e] = p.tw[e];
    const int n1 = threadIdx.x & 15, i = threadIdx.x >> 4;
    const int z = blockIdx.y, pr = blockIdx.x * 16 + i;
    const bool ok = pr < p.ny / 2;
    const float2* sp = p.spec + ((size_t)z * p.ny + 2 * (size_t)pr) * p.hn;
    float2 v[16];
#pragma unroll
    for (int n2 = 0; n2 < 16; ++n2) {
        const int k = n1 + 16 * n2, kk = k <= 128 ? k : 256 - k;
        float2 zk = make_float2(0.f, 0.f);
        if (ok) {
            const float2 xa = sp[kk], xb = sp[p.hn + kk];
            zk = k <= 128 ? make_float2(xa.x - xb.y, xa.y + xb.x) : make_float2(xa.x + xb.y, xb.x - xa.y);
        }
        v[n2] = zk;
    }
    __syncthreads();  // tw
    fs256<true>(v, scratch + i * kFsLine, n1, tw);
    if (!ok) return;
    float* out = p.out + ((size_t)z * p.ny + 2 * (size_t)pr) * 256;
#pragma unroll
    for (int k2 = 0; k2 < 16; ++k2) {
        out[n1 + 16 * k2] = v[k2].x;
        out[256 + n1 + 16 * k2] = v[k2].y;
    }
}

fbp_status log_pass256(fbp_context* ctx, int kind, const LogFftParams& p, cudaStream_t s) {
    const unsigned xg = cdiv(p.ny / 2, 16), cg = cdiv(p.hn, 16);
    switch (kind) {
        case 0:
            log_x_r2c256_kernel<<<dim3(xg, p.nz), kLogNT, 0, s>>>(p);
            FBP_CHECK_LAUNCH(ctx, "log_x_r2c256_kernel");
            return FBP_OK;
        case 4:
            log_x_c2r256_kernel<<<dim3(xg, p.nz), kLogNT, 0, s>>>(p);
            FBP_CHECK_LAUNCH(ctx, "log_x_c2r256_kernel");
            return FBP_OK;
        case 1:
        case 3:
            if (kind == 1) log_strided256_kernel<0><<<dim3(cg, p.nz), kLogNT, 0, s>>>(p, p.hn, (long long)p.ny * p.hn);
            else log_strided256_kernel<1><<<dim3(cg, p.nz), kLogNT, 0, s>>>(p, p.hn, (long long)p.ny * p.hn);
            FBP_CHECK_LAUNCH(ctx, "log_strided256_kernel");
            return FBP_OK;
        default:
            log_strided256_kernel<2><<<dim3(cg, p.ny), kLogNT, 0, s>>>(p, (long long)p.ny * p.hn, p.hn);
            FBP_CHECK_LAUNCH(ctx, "log_strided256_kernel");
            return FBP_OK;
    }
}

// One pass of the given kind for axis length 2^log2n.
// kind 0: x r2c, 1: y forward, 2: z forward * LoG * inverse, 3: y inverse, 4: x c2r.
template <int LOG2N>
fbp_status log_pass(fbp_context* ctx, int kind, LogFftParams p, cudaStream_t s) {
    constexpr int C = log_lines(LOG2N);
    constexpr size_t smem = log_smem<LOG2N>();
    FBP_TRY(stage_twiddles(ctx, LOG2N, s, &p.tw));
    if constexpr (LOG2N == 8) {
        static_assert(stage_table_size(8) == kFsTw && stage_radix_bits(8, 0) == 4 && stage_radix_bits(8, 4) == 4,
                      "the register path reads the radix-16 stage tables of n = 256");
        return log_pass256(ctx, kind, p, s);
    }
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
