// Shared-memory radix-2 line FFTs (see fft.cuh) and their host launcher.
#include "fft.cuh"

#include <cmath>
#include <vector>

namespace fbp {

constexpr int kFftThreads = 256;
constexpr int kFftSmemElems = 8192;  // complex elements per CTA (64 KiB)

int fft_lines_per_cta(int log2n) {
    const int n = 1 << log2n;
    return n >= kFftSmemElems ? 1 : kFftSmemElems / n;
}

fbp_status fft_twiddles(fbp_context* ctx, int log2n, cudaStream_t stream, const float2** out) {
    if (log2n < 1 || log2n > 15) return set_error(FBP_ERR_UNSUPPORTED, "FFT length must be 2..32768");
    if (!ctx->twiddles[log2n]) {
        const int n = 1 << log2n;
        std::vector<float2> h(n / 2);
        for (int k = 0; k < n / 2; ++k) {
            const double a = -2.0 * M_PI * (double)k / (double)n;
            h[k] = make_float2((float)std::cos(a), (float)std::sin(a));
        }
        void* d = nullptr;
        FBP_TRY_CUDA(cudaMalloc(&d, h.size() * sizeof(float2)));
        FBP_TRY_CUDA(cudaMemcpyAsync(d, h.data(), h.size() * sizeof(float2), cudaMemcpyHostToDevice, stream));
        FBP_TRY_CUDA(cudaStreamSynchronize(stream));  // h is a host temporary
        ctx->twiddles[log2n] = d;
    }
    *out = static_cast<const float2*>(ctx->twiddles[log2n]);
    return FBP_OK;
}

__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// In-place radix-2 DIT over C lines of n points held bit-reversed in x.
template <bool INV>
__device__ __forceinline__ void fft_stages(float2* x, const float2* tw, int log2n, int C) {
    const int n = 1 << log2n, half_n = n >> 1;
    for (int s = 0; s < log2n; ++s) {
        const int half = 1 << s;
        for (int b = threadIdx.x; b < C * half_n; b += blockDim.x) {
            const int line = b >> (log2n - 1);
            const int bb = b & (half_n - 1);
            const int pos = bb & (half - 1);
            const int i0 = ((bb >> s) << (s + 1)) + pos;
            float2 w = tw[pos << (log2n - 1 - s)];
            if (INV) w.y = -w.y;
            float2* xl = x + line * n;
            const float2 u = xl[i0];
            const float2 v = cmul(xl[i0 + half], w);
            xl[i0] = make_float2(u.x + v.x, u.y + v.y);
            xl[i0 + half] = make_float2(u.x - v.x, u.y - v.y);
        }
        __syncthreads();
    }
}

__device__ __forceinline__ int bitrev(int j, int log2n) { return (int)(__brev((unsigned)j) >> (32 - log2n)); }

// buildLoGKernel3D (transient_postprocessing.cuh:116-148) at full-grid index (x, y, z).
__device__ __forceinline__ float log_response(int x, int y, int z, int nx, int ny, int nz, float sigma) {
    const float fx = (x <= nx / 2) ? (float)x : (float)(x - nx);
    const float fy = (y <= ny / 2) ? (float)y : (float)(y - ny);
    const float fz = (z <= nz / 2) ? (float)z : (float)(z - nz);
    const float fxn = fx / nx, fyn = fy / ny, fzn = fz / nz;
    const float k2 = fxn * fxn + fyn * fyn + fzn * fzn;
    const float pi = 3.14159265358979323846f;
    return -4.0f * pi * pi * k2 * expf(-2.0f * pi * pi * sigma * sigma * k2);
}

template <int MODE, int LOAD, int STORE, int MUL>
__global__ void __launch_bounds__(kFftThreads) fft_lines_kernel(FftLineParams p) {
    extern __shared__ float2 sh[];
    const int log2n = p.log2n, n = 1 << log2n, C = p.lines;
    float2* x = sh;                 // [C][n]
    float2* tw = sh + (size_t)C * n;  // [n/2]
    for (int k = threadIdx.x; k < n / 2; k += blockDim.x) tw[k] = p.tw[k];
    const long long base = (long long)blockIdx.y * p.outer_stride + (long long)blockIdx.x * C * p.line_step;
    const bool contig = p.elem_stride == 1;

    // Load (bit-reversed placement).
    for (int idx = threadIdx.x; idx < C * n; idx += blockDim.x) {
        const int i = contig ? idx / n : idx % C;
        const int j = contig ? idx % n : idx / C;
        const long long off = base + (long long)i * p.line_step + (long long)j * p.elem_stride;
        float2 v;
        if (LOAD == LOAD_COMPLEX) {
            v = p.data[off];
        } else if (LOAD == LOAD_REAL) {
            v = make_float2(p.real_in[off], 0.f);
        } else {  // LOAD_RESAMPLE: row z' = blockIdx.y, y = blockIdx.x * C + i
            v = make_float2(0.f, 0.f);
            const int zp = blockIdx.y, y = blockIdx.x * C + i;
            if (j < p.n_valid && y < p.rs_ns) {
                float acc = 0.f;
                for (int k = p.rs_rowptr[zp]; k < p.rs_rowptr[zp + 1]; ++k) {
                    const int z = p.rs_col[k];
                    float g = 1.f;
                    if (p.rs_power > 0) {
                        const int gi = p.rs_grid_tiled ? (int)(((long long)z * p.rs_ns + y) % p.rs_m) : z;
                        const float lin = p.rs_m > 1 ? (float)((double)gi / (double)(p.rs_m - 1)) : 0.f;
                        const float l2 = lin * lin;
                        g = p.rs_power == 4 ? l2 * l2 : l2;
                    }
                    acc = fmaf(p.rs_val[k] * g, p.rs_src[z * p.rs_sz + y * p.rs_sy + j * p.rs_sx], acc);
                }
                v.x = acc;
            }
        }
        x[i * n + bitrev(j, log2n)] = v;
    }
    __syncthreads();
    fft_stages<MODE == FFT_INVERSE>(x, tw, log2n, C);

    if (MODE == FFT_FWD_MUL_INV) {
        for (int idx = threadIdx.x; idx < C * n; idx += blockDim.x) {
            const int i = idx / n, j = idx % n;
            const long long off = base + (long long)i * p.line_step + (long long)j * p.elem_stride;
            float2 m;
            if (MUL == MUL_ARRAY) {
                m = p.mul[off];
            } else {
                // Position of this element in the nx*ny*nz grid (x fastest).
                const long long e = off;
                const int gx = (int)(e % p.nx), gy = (int)((e / p.nx) % p.ny), gz = (int)(e / ((long long)p.nx * p.ny));
                m = make_float2(log_response(gx, gy, gz, p.nx, p.ny, p.nz, p.sigma), 0.f);
            }
            x[idx] = cmul(x[idx], m);
        }
        __syncthreads();
        // Back to bit-reversed order for the inverse transform.
        for (int idx = threadIdx.x; idx < C * n; idx += blockDim.x) {
            const int i = idx / n, j = idx % n, r = bitrev(j, log2n);
            if (j < r) {
                const float2 t = x[i * n + j];
                x[i * n + j] = x[i * n + r];
                x[i * n + r] = t;
            }
        }
        __syncthreads();
        fft_stages<true>(x, tw, log2n, C);
    }

    for (int idx = threadIdx.x; idx < C * n; idx += blockDim.x) {
        const int i = contig ? idx / n : idx % C;
        const int j = contig ? idx % n : idx / C;
        const long long off = base + (long long)i * p.line_step + (long long)j * p.elem_stride;
        const float2 v = x[i * n + j];
        if (STORE == STORE_COMPLEX) p.data[off] = make_float2(v.x * p.scale, v.y * p.scale);
        else p.real_out[off] = v.x * p.scale;
    }
}

template <int MODE, int LOAD, int STORE, int MUL>
static fbp_status fft_go(fbp_context* ctx, const FftLineParams& p, unsigned gx, unsigned gy, cudaStream_t stream) {
    const int n = 1 << p.log2n;
    const size_t smem = ((size_t)p.lines * n + n / 2) * sizeof(float2);
    auto k = fft_lines_kernel<MODE, LOAD, STORE, MUL>;
    FBP_TRY_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k<<<dim3(gx, gy), kFftThreads, smem, stream>>>(p);
    FBP_CHECK_LAUNCH(ctx, "fft_lines_kernel");
    return FBP_OK;
}

fbp_status fft_launch(fbp_context* ctx, const FftLineParams& p, int mode, int load, int store, int mul,
                      unsigned inner_blocks, unsigned outer_count, cudaStream_t stream) {
    if (inner_blocks == 0 || outer_count == 0) return FBP_OK;
    if (outer_count > 65535) return set_error(FBP_ERR_UNSUPPORTED, "FFT: too many outer lines");
#define FBP_FFT_CASE(M, L, S, U) \
    if (mode == M && load == L && store == S && mul == U) return fft_go<M, L, S, U>(ctx, p, inner_blocks, outer_count, stream);
    FBP_FFT_CASE(FFT_FORWARD, LOAD_COMPLEX, STORE_COMPLEX, MUL_NONE)
    FBP_FFT_CASE(FFT_INVERSE, LOAD_COMPLEX, STORE_COMPLEX, MUL_NONE)
    FBP_FFT_CASE(FFT_FORWARD, LOAD_REAL, STORE_COMPLEX, MUL_NONE)
    FBP_FFT_CASE(FFT_FORWARD, LOAD_RESAMPLE, STORE_COMPLEX, MUL_NONE)
    FBP_FFT_CASE(FFT_INVERSE, LOAD_COMPLEX, STORE_REAL, MUL_NONE)
    FBP_FFT_CASE(FFT_FWD_MUL_INV, LOAD_COMPLEX, STORE_COMPLEX, MUL_ARRAY)
    FBP_FFT_CASE(FFT_FWD_MUL_INV, LOAD_COMPLEX, STORE_COMPLEX, MUL_LOG)
#undef FBP_FFT_CASE
    return set_error(FBP_ERR_UNSUPPORTED, "FFT: unsupported kernel variant");
}

// ------------------------------------------------------- LoG in frequency --

static int ilog2_exact(uint32_t v) {
    if (v == 0 || (v & (v - 1))) return -1;
    int l = 0;
    while ((1u << l) < v) ++l;
    return l;
}

// LoGFFT::compute (PostprocessingFilters.cu:36-77): out = unnormalised
// inverse FFT of FFT(in) * LoG(k), done as full complex transforms of the real
// volume (equal to the reference's R2C/C2R pair for this real, symmetric
// response).  x-forward (real in), y-forward, z-forward * response * z-inverse,
// y-inverse, x-inverse (real part out).
fbp_status launch_log_fft(fbp_context* ctx, const float* in, float* out, uint32_t nx, uint32_t ny, uint32_t nz,
                          float sigma, cudaStream_t stream) {
    const int lx = ilog2_exact(nx), ly = ilog2_exact(ny), lz = ilog2_exact(nz);
    if (lx < 1 || ly < 1 || lz < 1 || lx > 12 || ly > 12 || lz > 12)
        return set_error(FBP_ERR_UNSUPPORTED, "LoG-FFT filter: sizes must be powers of two in [2, 4096]");
    void* buf = nullptr;
    FBP_TRY(workspace(ctx, WS_FFT_A, (size_t)nx * ny * nz * sizeof(float2), stream, &buf));
    FftLineParams p{};
    p.data = static_cast<float2*>(buf);
    p.scale = 1.f;
    p.nx = nx; p.ny = ny; p.nz = nz;
    p.sigma = sigma;
    // x axis: lines are rows (z, y); C rows per CTA along y.
    {
        p.log2n = lx;
        p.lines = std::min<int>(fft_lines_per_cta(lx), ny);
        FBP_TRY(fft_twiddles(ctx, lx, stream, &p.tw));
        p.elem_stride = 1; p.line_step = nx; p.outer_stride = (long long)nx * ny;
        p.real_in = in;
        FBP_TRY(fft_launch(ctx, p, FFT_FORWARD, LOAD_REAL, STORE_COMPLEX, MUL_NONE, cdiv(ny, p.lines), nz, stream));
    }
    // y axis: lines (z, x); C adjacent x per CTA.
    {
        p.log2n = ly;
        p.lines = std::min<int>(fft_lines_per_cta(ly), nx);
        FBP_TRY(fft_twiddles(ctx, ly, stream, &p.tw));
        p.elem_stride = nx; p.line_step = 1; p.outer_stride = (long long)nx * ny;
        FBP_TRY(fft_launch(ctx, p, FFT_FORWARD, LOAD_COMPLEX, STORE_COMPLEX, MUL_NONE, cdiv(nx, p.lines), nz, stream));
    }
    // z axis: lines (y, x); forward, response, inverse in one pass.
    {
        p.log2n = lz;
        p.lines = std::min<int>(fft_lines_per_cta(lz), nx);
        FBP_TRY(fft_twiddles(ctx, lz, stream, &p.tw));
        p.elem_stride = (long long)nx * ny; p.line_step = 1; p.outer_stride = nx;
        FBP_TRY(fft_launch(ctx, p, FFT_FWD_MUL_INV, LOAD_COMPLEX, STORE_COMPLEX, MUL_LOG, cdiv(nx, p.lines), ny, stream));
    }
    {
        p.log2n = ly;
        p.lines = std::min<int>(fft_lines_per_cta(ly), nx);
        FBP_TRY(fft_twiddles(ctx, ly, stream, &p.tw));
        p.elem_stride = nx; p.line_step = 1; p.outer_stride = (long long)nx * ny;
        FBP_TRY(fft_launch(ctx, p, FFT_INVERSE, LOAD_COMPLEX, STORE_COMPLEX, MUL_NONE, cdiv(nx, p.lines), nz, stream));
    }
    {
        p.log2n = lx;
        p.lines = std::min<int>(fft_lines_per_cta(lx), ny);
        FBP_TRY(fft_twiddles(ctx, lx, stream, &p.tw));
        p.elem_stride = 1; p.line_step = nx; p.outer_stride = (long long)nx * ny;
        p.real_out = out;
        FBP_TRY(fft_launch(ctx, p, FFT_INVERSE, LOAD_COMPLEX, STORE_REAL, MUL_NONE, cdiv(ny, p.lines), nz, stream));
    }
    return FBP_OK;
}

}  // namespace fbp
