// Shared-memory radix-2 line FFTs (see fft.cuh) and their host launcher.
#include "fft.cuh"
#include "fft_codelets.cuh"

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

// w^k for k in [0, n) from the half table tw[k] = exp(-2 pi i k / n), k < n/2.
template <bool INV>
__device__ __forceinline__ float2 twiddle(const float2* tw, int k, int half_n) {
    float2 w = k < half_n ? tw[k] : make_float2(-tw[k - half_n].x, -tw[k - half_n].y);
    if (INV) w.y = -w.y;
    return w;
}

// Stockham auto-sort FFT over C lines of n points in shared memory, natural
// order in and out (the radix-R formulation of Govindaraju et al., "High
// performance discrete Fourier transforms on graphics processors", SC 2008):
// a pass with stride Ns reads the R inputs x[j + r n/R] of butterfly j,
// multiplies input r by w^(r (j mod Ns) n / (Ns R)) (w = exp(-2 pi i / n)),
// takes an R-point DFT in registers and writes output k to
// x[(j / Ns) Ns R + (j mod Ns) + k Ns]; Ns grows by R per pass.  Radix-8
// passes, then one radix-4 or radix-2 pass.  Every thread holds at most 32
// complex values (C * n <= 8192 with 256 threads).
template <int R, bool INV>
__device__ __forceinline__ void stockham_pass(float2* x, const float2* tw, int log2n, int ns_log, int C) {
    constexpr int U = 32 / R;
    constexpr int RL = R == 8 ? 3 : (R == 4 ? 2 : 1);
    const int n = 1 << log2n, lb = log2n - RL, nb_line = 1 << lb, nb = C << lb;
    const int Ns = 1 << ns_log, LS = line_stride(n);
    const int tshift = log2n - ns_log - RL;  // n / (Ns R) = 2^tshift
    float2 v[U][R];
#pragma unroll
    for (int u = 0; u < U; ++u) {
        const int b = threadIdx.x + u * (int)blockDim.x;
        if (b < nb) {
            const int line = b >> lb, j = b & (nb_line - 1);
            const float2* xl = x + line * LS;
            const int jm = j & (Ns - 1);
#pragma unroll
            for (int r = 0; r < R; ++r) {
                float2 a = xl[pidx(j + r * nb_line)];
                if (r > 0 && jm > 0) a = cmul(a, twiddle<INV>(tw, (r * jm) << tshift, n >> 1));
                v[u][r] = a;
            }
            if (R == 8) dft8<INV>(v[u]);
            else if (R == 4) dft4<INV>(v[u][0], v[u][1], v[u][2], v[u][3]);
            else dft2<INV>(v[u][0], v[u][1]);
        }
    }
    __syncthreads();
#pragma unroll
    for (int u = 0; u < U; ++u) {
        const int b = threadIdx.x + u * (int)blockDim.x;
        if (b < nb) {
            const int line = b >> lb, j = b & (nb_line - 1);
            float2* xl = x + line * LS;
            const int d = ((j >> ns_log) << (ns_log + RL)) + (j & (Ns - 1));
#pragma unroll
            for (int r = 0; r < R; ++r) xl[pidx(d + r * Ns)] = v[u][r];
        }
    }
    __syncthreads();
}

template <bool INV>
__device__ __forceinline__ void fft_stages(float2* x, const float2* tw, int log2n, int C) {
    int done = 0;
    while (log2n - done >= 3) {
        stockham_pass<8, INV>(x, tw, log2n, done, C);
        done += 3;
    }
    if (log2n - done == 2) stockham_pass<4, INV>(x, tw, log2n, done, C);
    else if (log2n - done == 1) stockham_pass<2, INV>(x, tw, log2n, done, C);
}

// Element j of line i of this CTA's group.
__device__ __forceinline__ long long fft_offset(const FftLineParams& p, long long base, int i, int j) {
    return base + (long long)i * p.line_step + (long long)j * p.elem_stride;
}

template <int MODE, int LOAD, int STORE, int MUL>
__global__ void __launch_bounds__(kFftThreads, 3) fft_lines_kernel(FftLineParams p) {
    extern __shared__ float2 sh[];
    constexpr int EMAX = kFftSmemElems / kFftThreads;  // elements per thread
    const int log2n = p.log2n, n = 1 << log2n, C = p.lines, log2c = p.log2c, total = C * n;
    const int LS = line_stride(n);
    const int nv = p.n_valid > 0 ? p.n_valid : n;  // elements j >= nv are zero (not read)
    const int nst = p.n_store > 0 ? p.n_store : n; // elements j >= nst are not stored
    float2* x = sh;                    // [C][LS], padded lines
    float2* tw = sh + (size_t)C * LS;  // [n/2]
    for (int k = threadIdx.x; k < n / 2; k += blockDim.x) tw[k] = p.tw[k];
    const long long base = (long long)blockIdx.y * p.outer_stride + (long long)blockIdx.x * C * p.line_step;
    const bool contig = p.elem_stride == 1;

    // Load: every thread first issues all its loads (registers), then fills
    // shared memory, so the loads of a thread are in flight together.
    if (LOAD == LOAD_RESAMPLE) {
        // Row z' = blockIdx.y of the operator is the same for the whole CTA:
        // stage its entries, then accumulate every element term by term
        // (all of a term's source loads in flight together).
        constexpr int KMAX = 128;
        __shared__ int s_col[KMAX];
        __shared__ float s_val[KMAX];
        const int zp = blockIdx.y;
        const int k0 = p.rs_rowptr[zp], nk = p.rs_rowptr[zp + 1] - k0;
        for (int t = threadIdx.x; t < min(nk, KMAX); t += blockDim.x) {
            s_col[t] = p.rs_col[k0 + t];
            s_val[t] = p.rs_val[k0 + t];
        }
        __syncthreads();
        constexpr int EG = 8;  // elements per accumulation group
        for (int e0 = 0; e0 < EMAX; e0 += EG) {
            float acc[EG];
#pragma unroll
            for (int e = 0; e < EG; ++e) acc[e] = 0.f;
            for (int k = 0; k < nk; ++k) {
                const int z = k < KMAX ? s_col[k] : p.rs_col[k0 + k];
                const float vk = k < KMAX ? s_val[k] : p.rs_val[k0 + k];
#pragma unroll
                for (int e = 0; e < EG; ++e) {
                    const int idx = threadIdx.x + (e0 + e) * kFftThreads;
                    const int i = contig ? idx >> log2n : idx & (C - 1);
                    const int j = contig ? idx & (n - 1) : idx >> log2c;
                    const int y = blockIdx.x * C + i;
                    if (idx < total && j < nv && y < p.rs_ns) {
                        const float g = p.rs_power > 0 ? p.rs_gtab[p.rs_grid_tiled ? (z * p.rs_ns + y) % p.rs_m : z]
                                                       : 1.f;
                        acc[e] = fmaf(vk * g, p.rs_src[z * p.rs_sz + y * p.rs_sy + j * p.rs_sx], acc[e]);
                    }
                }
            }
#pragma unroll
            for (int e = 0; e < EG; ++e) {
                const int idx = threadIdx.x + (e0 + e) * kFftThreads;
                if (idx < total) {
                    const int i = contig ? idx >> log2n : idx & (C - 1);
                    const int j = contig ? idx & (n - 1) : idx >> log2c;
                    x[i * LS + pidx(j)] = make_float2(acc[e], 0.f);
                }
            }
        }
    } else {
        float2 r[EMAX];
#pragma unroll
        for (int e = 0; e < EMAX; ++e) {
            const int idx = threadIdx.x + e * kFftThreads;
            r[e] = make_float2(0.f, 0.f);
            if (idx < total) {
                const int i = contig ? idx >> log2n : idx & (C - 1);
                const int j = contig ? idx & (n - 1) : idx >> log2c;
                if (j < nv) {
                    if (LOAD == LOAD_COMPLEX) r[e] = p.data[fft_offset(p, base, i, j)];
                    else r[e] = make_float2(p.real_in[fft_offset(p, base, i, j)], 0.f);
                }
            }
        }
#pragma unroll
        for (int e = 0; e < EMAX; ++e) {
            const int idx = threadIdx.x + e * kFftThreads;
            if (idx < total) {
                const int i = contig ? idx >> log2n : idx & (C - 1);
                const int j = contig ? idx & (n - 1) : idx >> log2c;
                x[i * LS + pidx(j)] = r[e];
            }
        }
    }
    __syncthreads();
    fft_stages<MODE == FFT_INVERSE>(x, tw, log2n, C);

    if (MODE == FFT_FWD_MUL_INV) {
        float2 m[EMAX];
#pragma unroll
        for (int e = 0; e < EMAX; ++e) {
            const int idx = threadIdx.x + e * kFftThreads;
            m[e] = make_float2(0.f, 0.f);
            if (idx < total) {
                const int i = contig ? idx >> log2n : idx & (C - 1);
                const int j = contig ? idx & (n - 1) : idx >> log2c;
                const long long off = fft_offset(p, base, i, j);
                if (MUL == MUL_ARRAY) {
                    m[e] = p.mul[off];
                } else {
                    // Position of this element in the nx*ny*nz grid (x fastest).
                    const int gx = (int)(off % p.nx), gy = (int)((off / p.nx) % p.ny),
                              gz = (int)(off / ((long long)p.nx * p.ny));
                    m[e] = make_float2(log_response(gx, gy, gz, p.nx, p.ny, p.nz, p.sigma), 0.f);
                }
            }
        }
#pragma unroll
        for (int e = 0; e < EMAX; ++e) {
            const int idx = threadIdx.x + e * kFftThreads;
            if (idx < total) {
                const int i = contig ? idx >> log2n : idx & (C - 1);
                const int j = contig ? idx & (n - 1) : idx >> log2c;
                x[i * LS + pidx(j)] = cmul(x[i * LS + pidx(j)], m[e]);
            }
        }
        __syncthreads();
        fft_stages<true>(x, tw, log2n, C);
    }

    for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
        const int i = contig ? idx >> log2n : idx & (C - 1);
        const int j = contig ? idx & (n - 1) : idx >> log2c;
        if (j >= nst) continue;
        const long long off = fft_offset(p, base, i, j);
        const float2 v = x[i * LS + pidx(j)];
        if (STORE == STORE_COMPLEX) p.data[off] = make_float2(v.x * p.scale, v.y * p.scale);
        else p.real_out[off] = v.x * p.scale;
    }
}

template <int MODE, int LOAD, int STORE, int MUL>
static fbp_status fft_go(fbp_context* ctx, const FftLineParams& p, unsigned gx, unsigned gy, cudaStream_t stream) {
    const int n = 1 << p.log2n;
    if (p.lines < 1 || (p.lines & (p.lines - 1)) || (size_t)p.lines * n > (size_t)kFftSmemElems)
        return set_error(FBP_ERR_UNSUPPORTED, "FFT: lines per CTA must be a power of two within the tile");
    FftLineParams q = p;
    q.log2c = 0;
    while ((1 << q.log2c) < p.lines) ++q.log2c;
    const size_t smem = ((size_t)p.lines * line_stride(n) + n / 2) * sizeof(float2);
    auto k = fft_lines_kernel<MODE, LOAD, STORE, MUL>;
    // The largest tile any launch uses, set once per variant and device.
    static thread_local int attr_device = -1;
    if (attr_device != ctx->device) {
        const size_t most = ((size_t)kFftSmemElems * 17 / 16 + kFftSmemElems + kFftSmemElems / 2) * sizeof(float2);
        FBP_TRY_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)most));
        attr_device = ctx->device;
    }
    (void)smem;
    k<<<dim3(gx, gy), kFftThreads, smem, stream>>>(q);
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
// inverse FFT of FFT(in) * LoG(k).  Sizes the half-spectrum path of
// log_fft.cu covers go there; the rest run full complex transforms of the
// real volume here (equal to the reference's R2C/C2R pair for this real,
// symmetric response).  x-forward (real in), y-forward, z-forward * response * z-inverse,
// y-inverse, x-inverse (real part out).
fbp_status launch_log_fft(fbp_context* ctx, const float* in, float* out, uint32_t nx, uint32_t ny, uint32_t nz,
                          float sigma, cudaStream_t stream) {
    const int lx = ilog2_exact(nx), ly = ilog2_exact(ny), lz = ilog2_exact(nz);
    if (lx < 1 || ly < 1 || lz < 1 || lx > 12 || ly > 12 || lz > 12)
        return set_error(FBP_ERR_UNSUPPORTED, "LoG-FFT filter: sizes must be powers of two in [2, 4096]");
    if (log_fft_half_supported(nx, ny, nz)) return launch_log_fft_half(ctx, in, out, nx, ny, nz, sigma, stream);
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
