// Post-processing of the reconstructed volume: min-max normalisation and the
// LoG / Laplacian 3-D filters.
//
// Replaces Laser::normalizeMatrix (Laser.cu:317-339: two CUB reductions and
// normalizeReconstruction, transient_postprocessing.cuh:10-17) and
// PostprocessingFilters::compute (PostprocessingFilters.h:5-39,
// PostprocessingFilters.cu:12-98).  The convolutions keep the reference's tap
// order and FMA sequence, so FP32 outputs can match the reference kernels bit
// for bit; neighbourhoods come from a shared-memory tile instead of 125 (or
// k^3) global loads per voxel.
#include "fbp_internal.cuh"

#include <cmath>
#include <cstring>
#include <vector>

namespace fbp {

// ------------------------------------------------------- min-max reduction --

constexpr int kReduceThreads = 512;

__device__ __forceinline__ void block_minmax(float& mn, float& mx) {
    __shared__ float smn[32], smx[32];
    for (int o = 16; o > 0; o >>= 1) {
        mn = fminf(mn, __shfl_xor_sync(0xffffffffu, mn, o));
        mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    }
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) { smn[w] = mn; smx[w] = mx; }
    __syncthreads();
    const int nw = (blockDim.x + 31) >> 5;
    if (w == 0) {
        mn = l < nw ? smn[l] : INFINITY;
        mx = l < nw ? smx[l] : -INFINITY;
        for (int o = 16; o > 0; o >>= 1) {
            mn = fminf(mn, __shfl_xor_sync(0xffffffffu, mn, o));
            mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        }
    }
}

// Pass 1: per-block min/max into partials[2*b], partials[2*b+1].
__global__ void minmax_partial_kernel(const float* __restrict__ v, uint64_t n, float* __restrict__ partials) {
    float mn = INFINITY, mx = -INFINITY;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    // Vectorised body when the pointer is 16-byte aligned.
    if ((reinterpret_cast<uintptr_t>(v) & 15) == 0) {
        const float4* v4 = reinterpret_cast<const float4*>(v);
        const uint64_t n4 = n / 4;
        for (uint64_t j = i; j < n4; j += stride) {
            const float4 a = v4[j];
            mn = fminf(mn, fminf(fminf(a.x, a.y), fminf(a.z, a.w)));
            mx = fmaxf(mx, fmaxf(fmaxf(a.x, a.y), fmaxf(a.z, a.w)));
        }
        for (uint64_t j = n4 * 4 + i; j < n; j += stride) {
            mn = fminf(mn, v[j]);
            mx = fmaxf(mx, v[j]);
        }
    } else {
        for (uint64_t j = i; j < n; j += stride) {
            mn = fminf(mn, v[j]);
            mx = fmaxf(mx, v[j]);
        }
    }
    block_minmax(mn, mx);
    if (threadIdx.x == 0) {
        partials[2 * blockIdx.x] = mn;
        partials[2 * blockIdx.x + 1] = mx;
    }
}

// Pass 2: one block folds the partials into mm[0] = min, mm[1] = max.
__global__ void minmax_final_kernel(const float* __restrict__ partials, int nblocks, float* __restrict__ mm) {
    float mn = INFINITY, mx = -INFINITY;
    for (int i = threadIdx.x; i < nblocks; i += blockDim.x) {
        mn = fminf(mn, partials[2 * i]);
        mx = fmaxf(mx, partials[2 * i + 1]);
    }
    block_minmax(mn, mx);
    if (threadIdx.x == 0) {
        mm[0] = mn;
        mm[1] = mx;
    }
}

// Pass 3: normalizeReconstruction, v = (v - min) * safeRCP(max - min).
__global__ void normalize_apply_kernel(float* __restrict__ v, uint64_t n, const float* __restrict__ mm) {
    const float mn = mm[0];
    const float r = ref_safe_rcp(sub_rn(mm[1], mn));
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += stride)
        v[i] = mul_rn(sub_rn(v[i], mn), r);
}

int minmax_blocks(const fbp_context* ctx, uint64_t n) {
    const uint64_t want = (n + 4ull * kReduceThreads - 1) / (4ull * kReduceThreads);
    const uint64_t cap = (uint64_t)ctx->sm_count * 4;
    return (int)std::max<uint64_t>(1, std::min<uint64_t>(want, cap));
}

// Runs the three passes with caller-provided scratch: partials must hold
// 2*minmax_blocks(n) floats and mm two floats.
fbp_status normalize_with_scratch(fbp_context* ctx, float* v, uint64_t n, float* partials, float* mm,
                                  cudaStream_t stream) {
    const int nb = minmax_blocks(ctx, n);
    minmax_partial_kernel<<<nb, kReduceThreads, 0, stream>>>(v, n, partials);
    FBP_CHECK_LAUNCH(ctx, "minmax_partial_kernel");
    minmax_final_kernel<<<1, kReduceThreads, 0, stream>>>(partials, nb, mm);
    FBP_CHECK_LAUNCH(ctx, "minmax_final_kernel");
    const unsigned ab = (unsigned)std::min<uint64_t>(cdiv(n, 256), (uint64_t)ctx->sm_count * 8);
    normalize_apply_kernel<<<ab, 256, 0, stream>>>(v, n, mm);
    FBP_CHECK_LAUNCH(ctx, "normalize_apply_kernel");
    return FBP_OK;
}

fbp_status normalize_device(fbp_context* ctx, float* v, uint64_t n, cudaStream_t stream) {
    const int nb = minmax_blocks(ctx, n);
    void* ws = nullptr;
    FBP_TRY(workspace(ctx, WS_PARTIALS, (size_t)(2 * nb + 2) * sizeof(float), stream, &ws));
    float* partials = static_cast<float*>(ws);
    return normalize_with_scratch(ctx, v, n, partials, partials + 2 * nb, stream);
}

// ------------------------------------------------------------- LoG filter --

constexpr int kLogMaxK = 15;

// LoG taps passed by value (kernel parameters, so concurrent calls with
// different kernels do not share state): ksize^3 weights, ksize = 2H+1 or 2H+2.
template <int H>
struct LogTaps {
    float w[(2 * H + 2) * (2 * H + 2) * (2 * H + 2)];
};

// Output tile 8x8x8 per CTA, halo tile (8 + 2h)^3 in shared memory.
// Taps in the reference's order (kz, ky, kx innermost), sum = fma(v, w, sum)
// (LoGFilter, transient_postprocessing.cuh:52-83).
template <int H>
__global__ void __launch_bounds__(512) log_filter_kernel(const float* __restrict__ in, float* __restrict__ out,
                                                         uint32_t nx, uint32_t ny, uint32_t nz, int ksize,
                                                         const __grid_constant__ LogTaps<H> taps) {
    constexpr int E = 8 + 2 * H;
    extern __shared__ float tile[];  // [E][E][E]
    const int x0 = blockIdx.x * 8, y0 = blockIdx.y * 8, z0 = blockIdx.z * 8;
    const int tid = threadIdx.x + 8 * (threadIdx.y + 8 * threadIdx.z);
    constexpr int NE = E * E * E, B = 4;
    for (int i0 = tid; i0 < NE; i0 += B * 512) {
        float v[B];
#pragma unroll
        for (int u = 0; u < B; ++u) {
            const int i = i0 + u * 512;
            if (i < NE) {
                const int lx = i % E, ly = (i / E) % E, lz = i / (E * E);
                const int gx = min(max(x0 + lx - H, 0), (int)nx - 1);
                const int gy = min(max(y0 + ly - H, 0), (int)ny - 1);
                const int gz = min(max(z0 + lz - H, 0), (int)nz - 1);
                v[u] = in[((size_t)gz * ny + gy) * nx + gx];
            }
        }
#pragma unroll
        for (int u = 0; u < B; ++u)
            if (i0 + u * 512 < NE) tile[i0 + u * 512] = v[u];
    }
    __syncthreads();
    const int x = x0 + threadIdx.x, y = y0 + threadIdx.y, z = z0 + threadIdx.z;
    if (x >= (int)nx || y >= (int)ny || z >= (int)nz) return;
    float sum = 0.f;
    for (int kz = -H; kz <= H; ++kz)
        for (int ky = -H; ky <= H; ++ky) {
            const float* row = tile + ((threadIdx.z + H + kz) * E + (threadIdx.y + H + ky)) * E + threadIdx.x + H;
            const float* wrow = taps.w + ((kz + H) * ksize + (ky + H)) * ksize + H;
#pragma unroll
            for (int kx = -H; kx <= H; ++kx) sum = fma_rn(row[kx], wrow[kx], sum);
        }
    out[((size_t)z * ny + y) * nx + x] = sum;
}


// The same filter for odd ksize = 2H+1 with H <= 2, register-blocked along
// z: a thread walks the input planes of its columns once, keeping the K = 2H+1
// outputs a plane reaches in a rotating window of accumulators (output
// zo = pl - 2H + k sits in acc[k] and takes tap kz = 2H - k of plane pl;
// after the plane acc[0] is complete and the window shifts).  Each thread
// owns two columns, x and x + 16, as the halves of packed FP32 pairs: the
// tile holds (v[x], v[x + 16]) pairs, the taps (w, w), and one fma.rn.f32x2
// applies a tap to both outputs with the scalar rounding on each half.
// Every output still receives its terms in the reference's order (plane =
// kz ascending, then ky, then kx), so the result is bitwise that of
// log_filter_kernel at half an issue slot per tap and output.  Tile
// 32 x 8 x 16 outputs, 128 threads, 38 KB of shared memory.
template <int H>
struct LogTaps2 {
    unsigned long long w2[(2 * H + 1) * (2 * H + 1) * (2 * H + 1)];
};

template <int H>
__global__ void __launch_bounds__(128) log_filter_zpair_kernel(const float* __restrict__ in, float* __restrict__ out,
                                                               uint32_t nx, uint32_t ny, uint32_t nz,
                                                               const __grid_constant__ LogTaps2<H> taps) {
    constexpr int K = 2 * H + 1, TX = 32, HX = 16, TY = 8, TZ = 16;
    constexpr int EX = HX + 2 * H, EY = TY + 2 * H, EZ = TZ + 2 * H;
    __shared__ f32x2_t tile[EZ][EY][EX];
    const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY, z0 = blockIdx.z * TZ;
    const int tid = threadIdx.x + HX * threadIdx.y;
    constexpr int NT = HX * TY, NE = EX * EY * EZ, B = 8;
    for (int i0 = tid; i0 < NE; i0 += B * NT) {
        float va[B], vb[B];
#pragma unroll
        for (int u = 0; u < B; ++u) {
            const int i = i0 + u * NT;
            if (i < NE) {
                const int lx = i % EX, ly = (i / EX) % EY, lz = i / (EX * EY);
                const int ga = min(max(x0 + lx - H, 0), (int)nx - 1);
                const int gb = min(max(x0 + lx + HX - H, 0), (int)nx - 1);
                const int gy = min(max(y0 + ly - H, 0), (int)ny - 1);
                const int gz = min(max(z0 + lz - H, 0), (int)nz - 1);
                const size_t row = ((size_t)gz * ny + gy) * nx;
                va[u] = in[row + ga];
                vb[u] = in[row + gb];
            }
        }
#pragma unroll
        for (int u = 0; u < B; ++u)
            if (i0 + u * NT < NE) (&tile[0][0][0])[i0 + u * NT] = pack2(va[u], vb[u]);
    }
    __syncthreads();
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int xa = x0 + tx, xb = xa + HX, y = y0 + ty;
    const bool ok_a = xa < (int)nx && y < (int)ny, ok_b = xb < (int)nx && y < (int)ny;
    f32x2_t acc[K];
#pragma unroll
    for (int k = 0; k < K; ++k) acc[k] = 0ull;
#pragma unroll 1
    for (int pl = 0; pl < EZ; ++pl) {
#pragma unroll
        for (int ky = 0; ky < K; ++ky) {
            f32x2_t r[K];
#pragma unroll
            for (int kx = 0; kx < K; ++kx) r[kx] = tile[pl][ty + ky][tx + kx];
#pragma unroll
            for (int k = 0; k < K; ++k) {
                const int kz = 2 * H - k;
#pragma unroll
                for (int kx = 0; kx < K; ++kx) acc[k] = fma_rn2(r[kx], taps.w2[(kz * K + ky) * K + kx], acc[k]);
            }
        }
        const int zo = pl - 2 * H;  // acc[0] is complete
        if (zo >= 0 && z0 + zo < (int)nz) {
            float a, b;
            unpack2(acc[0], a, b);
            const size_t row = ((size_t)(z0 + zo) * ny + y) * nx;
            if (ok_a) out[row + xa] = a;
            if (ok_b) out[row + xb] = b;
        }
#pragma unroll
        for (int k = 0; k < K - 1; ++k) acc[k] = acc[k + 1];
        acc[K - 1] = 0ull;
    }
}

// ------------------------------------------------------- Laplacian filter --

// laplacianFilter (transient_postprocessing.cuh:21-50): k^3 * v - (sum of the
// k^3 box, zero outside the volume), box summed with x outermost, z innermost.
template <int H>
__global__ void __launch_bounds__(512) laplacian_filter_kernel(const float* __restrict__ in, float* __restrict__ out,
                                                               uint32_t nx, uint32_t ny, uint32_t nz, float k3) {
    constexpr int E = 8 + 2 * H;
    extern __shared__ float tile[];
    const int x0 = blockIdx.x * 8, y0 = blockIdx.y * 8, z0 = blockIdx.z * 8;
    const int tid = threadIdx.x + 8 * (threadIdx.y + 8 * threadIdx.z);
    for (int i = tid; i < E * E * E; i += 512) {
        const int lx = i % E, ly = (i / E) % E, lz = i / (E * E);
        const int gx = x0 + lx - H, gy = y0 + ly - H, gz = z0 + lz - H;
        float v = 0.f;
        if (gx >= 0 && gx < (int)nx && gy >= 0 && gy < (int)ny && gz >= 0 && gz < (int)nz)
            v = in[((size_t)gz * ny + gy) * nx + gx];
        tile[i] = v;
    }
    __syncthreads();
    const int x = x0 + threadIdx.x, y = y0 + threadIdx.y, z = z0 + threadIdx.z;
    if (x >= (int)nx || y >= (int)ny || z >= (int)nz) return;
    float lap = 0.f;
    for (int dx = -H; dx <= H; ++dx)
        for (int dy = -H; dy <= H; ++dy)
#pragma unroll
            for (int dz = -H; dz <= H; ++dz)
                lap = add_rn(lap, tile[((threadIdx.z + H + dz) * E + (threadIdx.y + H + dy)) * E + threadIdx.x + H + dx]);
    const float c = tile[((threadIdx.z + H) * E + (threadIdx.y + H)) * E + threadIdx.x + H];
    out[((size_t)z * ny + y) * nx + x] = fma_rn(k3, c, -lap);
}


// laplacianFilter (transient_postprocessing.cuh:21-50) register-blocked along
// z: a thread owns one (x, y) column of 32 outputs and adds the K^3
// neighbours of each in the reference's order (dx, dy, dz; zero outside the
// volume), then centre * K^3 - sum.  The outputs z and z + 16 are the halves
// of packed FP32 pairs: the tile holds (v[z], v[z + 16]) pairs along z, and
// one add.rn.f32x2 adds a neighbour to both sums, so the result is bitwise
// that of the scalar sum at half the add instructions.
template <int H>
__global__ void __launch_bounds__(128) laplacian_zpair_kernel(const float* __restrict__ in, float* __restrict__ out,
                                                              uint32_t nx, uint32_t ny, uint32_t nz, float k3) {
    constexpr int K = 2 * H + 1, TX = 32, TY = 4, TZ = 32, HZ = 16;
    constexpr int EX = TX + 2 * H, EY = TY + 2 * H, EZ2 = HZ + 2 * H;  // pairs (z, z + 16), z < EZ2
    __shared__ f32x2_t tile[EZ2][EY][EX];
    const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY, z0 = blockIdx.z * TZ;
    const int tid = threadIdx.x + TX * threadIdx.y;
    constexpr int NT = TX * TY, NE = EX * EY * EZ2, B = 8;
    for (int i0 = tid; i0 < NE; i0 += B * NT) {
        float va[B], vb[B];
#pragma unroll
        for (int u = 0; u < B; ++u) {
            const int i = i0 + u * NT;
            va[u] = vb[u] = 0.f;  // zero outside the volume
            if (i < NE) {
                const int lx = i % EX, ly = (i / EX) % EY, lz = i / (EX * EY);
                const int gx = x0 + lx - H, gy = y0 + ly - H, ga = z0 + lz - H, gb = ga + HZ;
                if (gx >= 0 && gx < (int)nx && gy >= 0 && gy < (int)ny) {
                    const size_t col = (size_t)gy * nx + gx, plane = (size_t)nx * ny;
                    if (ga >= 0 && ga < (int)nz) va[u] = in[ga * plane + col];
                    if (gb >= 0 && gb < (int)nz) vb[u] = in[gb * plane + col];
                }
            }
        }
#pragma unroll
        for (int u = 0; u < B; ++u)
            if (i0 + u * NT < NE) (&tile[0][0][0])[i0 + u * NT] = pack2(va[u], vb[u]);
    }
    __syncthreads();
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int x = x0 + tx, y = y0 + ty;
    if (x >= (int)nx || y >= (int)ny) return;
    f32x2_t lap[HZ];  // (sum of output z, sum of output z + 16)
#pragma unroll
    for (int z = 0; z < HZ; ++z) lap[z] = 0ull;
#pragma unroll 1
    for (int dx = 0; dx < K; ++dx) {
#pragma unroll 1
        for (int dy = 0; dy < K; ++dy) {
            f32x2_t c[EZ2];
#pragma unroll
            for (int z = 0; z < EZ2; ++z) c[z] = tile[z][ty + dy][tx + dx];
#pragma unroll
            for (int z = 0; z < HZ; ++z)
#pragma unroll
                for (int dz = 0; dz < K; ++dz) lap[z] = add_rn2(lap[z], c[z + dz]);
        }
    }
#pragma unroll
    for (int z = 0; z < HZ; ++z) {
        float la, lb, ca, cb;
        unpack2(lap[z], la, lb);
        unpack2(tile[z + H][ty + H][tx + H], ca, cb);  // (v[z + H], v[z + 16 + H]) of this column
        const size_t col = (size_t)y * nx + x, plane = (size_t)nx * ny;
        if (z0 + z < (int)nz) out[(z0 + z) * plane + col] = fma_rn(k3, ca, -la);
        if (z0 + z + HZ < (int)nz) out[(z0 + z + HZ) * plane + col] = fma_rn(k3, cb, -lb);
    }
}

fbp_status launch_log(fbp_context* ctx, const float* in, float* out, uint32_t nx, uint32_t ny, uint32_t nz, int ksize,
                      float sigma, cudaStream_t stream);
fbp_status launch_laplacian(fbp_context* ctx, const float* in, float* out, uint32_t nx, uint32_t ny, uint32_t nz,
                            int ksize, cudaStream_t stream);
fbp_status launch_log_fft(fbp_context* ctx, const float* in, float* out, uint32_t nx, uint32_t ny, uint32_t nz,
                          float sigma, cudaStream_t stream);

// Host-side LoG weights: PostprocessingFilters.cu:102-175 in float, same step order.
fbp_status log_weights_host(int size, float sigma, float* taps) {
    if (size <= 0 || !taps) return set_error(FBP_ERR_INVALID_ARG, "LoG weights: size must be > 0");
    const int half = (size - 1) / 2;
    const float var = sigma * sigma;
    const int n = size * size * size;
    std::vector<float> g(n), rr(n);
    float gmax = 0.0f;
    for (int kz = 0; kz < size; ++kz)
        for (int ky = 0; ky < size; ++ky)
            for (int kx = 0; kx < size; ++kx) {
                const float x = (float)(kx - half), y = (float)(ky - half), z = (float)(kz - half);
                const int i = kz * size * size + ky * size + kx;
                rr[i] = x * x + y * y + z * z;
                g[i] = std::exp(-(x * x + y * y + z * z) / (2.0f * var));
                gmax = std::max(g[i], gmax);
            }
    const float cutoff = 1.19209290e-07f * gmax;  // FLT_EPSILON * max
    float gsum = 0.0f;
    for (float& v : g) {
        if (v < cutoff) v = 0.0f;
        gsum += v;
    }
    if (gsum != 0.0f)
        for (float& v : g) v /= gsum;
    float lsum = 0.0f;
    for (int i = 0; i < n; ++i) {
        g[i] = g[i] * (rr[i] - 3.0f * var) / (var * var);
        lsum += g[i];
    }
    const float mean = lsum / (float)n;  // subtracted so the taps sum to zero
    for (int i = 0; i < n; ++i) taps[i] = g[i] - mean;
    return FBP_OK;
}

template <int H>
static fbp_status log_h(fbp_context* ctx, const float* in, float* out, uint32_t nx, uint32_t ny, uint32_t nz, int ksize,
                        const float* w, cudaStream_t stream) {
    LogTaps<H> taps{};
    for (int i = 0; i < ksize * ksize * ksize; ++i) taps.w[i] = w[i];
    if constexpr (H >= 1 && H <= 2) {
        if (ksize == 2 * H + 1) {
            LogTaps2<H> taps2{};
            for (int i = 0; i < ksize * ksize * ksize; ++i) {
                uint32_t b;
                std::memcpy(&b, &w[i], 4);
                taps2.w2[i] = ((unsigned long long)b << 32) | b;  // (w, w)
            }
            dim3 grid(cdiv(nx, 32), cdiv(ny, 8), cdiv(nz, 16));
            log_filter_zpair_kernel<H><<<grid, dim3(16, 8), 0, stream>>>(in, out, nx, ny, nz, taps2);
            FBP_CHECK_LAUNCH(ctx, "log_filter_zpair_kernel");
            return FBP_OK;
        }
    }
    constexpr int E = 8 + 2 * H;
    const size_t smem = sizeof(float) * E * E * E;
    FBP_TRY_CUDA(cudaFuncSetAttribute(log_filter_kernel<H>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    dim3 grid(cdiv(nx, 8), cdiv(ny, 8), cdiv(nz, 8));
    log_filter_kernel<H><<<grid, dim3(8, 8, 8), smem, stream>>>(in, out, nx, ny, nz, ksize, taps);
    FBP_CHECK_LAUNCH(ctx, "log_filter_kernel");
    return FBP_OK;
}

template <int H>
static fbp_status lap_h(fbp_context* ctx, const float* in, float* out, uint32_t nx, uint32_t ny, uint32_t nz, float k3,
                        cudaStream_t stream) {
    if constexpr (H <= 2) {
        const dim3 grid(cdiv(nx, 32), cdiv(ny, 4), cdiv(nz, 32));
        laplacian_zpair_kernel<H><<<grid, dim3(32, 4), 0, stream>>>(in, out, nx, ny, nz, k3);
        FBP_CHECK_LAUNCH(ctx, "laplacian_zpair_kernel");
        return FBP_OK;
    }
    constexpr int E = 8 + 2 * H;
    const size_t smem = sizeof(float) * E * E * E;
    FBP_TRY_CUDA(cudaFuncSetAttribute(laplacian_filter_kernel<H>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    dim3 grid(cdiv(nx, 8), cdiv(ny, 8), cdiv(nz, 8));
    laplacian_filter_kernel<H><<<grid, dim3(8, 8, 8), smem, stream>>>(in, out, nx, ny, nz, k3);
    FBP_CHECK_LAUNCH(ctx, "laplacian_filter_kernel");
    return FBP_OK;
}

fbp_status launch_log(fbp_context* ctx, const float* in, float* out, uint32_t nx, uint32_t ny, uint32_t nz, int ksize,
                      float sigma, cudaStream_t stream) {
    if (ksize < 1 || ksize > kLogMaxK)
        return set_error(FBP_ERR_UNSUPPORTED, "LoG filter: kernel size must be in [1, 15]");
    std::vector<float> w((size_t)ksize * ksize * ksize);
    FBP_TRY(log_weights_host(ksize, sigma, w.data()));
    // The reference's kernelHalf = (k - 1) / 2 (PostprocessingFilters.cu:25).
    switch ((ksize - 1) / 2) {
        case 0: return log_h<0>(ctx, in, out, nx, ny, nz, ksize, w.data(), stream);
        case 1: return log_h<1>(ctx, in, out, nx, ny, nz, ksize, w.data(), stream);
        case 2: return log_h<2>(ctx, in, out, nx, ny, nz, ksize, w.data(), stream);
        case 3: return log_h<3>(ctx, in, out, nx, ny, nz, ksize, w.data(), stream);
        case 4: return log_h<4>(ctx, in, out, nx, ny, nz, ksize, w.data(), stream);
        case 5: return log_h<5>(ctx, in, out, nx, ny, nz, ksize, w.data(), stream);
        case 6: return log_h<6>(ctx, in, out, nx, ny, nz, ksize, w.data(), stream);
        default: return log_h<7>(ctx, in, out, nx, ny, nz, ksize, w.data(), stream);
    }
}

fbp_status launch_laplacian(fbp_context* ctx, const float* in, float* out, uint32_t nx, uint32_t ny, uint32_t nz,
                            int ksize, cudaStream_t stream) {
    if (ksize < 1 || ksize > kLogMaxK)
        return set_error(FBP_ERR_UNSUPPORTED, "Laplacian filter: kernel size must be in [1, 15]");
    // laplacianFilter receives the size as a float and uses floor(size / 2)
    // for the half width and size^3 (as float products) for the centre weight.
    const float fs = (float)ksize;
    const float k3 = fs * fs * fs;
    switch ((int)std::floor(fs / 2.0f)) {
        case 0: return lap_h<0>(ctx, in, out, nx, ny, nz, k3, stream);
        case 1: return lap_h<1>(ctx, in, out, nx, ny, nz, k3, stream);
        case 2: return lap_h<2>(ctx, in, out, nx, ny, nz, k3, stream);
        case 3: return lap_h<3>(ctx, in, out, nx, ny, nz, k3, stream);
        case 4: return lap_h<4>(ctx, in, out, nx, ny, nz, k3, stream);
        case 5: return lap_h<5>(ctx, in, out, nx, ny, nz, k3, stream);
        case 6: return lap_h<6>(ctx, in, out, nx, ny, nz, k3, stream);
        default: return lap_h<7>(ctx, in, out, nx, ny, nz, k3, stream);
    }
}

}  // namespace fbp

using namespace fbp;

extern "C" fbp_status fbp_log_weights(int size, float sigma, float* w) {
    return guarded("fbp_log_weights", [&]() -> fbp_status {
        clear_error();
        return log_weights_host(size, sigma, w);
    });
}

extern "C" fbp_status fbp_normalize_minmax(fbp_context* ctx, float* v, uint64_t n, void* stream) {
    return guarded("fbp_normalize_minmax", [&]() -> fbp_status {
        clear_error();
        FBP_TRY(check_ctx(ctx));
        if (!v || n == 0) return set_error(FBP_ERR_INVALID_ARG, "fbp_normalize_minmax: null buffer or n == 0");
        return normalize_device(ctx, v, n, (cudaStream_t)stream);
    });
}

// ------------------------------------------ allocation-free normalisation --
//
// fbp_normalize_minmax_noalloc: the same three passes as fbp_normalize_minmax,
// but its scratch (one min/max pair per reduction block plus the final pair)
// lives in this file-scope array instead of context workspace, so the call
// allocates nothing and needs no fbp_context.  Every device that loads the
// library holds the array (8 KiB) until the process exits.  The partial pass
// strides over the input with up to 1024 blocks (4 per SM, like the context
// entry point), one partial slot each; inputs are limited to 2^30 elements.
// All calls on a device share the array: each call overwrites every slot it
// reads before reading it, and two calls that overlap on the GPU (different
// streams, no ordering between them) race on it.
namespace fbp {
constexpr int kNoAllocMaxBlocks = 1024;
constexpr uint64_t kNoAllocMaxElems = 1ull << 30;
static __device__ __align__(256) float g_noalloc_scratch[2 * kNoAllocMaxBlocks + 2];

// Device address of g_noalloc_scratch on the current device, looked up on
// every call (the first call on a device loads the module; later lookups are
// cheap, and a module reloaded after a device reset gets its new address).
// Host code must not pass the symbol itself to a kernel: on the host it only
// names a stand-in object.
static fbp_status noalloc_scratch(float** out) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return cuda_error(e, "fbp_normalize_minmax_noalloc: cudaGetSymbolAddress");
    *out = static_cast<float*>(p);
    return FBP_OK;
}
}  // namespace fbp

extern "C" fbp_status fbp_normalize_minmax_noalloc(float* v, uint64_t n, void* stream) {
    return guarded("fbp_normalize_minmax_noalloc", [&]() -> fbp_status {
        clear_error();
        if (!v || n == 0) return set_error(FBP_ERR_INVALID_ARG, "fbp_normalize_minmax_noalloc: null buffer or n == 0");
        if (n > kNoAllocMaxElems)
            return set_error(FBP_ERR_UNSUPPORTED,
                             "fbp_normalize_minmax_noalloc: n exceeds 2^30 elements (the static scratch holds 1024 "
                             "partial min/max pairs); use fbp_normalize_minmax");
        // An error left pending by earlier work is reported as such, not as
        // this call's launch failure (and left for the caller to clear).
        const cudaError_t pending = cudaPeekAtLastError();
        if (pending != cudaSuccess)
            return cuda_error(pending, "fbp_normalize_minmax_noalloc: a CUDA error was pending before the call");
        int dev = -1;
        FBP_TRY_CUDA(cudaGetDevice(&dev));
        cudaPointerAttributes attr{};
        FBP_TRY_CUDA(cudaPointerGetAttributes(&attr, v));
        if ((attr.type != cudaMemoryTypeDevice && attr.type != cudaMemoryTypeManaged) || attr.device != dev)
            return set_error(FBP_ERR_INVALID_ARG,
                             "fbp_normalize_minmax_noalloc: v is not device memory of the current device");
        float* scratch = nullptr;
        FBP_TRY(noalloc_scratch(&scratch));
        int sms = 0;
        FBP_TRY_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        cudaStream_t s = (cudaStream_t)stream;
        const uint64_t want = (n + 4ull * kReduceThreads - 1) / (4ull * kReduceThreads);
        const uint64_t cap = std::min<uint64_t>(kNoAllocMaxBlocks, 4ull * (uint64_t)std::max(sms, 1));
        const int nb = (int)std::max<uint64_t>(1, std::min(want, cap));
        float* mm = scratch + 2 * kNoAllocMaxBlocks;
        minmax_partial_kernel<<<nb, kReduceThreads, 0, s>>>(v, n, scratch);
        FBP_TRY_CUDA(cudaGetLastError());
        minmax_final_kernel<<<1, kReduceThreads, 0, s>>>(scratch, nb, mm);
        FBP_TRY_CUDA(cudaGetLastError());
        const unsigned ab = (unsigned)std::min<uint64_t>(cdiv(n, 256), 1216);
        normalize_apply_kernel<<<ab, 256, 0, s>>>(v, n, mm);
        FBP_TRY_CUDA(cudaGetLastError());
        return FBP_OK;
    });
}

extern "C" fbp_status fbp_postfilter(fbp_context* ctx, int kind, int kernel_size, float sigma, const float* in,
                                     float* out, uint32_t nx, uint32_t ny, uint32_t nz, void* stream) {
    return guarded("fbp_postfilter", [&]() -> fbp_status {
        clear_error();
        FBP_TRY(check_ctx(ctx));
        if (!in || !out) return set_error(FBP_ERR_INVALID_ARG, "fbp_postfilter: null buffer");
        if (nx == 0 || ny == 0 || nz == 0) return set_error(FBP_ERR_INVALID_ARG, "fbp_postfilter: empty volume");
        const size_t n = (size_t)nx * ny * nz;
        if (in == out && kind != FBP_FILTER_NONE)
            return set_error(FBP_ERR_INVALID_ARG, "fbp_postfilter: in and out must be different buffers");
        cudaStream_t s = (cudaStream_t)stream;
        switch (kind) {
            case FBP_FILTER_NONE:
                if (in != out) FBP_TRY_CUDA(cudaMemcpyAsync(out, in, n * sizeof(float), cudaMemcpyDeviceToDevice, s));
                return FBP_OK;
            case FBP_FILTER_LAPLACIAN: return launch_laplacian(ctx, in, out, nx, ny, nz, kernel_size, s);
            case FBP_FILTER_LOG: return launch_log(ctx, in, out, nx, ny, nz, kernel_size, sigma, s);
            case FBP_FILTER_LOG_FFT: return launch_log_fft(ctx, in, out, nx, ny, nz, sigma, s);
            default: return set_error(FBP_ERR_INVALID_ARG, "fbp_postfilter: unknown filter kind");
        }
    });
}
