// Learned MIS proposal: a 19 -> 64 -> 64 -> 64 -> 1 MLP (GELU) that scores,
// for every voxel tile of the gather, how much each square cluster of scan
// points contributes to it.  Per tile the scores become a distribution over
// clusters (softmax, mixed with a uniform share) that the sampled gather draws
// whole clusters from (FBP_MIS_LEARNED).
//
// The MLP runs on the fifth-generation tensor cores: BF16 weights and
// activations in shared memory, FP32 accumulators in TMEM (umma.cuh).  One CTA
// of 128 threads handles one tile; the tile's clusters are processed in
// blocks of 128 rows (one M=128 MMA tile, thread r owning row r when reading
// the accumulators back).
//
// Inputs of row (tile t, cluster c): the tile centre relative to the cluster
// centre (3 values, metres / 2) and 16 pooled transient features: the
// cluster's mean transient, pooled over 3.84 cm of path per bin, in the 16
// pooled bins around the tile-cluster round trip, as log(1 + v / mean).
//
// Training (project-written forward and backward kernels, Adam): the target
// of tile t is q_c proportional to sqrt(sum over the tile's voxels of F_vc^2),
// F_vc being cluster c's exact contribution to voxel v -- the proposal that
// minimises the summed variance of the cluster estimator; the loss is the
// cross-entropy -sum_c q_c log softmax(o)_c.  Numerics of both directions
// (the CPU oracle restates them): BF16 operands rounded from FP32 at every
// MMA input, FP32 accumulation, biases, GELU, the output layer and the
// softmax in FP32; per-CTA gradient partials reduced in a fixed order, so a
// step is deterministic.
#include "fbp_internal.cuh"
#include "bp_common.cuh"
#include "umma.cuh"

#include <algorithm>
#include <cmath>
#include <random>
#include <vector>

struct fbp_mlp {
    fbp_context* ctx = nullptr;
    float* params = nullptr;  // device FP32 master copy
    float* adam_m = nullptr;
    float* adam_v = nullptr;
    float* grad = nullptr;    // device [NPARAM + 1]: gradient, then the mean loss
    uint64_t step = 0;
};

namespace fbp {
namespace mlp {

constexpr int IN = 19, IN_PAD = 32, FEAT = 20, H = 64;
constexpr int R = 128;      // rows per tensor-core block
constexpr int MAXG = 1024;  // clusters per tile
constexpr int NTH = 128;    // threads per CTA
constexpr int OW1 = 0, OB1 = OW1 + H * IN_PAD, OW2 = OB1 + H, OB2 = OW2 + H * H, OW3 = OB2 + H,
              OB3 = OW3 + H * H, OW4 = OB3 + H, OB4 = OW4 + H, NPARAM = OB4 + 1;
constexpr float POOL_M = 0.0384f;
constexpr int WINDOW = 16;
constexpr uint32_t kWaitIter = 1u << 22;
constexpr float kSqrt2OverPi = 0.7978845608028654f;

__device__ __forceinline__ float gelu_f(float x) {
    const float u = kSqrt2OverPi * fmaf(0.044715f * x, x * x, x);
    return 0.5f * x * (1.f + tanhf(u));
}
__device__ __forceinline__ float gelu_d(float x) {
    const float x2 = x * x;
    const float t = tanhf(kSqrt2OverPi * fmaf(0.044715f * x, x2, x));
    return 0.5f * (1.f + t) + 0.5f * x * (1.f - t * t) * kSqrt2OverPi * fmaf(0.134145f, x2, 1.f);
}

__device__ __forceinline__ uint32_t pack_bf16(float a, float b) {
    const __nv_bfloat162 v = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<const uint32_t*>(&v);
}

// Row r (K values in v, K a multiple of 8) into a K-major operand.
template <int K>
__device__ __forceinline__ void store_row(uint8_t* base, uint32_t r, const float* v) {
#pragma unroll
    for (int k8 = 0; k8 < K; k8 += 8) {
        uint4 q;
        q.x = pack_bf16(v[k8 + 0], v[k8 + 1]);
        q.y = pack_bf16(v[k8 + 2], v[k8 + 3]);
        q.z = pack_bf16(v[k8 + 4], v[k8 + 5]);
        q.w = pack_bf16(v[k8 + 6], v[k8 + 7]);
        *reinterpret_cast<uint4*>(base + umma::kmajor_offset(r, k8, K)) = q;
    }
}

// Column r of a transposed operand: element (k, r) of a [K][R] K-major matrix.
template <int K>
__device__ __forceinline__ void store_col(uint8_t* base, uint32_t r, const float* v) {
#pragma unroll
    for (int k = 0; k < K; ++k)
        *reinterpret_cast<__nv_bfloat16*>(base + umma::kmajor_offset(k, r, R)) = __float2bfloat16_rn(v[k]);
}

// W [rows][K] (FP32, row stride K) -> K-major BF16 operand; transposed: the
// [K][rows] operand W^T.
__device__ void load_weight(uint8_t* dst, const float* __restrict__ W, int rows, int K, bool transposed) {
    for (int i = threadIdx.x; i < rows * K; i += blockDim.x) {
        const int r = i / K, k = i % K;
        const uint32_t off = transposed ? umma::kmajor_offset(k, r, rows) : umma::kmajor_offset(r, k, K);
        *reinterpret_cast<__nv_bfloat16*>(dst + off) = __float2bfloat16_rn(W[i]);
    }
}

// Shared state of the MLP kernels.
struct Sync {
    uint64_t* mbar;
    uint32_t phase;
    int* abort;
    int* status;
    // Issue-side: thread 0 has issued MMAs and committed; everybody waits.
    __device__ __forceinline__ bool wait() {
        bool ok = umma::mbar_wait(mbar, phase, kWaitIter);
        phase ^= 1u;
        if (!ok) {
            *abort = 1;
            if (status) atomicExch(status, (int)FBP_ERR_TIMEOUT);
        }
        umma::fence_after_sync();
        return ok;
    }
};

// z = A[128][K] * W[64][K]^T into TMEM columns [col, col+64).
template <int K>
__device__ __forceinline__ void issue_layer(uint32_t tmem, uint32_t col, const uint8_t* A, const uint8_t* W,
                                            uint64_t* mbar) {
    umma::fence_after_sync();
    const uint32_t a = umma::smem_u32(A), w = umma::smem_u32(W);
#pragma unroll
    for (int ks = 0; ks < K / 16; ++ks)
        umma::mma_bf16(tmem + col, umma::kslice_desc(a, K, 0, ks), umma::kslice_desc(w, K, 0, ks),
                       umma::idesc_bf16_f32(R, H), ks > 0);
    umma::commit(mbar);
}

// This thread's row of TMEM columns [col, col+64), + bias, through GELU.
__device__ __forceinline__ void load_act(uint32_t taddr, const float* b, float (&x)[H], float (&a)[H]) {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        float v[16];
        umma::tmem_ld16(taddr + q * 16, v);
#pragma unroll
        for (int j = 0; j < 16; ++j) {
            x[q * 16 + j] = v[j] + b[q * 16 + j];
            a[q * 16 + j] = gelu_f(x[q * 16 + j]);
        }
    }
}

// Features of one row into a0 (IN_PAD values, zero padded).
__device__ __forceinline__ void load_features(const float* __restrict__ feat, uint64_t tile, uint32_t c, uint32_t G,
                                              float (&a0)[IN_PAD]) {
#pragma unroll
    for (int k = 0; k < IN_PAD; ++k) a0[k] = 0.f;
    if (c < G) {
        const float4* f = reinterpret_cast<const float4*>(feat + (tile * G + c) * FEAT);
#pragma unroll
        for (int q = 0; q < FEAT / 4; ++q) {
            const float4 v = f[q];
            a0[4 * q + 0] = v.x;
            a0[4 * q + 1] = v.y;
            a0[4 * q + 2] = v.z;
            a0[4 * q + 3] = v.w;
        }
        a0[IN] = 0.f;  // the 20th stored value is padding
    }
}

// ---------------------------------------------------------------- inference
// Shared memory (bytes): A0 8K | A1 16K | A2 16K | W1 4K | W2 8K | W3 8K | floats.
constexpr int SI_A0 = 0, SI_A1 = 8192, SI_A2 = SI_A1 + 16384, SI_W1 = SI_A2 + 16384, SI_W2 = SI_W1 + 4096,
              SI_W3 = SI_W2 + 8192, SI_F = SI_W3 + 8192;
constexpr int SI_BYTES = SI_F + (4 * H + MAXG + 16) * 4 + 64;

// Forward of one 128-row block: the logits of its rows (FP32).
__device__ __forceinline__ float forward_block(uint8_t* sm, uint32_t tmem, Sync& sy, const float* b1, const float* b2,
                                               const float* b3, const float* w4, float b4,
                                               const float (&a0)[IN_PAD]) {
    const int tid = threadIdx.x, warp = tid >> 5;
    const uint32_t r = tid;
    const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16);
    store_row<IN_PAD>(sm + SI_A0, r, a0);
    umma::fence_smem_to_async();
    __syncthreads();
    float x[H], a[H];
    if (tid == 0) issue_layer<IN_PAD>(tmem, 0, sm + SI_A0, sm + SI_W1, sy.mbar);
    sy.wait();
    load_act(taddr, b1, x, a);
    store_row<H>(sm + SI_A1, r, a);
    umma::fence_before_sync();
    umma::fence_smem_to_async();
    __syncthreads();
    if (tid == 0) issue_layer<H>(tmem, 0, sm + SI_A1, sm + SI_W2, sy.mbar);
    sy.wait();
    load_act(taddr, b2, x, a);
    store_row<H>(sm + SI_A2, r, a);
    umma::fence_before_sync();
    umma::fence_smem_to_async();
    __syncthreads();
    if (tid == 0) issue_layer<H>(tmem, 0, sm + SI_A2, sm + SI_W3, sy.mbar);
    sy.wait();
    load_act(taddr, b3, x, a);
    float o = b4;
#pragma unroll
    for (int k = 0; k < H; ++k) o = fmaf(a[k], w4[k], o);
    umma::fence_before_sync();
    __syncthreads();
    return o;
}

// Inclusive scan of p[0..G) by the block (G <= MAXG, 128 threads, each a
// run of ceil(G / 128) consecutive elements).
__device__ void block_scan(float* p, uint32_t G, float* red) {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const uint32_t per = (G + NTH - 1) / NTH;
    const uint32_t i0 = tid * per, i1 = min(i0 + per, G);
    float s = 0.f;
    for (uint32_t i = i0; i < i1; ++i) s += p[i];
    const float own = s;
    for (int o = 1; o < 32; o <<= 1) {
        const float t = __shfl_up_sync(0xffffffffu, s, o);
        if (lane >= o) s += t;
    }
    if (lane == 31) red[warp] = s;
    __syncthreads();
    float run = s - own;  // exclusive prefix within the warp
    for (int w = 0; w < warp; ++w) run += red[w];
    __syncthreads();
    for (uint32_t i = i0; i < i1; ++i) {
        run += p[i];
        p[i] = run;
    }
    __syncthreads();
}

__global__ void __launch_bounds__(NTH) mlp_infer_kernel(const float* __restrict__ prm, const float* __restrict__ feat,
                                                        uint32_t G, float defensive, float* __restrict__ logits,
                                                        float* __restrict__ cdf, int* __restrict__ status) {
    extern __shared__ __align__(128) uint8_t sm[];
    float* fb = reinterpret_cast<float*>(sm + SI_F);
    float *b1 = fb, *b2 = fb + H, *b3 = fb + 2 * H, *w4 = fb + 3 * H, *s_o = fb + 4 * H, *red = s_o + MAXG;
    __shared__ uint64_t mbar;
    __shared__ uint32_t s_tmem;
    __shared__ int s_abort;
    const int tid = threadIdx.x, warp = tid >> 5;
    const uint64_t tile = blockIdx.x;

    if (warp == 0) {
        umma::tmem_alloc(&s_tmem, 64);
        umma::tmem_relinquish();
    }
    load_weight(sm + SI_W1, prm + OW1, H, IN_PAD, false);
    load_weight(sm + SI_W2, prm + OW2, H, H, false);
    load_weight(sm + SI_W3, prm + OW3, H, H, false);
    for (int i = tid; i < H; i += NTH) {
        b1[i] = prm[OB1 + i];
        b2[i] = prm[OB2 + i];
        b3[i] = prm[OB3 + i];
        w4[i] = prm[OW4 + i];
    }
    if (tid == 0) {
        umma::mbar_init(&mbar, 1);
        s_abort = 0;
    }
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
    const uint32_t tmem = s_tmem;
    const float b4 = prm[OB4];
    Sync sy{&mbar, 0u, &s_abort, status};

    const uint32_t nb = (G + R - 1) / R;
    for (uint32_t h = 0; h < nb; ++h) {
        float a0[IN_PAD];
        const uint32_t c = h * R + tid;
        load_features(feat, tile, c, G, a0);
        const float o = forward_block(sm, tmem, sy, b1, b2, b3, w4, b4, a0);
        if (s_abort) break;
        if (c < G) s_o[c] = o;
    }
    __syncthreads();
    if (!s_abort) {
        if (logits)
            for (uint32_t c = tid; c < G; c += NTH) logits[tile * G + c] = s_o[c];
        if (cdf) {
            // Softmax over the tile's clusters, mixed with a uniform share.
            float m = -INFINITY;
            for (uint32_t c = tid; c < G; c += NTH) m = fmaxf(m, s_o[c]);
            for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
            if ((tid & 31) == 0) red[8 + warp] = m;
            __syncthreads();
            m = fmaxf(fmaxf(red[8], red[9]), fmaxf(red[10], red[11]));
            float s = 0.f;
            for (uint32_t c = tid; c < G; c += NTH) {
                const float e = expf(s_o[c] - m);
                s_o[c] = e;
                s += e;
            }
            for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
            __syncthreads();
            if ((tid & 31) == 0) red[8 + warp] = s;
            __syncthreads();
            s = (red[8] + red[9]) + (red[10] + red[11]);
            const float scale = (1.f - defensive) / s, uni = defensive / (float)G;
            for (uint32_t c = tid; c < G; c += NTH) s_o[c] = fmaf(s_o[c], scale, uni);
            __syncthreads();
            block_scan(s_o, G, red);
            for (uint32_t c = tid; c < G; c += NTH) cdf[tile * G + c] = c + 1 == G ? 1.f : fminf(s_o[c], 1.f);
        }
    }
    umma::fence_before_sync();
    __syncthreads();
    if (warp == 0) umma::tmem_dealloc(tmem, 64);
}

// ----------------------------------------------------------------- training
// Shared memory (bytes).  DZT comes first: the dW products read it as an
// M=128 operand whose rows 64..127 (the next 16 KB, in bounds) are ignored.
constexpr int ST_DZT = 0, ST_DZ = 16384, ST_A0 = 32768, ST_A0T = ST_A0 + 8192, ST_A1 = ST_A0T + 8192,
              ST_A1T = ST_A1 + 16384, ST_A2 = ST_A1T + 16384, ST_A2T = ST_A2 + 16384, ST_W1 = ST_A2T + 16384,
              ST_W2 = ST_W1 + 4096, ST_W3 = ST_W2 + 8192, ST_W2T = ST_W3 + 8192, ST_W3T = ST_W2T + 8192,
              ST_F = ST_W3T + 8192;
// floats: b1 b2 b3 w4 | logits/g [256] | per-warp partial sums [4][4*64+1] | red[16]
constexpr int ST_NF = 4 * H + MAXG + 4 * (4 * H + 1) + 16;
constexpr int ST_BYTES = ST_F + ST_NF * 4;
// TMEM columns.
constexpr uint32_t TC_Z1 = 0, TC_Z2 = 64, TC_Z3 = 128, TC_DA = 192, TC_DW1 = 256, TC_DW2 = 320, TC_DW3 = 384;

// dW[n][k] (+)= sum_r DZT[n][r] * AT[k][r] (M=128 with rows >= 64 ignored),
// then da[r][k] = sum_n DZ[r][n] * WT[k][n] when WT is given.
template <int KIN>
__device__ __forceinline__ void issue_backward(uint32_t tmem, uint32_t dw_col, bool acc, const uint8_t* DZT,
                                               const uint8_t* AT, const uint8_t* DZ, const uint8_t* WT, uint64_t* mbar) {
    umma::fence_after_sync();
    const uint32_t dzt = umma::smem_u32(DZT), at = umma::smem_u32(AT);
#pragma unroll
    for (int ks = 0; ks < R / 16; ++ks)
        umma::mma_bf16(tmem + dw_col, umma::kslice_desc(dzt, R, 0, ks), umma::kslice_desc(at, R, 0, ks),
                       umma::idesc_bf16_f32(R, KIN), (acc || ks > 0) ? 1u : 0u);
    if (WT) {
        const uint32_t dz = umma::smem_u32(DZ), wt = umma::smem_u32(WT);
#pragma unroll
        for (int ks = 0; ks < H / 16; ++ks)
            umma::mma_bf16(tmem + TC_DA, umma::kslice_desc(dz, H, 0, ks), umma::kslice_desc(wt, H, 0, ks),
                           umma::idesc_bf16_f32(R, H), ks > 0);
    }
    umma::commit(mbar);
}

// Sum of v[0..n) over the block's 128 rows into part[warp][..] (then reduced
// in warp order by the caller): deterministic.
template <int N>
__device__ __forceinline__ void warp_sums(const float* v, float* part) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int k = 0; k < N; ++k) {
        float s = v[k];
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == 0) part[k] += s;
    }
}

// One CTA per tile of the minibatch: loss and gradient partials of its rows.
// grad_part[blockIdx.x][NPARAM + 1] (the last entry is the tile's loss), all
// scaled by 1/nbatch.
__global__ void __launch_bounds__(NTH) mlp_train_kernel(const float* __restrict__ prm, const float* __restrict__ feat,
                                                        const float* __restrict__ labels,
                                                        const uint32_t* __restrict__ idx, uint32_t nbatch, uint32_t G,
                                                        float* __restrict__ grad_part, int* __restrict__ status) {
    extern __shared__ __align__(128) uint8_t sm[];
    float* fb = reinterpret_cast<float*>(sm + ST_F);
    float *b1 = fb, *b2 = fb + H, *b3 = fb + 2 * H, *w4 = fb + 3 * H, *s_g = fb + 4 * H;
    float* part = s_g + MAXG;                    // [4 warps][3*64 bias + 64 w4 + 1 b4]
    float* red = part + 4 * (4 * H + 1);
    __shared__ uint64_t mbar;
    __shared__ uint32_t s_tmem;
    __shared__ int s_abort;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const uint64_t tile = idx[blockIdx.x];
    const float inv_n = 1.f / (float)nbatch;

    if (warp == 0) {
        umma::tmem_alloc(&s_tmem, 512);
        umma::tmem_relinquish();
    }
    load_weight(sm + ST_W1, prm + OW1, H, IN_PAD, false);
    load_weight(sm + ST_W2, prm + OW2, H, H, false);
    load_weight(sm + ST_W3, prm + OW3, H, H, false);
    load_weight(sm + ST_W2T, prm + OW2, H, H, true);
    load_weight(sm + ST_W3T, prm + OW3, H, H, true);
    for (int i = tid; i < H; i += NTH) {
        b1[i] = prm[OB1 + i];
        b2[i] = prm[OB2 + i];
        b3[i] = prm[OB3 + i];
        w4[i] = prm[OW4 + i];
    }
    for (int i = tid; i < 4 * (4 * H + 1); i += NTH) part[i] = 0.f;
    if (tid == 0) {
        umma::mbar_init(&mbar, 1);
        s_abort = 0;
    }
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
    const uint32_t tmem = s_tmem;
    const uint32_t tl = tmem + ((uint32_t)(warp * 32) << 16);  // this warp's lanes
    const float b4 = prm[OB4];
    Sync sy{&mbar, 0u, &s_abort, status};
    const uint32_t nb = (G + R - 1) / R;

    // Pass 1: logits of every row (layers reuse TMEM columns Z1).
    for (uint32_t h = 0; h < nb && !s_abort; ++h) {
        float a0[IN_PAD];
        const uint32_t c = h * R + tid;
        load_features(feat, tile, c, G, a0);
        store_row<IN_PAD>(sm + ST_A0, tid, a0);
        umma::fence_smem_to_async();
        __syncthreads();
        float x[H], a[H];
        if (tid == 0) issue_layer<IN_PAD>(tmem, TC_Z1, sm + ST_A0, sm + ST_W1, sy.mbar);
        sy.wait();
        load_act(tl + TC_Z1, b1, x, a);
        store_row<H>(sm + ST_A1, tid, a);
        umma::fence_before_sync();
        umma::fence_smem_to_async();
        __syncthreads();
        if (tid == 0) issue_layer<H>(tmem, TC_Z2, sm + ST_A1, sm + ST_W2, sy.mbar);
        sy.wait();
        load_act(tl + TC_Z2, b2, x, a);
        store_row<H>(sm + ST_A2, tid, a);
        umma::fence_before_sync();
        umma::fence_smem_to_async();
        __syncthreads();
        if (tid == 0) issue_layer<H>(tmem, TC_Z3, sm + ST_A2, sm + ST_W3, sy.mbar);
        sy.wait();
        load_act(tl + TC_Z3, b3, x, a);
        float o = b4;
#pragma unroll
        for (int k = 0; k < H; ++k) o = fmaf(a[k], w4[k], o);
        if (c < G) s_g[c] = o;
        umma::fence_before_sync();
        __syncthreads();
    }

    // Softmax cross-entropy against the tile's labels: g = (p - q) / nbatch.
    float loss = 0.f;
    {
        float m = -INFINITY;
        for (uint32_t c = tid; c < G; c += NTH) m = fmaxf(m, s_g[c]);
        for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
        if (lane == 0) red[warp] = m;
        __syncthreads();
        m = fmaxf(fmaxf(red[0], red[1]), fmaxf(red[2], red[3]));
        float s = 0.f;
        for (uint32_t c = tid; c < G; c += NTH) s += expf(s_g[c] - m);
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        __syncthreads();
        if (lane == 0) red[warp] = s;
        __syncthreads();
        s = (red[0] + red[1]) + (red[2] + red[3]);
        const float lse = m + logf(s);
        float l = 0.f;
        for (uint32_t c = tid; c < G; c += NTH) {
            const float q = labels[tile * G + c];
            const float lp = s_g[c] - lse;
            l -= q * lp;
            s_g[c] = (expf(lp) - q) * inv_n;
        }
        for (int o = 16; o > 0; o >>= 1) l += __shfl_xor_sync(0xffffffffu, l, o);
        __syncthreads();
        if (lane == 0) red[warp] = l;
        __syncthreads();
        loss = ((red[0] + red[1]) + (red[2] + red[3])) * inv_n;
    }

    // Pass 2, per block: forward keeping the operands, then backward.
    float* pw = part + warp * (4 * H + 1);
    for (uint32_t h = 0; h < nb && !s_abort; ++h) {
        const uint32_t c = h * R + tid;
        float a0[IN_PAD];
        load_features(feat, tile, c, G, a0);
        store_row<IN_PAD>(sm + ST_A0, tid, a0);
        store_col<IN_PAD>(sm + ST_A0T, tid, a0);
        umma::fence_smem_to_async();
        __syncthreads();
        float x[H], a[H];
        if (tid == 0) issue_layer<IN_PAD>(tmem, TC_Z1, sm + ST_A0, sm + ST_W1, sy.mbar);
        sy.wait();
        load_act(tl + TC_Z1, b1, x, a);
        store_row<H>(sm + ST_A1, tid, a);
        store_col<H>(sm + ST_A1T, tid, a);
        umma::fence_before_sync();
        umma::fence_smem_to_async();
        __syncthreads();
        if (tid == 0) issue_layer<H>(tmem, TC_Z2, sm + ST_A1, sm + ST_W2, sy.mbar);
        sy.wait();
        load_act(tl + TC_Z2, b2, x, a);
        store_row<H>(sm + ST_A2, tid, a);
        store_col<H>(sm + ST_A2T, tid, a);
        umma::fence_before_sync();
        umma::fence_smem_to_async();
        __syncthreads();
        if (tid == 0) issue_layer<H>(tmem, TC_Z3, sm + ST_A2, sm + ST_W3, sy.mbar);
        sy.wait();
        // Output layer and layer 3's input gradient.
        load_act(tl + TC_Z3, b3, x, a);
        const float g = c < G ? s_g[c] : 0.f;
        float d[H];
#pragma unroll
        for (int k = 0; k < H; ++k) {
            d[k] = g * w4[k] * gelu_d(x[k]);
            a[k] *= g;  // dw4 contribution
        }
        warp_sums<H>(a, pw + 3 * H);
        {
            float gs = g;
            for (int o = 16; o > 0; o >>= 1) gs += __shfl_xor_sync(0xffffffffu, gs, o);
            if (lane == 0) pw[4 * H] += gs;
        }
        warp_sums<H>(d, pw + 2 * H);
        store_row<H>(sm + ST_DZ, tid, d);
        store_col<H>(sm + ST_DZT, tid, d);
        umma::fence_before_sync();
        umma::fence_smem_to_async();
        __syncthreads();
        // dW3 += dz3^T a2 ; da2 = dz3 W3
        if (tid == 0) issue_backward<H>(tmem, TC_DW3, h > 0, sm + ST_DZT, sm + ST_A2T, sm + ST_DZ, sm + ST_W3T, sy.mbar);
        sy.wait();
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            float v[16], z[16];
            umma::tmem_ld16(tl + TC_DA + q * 16, v);
            umma::tmem_ld16(tl + TC_Z2 + q * 16, z);
#pragma unroll
            for (int j = 0; j < 16; ++j) d[q * 16 + j] = v[j] * gelu_d(z[j] + b2[q * 16 + j]);
        }
        warp_sums<H>(d, pw + H);
        store_row<H>(sm + ST_DZ, tid, d);
        store_col<H>(sm + ST_DZT, tid, d);
        umma::fence_before_sync();
        umma::fence_smem_to_async();
        __syncthreads();
        // dW2 += dz2^T a1 ; da1 = dz2 W2
        if (tid == 0) issue_backward<H>(tmem, TC_DW2, h > 0, sm + ST_DZT, sm + ST_A1T, sm + ST_DZ, sm + ST_W2T, sy.mbar);
        sy.wait();
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            float v[16], z[16];
            umma::tmem_ld16(tl + TC_DA + q * 16, v);
            umma::tmem_ld16(tl + TC_Z1 + q * 16, z);
#pragma unroll
            for (int j = 0; j < 16; ++j) d[q * 16 + j] = v[j] * gelu_d(z[j] + b1[q * 16 + j]);
        }
        warp_sums<H>(d, pw);
        store_col<H>(sm + ST_DZT, tid, d);
        umma::fence_before_sync();
        umma::fence_smem_to_async();
        __syncthreads();
        // dW1 += dz1^T a0
        if (tid == 0) issue_backward<IN_PAD>(tmem, TC_DW1, h > 0, sm + ST_DZT, sm + ST_A0T, nullptr, nullptr, sy.mbar);
        sy.wait();
        umma::fence_before_sync();
        __syncthreads();
    }

    // Write the partials: weights from TMEM (rows n = 0..63 live in the lanes
    // of warps 0 and 1), biases and w4 from the per-warp sums.
    float* out = grad_part + (uint64_t)blockIdx.x * (NPARAM + 1);
    if (!s_abort) {
        if (warp < 2) {
            const uint32_t n = tid;
            for (int q = 0; q < IN_PAD / 16; ++q) {
                float v[16];
                umma::tmem_ld16(tl + TC_DW1 + q * 16, v);
                for (int j = 0; j < 16; ++j) out[OW1 + n * IN_PAD + q * 16 + j] = v[j];
            }
            for (int q = 0; q < 4; ++q) {
                float v[16];
                umma::tmem_ld16(tl + TC_DW2 + q * 16, v);
                for (int j = 0; j < 16; ++j) out[OW2 + n * H + q * 16 + j] = v[j];
                umma::tmem_ld16(tl + TC_DW3 + q * 16, v);
                for (int j = 0; j < 16; ++j) out[OW3 + n * H + q * 16 + j] = v[j];
            }
        }
        __syncthreads();
        for (int i = tid; i < 4 * H + 1; i += NTH) {
            const float s = ((part[i] + part[(4 * H + 1) + i]) + part[2 * (4 * H + 1) + i]) + part[3 * (4 * H + 1) + i];
            int dst;
            if (i < H) dst = OB1 + i;
            else if (i < 2 * H) dst = OB2 + (i - H);
            else if (i < 3 * H) dst = OB3 + (i - 2 * H);
            else if (i < 4 * H) dst = OW4 + (i - 3 * H);
            else dst = OB4;
            out[dst] = s;
        }
        if (tid == 0) out[NPARAM] = loss;
    }
    umma::fence_before_sync();
    __syncthreads();
    if (warp == 0) umma::tmem_dealloc(tmem, 512);
}

// grad[p] = sum over CTAs of the partials, in CTA order.
__global__ void grad_reduce_kernel(const float* __restrict__ part, uint32_t nparts, float* __restrict__ grad) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p > (uint32_t)NPARAM) return;
    float s = 0.f;
    for (uint32_t b = 0; b < nparts; ++b) s += part[(uint64_t)b * (NPARAM + 1) + p];
    grad[p] = s;
}

__global__ void adam_kernel(float* __restrict__ prm, float* __restrict__ m, float* __restrict__ v,
                            const float* __restrict__ g, float lr, float b1, float b2, float eps, float c1, float c2) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= (uint32_t)NPARAM) return;
    const float gp = g[p];
    const float mp = fmaf(b1, m[p], (1.f - b1) * gp);
    const float vp = fmaf(b2, v[p], (1.f - b2) * gp * gp);
    m[p] = mp;
    v[p] = vp;
    prm[p] -= lr * (mp * c1) / (sqrtf(vp * c2) + eps);
}

// ----------------------------------------------------- capture -> features
// Pooled bins of a capture's profiles.
__host__ __device__ inline uint32_t pool_bins(float time_step) {
    const float r = POOL_M / time_step;
    return r < 1.5f ? 1u : (uint32_t)(r + 0.5f);
}

struct ClusterGeo {
    uint32_t n_side, cs, cpr, G;
};

__host__ __device__ inline ClusterGeo cluster_geo(uint32_t n_side, uint32_t cs) {
    ClusterGeo g;
    g.n_side = n_side;
    g.cs = cs;
    g.cpr = (n_side + cs - 1) / cs;
    g.G = g.cpr * g.cpr;
    return g;
}

// Per cluster: mean pooled profile prof[c][j] and centre (x, y, z, points).
template <typename S>
__global__ void cluster_profiles_kernel(const S* __restrict__ cube, int time_major, uint32_t L, uint32_t T,
                                        const float* __restrict__ laser_xyz, ClusterGeo cg, uint32_t pool, uint32_t J,
                                        float* __restrict__ prof, float4* __restrict__ centre) {
    const uint32_t c = blockIdx.x;
    const uint32_t cx = c % cg.cpr, cz = c / cg.cpr;
    const uint32_t x0 = cx * cg.cs, z0 = cz * cg.cs;
    const uint32_t w = min(cg.cs, cg.n_side - x0), hgt = min(cg.cs, cg.n_side - z0);
    const uint32_t npts = w * hgt;
    const float inv = 1.f / (float)npts;
    for (uint32_t j = threadIdx.x; j < J; j += blockDim.x) {
        float s = 0.f;
        const uint32_t t0 = j * pool, t1 = min(t0 + pool, T);
        for (uint32_t iz = 0; iz < hgt; ++iz)
            for (uint32_t ix = 0; ix < w; ++ix) {
                const uint64_t l = (uint64_t)(z0 + iz) * cg.n_side + x0 + ix;
                if (l >= L) continue;
                for (uint32_t t = t0; t < t1; ++t)
                    s += to_f32(time_major ? cube[(uint64_t)t * L + l] : cube[l * T + t]);
            }
        prof[(uint64_t)c * J + j] = s * inv;
    }
    if (threadIdx.x == 0) {
        float sx = 0.f, sy = 0.f, sz = 0.f;
        for (uint32_t iz = 0; iz < hgt; ++iz)
            for (uint32_t ix = 0; ix < w; ++ix) {
                const uint64_t l = (uint64_t)(z0 + iz) * cg.n_side + x0 + ix;
                if (l >= L) continue;
                sx += laser_xyz[3 * l];
                sy += laser_xyz[3 * l + 1];
                sz += laser_xyz[3 * l + 2];
            }
        centre[c] = make_float4(sx * inv, sy * inv, sz * inv, (float)npts);
    }
}

// Mean of the profiles (one block, fixed order).
__global__ void profile_mean_kernel(const float* __restrict__ prof, uint64_t n, float* __restrict__ mean) {
    __shared__ double red[256];
    double s = 0.0;
    for (uint64_t i = threadIdx.x; i < n; i += blockDim.x) s += prof[i];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) mean[0] = (float)(red[0] / (double)n) + 1e-30f;
}

struct TileGeo {
    uint32_t gx, gy;           // tiles along vx, vy
    float hmin[3], vs[3];
    uint32_t res[3];
    float t0, path_per_bin;    // metres of path per pooled bin
    int bounce;
    float lpos[3], spos[3];
};

__device__ inline float3 tile_centre(const TileGeo& tg, uint32_t tile) {
    const uint32_t bx = tile % tg.gx, by = (tile / tg.gx) % tg.gy, bz = tile / (tg.gx * tg.gy);
    const uint32_t x0 = bx * 8, y0 = by * 16, z0 = bz * 16;
    const float nx = (float)min(8u, tg.res[0] - x0), ny = (float)min(16u, tg.res[1] - y0),
                nz = (float)min(16u, tg.res[2] - z0);
    // Voxel (vx, vy, vz) sits at hmin + (vx, vz, vy) * vs + vs / 2.
    return make_float3(tg.hmin[0] + tg.vs[0] * ((float)x0 + 0.5f * nx),
                       tg.hmin[1] + tg.vs[1] * ((float)z0 + 0.5f * nz),
                       tg.hmin[2] + tg.vs[2] * ((float)y0 + 0.5f * ny));
}

__global__ void features_kernel(const float* __restrict__ prof, const float4* __restrict__ centre,
                                const float* __restrict__ mean, uint32_t G, uint32_t J, TileGeo tg, uint32_t ntotal,
                                const uint32_t* __restrict__ tiles, float* __restrict__ feat,
                                int* __restrict__ status) {
    const uint64_t ti = blockIdx.x;
    const uint32_t tile = tiles ? tiles[ti] : (uint32_t)ti;
    if (tile >= ntotal) {  // not a tile of this volume: zero rows, report
        for (uint32_t i = threadIdx.x; i < G * FEAT; i += blockDim.x) feat[ti * G * FEAT + i] = 0.f;
        if (threadIdx.x == 0) atomicExch(status, (int)FBP_ERR_DEVICE);
        return;
    }
    const float3 tc = tile_centre(tg, tile);
    const float inv_mean = 1.f / mean[0];
    for (uint32_t c = threadIdx.x; c < G; c += blockDim.x) {
        const float4 cc = centre[c];
        float f[FEAT];
        const float dx = tc.x - cc.x, dy = tc.y - cc.y, dz = tc.z - cc.z;
        f[0] = 0.5f * dx;
        f[1] = 0.5f * dy;
        f[2] = 0.5f * dz;
        float path = 2.f * sqrtf(dx * dx + dy * dy + dz * dz) - tg.t0;
        if (tg.bounce) {
            const float ax = tg.lpos[0] - cc.x, ay = tg.lpos[1] - cc.y, az = tg.lpos[2] - cc.z;
            const float sx = tg.spos[0] - cc.x, sy = tg.spos[1] - cc.y, sz = tg.spos[2] - cc.z;
            path += sqrtf(ax * ax + ay * ay + az * az) + sqrtf(sx * sx + sy * sy + sz * sz);
        }
        const int j0 = (int)floorf(path / tg.path_per_bin) - WINDOW / 2;
        for (int k = 0; k < WINDOW; ++k) {
            const int j = j0 + k;
            const float v = (j >= 0 && j < (int)J) ? prof[(uint64_t)c * J + j] : 0.f;
            f[3 + k] = log1pf(fmaxf(v, 0.f) * inv_mean);
        }
        f[IN] = 0.f;
        float4* o = reinterpret_cast<float4*>(feat + (ti * G + c) * FEAT);
#pragma unroll
        for (int q = 0; q < FEAT / 4; ++q) o[q] = make_float4(f[4 * q], f[4 * q + 1], f[4 * q + 2], f[4 * q + 3]);
    }
}

// Labels: q_c proportional to sqrt(sum_v F_vc^2) over the tile's voxels, F_vc
// = sum over cluster c's scan points of I(l, bin) * safeRCP(dist^2) with the
// reference kernel's arithmetic (transient_reconstruction.cuh:93-136).
template <typename S>
__global__ void __launch_bounds__(256) labels_kernel(const S* __restrict__ cube, int time_major, fbp_recon_info in,
                                                     const float4* __restrict__ scan, ClusterGeo cg, uint32_t gx,
                                                     uint32_t gy, uint32_t ntotal, const uint32_t* __restrict__ tiles,
                                                     float* __restrict__ labels, int* __restrict__ status) {
    __shared__ float s2[8][MAXG];
    __shared__ float red[8];
    const uint32_t tile = tiles[blockIdx.x];
    if (tile >= ntotal) {  // not a tile of this volume: uniform target, report
        for (uint32_t c = threadIdx.x; c < cg.G; c += blockDim.x) labels[(uint64_t)blockIdx.x * cg.G + c] = 1.f / (float)cg.G;
        if (threadIdx.x == 0) atomicExch(status, (int)FBP_ERR_DEVICE);
        return;
    }
    const uint32_t bx = tile % gx, by = (tile / gx) % gy, bz = tile / (gx * gy);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const uint32_t Vx = in.voxel_res[0], Vy = in.voxel_res[1], Vz = in.voxel_res[2];
    const uint32_t L = in.num_laser_targets, T = in.num_time_bins;
    const uint32_t vy = by * 16 + (tid & 15), vz = bz * 16 + (tid >> 4);
    const bool row_ok = vy < Vy && vz < Vz;
    float px[8];
    for (int k = 0; k < 8; ++k) px[k] = ref_voxel_coord(min(bx * 8 + k, Vx - 1), in.voxel_size[0], in.hidden_min[0]);
    const float py = ref_voxel_coord(min(vz, Vz - 1), in.voxel_size[1], in.hidden_min[1]);
    const float pz = ref_voxel_coord(min(vy, Vy - 1), in.voxel_size[2], in.hidden_min[2]);
    const float rcp_dt = rcp_approx(in.time_step);
    const bool bounce = in.discard_first_last_bounces == 0;
    for (uint32_t c = 0; c < cg.G; ++c) {
        const uint32_t cx = c % cg.cpr, cz = c / cg.cpr;
        const uint32_t x0 = cx * cg.cs, z0 = cz * cg.cs;
        const uint32_t w = min(cg.cs, cg.n_side - x0), hgt = min(cg.cs, cg.n_side - z0);
        float F[8];
        for (int k = 0; k < 8; ++k) F[k] = 0.f;
        for (uint32_t iz = 0; iz < hgt; ++iz)
            for (uint32_t ix = 0; ix < w; ++ix) {
                const uint32_t l = (z0 + iz) * cg.n_side + x0 + ix;
                if (l >= L) continue;
                const float4 g = scan[l];
                for (int k = 0; k < 8; ++k) {
                    float dist = fma_rn(sqrt_approx(ref_dot3(sub_rn(px[k], g.x), sub_rn(py, g.y), sub_rn(pz, g.z))),
                                        2.f, -in.time_offset);
                    if (bounce) dist = add_rn(dist, g.w);
                    const int b = __float2int_rz(ref_bin_ratio(dist, rcp_dt));
                    if (b < 0 || b >= (int)T) continue;
                    const float I = to_f32(time_major ? cube[(uint64_t)b * L + l] : cube[(uint64_t)l * T + b]);
                    if (I > FBP_EPS) F[k] = fmaf(I, ref_safe_rcp(mul_rn(dist, dist)), F[k]);
                }
            }
        float s = 0.f;
        if (row_ok)
            for (int k = 0; k < 8; ++k)
                if (bx * 8 + k < Vx) s = fmaf(F[k], F[k], s);
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == 0) s2[warp][c] = s;
    }
    __syncthreads();
    // q_c = sqrt(S2_c) / sum (uniform when the tile receives nothing).
    float local = 0.f;
    for (uint32_t c = tid; c < cg.G; c += blockDim.x) {
        float t = 0.f;
        for (int w = 0; w < 8; ++w) t += s2[w][c];
        t = sqrtf(t);
        s2[0][c] = t;
        local += t;
    }
    for (int o = 16; o > 0; o >>= 1) local += __shfl_xor_sync(0xffffffffu, local, o);
    if (lane == 0) red[warp] = local;
    __syncthreads();
    float tot = 0.f;
    for (int w = 0; w < 8; ++w) tot += red[w];
    for (uint32_t c = tid; c < cg.G; c += blockDim.x)
        labels[(uint64_t)blockIdx.x * cg.G + c] = tot > 0.f ? s2[0][c] / tot : 1.f / (float)cg.G;
}

// ------------------------------------------------------------------- host

fbp_status check_clusters(const fbp_recon_info* info, uint32_t cluster_side, uint32_t scan_side, ClusterGeo* cg,
                          const char* who) {
    if (!info) return set_error(FBP_ERR_INVALID_ARG, std::string(who) + ": null info");
    if (cluster_side == 0 || scan_side == 0 || (uint64_t)scan_side * scan_side != info->num_laser_targets)
        return set_error(FBP_ERR_INVALID_ARG,
                         std::string(who) + ": scan_side^2 must equal the scan points and cluster_side be > 0");
    *cg = cluster_geo(scan_side, cluster_side);
    if (cg->G > (uint32_t)MAXG)
        return set_error(FBP_ERR_UNSUPPORTED, std::string(who) + ": more than 1024 clusters per capture");
    return FBP_OK;
}

TileGeo tile_geo(const fbp_recon_info& in) {
    TileGeo tg{};
    tg.gx = cdiv(in.voxel_res[0], 8);
    tg.gy = cdiv(in.voxel_res[1], 16);
    for (int k = 0; k < 3; ++k) {
        tg.hmin[k] = in.hidden_min[k];
        tg.vs[k] = in.voxel_size[k];
        tg.res[k] = in.voxel_res[k];
        tg.lpos[k] = in.laser_position[k];
        tg.spos[k] = in.sensor_position[k];
    }
    tg.t0 = in.time_offset;
    tg.path_per_bin = in.time_step * (float)pool_bins(in.time_step);
    tg.bounce = in.discard_first_last_bounces == 0;
    return tg;
}

uint64_t num_tiles(const fbp_recon_info& in) {
    return (uint64_t)cdiv(in.voxel_res[0], 8) * cdiv(in.voxel_res[1], 16) * cdiv(in.voxel_res[2], 16);
}

template <typename S>
fbp_status profiles_typed(fbp_context* ctx, const fbp_recon_info& in, const void* cube, int layout,
                          const float* laser_xyz, const ClusterGeo& cg, cudaStream_t s, float** prof, float4** centre,
                          float** mean, uint32_t* J_out) {
    const uint32_t pool = pool_bins(in.time_step);
    const uint32_t J = cdiv(in.num_time_bins, pool);
    const size_t prof_bytes = ((size_t)cg.G * J * sizeof(float) + 255) & ~size_t(255);
    const size_t centre_bytes = (size_t)cg.G * sizeof(float4);
    void* ws = nullptr;
    FBP_TRY(workspace(ctx, WS_MLP_PROFILES, prof_bytes + centre_bytes + 256, s, &ws));
    *prof = static_cast<float*>(ws);
    *centre = reinterpret_cast<float4*>(static_cast<char*>(ws) + prof_bytes);
    *mean = reinterpret_cast<float*>(static_cast<char*>(ws) + prof_bytes + centre_bytes);
    cluster_profiles_kernel<S><<<cg.G, 128, 0, s>>>(static_cast<const S*>(cube), layout == FBP_LAYOUT_TIME_MAJOR,
                                                    in.num_laser_targets, in.num_time_bins, laser_xyz, cg, pool, J,
                                                    *prof, *centre);
    FBP_CHECK_LAUNCH(ctx, "cluster_profiles_kernel");
    profile_mean_kernel<<<1, 256, 0, s>>>(*prof, (uint64_t)cg.G * J, *mean);
    FBP_CHECK_LAUNCH(ctx, "profile_mean_kernel");
    *J_out = J;
    return FBP_OK;
}

fbp_status validate_capture(const fbp_recon_info* info, const void* cube, int dtype, int layout,
                            const float* laser_xyz, const char* who) {
    FBP_TRY(validate_info(info, false, who));
    if (!cube || !laser_xyz) return set_error(FBP_ERR_INVALID_ARG, std::string(who) + ": null buffer");
    if (layout != FBP_LAYOUT_TIME_MAJOR && layout != FBP_LAYOUT_TIME_INNER)
        return set_error(FBP_ERR_INVALID_ARG, std::string(who) + ": unknown layout");
    if (dtype != FBP_F32 && dtype != FBP_BF16 && dtype != FBP_F16)
        return set_error(FBP_ERR_INVALID_ARG, std::string(who) + ": unknown dtype");
    return FBP_OK;
}

fbp_status set_smem(const void* k, int bytes) {
    FBP_TRY_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
    return FBP_OK;
}

}  // namespace mlp
}  // namespace fbp

using namespace fbp;
using namespace fbp::mlp;

extern "C" uint32_t fbp_mlp_num_params(void) { return (uint32_t)NPARAM; }

extern "C" fbp_status fbp_mlp_create(fbp_context* ctx, uint64_t seed, fbp_mlp** out) {
    return guarded("fbp_mlp_create", [&]() -> fbp_status {
        clear_error();
        FBP_TRY(check_ctx(ctx));
        if (!out) return set_error(FBP_ERR_INVALID_ARG, "fbp_mlp_create: null output");
        *out = nullptr;
        fbp_mlp* m = new (std::nothrow) fbp_mlp();
        if (!m) return set_error(FBP_ERR_OOM, "fbp_mlp_create: host allocation failed");
        m->ctx = ctx;
        const size_t bytes = (size_t)NPARAM * sizeof(float);
        if (cudaMalloc(&m->params, bytes) != cudaSuccess || cudaMalloc(&m->adam_m, bytes) != cudaSuccess ||
            cudaMalloc(&m->adam_v, bytes) != cudaSuccess || cudaMalloc(&m->grad, bytes + sizeof(float)) != cudaSuccess) {
            cudaFree(m->params);
            cudaFree(m->adam_m);
            cudaFree(m->adam_v);
            cudaFree(m->grad);
            delete m;
            return set_error(FBP_ERR_OOM, "fbp_mlp_create: device allocation failed");
        }
        // Uniform(-1/sqrt(fan_in), 1/sqrt(fan_in)) weights, zero biases; the
        // padded input columns of layer 1 stay zero.
        std::vector<float> h(NPARAM, 0.f);
        std::mt19937_64 rng(seed);
        auto fill = [&](int off, int rows, int cols, int used, float bound) {
            std::uniform_real_distribution<float> u(-bound, bound);
            for (int r = 0; r < rows; ++r)
                for (int c = 0; c < cols; ++c) h[off + r * cols + c] = c < used ? u(rng) : 0.f;
        };
        fill(OW1, H, IN_PAD, IN, 1.f / std::sqrt((float)IN));
        fill(OW2, H, H, H, 1.f / std::sqrt((float)H));
        fill(OW3, H, H, H, 1.f / std::sqrt((float)H));
        fill(OW4, 1, H, H, 1.f / std::sqrt((float)H));
        cudaMemcpy(m->params, h.data(), bytes, cudaMemcpyHostToDevice);
        cudaMemset(m->adam_m, 0, bytes);
        cudaMemset(m->adam_v, 0, bytes);
        if (cudaGetLastError() != cudaSuccess) {
            fbp_mlp_destroy(m);
            return set_error(FBP_ERR_CUDA, "fbp_mlp_create: initialisation failed");
        }
        *out = m;
        return FBP_OK;
    });
}

extern "C" fbp_status fbp_mlp_destroy(fbp_mlp* m) {
    return guarded("fbp_mlp_destroy", [&]() -> fbp_status {
        clear_error();
        if (!m) return FBP_OK;
        cudaFree(m->params);
        cudaFree(m->adam_m);
        cudaFree(m->adam_v);
        cudaFree(m->grad);
        delete m;
        return FBP_OK;
    });
}

extern "C" fbp_status fbp_mlp_get_params(const fbp_mlp* m, float* host, uint32_t n) {
    return guarded("fbp_mlp_get_params", [&]() -> fbp_status {
        clear_error();
        if (!m || !host || n != (uint32_t)NPARAM) return set_error(FBP_ERR_INVALID_ARG, "fbp_mlp_get_params: bad arguments");
        FBP_TRY_CUDA(cudaMemcpy(host, m->params, n * sizeof(float), cudaMemcpyDeviceToHost));
        return FBP_OK;
    });
}

extern "C" fbp_status fbp_mlp_set_params(fbp_mlp* m, const float* host, uint32_t n) {
    return guarded("fbp_mlp_set_params", [&]() -> fbp_status {
        clear_error();
        if (!m || !host || n != (uint32_t)NPARAM) return set_error(FBP_ERR_INVALID_ARG, "fbp_mlp_set_params: bad arguments");
        FBP_TRY_CUDA(cudaMemcpy(m->params, host, n * sizeof(float), cudaMemcpyHostToDevice));
        FBP_TRY_CUDA(cudaMemset(m->adam_m, 0, n * sizeof(float)));
        FBP_TRY_CUDA(cudaMemset(m->adam_v, 0, n * sizeof(float)));
        m->step = 0;
        return FBP_OK;
    });
}

extern "C" fbp_status fbp_mlp_features(fbp_context* ctx, const fbp_recon_info* info, const void* cube, int dtype,
                                       int layout, const float* laser_xyz, uint32_t cluster_side, uint32_t scan_side,
                                       const uint32_t* tiles, uint32_t ntiles, float* features, void* stream) {
    return guarded("fbp_mlp_features", [&]() -> fbp_status {
        clear_error();
        FBP_TRY(check_ctx(ctx));
        FBP_TRY(validate_capture(info, cube, dtype, layout, laser_xyz, "fbp_mlp_features"));
        ClusterGeo cg;
        FBP_TRY(check_clusters(info, cluster_side, scan_side, &cg, "fbp_mlp_features"));
        if (!features) return set_error(FBP_ERR_INVALID_ARG, "fbp_mlp_features: null output");
        const uint64_t nt = tiles ? ntiles : num_tiles(*info);
        if (nt == 0) return FBP_OK;
        if (nt > 0x7FFFFFFFull) return set_error(FBP_ERR_UNSUPPORTED, "fbp_mlp_features: too many tiles");
        cudaStream_t s = (cudaStream_t)stream;
        float *prof, *mean;
        float4* centre;
        uint32_t J;
        switch (dtype) {
            case FBP_F32: FBP_TRY(profiles_typed<float>(ctx, *info, cube, layout, laser_xyz, cg, s, &prof, &centre, &mean, &J)); break;
            case FBP_BF16: FBP_TRY(profiles_typed<__nv_bfloat16>(ctx, *info, cube, layout, laser_xyz, cg, s, &prof, &centre, &mean, &J)); break;
            default: FBP_TRY(profiles_typed<__half>(ctx, *info, cube, layout, laser_xyz, cg, s, &prof, &centre, &mean, &J)); break;
        }
        features_kernel<<<(unsigned)nt, 256, 0, s>>>(prof, centre, mean, cg.G, J, tile_geo(*info),
                                                     (uint32_t)num_tiles(*info), tiles, features, ctx->status_dev);
        FBP_CHECK_LAUNCH(ctx, "features_kernel");
        return FBP_OK;
    });
}

extern "C" fbp_status fbp_mlp_labels(fbp_context* ctx, const fbp_recon_info* info, const void* cube, int dtype,
                                     int layout, const float* laser_xyz, uint32_t cluster_side, uint32_t scan_side,
                                     const uint32_t* tiles, uint32_t ntiles, float* labels, void* stream) {
    return guarded("fbp_mlp_labels", [&]() -> fbp_status {
        clear_error();
        FBP_TRY(check_ctx(ctx));
        FBP_TRY(validate_capture(info, cube, dtype, layout, laser_xyz, "fbp_mlp_labels"));
        ClusterGeo cg;
        FBP_TRY(check_clusters(info, cluster_side, scan_side, &cg, "fbp_mlp_labels"));
        if (!tiles || !labels) return set_error(FBP_ERR_INVALID_ARG, "fbp_mlp_labels: null tiles or output");
        if (ntiles == 0) return FBP_OK;
        cudaStream_t s = (cudaStream_t)stream;
        const float4* scan;
        const float *xs, *ys, *zs;
        FBP_TRY(build_tables(ctx, *info, laser_xyz, s, &scan, &xs, &ys, &zs));
        const uint32_t gx = cdiv(info->voxel_res[0], 8), gy = cdiv(info->voxel_res[1], 16);
        const uint32_t nall = (uint32_t)std::min<uint64_t>(num_tiles(*info), 0xFFFFFFFFull);
        const int tm = layout == FBP_LAYOUT_TIME_MAJOR;
        switch (dtype) {
            case FBP_F32:
                labels_kernel<float><<<ntiles, 256, 0, s>>>(static_cast<const float*>(cube), tm, *info, scan, cg, gx, gy, nall, tiles, labels, ctx->status_dev);
                break;
            case FBP_BF16:
                labels_kernel<__nv_bfloat16><<<ntiles, 256, 0, s>>>(static_cast<const __nv_bfloat16*>(cube), tm, *info, scan, cg, gx, gy, nall, tiles, labels, ctx->status_dev);
                break;
            default:
                labels_kernel<__half><<<ntiles, 256, 0, s>>>(static_cast<const __half*>(cube), tm, *info, scan, cg, gx, gy, nall, tiles, labels, ctx->status_dev);
                break;
        }
        FBP_CHECK_LAUNCH(ctx, "labels_kernel");
        return FBP_OK;
    });
}

extern "C" fbp_status fbp_mlp_forward(fbp_context* ctx, const fbp_mlp* m, const float* features, uint32_t ntiles,
                                      uint32_t G, float* logits, float defensive, float* tile_cdf, void* stream) {
    return guarded("fbp_mlp_forward", [&]() -> fbp_status {
        clear_error();
        FBP_TRY(check_ctx(ctx));
        if (!m || !features || (!logits && !tile_cdf)) return set_error(FBP_ERR_INVALID_ARG, "fbp_mlp_forward: null argument");
        if (G == 0 || G > (uint32_t)MAXG) return set_error(FBP_ERR_UNSUPPORTED, "fbp_mlp_forward: G must be in 1..1024");
        if (!(defensive >= 0.f && defensive <= 1.f)) return set_error(FBP_ERR_INVALID_ARG, "fbp_mlp_forward: defensive share not in [0, 1]");
        if (ntiles == 0) return FBP_OK;
        FBP_TRY(set_smem((const void*)mlp_infer_kernel, SI_BYTES));
        mlp_infer_kernel<<<ntiles, NTH, SI_BYTES, (cudaStream_t)stream>>>(m->params, features, G, defensive, logits,
                                                                           tile_cdf, ctx->status_dev);
        FBP_CHECK_LAUNCH(ctx, "mlp_infer_kernel");
        return FBP_OK;
    });
}

namespace {

fbp_status gradients(fbp_context* ctx, const fbp_mlp* m, const float* features, const float* labels,
                     const uint32_t* idx, uint32_t nbatch, uint32_t G, float* grad, cudaStream_t s) {
    if (!features || !labels || !idx || !grad || nbatch == 0)
        return set_error(FBP_ERR_INVALID_ARG, "fbp_mlp: null argument or empty batch");
    if (G == 0 || G > (uint32_t)MAXG) return set_error(FBP_ERR_UNSUPPORTED, "fbp_mlp: G must be in 1..1024");
    void* part = nullptr;
    FBP_TRY(workspace(ctx, WS_MLP_PARTIALS, (size_t)nbatch * (NPARAM + 1) * sizeof(float), s, &part));
    FBP_TRY(set_smem((const void*)mlp_train_kernel, ST_BYTES));
    mlp_train_kernel<<<nbatch, NTH, ST_BYTES, s>>>(m->params, features, labels, idx, nbatch, G,
                                                   static_cast<float*>(part), ctx->status_dev);
    FBP_CHECK_LAUNCH(ctx, "mlp_train_kernel");
    grad_reduce_kernel<<<cdiv(NPARAM + 1, 256), 256, 0, s>>>(static_cast<const float*>(part), nbatch, grad);
    FBP_CHECK_LAUNCH(ctx, "grad_reduce_kernel");
    return FBP_OK;
}

}  // namespace

extern "C" fbp_status fbp_mlp_gradients(fbp_context* ctx, const fbp_mlp* m, const float* features,
                                        const float* labels, const uint32_t* idx, uint32_t nbatch, uint32_t G,
                                        float* grad_loss, void* stream) {
    return guarded("fbp_mlp_gradients", [&]() -> fbp_status {
        clear_error();
        FBP_TRY(check_ctx(ctx));
        if (!m) return set_error(FBP_ERR_INVALID_ARG, "fbp_mlp_gradients: null network");
        return gradients(ctx, m, features, labels, idx, nbatch, G, grad_loss, (cudaStream_t)stream);
    });
}

extern "C" fbp_status fbp_mlp_train_step(fbp_context* ctx, fbp_mlp* m, const float* features, const float* labels,
                                         const uint32_t* idx, uint32_t nbatch, uint32_t G, float lr, float* loss,
                                         void* stream) {
    return guarded("fbp_mlp_train_step", [&]() -> fbp_status {
        clear_error();
        FBP_TRY(check_ctx(ctx));
        if (!m) return set_error(FBP_ERR_INVALID_ARG, "fbp_mlp_train_step: null network");
        if (!(lr > 0.f)) return set_error(FBP_ERR_INVALID_ARG, "fbp_mlp_train_step: learning rate must be > 0");
        cudaStream_t s = (cudaStream_t)stream;
        FBP_TRY(gradients(ctx, m, features, labels, idx, nbatch, G, m->grad, s));
        m->step += 1;
        const float b1 = 0.9f, b2 = 0.999f;
        const float c1 = (float)(1.0 / (1.0 - std::pow((double)b1, (double)m->step)));
        const float c2 = (float)(1.0 / (1.0 - std::pow((double)b2, (double)m->step)));
        adam_kernel<<<cdiv(NPARAM, 256), 256, 0, s>>>(m->params, m->adam_m, m->adam_v, m->grad, lr, b1, b2, 1e-8f, c1, c2);
        FBP_CHECK_LAUNCH(ctx, "adam_kernel");
        if (loss) FBP_TRY_CUDA(cudaMemcpyAsync(loss, m->grad + NPARAM, sizeof(float), cudaMemcpyDeviceToDevice, s));
        return FBP_OK;
    });
}

extern "C" fbp_status fbp_mlp_tile_count(const fbp_recon_info* info, uint32_t* ntiles) {
    return guarded("fbp_mlp_tile_count", [&]() -> fbp_status {
        clear_error();
        if (!info || !ntiles) return set_error(FBP_ERR_INVALID_ARG, "fbp_mlp_tile_count: null argument");
        const uint64_t n = num_tiles(*info);
        if (n > 0xFFFFFFFFull) return set_error(FBP_ERR_UNSUPPORTED, "fbp_mlp_tile_count: too many tiles");
        *ntiles = (uint32_t)n;
        return FBP_OK;
    });
}
