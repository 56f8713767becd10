// Confocal backprojection as a voxel-tiled gather.
//
// Replaces Laser::reconstructAABBConfocal (Laser.cu:482-498) and
// backprojectConfocalVoxel (transient_reconstruction.cuh:93-136).  The
// reference launches one thread per (voxel, scan point) pair and adds each
// contribution with a global FP32 atomic.  Here one CTA owns a tile of voxels
// and walks all scan points; for every scan point it stages only the window
// of time bins the tile can reach into shared memory (cp.async), so each
// pair costs a shared-memory load instead of a global gather + atomic, and the
// sum order is fixed (reproducible run to run).
//
// Data layout in HBM (per call, in the context's scratch):
//   rows   [L][row_pitch] of the storage type: one padded row per scan point,
//          time innermost, values <= 1e-5 already replaced by 0 (the
//          reference skips them), zeros in [T, row_pitch).
//   scan   [L] float4 (x, y, z, bounce)   bounce = |l-laser|+|l-sensor| or 0
//   axes   xs[Vx], ys[Vz], zs[Vy]         voxel-centre coordinates
#include "fbp_internal.cuh"
#include "bp_common.cuh"

#include <algorithm>
#include <cmath>

namespace fbp {

// ------------------------------------------------------------ prep kernels --

__global__ void axis_tables_kernel(float* __restrict__ xs, float* __restrict__ ys, float* __restrict__ zs,
                                   uint32_t Vx, uint32_t Vy, uint32_t Vz, float mnx, float mny, float mnz, float sx,
                                   float sy, float sz) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    // transient_reconstruction.cuh:106: (vx, vz, vy) drive world (x, y, z).
    if (i < Vx) xs[i] = ref_voxel_coord(i, sx, mnx);
    if (i < Vz) ys[i] = ref_voxel_coord(i, sy, mny);
    if (i < Vy) zs[i] = ref_voxel_coord(i, sz, mnz);
}

// Per scan point (x, y, z, bounce): transient_reconstruction.cuh:109-110.
__global__ void scan_table_kernel(float4* __restrict__ out, const float* __restrict__ xyz, uint32_t n, int discard,
                                  float ax, float ay, float az, float bx, float by, float bz, int confocal_pair) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float x = xyz[3 * (size_t)i], y = xyz[3 * (size_t)i + 1], z = xyz[3 * (size_t)i + 2];
    float b = 0.f;
    if (discard == 0) {
        // confocal: |l - laserPos| + |l - sensorPos|; exhaustive tables carry
        // one distance each (|l - laserPos| or |s - sensorPos|).
        const float d1 = ref_distance(x, y, z, ax, ay, az);
        b = confocal_pair ? add_rn(d1, ref_distance(x, y, z, bx, by, bz)) : d1;
    }
    out[i] = make_float4(x, y, z, b);
}

// Rows from a time-innermost cube: copy, threshold, pad.
template <typename S>
__global__ void rows_from_time_inner_kernel(S* __restrict__ rows, const S* __restrict__ cube, uint32_t L, uint32_t T,
                                            uint32_t pitch) {
    const uint64_t n = (uint64_t)L * pitch;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t l = (uint32_t)(i / pitch), t = (uint32_t)(i % pitch);
        S v = from_f32<S>(0.f);
        if (t < T) {
            const S c = cube[(uint64_t)l * T + t];
            if (to_f32(c) > FBP_EPS) v = c;
        }
        rows[i] = v;
    }
}

// Rows from a time-major cube (cube[t*L + l]): tiled transpose through shared
// memory so both the read and the write are coalesced.
template <typename S>
__global__ void rows_from_time_major_kernel(S* __restrict__ rows, const S* __restrict__ cube, uint32_t L, uint32_t T,
                                            uint32_t pitch) {
    __shared__ float tile[32][33];
    const uint32_t l0 = blockIdx.x * 32, t0 = blockIdx.y * 32;
    for (int j = threadIdx.y; j < 32; j += blockDim.y) {
        const uint32_t t = t0 + j, l = l0 + threadIdx.x;
        float v = 0.f;
        if (t < T && l < L) {
            v = to_f32(cube[(uint64_t)t * L + l]);
            if (!(v > FBP_EPS)) v = 0.f;
        }
        tile[j][threadIdx.x] = v;
    }
    __syncthreads();
    for (int j = threadIdx.y; j < 32; j += blockDim.y) {
        const uint32_t l = l0 + j, t = t0 + threadIdx.x;
        if (l < L && t < pitch) rows[(uint64_t)l * pitch + t] = from_f32<S>(tile[threadIdx.x][j]);
    }
}

// Zero the padding columns [roundup(T,32), pitch) the transpose grid does not cover.
template <typename S>
__global__ void rows_zero_tail_kernel(S* __restrict__ rows, uint32_t L, uint32_t from, uint32_t pitch) {
    const uint32_t w = pitch - from;
    const uint64_t n = (uint64_t)L * w;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        rows[(i / w) * pitch + from + (i % w)] = from_f32<S>(0.f);
}

// ----------------------------------------------------------- gather kernel --

// Arithmetic paths of the pair loop (all reproduce the reference's bins):
//   PATH_2D     time_offset == 0, no bounce terms: dist = 2d exactly, so
//               x = d * (2 rcp(dt)) and the weight is rcp(d^2) = 4 rcp(dist^2);
//               the stage's partial sum is scaled by 1/4 (exact).
//   PATH_FAST   time_offset <= 0 (every path >= 0): dist = fma(d, 2, -t0) [+ bounce].
//   PATH_EXACT  time_offset > 0: negative paths possible, bin by conversion.
// In PATH_2D / PATH_FAST the bin is floor(x) - a via a round-toward-zero add of
// 2^23 - a; without CLAMP the window planner guarantees every bin of the tile
// lies inside its window, so the -2^23 bias folds into the shared-memory base.
enum { PATH_2D = 0, PATH_FAST = 1, PATH_EXACT = 2 };

template <typename S>
__device__ __forceinline__ float lds_elem(uint32_t addr);
template <>
__device__ __forceinline__ float lds_elem<float>(uint32_t addr) {
    float v;
    asm volatile("ld.shared.f32 %0, [%1];" : "=f"(v) : "r"(addr));
    return v;
}
template <>
__device__ __forceinline__ float lds_elem<__nv_bfloat16>(uint32_t addr) {
    unsigned short v;
    asm volatile("ld.shared.u16 %0, [%1];" : "=h"(v) : "r"(addr));
    return __uint_as_float((uint32_t)v << 16);
}
template <>
__device__ __forceinline__ float lds_elem<__half>(uint32_t addr) {
    unsigned short v;
    asm volatile("ld.shared.u16 %0, [%1];" : "=h"(v) : "r"(addr));
    return __half2float(__ushort_as_half(v));
}

template <typename S> struct ElemShift;
template <> struct ElemShift<float> { static constexpr int value = 2; };
template <> struct ElemShift<__nv_bfloat16> { static constexpr int value = 1; };
template <> struct ElemShift<__half> { static constexpr int value = 1; };

// One staged stage of scan points against a thread's KV voxels (consecutive
// along x, sharing the y/z offsets).
template <typename S, int KV, int PATH, bool BOUNCE, bool CLAMP, bool SAFE, bool WEIGHTED>
__device__ __forceinline__ void confocal_stage(const float4* __restrict__ geo, const int2* __restrict__ meta,
                                               const float* __restrict__ wts, int nl, const float (&px)[KV], float py,
                                               float pz, float neg_t0, float rcp_dt, uint32_t slot_w,
                                               float (&acc)[KV]) {
    constexpr int SH = ElemShift<S>::value;
    const float rcp2 = 2.f * rcp_dt;  // exact
#pragma unroll 2
    for (int i = 0; i < nl; ++i) {
        const float4 g = geo[i];
        const int2 m = meta[i];  // (bin bias: float 2^23 - a, or a; slot shared address)
        const float wl = WEIGHTED ? wts[i] : 1.f;
        const float dy = sub_rn(py, g.y), dz = sub_rn(pz, g.z);
        const float dy2 = mul_rn(dy, dy);
#pragma unroll
        for (int k = 0; k < KV; ++k) {
            const float dx = sub_rn(px[k], g.x);
            const float d = sqrt_approx(fma_rn(dz, dz, fma_rn(dx, dx, dy2)));
            float x, dist = 0.f;
            if (PATH == PATH_2D && !SAFE) {
                x = mul_rn(d, rcp2);
            } else {
                dist = fma_rn(d, 2.f, neg_t0);
                if (BOUNCE) dist = add_rn(dist, g.w);
                x = ref_bin_ratio(dist, rcp_dt);
            }
            uint32_t addr;
            if (PATH == PATH_EXACT) {
                const int b = __float2int_rz(x);  // static_cast<int>, like the reference
                addr = (uint32_t)m.y + (min((uint32_t)(b - m.x), slot_w) << SH);
            } else {
                const uint32_t bits = __float_as_uint(add_rz(x, __int_as_float(m.x)));
                if (CLAMP) addr = (uint32_t)m.y + (min(bits - 0x4B000000u, slot_w) << SH);
                else addr = (uint32_t)m.y + (bits << SH);  // bias folded into m.y
            }
            float I = lds_elem<S>(addr);
            if (WEIGHTED) I *= wl;
            float w;
            if (PATH == PATH_2D && !SAFE) w = rcp_approx(mul_rn(d, d));
            else w = SAFE ? ref_safe_rcp(mul_rn(dist, dist)) : rcp_approx(mul_rn(dist, dist));
            acc[k] = fmaf(I, w, acc[k]);
        }
    }
}

// The main kernel.  One CTA of 32*WY*WZ threads owns a tile of KV (x) x 8*WY
// (rows) x 4*WZ (depth slices) voxels; a warp covers 8 rows x 4 slices, a
// thread KV consecutive voxels along x.  Scan points (or, SAMPLED, K scan
// points drawn per tile) are walked in stages of up to 32: one warp plans the
// bin windows of the stage, all threads copy them from the padded rows into
// shared memory with cp.async (double buffered), then every thread runs the
// pair loop against the staged windows.  FP32 partials per stage, Kahan
// across stages.
template <typename S, int KV, int WY, int WZ, int PATH, bool BOUNCE, bool SAMPLED, bool CLAMP>
__global__ void __launch_bounds__(32 * WY * WZ)
confocal_gather_kernel(ConfocalGatherParams p) {
    constexpr int NT = 32 * WY * WZ;
    constexpr int CHMAX = 32;
    constexpr int ALIGN = 16 / sizeof(S);  // elements per 16-byte copy
    constexpr int SH = ElemShift<S>::value;
    constexpr int TY = 8 * WY, TZ = 4 * WZ;
    const int CH = p.ch;

    extern __shared__ __align__(16) unsigned char smem_raw[];
    const uint32_t slot_stride = p.slot_w + ALIGN;  // sentinel element(s) at slot_w
    float4* s_geo = reinterpret_cast<float4*>(smem_raw);         // [2][CHMAX]
    int2* s_meta = reinterpret_cast<int2*>(s_geo + 2 * CHMAX);   // [2][CHMAX]
    int* s_cnt = reinterpret_cast<int*>(s_meta + 2 * CHMAX);     // [2][CHMAX]
    int* s_src = s_cnt + 2 * CHMAX;                              // [2][CHMAX]
    int* s_row = s_src + 2 * CHMAX;                              // [2][CHMAX]
    float* s_w = reinterpret_cast<float*>(s_row + 2 * CHMAX);    // [2][CHMAX]
    int* s_flag = reinterpret_cast<int*>(s_w + 2 * CHMAX);       // [2]
    const size_t slots_off = ConfocalGatherParams::meta_bytes(CHMAX);
    S* s_slots = reinterpret_cast<S*>(smem_raw + slots_off);     // [2][CH][slot_stride], then the zero slot
    const uint32_t sbase = (uint32_t)__cvta_generic_to_shared(smem_raw);
    const uint32_t zero_slot = 2u * CH * slot_stride;            // element index of the all-zero slot

    const int tid = threadIdx.x;
    const int lane = tid & 31, warp = tid >> 5;
    const int wy = warp % WY, wz = warp / WY;

    const uint32_t tx0 = blockIdx.x * KV, ty0 = blockIdx.y * TY, tz0 = blockIdx.z * TZ;
    const uint32_t vy = ty0 + wy * 8 + (lane & 7);
    const uint32_t vz = tz0 + wz * 4 + (lane >> 3);
    const bool row_ok = vy < p.Vy && vz < p.Vz;

    // Tile AABB of voxel centres (clamped to the volume).
    const uint32_t tx1 = min(tx0 + KV, p.Vx) - 1, ty1 = min(ty0 + TY, p.Vy) - 1, tz1 = min(tz0 + TZ, p.Vz) - 1;
    const float bx0 = fminf(p.xs[tx0], p.xs[tx1]), bx1 = fmaxf(p.xs[tx0], p.xs[tx1]);
    const float by0 = fminf(p.ys[tz0], p.ys[tz1]), by1 = fmaxf(p.ys[tz0], p.ys[tz1]);
    const float bz0 = fminf(p.zs[ty0], p.zs[ty1]), bz1 = fmaxf(p.zs[ty0], p.zs[ty1]);

    const float py = p.ys[min(vz, p.Vz - 1)];
    const float pz = p.zs[min(vy, p.Vy - 1)];
    float px[KV];
#pragma unroll
    for (int k = 0; k < KV; ++k) px[k] = p.xs[min(tx0 + k, p.Vx - 1)];

    const float rcp_dt = rcp_approx(p.dt);
    const float neg_t0 = -p.t0;

    // Sentinels of every slot and the whole zero slot.
    for (int i = tid; i < 2 * CH * ALIGN; i += NT) {
        const int slot = i / ALIGN, e = i % ALIGN;
        s_slots[(size_t)slot * slot_stride + p.slot_w + e] = from_f32<S>(0.f);
    }
    for (uint32_t i = tid; i < slot_stride; i += NT) s_slots[zero_slot + i] = from_f32<S>(0.f);

    const uint32_t nitems = SAMPLED ? p.smp.K : p.L;
    const uint32_t nchunks = (nitems + CH - 1) / CH;
    const unsigned long long tile_id =
        ((unsigned long long)blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x;

    // Plan a stage: bin window of each scan point (threads < CH, all in warp 0).
    auto plan_chunk = [&](uint32_t c, int buf) {
        if (tid < CH) {
            const uint32_t item = c * CH + tid;
            uint32_t l = item;
            float wgt = 1.f;
            if (SAMPLED && item < nitems) {
                const float u1 = hash_uniform(p.smp.seed, tile_id, item, 0);
                const float u2 = hash_uniform(p.smp.seed, tile_id, item, 1);
                float pl;
                if (p.smp.mode == SAMPLE_UNIFORM) {
                    l = min((uint32_t)(u1 * (float)p.L), p.L - 1);
                    pl = 1.f / (float)p.L;
                } else if (p.smp.mode == SAMPLE_ALIAS) {
                    const uint32_t kk = min((uint32_t)(u1 * (float)p.L), p.L - 1);
                    l = u2 < p.smp.prob[kk] ? kk : p.smp.alias[kk];
                    pl = p.smp.pl[l];
                } else {
                    // Cluster from the tile's CDF (binary search), then uniform inside it.
                    const float* cdf = p.smp.tile_cdf + tile_id * p.smp.G;
                    uint32_t lo = 0, hi = p.smp.G - 1;
                    while (lo < hi) {
                        const uint32_t mid = (lo + hi) >> 1;
                        if (u1 < cdf[mid]) hi = mid; else lo = mid + 1;
                    }
                    const float pc = cdf[lo] - (lo > 0 ? cdf[lo - 1] : 0.f);
                    const uint32_t cs = p.smp.cluster_side, cpr = (p.smp.n_side + cs - 1) / cs;
                    const uint32_t cx = lo % cpr, cz = lo / cpr;
                    const uint32_t w0 = min(cs, p.smp.n_side - cx * cs), h0 = min(cs, p.smp.n_side - cz * cs);
                    const uint32_t inner = min((uint32_t)(u2 * (float)(w0 * h0)), w0 * h0 - 1);
                    l = (cz * cs + inner / w0) * p.smp.n_side + cx * cs + inner % w0;
                    pl = pc / (float)(w0 * h0);
                }
                wgt = pl > 0.f ? 1.f / ((float)nitems * pl) : 0.f;
            }
            float4 g = make_float4(0.f, 0.f, 0.f, 0.f);
            int cnt = 0, src = 0, near = 0, a = 0;
            bool skip = true;
            if (item < nitems && l < p.L) {
                g = p.scan[l];
                // Nearest and farthest voxel-centre distance of the tile.
                const float cx = fminf(fmaxf(g.x, bx0), bx1), cy = fminf(fmaxf(g.y, by0), by1),
                            cz = fminf(fmaxf(g.z, bz0), bz1);
                const float dmin = sqrtf((g.x - cx) * (g.x - cx) + (g.y - cy) * (g.y - cy) + (g.z - cz) * (g.z - cz));
                const float fx = fmaxf(fabsf(g.x - bx0), fabsf(g.x - bx1)), fy = fmaxf(fabsf(g.y - by0), fabsf(g.y - by1)),
                            fz = fmaxf(fabsf(g.z - bz0), fabsf(g.z - bz1));
                const float dmax = sqrtf(fx * fx + fy * fy + fz * fz);
                const float bnc = BOUNCE ? g.w : 0.f;
                const float pmin = 2.f * dmin + neg_t0 + bnc, pmax = 2.f * dmax + neg_t0 + bnc;
                // Paths this short make dist^2 <= EPS possible: use safeRCP's branch.
                near = pmin < 0.0035f;
                // Conservative bin range with a 2-bin margin for rounding.
                const int blo = (int)fmaxf(fminf(floorf(pmin * rcp_dt), 1.0e9f), -1.0e9f) - 2;
                const int bhi = (int)fmaxf(fminf(floorf(pmax * rcp_dt), 1.0e9f), -1.0e9f) + 2;
                a = max(blo, 0) & ~(ALIGN - 1);
                skip = bhi < 0 || blo >= (int)p.T;  // no bin of this tile is inside [0, T)
                if (!skip) {
                    if (CLAMP) a = min(a, (int)(p.row_pitch - p.slot_w));
                    const int hi = min(bhi + 1, (int)p.row_pitch);
                    cnt = (max(hi - a, 0) + ALIGN - 1) & ~(ALIGN - 1);
                    if (cnt > (int)p.slot_w) {
                        if (CLAMP) {
                            // Capped window: bins past it map to the sentinel; only an
                            // uncovered valid bin would be an error.
                            if (min(bhi + 1, (int)p.T) - a > (int)p.slot_w) atomicExch(p.status, (int)FBP_ERR_DEVICE);
                            cnt = (int)p.slot_w;
                        } else {
                            // The planner's span bound failed: read zeros, report.
                            atomicExch(p.status, (int)FBP_ERR_DEVICE);
                            skip = true;
                            cnt = 0;
                        }
                    }
                    src = a;
                }
            }
            // Slot of this scan point (or the zero slot) as a shared address.
            const uint32_t slot_elem = skip ? zero_slot : (uint32_t)(buf * CH + tid) * slot_stride;
            uint32_t saddr = sbase + (uint32_t)slots_off + (slot_elem << SH);
            int bias;
            if (PATH == PATH_EXACT) {
                bias = a;
            } else {
                bias = __float_as_int((float)(8388608 - a));
                if (!CLAMP) saddr -= (0x4B000000u << SH);
            }
            if (item >= nitems || l >= p.L) {
                // Beyond the last scan point: x + 0 < 2^23 lands on the sentinel
                // (CLAMP) or, unclamped, reads the zero slot at index 0.
                bias = PATH == PATH_EXACT ? 0x40000000 : 0;
                saddr = sbase + (uint32_t)slots_off + (zero_slot << SH);
                if (!CLAMP && PATH != PATH_EXACT) saddr -= (__float_as_uint(0.f) << SH);
                g = make_float4(3.0e18f, 3.0e18f, 3.0e18f, 0.f);  // far away: x is huge
                wgt = 0.f;
            }
            s_geo[buf * CHMAX + tid] = g;
            s_meta[buf * CHMAX + tid] = make_int2(bias, (int)saddr);
            s_cnt[buf * CHMAX + tid] = cnt;
            s_src[buf * CHMAX + tid] = src;
            s_row[buf * CHMAX + tid] = (int)l;
            s_w[buf * CHMAX + tid] = wgt;
            const unsigned any_near = __ballot_sync(CH >= 32 ? 0xffffffffu : ((1u << CH) - 1u), near);
            if (tid == 0) s_flag[buf] = any_near != 0;
        }
    };

    // Copy a stage's windows (all threads).
    auto copy_chunk = [&](int buf) {
        const uint32_t vecs_per_slot = p.slot_w / ALIGN;
        for (uint32_t i = tid; i < CH * vecs_per_slot; i += NT) {
            const uint32_t s = i / vecs_per_slot, j = i - s * vecs_per_slot;
            if ((int)(j * ALIGN) < s_cnt[buf * CHMAX + s]) {
                const uint32_t l = (uint32_t)s_row[buf * CHMAX + s];
                const S* src = static_cast<const S*>(p.rows) + (size_t)l * p.row_pitch + s_src[buf * CHMAX + s] + j * ALIGN;
                S* dst = s_slots + (size_t)(buf * CH + s) * slot_stride + j * ALIGN;
                cp_async_16(dst, src);
            }
        }
        cp_async_commit();
    };

    float acc[KV], ksum[KV], kcomp[KV];
#pragma unroll
    for (int k = 0; k < KV; ++k) acc[k] = ksum[k] = kcomp[k] = 0.f;

    if (nchunks > 0) {
        plan_chunk(0, 0);
        __syncthreads();
        copy_chunk(0);
    }

    for (uint32_t c = 0; c < nchunks; ++c) {
        const int buf = c & 1;
        __syncthreads();  // every thread is done with stage c-1, whose buffers plan(c+1) reuses
        if (c + 1 < nchunks) plan_chunk(c + 1, buf ^ 1);
        __syncthreads();  // plan(c+1) visible to the copy loop
        if (c + 1 < nchunks) {
            copy_chunk(buf ^ 1);
            cp_async_wait<1>();
        } else {
            cp_async_wait<0>();
        }
        __syncthreads();  // stage c's windows visible

        const float4* geo = s_geo + buf * CHMAX;
        const int2* meta = s_meta + buf * CHMAX;
        const float* wts = s_w + buf * CHMAX;
        const bool safe = s_flag[buf] != 0;
        const int nl = (int)min((uint32_t)CH, nitems - c * CH);
        float scale = 1.f;
        if (!safe) {
            confocal_stage<S, KV, PATH, BOUNCE, CLAMP, false, SAMPLED>(geo, meta, wts, nl, px, py, pz, neg_t0, rcp_dt,
                                                                        p.slot_w, acc);
            if (PATH == PATH_2D) scale = 0.25f;  // w was rcp(d^2) = 4 rcp(dist^2)
        } else {
            confocal_stage<S, KV, PATH, BOUNCE, CLAMP, true, SAMPLED>(geo, meta, wts, nl, px, py, pz, neg_t0, rcp_dt,
                                                                       p.slot_w, acc);
        }

        // Compensated (Kahan) fold of this stage's partial sums.
#pragma unroll
        for (int k = 0; k < KV; ++k) {
            const float y = sub_rn(mul_rn(acc[k], scale), kcomp[k]);
            const float t = add_rn(ksum[k], y);
            kcomp[k] = sub_rn(sub_rn(t, ksum[k]), y);
            ksum[k] = t;
            acc[k] = 0.f;
        }
    }

    if (row_ok) {
        float* out = p.volume + ((size_t)vz * p.Vy + vy) * p.Vx + tx0;
#pragma unroll
        for (int k = 0; k < KV; ++k)
            if (tx0 + k < p.Vx) out[k] = ksum[k];
    }
}

// ------------------------------------------------------------ host driver --

namespace {

template <typename S>
fbp_status prepare_rows(fbp_context* ctx, const void* cube, int layout, uint32_t L, uint32_t T, uint32_t pitch,
                        cudaStream_t stream, S** rows_out) {
    void* rows = nullptr;
    FBP_TRY(workspace(ctx, WS_CUBE_ROWS, (size_t)L * pitch * sizeof(S), stream, &rows));
    S* r = static_cast<S*>(rows);
    const S* c = static_cast<const S*>(cube);
    if (layout == FBP_LAYOUT_TIME_INNER) {
        const uint64_t n = (uint64_t)L * pitch;
        const unsigned blocks = (unsigned)std::min<uint64_t>(cdiv(n, 256), (uint64_t)ctx->sm_count * 16);
        rows_from_time_inner_kernel<S><<<blocks, 256, 0, stream>>>(r, c, L, T, pitch);
        FBP_CHECK_LAUNCH(ctx, "rows_from_time_inner_kernel");
    } else {
        const uint32_t tcover = std::min<uint32_t>(pitch, (T + 31) / 32 * 32);
        dim3 grid(cdiv(L, 32), cdiv(tcover, 32));
        rows_from_time_major_kernel<S><<<grid, dim3(32, 8), 0, stream>>>(r, c, L, T, pitch);
        FBP_CHECK_LAUNCH(ctx, "rows_from_time_major_kernel");
        if (tcover < pitch) {
            const uint64_t n = (uint64_t)L * (pitch - tcover);
            const unsigned blocks = (unsigned)std::min<uint64_t>(cdiv(n, 256), (uint64_t)ctx->sm_count * 16);
            rows_zero_tail_kernel<S><<<blocks, 256, 0, stream>>>(r, L, tcover, pitch);
            FBP_CHECK_LAUNCH(ctx, "rows_zero_tail_kernel");
        }
    }
    *rows_out = r;
    return FBP_OK;
}

constexpr int kKV = 8, kWY = 2, kWZ = 4;

template <typename S, int PATH, bool BOUNCE, bool SAMPLED, bool CLAMP>
fbp_status go_confocal(fbp_context* ctx, const ConfocalGatherParams& p, dim3 grid, size_t smem, cudaStream_t stream) {
    auto kernel = confocal_gather_kernel<S, kKV, kWY, kWZ, PATH, BOUNCE, SAMPLED, CLAMP>;
    FBP_TRY_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    kernel<<<grid, 32 * kWY * kWZ, smem, stream>>>(p);
    FBP_CHECK_LAUNCH(ctx, "confocal_gather_kernel");
    return FBP_OK;
}

template <typename S, bool SAMPLED>
fbp_status dispatch_confocal(fbp_context* ctx, const ConfocalGatherParams& p, dim3 grid, size_t smem,
                             cudaStream_t stream, bool bounce, float t0, bool capped) {
    if (t0 > 0.f) {
        if (bounce) return go_confocal<S, PATH_EXACT, true, SAMPLED, true>(ctx, p, grid, smem, stream);
        return go_confocal<S, PATH_EXACT, false, SAMPLED, true>(ctx, p, grid, smem, stream);
    }
    if (!bounce && t0 == 0.f) {
        if (capped) return go_confocal<S, PATH_2D, false, SAMPLED, true>(ctx, p, grid, smem, stream);
        return go_confocal<S, PATH_2D, false, SAMPLED, false>(ctx, p, grid, smem, stream);
    }
    if (bounce) {
        if (capped) return go_confocal<S, PATH_FAST, true, SAMPLED, true>(ctx, p, grid, smem, stream);
        return go_confocal<S, PATH_FAST, true, SAMPLED, false>(ctx, p, grid, smem, stream);
    }
    if (capped) return go_confocal<S, PATH_FAST, false, SAMPLED, true>(ctx, p, grid, smem, stream);
    return go_confocal<S, PATH_FAST, false, SAMPLED, false>(ctx, p, grid, smem, stream);
}

template <typename S>
fbp_status launch_confocal(fbp_context* ctx, const fbp_recon_info& in, const void* cube, int layout,
                           const float* laser_xyz, float* volume, cudaStream_t stream, const SampleParams* smp) {
    const uint32_t L = in.num_laser_targets, T = in.num_time_bins;
    const uint32_t Vx = in.voxel_res[0], Vy = in.voxel_res[1], Vz = in.voxel_res[2];
    constexpr int ALIGN = 16 / sizeof(S);

    // World extents of the largest tile (clamped to the volume).
    const double ex = (double)std::min<uint32_t>(kKV, Vx) * std::fabs(in.voxel_size[0]);
    const double ey = (double)std::min<uint32_t>(4 * kWZ, Vz) * std::fabs(in.voxel_size[1]);
    const double ez = (double)std::min<uint32_t>(8 * kWY, Vy) * std::fabs(in.voxel_size[2]);
    WindowPlan wp;
    FBP_TRY(plan_window(ctx, ex, ey, ez, in.time_step, T, ALIGN, sizeof(S), ConfocalGatherParams::meta_bytes(32), &wp,
                        "fbp_backproject_confocal"));

    S* rows = nullptr;
    FBP_TRY(prepare_rows<S>(ctx, cube, layout, L, T, wp.pitch, stream, &rows));

    ConfocalGatherParams p{};
    FBP_TRY(build_tables(ctx, in, laser_xyz, stream, &p.scan, &p.xs, &p.ys, &p.zs));
    p.rows = rows;
    p.volume = volume;
    p.status = ctx->status_dev;
    p.Vx = Vx; p.Vy = Vy; p.Vz = Vz; p.L = L; p.T = T;
    p.t0 = in.time_offset;
    p.dt = in.time_step;
    p.row_pitch = wp.pitch;
    p.slot_w = wp.slot_w;
    p.ch = wp.ch;
    if (smp) p.smp = *smp;
    dim3 grid(cdiv(Vx, kKV), cdiv(Vy, 8 * kWY), cdiv(Vz, 4 * kWZ));
    const bool bounce = in.discard_first_last_bounces == 0;
    if (smp) return dispatch_confocal<S, true>(ctx, p, grid, wp.smem, stream, bounce, in.time_offset, wp.capped);
    return dispatch_confocal<S, false>(ctx, p, grid, wp.smem, stream, bounce, in.time_offset, wp.capped);
}

}  // namespace

// Tile grid of the confocal gather (also the MIS sampling tiles).
void confocal_tile_grid(const fbp_recon_info& in, uint32_t out[3]) {
    out[0] = cdiv(in.voxel_res[0], kKV);
    out[1] = cdiv(in.voxel_res[1], 8 * kWY);
    out[2] = cdiv(in.voxel_res[2], 4 * kWZ);
}

fbp_status confocal_gather(fbp_context* ctx, const fbp_recon_info& in, const void* cube, int dtype, int layout,
                           const float* laser_xyz, float* volume, cudaStream_t s, const SampleParams* smp) {
    switch (dtype) {
        case FBP_F32: return launch_confocal<float>(ctx, in, cube, layout, laser_xyz, volume, s, smp);
        case FBP_BF16: return launch_confocal<__nv_bfloat16>(ctx, in, cube, layout, laser_xyz, volume, s, smp);
        case FBP_F16: return launch_confocal<__half>(ctx, in, cube, layout, laser_xyz, volume, s, smp);
        default: return set_error(FBP_ERR_INVALID_ARG, "unknown dtype");
    }
}

fbp_status build_tables(fbp_context* ctx, const fbp_recon_info& in, const float* laser_xyz, cudaStream_t stream,
                        const float4** scan, const float** xs, const float** ys, const float** zs) {
    const uint32_t L = in.num_laser_targets;
    const uint32_t Vx = in.voxel_res[0], Vy = in.voxel_res[1], Vz = in.voxel_res[2];
    void* sp = nullptr;
    void* ap = nullptr;
    FBP_TRY(workspace(ctx, WS_SCAN_TABLE, (size_t)L * sizeof(float4), stream, &sp));
    FBP_TRY(workspace(ctx, WS_AXIS_TABLES, (size_t)(Vx + Vy + Vz) * sizeof(float), stream, &ap));
    float4* s = static_cast<float4*>(sp);
    float* a = static_cast<float*>(ap);
    scan_table_kernel<<<cdiv(L, 256), 256, 0, stream>>>(
        s, laser_xyz, L, (int)in.discard_first_last_bounces, in.laser_position[0], in.laser_position[1],
        in.laser_position[2], in.sensor_position[0], in.sensor_position[1], in.sensor_position[2], 1);
    FBP_CHECK_LAUNCH(ctx, "scan_table_kernel");
    const uint32_t vmax = std::max(Vx, std::max(Vy, Vz));
    axis_tables_kernel<<<cdiv(vmax, 256), 256, 0, stream>>>(a, a + Vx, a + Vx + Vz, Vx, Vy, Vz, in.hidden_min[0],
                                                            in.hidden_min[1], in.hidden_min[2], in.voxel_size[0],
                                                            in.voxel_size[1], in.voxel_size[2]);
    FBP_CHECK_LAUNCH(ctx, "axis_tables_kernel");
    *scan = s;
    *xs = a;
    *ys = a + Vx;
    *zs = a + Vx + Vz;
    return FBP_OK;
}

fbp_status plan_window(const fbp_context* ctx, double ex, double ey, double ez, double time_step, uint32_t T, int align,
                       size_t elem_bytes, size_t meta_bytes, WindowPlan* out, const char* who) {
    const double diag = std::sqrt(ex * ex + ey * ey + ez * ez);
    // Round trip across the tile, a 2-bin margin on each side, alignment slack.
    const double span = 2.0 * diag / std::fabs(time_step) + 8.0 + align;
    const uint32_t t_round = (T + align - 1) / align * align;
    const uint32_t cap = t_round + align;
    uint32_t slot_w = span < (double)cap ? ((uint32_t)std::ceil(span) + align - 1) / align * align : cap;
    if (slot_w > cap) slot_w = cap;
    out->slot_w = slot_w;
    out->capped = slot_w == cap;
    out->pitch = t_round + slot_w;
    const size_t per_stage = (size_t)2 * (slot_w + align) * elem_bytes;  // double-buffered, per scan point
    const size_t zero_slot = (size_t)(slot_w + align) * elem_bytes;
    int ch = 32;
    while (ch > 1 && meta_bytes + (size_t)ch * per_stage + zero_slot > (size_t)ctx->smem_optin) ch >>= 1;
    if (meta_bytes + (size_t)ch * per_stage + zero_slot > (size_t)ctx->smem_optin)
        return set_error(FBP_ERR_UNSUPPORTED, std::string(who) + ": time-bin window too large for shared memory");
    out->ch = ch;
    out->smem = meta_bytes + (size_t)ch * per_stage + zero_slot;
    return FBP_OK;
}

fbp_status validate_info(const fbp_recon_info* info, bool need_sensors, const char* who) {
    if (!info) return set_error(FBP_ERR_INVALID_ARG, std::string(who) + ": null info");
    const fbp_recon_info& in = *info;
    if (in.num_laser_targets == 0 || in.num_time_bins == 0 || (need_sensors && in.num_sensor_targets == 0))
        return set_error(FBP_ERR_INVALID_ARG, std::string(who) + ": empty capture (zero scan points or bins)");
    if (in.voxel_res[0] == 0 || in.voxel_res[1] == 0 || in.voxel_res[2] == 0)
        return set_error(FBP_ERR_INVALID_ARG, std::string(who) + ": zero voxel resolution");
    if (!(std::isfinite(in.time_step) && in.time_step > 0.f))
        return set_error(FBP_ERR_INVALID_ARG, std::string(who) + ": time_step must be finite and > 0");
    if (in.num_time_bins >= (1u << 22))
        return set_error(FBP_ERR_UNSUPPORTED, std::string(who) + ": more than 2^22 time bins");
    const uint64_t V = (uint64_t)in.voxel_res[0] * in.voxel_res[1] * in.voxel_res[2];
    if (V >= (1ull << 32)) return set_error(FBP_ERR_UNSUPPORTED, std::string(who) + ": more than 2^32 voxels");
    for (int k = 0; k < 3; ++k)
        if (!std::isfinite(in.hidden_min[k]) || !std::isfinite(in.voxel_size[k]))
            return set_error(FBP_ERR_INVALID_ARG, std::string(who) + ": non-finite volume geometry");
    if (!std::isfinite(in.time_offset)) return set_error(FBP_ERR_INVALID_ARG, std::string(who) + ": non-finite time_offset");
    return FBP_OK;
}

}  // namespace fbp

using namespace fbp;

extern "C" fbp_status fbp_backproject_confocal(fbp_context* ctx, const fbp_recon_info* info, const void* cube,
                                               int dtype, int layout, const float* laser_xyz, float* volume,
                                               void* stream) {
    clear_error();
    FBP_TRY(check_ctx(ctx));
    FBP_TRY(validate_info(info, false, "fbp_backproject_confocal"));
    if (!cube || !laser_xyz || !volume) return set_error(FBP_ERR_INVALID_ARG, "fbp_backproject_confocal: null buffer");
    if (layout != FBP_LAYOUT_TIME_MAJOR && layout != FBP_LAYOUT_TIME_INNER)
        return set_error(FBP_ERR_INVALID_ARG, "fbp_backproject_confocal: unknown layout");
    if (dtype != FBP_F32 && dtype != FBP_BF16 && dtype != FBP_F16)
        return set_error(FBP_ERR_INVALID_ARG, "fbp_backproject_confocal: unknown dtype");
    return confocal_gather(ctx, *info, cube, dtype, layout, laser_xyz, volume, (cudaStream_t)stream, nullptr);
}

// ------------------------------------------------------------ diagnostics --

namespace fbp {

__device__ __forceinline__ void voxel_of(int64_t v, uint32_t Vx, uint32_t Vy, uint32_t& vx, uint32_t& vy, uint32_t& vz) {
    const uint64_t slice = (uint64_t)Vx * Vy;
    vz = (uint32_t)(v / slice);
    const uint32_t r = (uint32_t)(v % slice);
    vy = r / Vx;
    vx = r % Vx;
}

__global__ void debug_confocal_bins_kernel(fbp_recon_info in, const float4* __restrict__ scan,
                                           const int64_t* __restrict__ vidx, uint64_t nv, int32_t* __restrict__ bins) {
    const uint64_t L = in.num_laser_targets;
    const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i >= nv * L) return;
    const uint64_t vi = i / L, l = i % L;
    uint32_t vx, vy, vz;
    voxel_of(vidx[vi], in.voxel_res[0], in.voxel_res[1], vx, vy, vz);
    const float px = ref_voxel_coord(vx, in.voxel_size[0], in.hidden_min[0]);
    const float py = ref_voxel_coord(vz, in.voxel_size[1], in.hidden_min[1]);
    const float pz = ref_voxel_coord(vy, in.voxel_size[2], in.hidden_min[2]);
    const float4 g = scan[l];
    float dist = fma_rn(sqrt_approx(ref_dot3(sub_rn(px, g.x), sub_rn(py, g.y), sub_rn(pz, g.z))), 2.f, -in.time_offset);
    if (in.discard_first_last_bounces == 0) dist = add_rn(dist, g.w);
    const int b = __float2int_rz(ref_bin_ratio(dist, rcp_approx(in.time_step)));
    bins[i] = (b >= 0 && b < (int)in.num_time_bins) ? b : -1;
}

__global__ void debug_exhaustive_bins_kernel(fbp_recon_info in, const float4* __restrict__ lscan,
                                             const float4* __restrict__ sscan, const int64_t* __restrict__ vidx,
                                             uint64_t nv, int32_t* __restrict__ bins) {
    const uint64_t L = in.num_laser_targets, S = in.num_sensor_targets;
    const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i >= nv * L * S) return;
    const uint64_t vi = i / (L * S), l = (i / S) % L, s = i % S;
    uint32_t vx, vy, vz;
    voxel_of(vidx[vi], in.voxel_res[0], in.voxel_res[1], vx, vy, vz);
    const float px = ref_voxel_coord(vx, in.voxel_size[0], in.hidden_min[0]);
    const float py = ref_voxel_coord(vz, in.voxel_size[1], in.hidden_min[1]);
    const float pz = ref_voxel_coord(vy, in.voxel_size[2], in.hidden_min[2]);
    const float4 lg = lscan[l], sg = sscan[s];
    const float dl = sqrt_approx(ref_dot3(sub_rn(px, lg.x), sub_rn(py, lg.y), sub_rn(pz, lg.z)));
    const float ds = sqrt_approx(ref_dot3(sub_rn(px, sg.x), sub_rn(py, sg.y), sub_rn(pz, sg.z)));
    float dist = sub_rn(add_rn(dl, ds), in.time_offset);
    if (in.discard_first_last_bounces == 0) dist = add_rn(dist, add_rn(lg.w, sg.w));
    const int b = __float2int_rz(ref_bin_ratio(dist, rcp_approx(in.time_step)));
    bins[i] = (b >= 0 && b < (int)in.num_time_bins) ? b : -1;
}

}  // namespace fbp

extern "C" fbp_status fbp_debug_confocal_bins(fbp_context* ctx, const fbp_recon_info* info, const float* laser_xyz,
                                              const int64_t* voxel_idx, uint64_t num_voxels, int32_t* bins,
                                              void* stream) {
    clear_error();
    FBP_TRY(check_ctx(ctx));
    FBP_TRY(validate_info(info, false, "fbp_debug_confocal_bins"));
    if (!laser_xyz || !voxel_idx || !bins) return set_error(FBP_ERR_INVALID_ARG, "fbp_debug_confocal_bins: null buffer");
    cudaStream_t s = (cudaStream_t)stream;
    const float4* scan;
    const float *xs, *ys, *zs;
    FBP_TRY(build_tables(ctx, *info, laser_xyz, s, &scan, &xs, &ys, &zs));
    const uint64_t n = num_voxels * info->num_laser_targets;
    if (n == 0) return FBP_OK;
    debug_confocal_bins_kernel<<<cdiv(n, 256), 256, 0, s>>>(*info, scan, voxel_idx, num_voxels, bins);
    FBP_CHECK_LAUNCH(ctx, "debug_confocal_bins_kernel");
    return FBP_OK;
}

extern "C" fbp_status fbp_debug_exhaustive_bins(fbp_context* ctx, const fbp_recon_info* info, const float* laser_xyz,
                                                const float* sensor_xyz, const int64_t* voxel_idx, uint64_t num_voxels,
                                                int32_t* bins, void* stream) {
    clear_error();
    FBP_TRY(check_ctx(ctx));
    FBP_TRY(validate_info(info, true, "fbp_debug_exhaustive_bins"));
    if (!laser_xyz || !sensor_xyz || !voxel_idx || !bins)
        return set_error(FBP_ERR_INVALID_ARG, "fbp_debug_exhaustive_bins: null buffer");
    cudaStream_t s = (cudaStream_t)stream;
    const uint32_t L = info->num_laser_targets, Sn = info->num_sensor_targets;
    void* lp = nullptr;
    void* sp = nullptr;
    FBP_TRY(workspace(ctx, WS_SCAN_TABLE, (size_t)L * sizeof(float4), s, &lp));
    FBP_TRY(workspace(ctx, WS_SENSOR_TABLE, (size_t)Sn * sizeof(float4), s, &sp));
    scan_table_kernel<<<cdiv(L, 256), 256, 0, s>>>(static_cast<float4*>(lp), laser_xyz, L,
                                                  (int)info->discard_first_last_bounces, info->laser_position[0],
                                                  info->laser_position[1], info->laser_position[2], 0.f, 0.f, 0.f, 0);
    FBP_CHECK_LAUNCH(ctx, "scan_table_kernel");
    scan_table_kernel<<<cdiv(Sn, 256), 256, 0, s>>>(static_cast<float4*>(sp), sensor_xyz, Sn,
                                                   (int)info->discard_first_last_bounces, info->sensor_position[0],
                                                   info->sensor_position[1], info->sensor_position[2], 0.f, 0.f, 0.f, 0);
    FBP_CHECK_LAUNCH(ctx, "scan_table_kernel");
    const uint64_t n = num_voxels * L * Sn;
    if (n == 0) return FBP_OK;
    debug_exhaustive_bins_kernel<<<cdiv(n, 256), 256, 0, s>>>(*info, static_cast<const float4*>(lp),
                                                             static_cast<const float4*>(sp), voxel_idx, num_voxels,
                                                             bins);
    FBP_CHECK_LAUNCH(ctx, "debug_exhaustive_bins_kernel");
    return FBP_OK;
}
