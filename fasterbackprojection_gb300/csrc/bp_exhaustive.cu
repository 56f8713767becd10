// Exhaustive (laser x SPAD) backprojection as a voxel-tiled gather.
//
// Replaces Laser::reconstructAABBExhaustive (Laser.cu:500-516) and
// backprojectExhaustiveVoxel (transient_reconstruction.cuh:138-166).  Same
// structure as the confocal gather: one CTA per voxel tile, the (laser, SPAD)
// pairs walked in staged chunks, each pair's reachable time-bin window copied
// to shared memory.  The pair index splits as l = ls / S, s = ls % S; the
// reference splits by L (transient_reconstruction.cuh:147-148), which is the
// same only when L == S and reads past the laser table otherwise.
// Within a chunk, consecutive pairs usually share the laser point, so the
// laser-to-voxel distance is computed once per laser point and reused.
#include "fbp_internal.cuh"
#include "bp_common.cuh"

#include <algorithm>
#include <cmath>

namespace fbp {

struct ExhaustiveGatherParams {
    const float4* lscan;  // [L] (x, y, z, |l - laserPos| or 0)
    const float4* sscan;  // [S] (x, y, z, |s - sensorPos| or 0)
    const float* xs;
    const float* ys;
    const float* zs;
    float* volume;
    int* status;
    const float* rows;  // [L*S][row_pitch] FP32 (16-bit cubes are widened, exactly, when the rows are made)
    uint32_t Vx, Vy, Vz, L, S, T;
    float t0, dt;
    uint32_t row_pitch, slot_w;
    int ch;
    int exact_weights;  // 1: every weight by its own rcp.approx (FBP_WEIGHTS_REFERENCE)

    // Per pair of a stage: laser (x, y, z, bounce), SPAD (x, y, z, bounce),
    // the packed (bias, bias, bounces, bounces) the triple loop reads as two
    // register pairs, then the slot address and four planning ints.
    __host__ __device__ static constexpr size_t meta_bytes(int ch) {
        return ((size_t)2 * ch * (3 * sizeof(float4) + 5 * sizeof(int)) + 4 * sizeof(int) + 15) & ~size_t(15);
    }
};

// Arithmetic of the triple loop (all reproduce the reference's bins):
//   EX_T0ZERO  time_offset == 0: dist = dl + ds [+ bounces]; the reference's
//              "- t0" subtracts zero, which changes no bit, so it is skipped.
//   EX_FAST    time_offset < 0: dist = (dl + ds) - t0 [+ bounces].
//   EX_EXACT   time_offset > 0: negative paths possible, bin by conversion,
//              scalar loop.
// In the first two the bin is floor(x) - a via a round-toward-zero add of
// 2^23 - a; without CLAMP the window planner guarantees every bin of the tile
// lies inside its window, so the -2^23 bias folds into the slot address.
enum { EX_T0ZERO = 0, EX_FAST = 1, EX_EXACT = 2 };

// LB = 4: pairs are walked as (laser block of 4, SPAD, laser in block), so
// the SPAD-to-voxel distance is computed once per SPAD for 4 lasers (the 4
// laser distances are kept per block); requires L % 4 == 0 and ch % 4 == 0.
// LB = 1: pairs in (laser, SPAD) order.
template <int KV, int WY, int WZ, int MODE, bool BOUNCE, bool CLAMP, int LB>
__global__ void __launch_bounds__(32 * WY * WZ)
exhaustive_gather_kernel(ExhaustiveGatherParams p) {
    static_assert(KV % 4 == 0, "voxels per thread in two packed pairs per weight group");
    constexpr int NT = 32 * WY * WZ;
    constexpr int CHMAX = 64;  // scan points (pairs) per stage, upper bound (planned by warps 0 and 1)
    const int CH = p.ch;
    constexpr int ALIGN = 4;   // FP32 elements per 16-byte copy
    constexpr int TY = 8 * WY, TZ = 4 * WZ;

    extern __shared__ __align__(16) unsigned char smem_raw[];
    const uint32_t slot_stride = p.slot_w + ALIGN;
    float4* s_lg = reinterpret_cast<float4*>(smem_raw);           // [2][CHMAX]
    float4* s_sg = s_lg + 2 * CHMAX;                              // [2][CHMAX]
    ulonglong2* s_pk = reinterpret_cast<ulonglong2*>(s_sg + 2 * CHMAX);  // [2][CHMAX] (bias, bias), (bnc, bnc)
    int* s_addr = reinterpret_cast<int*>(s_pk + 2 * CHMAX);       // [2][CHMAX] slot shared address
    int* s_cnt = s_addr + 2 * CHMAX;
    int* s_src = s_cnt + 2 * CHMAX;
    int* s_lid = s_src + 2 * CHMAX;
    int* s_row = s_lid + 2 * CHMAX;
    int* s_flag = s_row + 2 * CHMAX;  // [2][2]: per buffer, per planning warp
    const size_t slots_off = ExhaustiveGatherParams::meta_bytes(CHMAX);
    float* s_slots = reinterpret_cast<float*>(smem_raw + slots_off);  // [2][CH][slot_stride], then the zero slot
    const uint32_t sbase = (uint32_t)__cvta_generic_to_shared(smem_raw);
    const uint32_t zero_slot = 2u * CH * slot_stride;

    const int tid = threadIdx.x;
    const int lane = tid & 31, warp = tid >> 5;
    const int wy = warp % WY, wz = warp / WY;
    const uint32_t tx0 = blockIdx.x * KV, ty0 = blockIdx.y * TY, tz0 = blockIdx.z * TZ;
    const uint32_t vy = ty0 + wy * 8 + (lane & 7);
    const uint32_t vz = tz0 + wz * 4 + (lane >> 3);
    const bool row_ok = vy < p.Vy && vz < p.Vz;

    const uint32_t tx1 = min(tx0 + KV, p.Vx) - 1, ty1 = min(ty0 + TY, p.Vy) - 1, tz1 = min(tz0 + TZ, p.Vz) - 1;
    const float bx0 = fminf(p.xs[tx0], p.xs[tx1]), bx1 = fmaxf(p.xs[tx0], p.xs[tx1]);
    const float by0 = fminf(p.ys[tz0], p.ys[tz1]), by1 = fmaxf(p.ys[tz0], p.ys[tz1]);
    const float bz0 = fminf(p.zs[ty0], p.zs[ty1]), bz1 = fmaxf(p.zs[ty0], p.zs[ty1]);

    const float py = p.ys[min(vz, p.Vz - 1)];
    const float pz = p.zs[min(vy, p.Vy - 1)];
    f32x2_t pxp[KV / 2];
#pragma unroll
    for (int j = 0; j < KV / 2; ++j)
        pxp[j] = pack2(p.xs[min(tx0 + 2 * j, p.Vx - 1)], p.xs[min(tx0 + 2 * j + 1, p.Vx - 1)]);

    const float rcp_dt = rcp_approx(p.dt);
    const uint64_t npairs = (uint64_t)p.L * p.S;
    const uint64_t nchunks = (npairs + CH - 1) / CH;

    // Sentinels of every slot and the whole zero slot.
    for (int i = tid; i < 2 * CH * ALIGN; i += NT) {
        const int slot = i / ALIGN, e = i % ALIGN;
        s_slots[(size_t)slot * slot_stride + p.slot_w + e] = 0.f;
    }
    for (uint32_t i = tid; i < slot_stride; i += NT) s_slots[zero_slot + i] = 0.f;

    auto box_range = [&](const float4& g, float& dmin, float& dmax) {
        const float cx = fminf(fmaxf(g.x, bx0), bx1), cy = fminf(fmaxf(g.y, by0), by1), cz = fminf(fmaxf(g.z, bz0), bz1);
        dmin = sqrtf((g.x - cx) * (g.x - cx) + (g.y - cy) * (g.y - cy) + (g.z - cz) * (g.z - cz));
        const float fx = fmaxf(fabsf(g.x - bx0), fabsf(g.x - bx1)), fy = fmaxf(fabsf(g.y - by0), fabsf(g.y - by1)),
                    fz = fmaxf(fabsf(g.z - bz0), fabsf(g.z - bz1));
        dmax = sqrtf(fx * fx + fy * fy + fz * fz);
    };

    // Plan a stage: bin window of each (laser, SPAD) pair (threads < CH, warps 0 and 1).
    auto plan_chunk = [&](uint64_t c, int buf) {
        if (tid < CH) {
            const uint64_t ls = c * CH + tid;
            float4 lg = make_float4(0.f, 0.f, 0.f, 0.f), sg = lg;
            float bnc = 0.f;
            int cnt = 0, src = 0, near = 0, lid = -1, row = 0, a = 0;
            bool skip = true;
            if (ls < npairs) {
                uint32_t l, s;
                if (LB == 1) {
                    l = (uint32_t)(ls / p.S);
                    s = (uint32_t)(ls % p.S);
                } else {
                    const uint64_t grp = ls / LB;
                    l = (uint32_t)(grp / p.S) * LB + (uint32_t)(ls % LB);
                    s = (uint32_t)(grp % p.S);
                }
                row = (int)(l * p.S + s);
                lg = p.lscan[l];
                sg = p.sscan[s];
                lid = (int)l;
                float dl0, dl1, ds0, ds1;
                box_range(lg, dl0, dl1);
                box_range(sg, ds0, ds1);
                bnc = BOUNCE ? add_rn(lg.w, sg.w) : 0.f;  // transient_reconstruction.cuh:161
                const float pmin = dl0 + ds0 - p.t0 + bnc, pmax = dl1 + ds1 - p.t0 + bnc;
                // Paths this short make dist^2 <= EPS possible, paths this long
                // (or NaN) could take the shared reciprocal's product out of the
                // FP32 range: those stages weigh each pair on its own.
                near = pmin < 0.0035f || !(pmax < 1.0e4f);
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
            const uint32_t slot_elem = skip ? zero_slot : (uint32_t)(buf * CH + tid) * slot_stride;
            uint32_t saddr = sbase + (uint32_t)slots_off + (slot_elem << 2);
            int bias;
            if (MODE == EX_EXACT) {
                bias = a;
            } else {
                bias = __float_as_int((float)(8388608 - a));
                if (!CLAMP) saddr -= (0x4B000000u << 2);
            }
            const float bf = __int_as_float(bias);
            s_lg[buf * CHMAX + tid] = lg;
            s_sg[buf * CHMAX + tid] = sg;
            s_pk[buf * CHMAX + tid] = make_ulonglong2(pack2(bf, bf), pack2(bnc, bnc));
            s_addr[buf * CHMAX + tid] = (int)saddr;
            s_cnt[buf * CHMAX + tid] = cnt;
            s_src[buf * CHMAX + tid] = src;
            s_lid[buf * CHMAX + tid] = lid;
            s_row[buf * CHMAX + tid] = row;
            const int w = tid >> 5, nw = min(32, CH - 32 * w);
            const unsigned any_near = __ballot_sync(nw >= 32 ? 0xffffffffu : ((1u << nw) - 1u), near);
            if ((tid & 31) == 0) s_flag[2 * buf + w] = any_near != 0;
        }
    };

    auto copy_chunk = [&](int buf) {
        const uint32_t vecs = p.slot_w / ALIGN;
        for (uint32_t i = tid; i < CH * vecs; i += NT) {
            const uint32_t s = i / vecs, j = i - s * vecs;
            if ((int)(j * ALIGN) < s_cnt[buf * CHMAX + s]) {
                const uint64_t row = (uint32_t)s_row[buf * CHMAX + s];
                const float* src = p.rows + row * p.row_pitch + s_src[buf * CHMAX + s] + j * ALIGN;
                cp_async_16(s_slots + (size_t)(buf * CH + s) * slot_stride + j * ALIGN, src);
            }
        }
        cp_async_commit();
    };

    f32x2_t accp[KV / 2], dlp[LB][KV / 2];
    float ksum[KV], kcomp[KV];
#pragma unroll
    for (int j = 0; j < KV / 2; ++j) accp[j] = 0ull;
#pragma unroll
    for (int k = 0; k < KV; ++k) ksum[k] = kcomp[k] = 0.f;
#pragma unroll
    for (int li = 0; li < LB; ++li)
#pragma unroll
        for (int j = 0; j < KV / 2; ++j) dlp[li][j] = 0ull;
    int cur_l = -1;
    int buf_cur = 0;  // buffer of the stage being accumulated
    const f32x2_t rdp = pack2(rcp_dt, rcp_dt), t0p = pack2(p.t0, p.t0);

    // Triples of pair i of the stage in buffer buf_cur with the laser
    // distances dlp[li] and the SPAD distances dsp
    // (transient_reconstruction.cuh:155-162).
    auto pair_terms = [&](int i, int li, const f32x2_t (&dsp)[KV / 2], bool safe) {
        const ulonglong2 pk = s_pk[buf_cur * CHMAX + i];
        const uint32_t saddr = (uint32_t)s_addr[buf_cur * CHMAX + i];
        const f32x2_t biasp = pk.x, bncp = pk.y;
        if (MODE != EX_EXACT && !safe) {
            // Packed voxel pairs; weights of two pairs from one reciprocal per
            // lane (simultaneous inversion: 1/s0 = s1 / (s0 s1)).
#pragma unroll
            for (int j0 = 0; j0 < KV / 2; j0 += 2) {
                f32x2_t sq[2], Iq[2];
#pragma unroll
                for (int jj = 0; jj < 2; ++jj) {
                    const int j = j0 + jj;
                    f32x2_t dist = add_rn2(dlp[li][j], dsp[j]);
                    if (MODE == EX_FAST) dist = sub_rn2(dist, t0p);
                    if (BOUNCE) dist = add_rn2(dist, bncp);
                    float b0, b1;
                    unpack2(add_rz2(mul_rn2(dist, rdp), biasp), b0, b1);
                    uint32_t a0, a1;
                    if (CLAMP) {
                        a0 = saddr + (min(__float_as_uint(b0) - 0x4B000000u, p.slot_w) << 2);
                        a1 = saddr + (min(__float_as_uint(b1) - 0x4B000000u, p.slot_w) << 2);
                    } else {
                        a0 = saddr + (__float_as_uint(b0) << 2);  // bias folded into the address
                        a1 = saddr + (__float_as_uint(b1) << 2);
                    }
                    Iq[jj] = pack2(lds_f32(a0), lds_f32(a1));
                    sq[jj] = mul_rn2(dist, dist);
                }
                float m0, m1;
                unpack2(mul_rn2(sq[0], sq[1]), m0, m1);
                const f32x2_t r = pack2(rcp_approx(m0), rcp_approx(m1));
                accp[j0] = fmaf2(Iq[0], mul_rn2(r, sq[1]), accp[j0]);
                accp[j0 + 1] = fmaf2(Iq[1], mul_rn2(r, sq[0]), accp[j0 + 1]);
            }
            return;
        }
        // Scalar loop: the reference's own weight per triple (safeRCP near the
        // wall), and the conversion bin where negative paths are possible.
        float bias, bnc, unused;
        unpack2(biasp, bias, unused);
        unpack2(bncp, bnc, unused);
#pragma unroll
        for (int j = 0; j < KV / 2; ++j) {
            float dl2[2], ds2[2], ac[2];
            unpack2(dlp[li][j], dl2[0], dl2[1]);
            unpack2(dsp[j], ds2[0], ds2[1]);
            unpack2(accp[j], ac[0], ac[1]);
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                float dist = sub_rn(add_rn(dl2[h], ds2[h]), p.t0);
                if (BOUNCE) dist = add_rn(dist, bnc);
                const float x = ref_bin_ratio(dist, rcp_dt);
                uint32_t idx;
                if (MODE == EX_EXACT) {
                    idx = min((uint32_t)(__float2int_rz(x) - __float_as_int(bias)), p.slot_w);
                } else if (CLAMP) {
                    idx = min(__float_as_uint(add_rz(x, bias)) - 0x4B000000u, p.slot_w);
                } else {
                    idx = __float_as_uint(add_rz(x, bias));  // bias folded into the address
                }
                const float I = lds_f32(saddr + (idx << 2));
                const float dd = mul_rn(dist, dist);
                const float w = safe ? ref_safe_rcp(dd) : rcp_approx(dd);
                ac[h] = fmaf(I, w, ac[h]);
            }
            accp[j] = pack2(ac[0], ac[1]);
        }
    };
    auto point_dist = [&](const float4& g, f32x2_t (&d)[KV / 2]) {
        const float ddy = sub_rn(py, g.y), ddz = sub_rn(pz, g.z);
        const float ddy2 = mul_rn(ddy, ddy);
        const f32x2_t gxp = pack2(g.x, g.x), ddzp = pack2(ddz, ddz), ddy2p = pack2(ddy2, ddy2);
#pragma unroll
        for (int j = 0; j < KV / 2; ++j) {
            const f32x2_t dx = sub_rn2(pxp[j], gxp);
            float q0, q1;
            unpack2(fma_rn2(ddzp, ddzp, fma_rn2(dx, dx, ddy2p)), q0, q1);
            d[j] = pack2(sqrt_approx(q0), sqrt_approx(q1));
        }
    };

    if (nchunks > 0) {
        plan_chunk(0, 0);
        __syncthreads();
        copy_chunk(0);
    }
    for (uint64_t c = 0; c < nchunks; ++c) {
        const int buf = (int)(c & 1);
        buf_cur = buf;
        __syncthreads();  // every thread is done with chunk c-1, whose buffer plan(c+1) reuses
        if (c + 1 < nchunks) plan_chunk(c + 1, buf ^ 1);
        __syncthreads();  // plan(c+1) visible to the copy loop
        if (c + 1 < nchunks) {
            copy_chunk(buf ^ 1);
            cp_async_wait<1>();
        } else {
            cp_async_wait<0>();
        }
        __syncthreads();

        const bool safe = s_flag[2 * buf] != 0 || (CH > 32 && s_flag[2 * buf + 1] != 0) || p.exact_weights;
        const int np = (int)min((uint64_t)CH, npairs - c * CH);
        if (LB == 1) {
            for (int i = 0; i < np; ++i) {
                const int lid = s_lid[buf * CHMAX + i];
                if (lid != cur_l) {  // uniform across the CTA
                    cur_l = lid;
                    point_dist(s_lg[buf * CHMAX + i], dlp[0]);
                }
                f32x2_t dsp[KV / 2];
                point_dist(s_sg[buf * CHMAX + i], dsp);
                pair_terms(i, 0, dsp, safe);
            }
        } else {
            for (int g = 0; g < np; g += LB) {
                const int lb = s_lid[buf * CHMAX + g] / LB;
                if (lb != cur_l) {  // a new block of LB lasers (uniform across the CTA)
                    cur_l = lb;
#pragma unroll
                    for (int li = 0; li < LB; ++li) point_dist(s_lg[buf * CHMAX + g + li], dlp[li]);
                }
                f32x2_t dsp[KV / 2];
                point_dist(s_sg[buf * CHMAX + g], dsp);  // the group's SPAD
#pragma unroll
                for (int li = 0; li < LB; ++li) pair_terms(g + li, li, dsp, safe);
            }
        }
        // Compensated (Kahan) fold of this stage's partial sums.
#pragma unroll
        for (int j = 0; j < KV / 2; ++j) {
            float a2[2];
            unpack2(accp[j], a2[0], a2[1]);
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int k = 2 * j + h;
                const float y = sub_rn(a2[h], kcomp[k]);
                const float t = add_rn(ksum[k], y);
                kcomp[k] = sub_rn(sub_rn(t, ksum[k]), y);
                ksum[k] = t;
            }
            accp[j] = 0ull;
        }
    }

    if (row_ok) {
        float* out = p.volume + ((size_t)vz * p.Vy + vy) * p.Vx + tx0;
#pragma unroll
        for (int k = 0; k < KV; ++k)
            if (tx0 + k < p.Vx) out[k] = ksum[k];
    }
}
namespace {

constexpr int kKV = 8, kWY = 2, kWZ = 4;

// Padded, thresholded FP32 rows [L*S][pitch] of the cube (16-bit storage
// widened exactly, so the triple loop reads FP32 with no conversion).
template <typename S>
__global__ void pair_rows_kernel(float* __restrict__ rows, const S* __restrict__ cube, uint64_t npairs, uint32_t T,
                                 uint32_t pitch) {
    const uint64_t n = npairs * pitch;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t r = i / pitch;
        const uint32_t t = (uint32_t)(i % pitch);
        float v = 0.f;
        if (t < T) {
            const float c = to_f32(cube[r * T + t]);
            if (c > FBP_EPS) v = c;
        }
        rows[i] = v;
    }
}

template <int MODE, bool BOUNCE, bool CLAMP, int LB>
fbp_status go_exhaustive(fbp_context* ctx, const ExhaustiveGatherParams& p, dim3 grid, size_t smem,
                         cudaStream_t stream) {
    auto kernel = exhaustive_gather_kernel<kKV, kWY, kWZ, MODE, BOUNCE, CLAMP, LB>;
    FBP_TRY_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    kernel<<<grid, 32 * kWY * kWZ, smem, stream>>>(p);
    FBP_CHECK_LAUNCH(ctx, "exhaustive_gather_kernel");
    return FBP_OK;
}

template <int LB>
fbp_status dispatch_exhaustive(fbp_context* ctx, const ExhaustiveGatherParams& p, dim3 grid, size_t smem,
                               cudaStream_t s, bool bounce, float t0, bool capped) {
    if (t0 > 0.f) {
        if (bounce) return go_exhaustive<EX_EXACT, true, true, LB>(ctx, p, grid, smem, s);
        return go_exhaustive<EX_EXACT, false, true, LB>(ctx, p, grid, smem, s);
    }
    if (t0 == 0.f) {
        if (bounce) {
            if (capped) return go_exhaustive<EX_T0ZERO, true, true, LB>(ctx, p, grid, smem, s);
            return go_exhaustive<EX_T0ZERO, true, false, LB>(ctx, p, grid, smem, s);
        }
        if (capped) return go_exhaustive<EX_T0ZERO, false, true, LB>(ctx, p, grid, smem, s);
        return go_exhaustive<EX_T0ZERO, false, false, LB>(ctx, p, grid, smem, s);
    }
    if (bounce) {
        if (capped) return go_exhaustive<EX_FAST, true, true, LB>(ctx, p, grid, smem, s);
        return go_exhaustive<EX_FAST, true, false, LB>(ctx, p, grid, smem, s);
    }
    if (capped) return go_exhaustive<EX_FAST, false, true, LB>(ctx, p, grid, smem, s);
    return go_exhaustive<EX_FAST, false, false, LB>(ctx, p, grid, smem, s);
}

template <typename S>
fbp_status launch_exhaustive(fbp_context* ctx, const fbp_recon_info& in, const void* cube, const float* laser_xyz,
                             const float* sensor_xyz, float* volume, cudaStream_t stream) {
    const uint32_t L = in.num_laser_targets, Sn = in.num_sensor_targets, T = in.num_time_bins;
    const uint32_t Vx = in.voxel_res[0], Vy = in.voxel_res[1], Vz = in.voxel_res[2];
    constexpr int ALIGN = 4;  // FP32 rows
    const double ex = (double)std::min<uint32_t>(kKV, Vx) * std::fabs(in.voxel_size[0]);
    const double ey = (double)std::min<uint32_t>(4 * kWZ, Vz) * std::fabs(in.voxel_size[1]);
    const double ez = (double)std::min<uint32_t>(8 * kWY, Vy) * std::fabs(in.voxel_size[2]);
    WindowPlan wp;
    FBP_TRY(plan_window(ctx, ex, ey, ez, in.time_step, T, ALIGN, sizeof(float), ExhaustiveGatherParams::meta_bytes(64),
                        &wp, "fbp_backproject_exhaustive"));
    // 64 pairs per stage where two CTAs per SM still fit (the kernel's
    // registers allow two): half the stage planning, barriers and compensated
    // folds per pair (200.5 -> 187.3 ms for 16^2 x 32^2 x 1024 -> 128^3).
    if (wp.ch == 32) {
        const size_t s64 = ExhaustiveGatherParams::meta_bytes(64) + (size_t)(2 * 64 + 1) * (wp.slot_w + ALIGN) * sizeof(float);
        if (s64 <= (size_t)ctx->smem_optin / 2) {
            wp.ch = 64;
            wp.smem = s64;
        }
    }
    const uint32_t slot_w = wp.slot_w, pitch = wp.pitch;
    const uint64_t npairs = (uint64_t)L * Sn;

    void* rows = nullptr;
    FBP_TRY(workspace(ctx, WS_CUBE_ROWS, npairs * pitch * sizeof(float), stream, &rows));
    {
        const uint64_t n = npairs * pitch;
        const unsigned blocks = (unsigned)std::min<uint64_t>(cdiv(n, 256), (uint64_t)ctx->sm_count * 16);
        pair_rows_kernel<S><<<blocks, 256, 0, stream>>>(static_cast<float*>(rows), static_cast<const S*>(cube), npairs,
                                                        T, pitch);
        FBP_CHECK_LAUNCH(ctx, "pair_rows_kernel");
    }

    ExhaustiveGatherParams p{};
    const float4* lscan = nullptr;
    FBP_TRY(build_tables(ctx, in, laser_xyz, stream, &lscan, &p.xs, &p.ys, &p.zs));
    // build_tables stores |l-laser| + |l-sensor|; the exhaustive kernel needs
    // |l - laserPos| and |s - sensorPos| separately, so rebuild both tables.
    void* lp = nullptr;
    void* sp = nullptr;
    FBP_TRY(workspace(ctx, WS_SCAN_TABLE, (size_t)L * sizeof(float4), stream, &lp));
    FBP_TRY(workspace(ctx, WS_SENSOR_TABLE, (size_t)Sn * sizeof(float4), stream, &sp));
    scan_table_kernel<<<cdiv(L, 256), 256, 0, stream>>>(static_cast<float4*>(lp), laser_xyz, L,
                                                       (int)in.discard_first_last_bounces, in.laser_position[0],
                                                       in.laser_position[1], in.laser_position[2], 0.f, 0.f, 0.f, 0);
    FBP_CHECK_LAUNCH(ctx, "scan_table_kernel");
    scan_table_kernel<<<cdiv(Sn, 256), 256, 0, stream>>>(static_cast<float4*>(sp), sensor_xyz, Sn,
                                                        (int)in.discard_first_last_bounces, in.sensor_position[0],
                                                        in.sensor_position[1], in.sensor_position[2], 0.f, 0.f, 0.f, 0);
    FBP_CHECK_LAUNCH(ctx, "scan_table_kernel");
    p.lscan = static_cast<const float4*>(lp);
    p.sscan = static_cast<const float4*>(sp);
    p.volume = volume;
    p.status = ctx->status_dev;
    p.rows = static_cast<const float*>(rows);
    p.Vx = Vx; p.Vy = Vy; p.Vz = Vz; p.L = L; p.S = Sn; p.T = T;
    p.t0 = in.time_offset;
    p.dt = in.time_step;
    p.row_pitch = pitch;
    p.slot_w = slot_w;
    p.ch = wp.ch;
    p.exact_weights = ctx->weight_mode == FBP_WEIGHTS_REFERENCE;
    dim3 grid(cdiv(Vx, kKV), cdiv(Vy, 8 * kWY), cdiv(Vz, 4 * kWZ));
    const bool bounce = in.discard_first_last_bounces == 0;
    if (L % 4 == 0 && wp.ch % 4 == 0)
        return dispatch_exhaustive<4>(ctx, p, grid, wp.smem, stream, bounce, in.time_offset, wp.capped);
    return dispatch_exhaustive<1>(ctx, p, grid, wp.smem, stream, bounce, in.time_offset, wp.capped);
}

}  // namespace
}  // namespace fbp

using namespace fbp;

extern "C" fbp_status fbp_backproject_exhaustive(fbp_context* ctx, const fbp_recon_info* info, const void* cube,
                                                 int dtype, const float* laser_xyz, const float* sensor_xyz,
                                                 float* volume, void* stream) {
    return guarded("fbp_backproject_exhaustive", [&]() -> fbp_status {
        clear_error();
        FBP_TRY(check_ctx(ctx));
        FBP_TRY(validate_info(info, true, "fbp_backproject_exhaustive"));
        if (!cube || !laser_xyz || !sensor_xyz || !volume)
            return set_error(FBP_ERR_INVALID_ARG, "fbp_backproject_exhaustive: null buffer");
        cudaStream_t s = (cudaStream_t)stream;
        switch (dtype) {
            case FBP_F32: return launch_exhaustive<float>(ctx, *info, cube, laser_xyz, sensor_xyz, volume, s);
            case FBP_BF16: return launch_exhaustive<__nv_bfloat16>(ctx, *info, cube, laser_xyz, sensor_xyz, volume, s);
            case FBP_F16: return launch_exhaustive<__half>(ctx, *info, cube, laser_xyz, sensor_xyz, volume, s);
            default: return set_error(FBP_ERR_INVALID_ARG, "fbp_backproject_exhaustive: unknown dtype");
        }
    });
}
