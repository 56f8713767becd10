// Device code of the confocal gather, shared by the one-capture kernel
// (bp_confocal.cu) and the persistent multi-capture kernel (batch.cu).
#pragma once

#include "bp_common.cuh"

namespace fbp {

// Arithmetic paths of the pair loop (all reproduce the reference's bins):
//   PATH_2D     time_offset == 0, no bounce terms: dist = 2d exactly, so
//               x = d * (2 rcp(dt)) and the weight is rcp(d^2) = 4 rcp(dist^2);
//               the stage's partial sum is scaled by 1/4 (exact).
//   PATH_FAST   time_offset <= 0 (every path >= 0): dist = fma(d, 2, -t0) [+ bounce].
//   PATH_EXACT  time_offset > 0: negative paths possible, bin by conversion.
// In PATH_2D / PATH_FAST the bin is floor(x) - a via a round-toward-zero add of
// 2^23 - a; without CLAMP the window planner guarantees every bin of the tile
// lies inside its window, so the -2^23 bias folds into the shared-memory base.
//   PATH_SCATTER + j  the reference's ACCUMULATE_VOXEL_SCATTERING variant
//               (transient_reconstruction.cuh:112-126): every bin of the
//               path range dist -/+ the voxel's half diagonal, stepped by
//               (dt + EPS) in float like the reference.  The first 2 + j
//               steps run unrolled and predicated (the voxels' walks
//               interleave), any further ones in a loop; bins by the same
//               round-toward-zero add (the path is never negative).
//   PATH_SCATTER + 3 + j  the same where every walk takes at least 2 + j
//               steps: the host checks (1 + j) (dt + EPS) + 1e-4 m < the
//               voxel diagonal, and stages with a path under 3.5 mm past
//               the half diagonal or of 64 m or more take the predicated
//               reference loop, so the unrolled steps add unconditionally
//               (the rounding of dd over four steps stays below 2e-5 m).
enum { PATH_2D = 0, PATH_FAST = 1, PATH_EXACT = 2, PATH_SCATTER = 3 };
constexpr int kScatterMaxPrefix = 4;
constexpr int kScatterForms = kScatterMaxPrefix - 1;  // prefixes 2, 3, 4
__host__ __device__ constexpr bool is_scatter(int path) { return path >= PATH_SCATTER; }
__host__ __device__ constexpr int scatter_prefix(int path) { return (path - PATH_SCATTER) % kScatterForms + 2; }
__host__ __device__ constexpr bool scatter_free(int path) { return path - PATH_SCATTER >= kScatterForms; }

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
__device__ __forceinline__ void confocal_stage(const float4* __restrict__ geo, const ulonglong2* __restrict__ geo2,
                                               const int2* __restrict__ meta, const float* __restrict__ wts, int nl, const float (&px)[KV], float py,
                                               float pz, float neg_t0, float rcp_dt, uint32_t slot_w,
                                               float (&acc)[KV], float ext = 0.f, float step = 0.f,
                                               bool tail = true) {
    constexpr int SH = ElemShift<S>::value;
    const float rcp2 = 2.f * rcp_dt;  // exact
    if constexpr (is_scatter(PATH)) {
        constexpr int SP = scatter_prefix(PATH);
        static_assert(SP >= 1 && SP <= kScatterMaxPrefix, "prefix within the step bound");
        const int max_it = (int)(2.f * ext / step) + 4;  // >= 4 >= SP
        // The reference adds I * w per bin with an atomic: one rounding for
        // the product, one for the sum, in bin order.  The count bound only
        // matters where dist is so large that adding the step no longer
        // changes it (no such path reaches a bin).  Once dd >= dmax it stays
        // there, so a predicated step past the end only reads (the clamped
        // index keeps it inside the slot).
        for (int i = 0; i < nl; ++i) {
            const float4 g = geo[i];
            const int2 m = meta[i];  // (float 2^23 - a for window start bin a, slot shared address)
            const float bias = __int_as_float(m.x);
            const float wl = WEIGHTED ? wts[i] : 1.f;
            const float dy = sub_rn(py, g.y), dz = sub_rn(pz, g.z);
            const float dy2 = mul_rn(dy, dy);
            auto bin_at = [&](float dd) -> uint32_t {
                const uint32_t bits = __float_as_uint(add_rz(ref_bin_ratio(dd, rcp_dt), bias));
                if (CLAMP) return (uint32_t)m.y + (min(bits - 0x4B000000u, slot_w) << SH);
                return (uint32_t)m.y + (bits << SH);  // every read inside the planned window; bias folded into m.y
            };
            // Steps SP.. of one walk (rare: a diagonal longer than the planned steps).
            auto walk_rest = [&](float a, float dd, float dmax, float w) -> float {
                for (int it = SP; dd < dmax && it < max_it; ++it) {
                    float I = lds_elem<S>(bin_at(dd));
                    if (WEIGHTED) I *= wl;
                    a = add_rn(a, mul_rn(I, w));
                    dd = add_rn(dd, step);
                }
                return a;
            };
            if constexpr (!SAFE && KV % 2 == 0) {
                // Voxel pairs (k, k + 1) in packed FP32 pairs, step by step.
                const f32x2_t gxp = pack2(g.x, g.x), dy2p = pack2(dy2, dy2), dzp = pack2(dz, dz);
                const f32x2_t gwp = pack2(g.w, g.w), extp = pack2(ext, ext), stepp = pack2(step, step);
                const f32x2_t rdp = pack2(rcp_dt, rcp_dt), biasp = pack2(bias, bias), wlp = pack2(wl, wl);
#pragma unroll
                for (int j = 0; j < KV / 2; ++j) {
                    const f32x2_t dx = sub_rn2(pack2(px[2 * j], px[2 * j + 1]), gxp);
                    float q0, q1, s0, s1, e0, e1, h0, h1;
                    unpack2(fma_rn2(dzp, dzp, fma_rn2(dx, dx, dy2p)), q0, q1);
                    f32x2_t dist = fma_rn2(pack2(sqrt_approx(q0), sqrt_approx(q1)), pack2(2.f, 2.f),
                                           pack2(neg_t0, neg_t0));
                    if (BOUNCE) dist = add_rn2(dist, gwp);
                    unpack2(mul_rn2(dist, dist), s0, s1);
                    const f32x2_t w = pack2(rcp_approx(s0), rcp_approx(s1));
                    unpack2(sub_rn2(dist, extp), e0, e1);
                    unpack2(add_rn2(dist, extp), h0, h1);  // dmax
                    f32x2_t dd = pack2(fmaxf(0.f, e0), fmaxf(0.f, e1));
                    float a0 = acc[2 * j], a1 = acc[2 * j + 1];
#pragma unroll
                    for (int it = 0; it < SP; ++it) {
                        float d0, d1, b0, b1, p0, p1;
                        unpack2(dd, d0, d1);
                        unpack2(add_rz2(mul_rn2(dd, rdp), biasp), b0, b1);
                        const uint32_t i0 = CLAMP ? min(__float_as_uint(b0) - 0x4B000000u, slot_w) : __float_as_uint(b0);
                        const uint32_t i1 = CLAMP ? min(__float_as_uint(b1) - 0x4B000000u, slot_w) : __float_as_uint(b1);
                        f32x2_t I = pack2(lds_elem<S>((uint32_t)m.y + (i0 << SH)),
                                          lds_elem<S>((uint32_t)m.y + (i1 << SH)));
                        if (WEIGHTED) I = mul_rn2(I, wlp);
                        unpack2(mul_rn2(I, w), p0, p1);
                        if constexpr (scatter_free(PATH)) {
                            a0 = add_rn(a0, p0);  // dd < dmax holds for every unrolled step
                            a1 = add_rn(a1, p1);
                        } else {
                            a0 = add_rn_if_lt(a0, p0, d0, h0);
                            a1 = add_rn_if_lt(a1, p1, d1, h1);
                        }
                        dd = add_rn2(dd, stepp);
                    }
                    if (scatter_free(PATH) && !tail) {
                        // Every walk is exactly the unrolled steps long.
                        acc[2 * j] = a0;
                        acc[2 * j + 1] = a1;
                        continue;
                    }
                    float d0, d1, w0, w1;
                    unpack2(dd, d0, d1);
                    unpack2(w, w0, w1);
                    acc[2 * j] = walk_rest(a0, d0, h0, w0);
                    acc[2 * j + 1] = walk_rest(a1, d1, h1, w1);
                }
            } else {
#pragma unroll
                for (int k = 0; k < KV; ++k) {
                    const float dx = sub_rn(px[k], g.x);
                    const float d = sqrt_approx(fma_rn(dz, dz, fma_rn(dx, dx, dy2)));
                    float dist = fma_rn(d, 2.f, neg_t0);
                    if (BOUNCE) dist = add_rn(dist, g.w);
                    const float w = SAFE ? ref_safe_rcp(mul_rn(dist, dist)) : rcp_approx(mul_rn(dist, dist));
                    float dd = fmaxf(0.f, sub_rn(dist, ext));
                    const float dmax = add_rn(dist, ext);
                    float a = acc[k];
#pragma unroll
                    for (int it = 0; it < SP; ++it) {
                        float I = lds_elem<S>(bin_at(dd));
                        if (WEIGHTED) I *= wl;
                        a = add_rn_if_lt(a, mul_rn(I, w), dd, dmax);
                        dd = add_rn(dd, step);
                    }
                    acc[k] = walk_rest(a, dd, dmax, w);
                }
            }
        }
        return;
    }
    if constexpr (!is_scatter(PATH) && !SAFE && KV % 4 == 0) {
        // Voxel pairs (k, k + 1) in packed FP32 pairs: the bins are the scalar
        // loop's operations, bit for bit, at half the FP32 instructions.
        //
        // Weights by simultaneous inversion (P. L. Montgomery, "Speeding the
        // Pollard and elliptic curve methods of factorization", Math. Comp. 48
        // (1987), section 10.3.1): the squared paths s_0, s_1 of two packed
        // pairs share ONE reciprocal per lane, r = 1 / (s_0 s_1), and
        // 1 / s_0 = r s_1, 1 / s_1 = r s_0 (G = 4 pairs would use a product
        // tree: 1 / s_0 = (r s_2 s_3) s_1).  That is one rcp.approx per two
        // voxels instead of one per voxel: the bin's sqrt.approx and the
        // weight's rcp.approx were the only MUFU operations per pair, and the
        // MUFU pipe bounded the loop.  Each weight carries at most ~2 ulp (the
        // rounded product, the approximate reciprocal, one rounded multiply)
        // instead of rcp.approx's own ~1 ulp.  G = 2 measured faster than
        // G = 4 (whose extra multiplies load the FMA pipe, which the packed
        // pairs already keep busy).  Stages where a product could leave the
        // normal FP32 range (paths under 3.5 mm or over 10 km) take the scalar
        // loop with the reference's safeRCP.
        constexpr int G = 2;
        f32x2_t pxp[KV / 2], accp[KV / 2];
#pragma unroll
        for (int j = 0; j < KV / 2; ++j) {
            pxp[j] = pack2(px[2 * j], px[2 * j + 1]);
            accp[j] = pack2(acc[2 * j], acc[2 * j + 1]);
        }
        const f32x2_t pyp = pack2(py, py), pzp = pack2(pz, pz);
        const f32x2_t rcp2p = pack2(rcp2, rcp2), rdp = pack2(rcp_dt, rcp_dt), two = pack2(2.f, 2.f);
        const f32x2_t nt0p = pack2(neg_t0, neg_t0);
#pragma unroll 2
        for (int i = 0; i < nl; ++i) {
            // (x, x, y, y), (z, z, bias, bias), (bounce, bounce, w, w) as register pairs.
            const ulonglong2 ga = geo2[3 * i], gb = geo2[3 * i + 1];
            const uint32_t m_addr = (uint32_t)meta[i].y;
            const int m_bias = meta[i].x;
            const f32x2_t gxp = ga.x, biasp = gb.y;
            const f32x2_t dyp = sub_rn2(pyp, ga.y), dzp = sub_rn2(pzp, gb.x);
            const f32x2_t dy2p = mul_rn2(dyp, dyp);
            f32x2_t gwp = 0ull, wlp = 0ull;
            if (BOUNCE || WEIGHTED) {
                const ulonglong2 gc = geo2[3 * i + 2];
                gwp = gc.x;
                wlp = gc.y;
            }
#pragma unroll
            for (int j0 = 0; j0 < KV / 2; j0 += G) {
                f32x2_t sq[G], Iq[G];
#pragma unroll
                for (int jj = 0; jj < G; ++jj) {
                    const int j = j0 + jj;
                    const f32x2_t dx = sub_rn2(pxp[j], gxp);
                    float q0, q1;
                    unpack2(fma_rn2(dzp, dzp, fma_rn2(dx, dx, dy2p)), q0, q1);
                    const f32x2_t d = pack2(sqrt_approx(q0), sqrt_approx(q1));
                    f32x2_t x;
                    if (PATH == PATH_2D) {
                        x = mul_rn2(d, rcp2p);
                        sq[jj] = mul_rn2(d, d);
                    } else {
                        f32x2_t dist = fma_rn2(d, two, nt0p);
                        if (BOUNCE) dist = add_rn2(dist, gwp);
                        x = mul_rn2(dist, rdp);
                        sq[jj] = mul_rn2(dist, dist);
                    }
                    uint32_t a0, a1;
                    if (PATH == PATH_EXACT) {
                        float x0, x1;
                        unpack2(x, x0, x1);
                        const int b0 = __float2int_rz(x0), b1 = __float2int_rz(x1);  // static_cast<int>
                        a0 = m_addr + (min((uint32_t)(b0 - m_bias), slot_w) << SH);
                        a1 = m_addr + (min((uint32_t)(b1 - m_bias), slot_w) << SH);
                    } else {
                        float b0, b1;
                        unpack2(add_rz2(x, biasp), b0, b1);
                        if (CLAMP) {
                            a0 = m_addr + (min(__float_as_uint(b0) - 0x4B000000u, slot_w) << SH);
                            a1 = m_addr + (min(__float_as_uint(b1) - 0x4B000000u, slot_w) << SH);
                        } else {
                            a0 = m_addr + (__float_as_uint(b0) << SH);  // bias folded into the address
                            a1 = m_addr + (__float_as_uint(b1) << SH);
                        }
                    }
                    Iq[jj] = pack2(lds_elem<S>(a0), lds_elem<S>(a1));
                    if (WEIGHTED) Iq[jj] = mulf2(Iq[jj], wlp);
                }
                if constexpr (G == 4) {
                    const f32x2_t p01 = mul_rn2(sq[0], sq[1]), p23 = mul_rn2(sq[2], sq[3]);
                    float m0, m1;
                    unpack2(mul_rn2(p01, p23), m0, m1);
                    const f32x2_t r = pack2(rcp_approx(m0), rcp_approx(m1));
                    const f32x2_t r01 = mul_rn2(r, p23), r23 = mul_rn2(r, p01);  // 1/(s0 s1), 1/(s2 s3)
                    accp[j0 + 0] = fmaf2(Iq[0], mul_rn2(r01, sq[1]), accp[j0 + 0]);
                    accp[j0 + 1] = fmaf2(Iq[1], mul_rn2(r01, sq[0]), accp[j0 + 1]);
                    accp[j0 + 2] = fmaf2(Iq[2], mul_rn2(r23, sq[3]), accp[j0 + 2]);
                    accp[j0 + 3] = fmaf2(Iq[3], mul_rn2(r23, sq[2]), accp[j0 + 3]);
                } else {
                    float m0, m1;
                    unpack2(mul_rn2(sq[0], sq[1]), m0, m1);
                    const f32x2_t r = pack2(rcp_approx(m0), rcp_approx(m1));
                    accp[j0 + 0] = fmaf2(Iq[0], mul_rn2(r, sq[1]), accp[j0 + 0]);
                    accp[j0 + 1] = fmaf2(Iq[1], mul_rn2(r, sq[0]), accp[j0 + 1]);
                }
            }
        }
#pragma unroll
        for (int j = 0; j < KV / 2; ++j) unpack2(accp[j], acc[2 * j], acc[2 * j + 1]);
        return;
    }
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
__device__ __forceinline__ void confocal_tile(const ConfocalGatherParams& p, uint32_t bx, uint32_t by, uint32_t bz,
                                              unsigned long long tile_id) {
    constexpr int NT = 32 * WY * WZ;
    constexpr int CHMAX = 32;
    constexpr int ALIGN = 16 / sizeof(S);  // elements per 16-byte copy
    constexpr int SH = ElemShift<S>::value;
    constexpr int TY = 8 * WY, TZ = 4 * WZ;
    const int CH = p.ch;

    extern __shared__ __align__(16) unsigned char smem_raw[];
    const uint32_t slot_stride = p.slot_w + ALIGN;  // sentinel element(s) at slot_w
    float4* s_geo = reinterpret_cast<float4*>(smem_raw);         // [2][CHMAX]
    ulonglong2* s_geo2 = reinterpret_cast<ulonglong2*>(s_geo + 2 * CHMAX);  // [2][CHMAX][kPackedGeo]
    constexpr int PG = ConfocalGatherParams::kPackedGeo;
    int2* s_meta = reinterpret_cast<int2*>(s_geo2 + 2 * CHMAX * PG);  // [2][CHMAX]
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

    const uint32_t tx0 = bx * KV, ty0 = by * TY, tz0 = bz * TZ;
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
    // PATH_SCATTER: length(voxelSize) / 2 and the step timeStep + EPS, in the
    // reference's FP32 arithmetic (transient_reconstruction.cuh:113-125).
    const float scat_ext = is_scatter(PATH) ? mul_rn(0.5f, sqrt_approx(ref_dot3(p.vs[0], p.vs[1], p.vs[2]))) : 0.f;
    const float scat_step = is_scatter(PATH) ? add_rn(p.dt, FBP_EPS) : 0.f;

    // Sentinels of every slot and the whole zero slot.
    for (int i = tid; i < 2 * CH * ALIGN; i += NT) {
        const int slot = i / ALIGN, e = i % ALIGN;
        s_slots[(size_t)slot * slot_stride + p.slot_w + e] = from_f32<S>(0.f);
    }
    for (uint32_t i = tid; i < slot_stride; i += NT) s_slots[zero_slot + i] = from_f32<S>(0.f);

    // SAMPLE_CLUSTERS: this tile's clusters, drawn by systematic sampling from
    // its CDF (K positions (k + u) / K), duplicates merged; each chosen
    // cluster is gathered whole with weight hits / (K p_c).
    uint32_t nitems = SAMPLED ? p.smp.K : p.L;
    const uint32_t* s_clu = nullptr;
    const float* s_cw = nullptr;
    if constexpr (SAMPLED) {
        __shared__ uint32_t clu[kMaxClusterSamples];
        __shared__ float cw[kMaxClusterSamples];
        __shared__ uint32_t ncl;
        if (p.smp.mode == SAMPLE_CLUSTERS) {
            const uint32_t K = p.smp.K, G = p.smp.G;
            const float* cdf = p.smp.tile_cdf ? p.smp.tile_cdf + tile_id * G : nullptr;
            if (warp == 0) {
                const float u = hash_uniform(p.smp.seed, tile_id, 0xFFFFFFFFu, 2);
                for (uint32_t k = lane; k < K; k += 32) {
                    const float x = ((float)k + u) / (float)K;
                    uint32_t c;
                    if (cdf) {
                        uint32_t lo = 0, hi = G - 1;  // first c with x < cdf[c]
                        while (lo < hi) {
                            const uint32_t mid = (lo + hi) >> 1;
                            if (x < cdf[mid]) hi = mid; else lo = mid + 1;
                        }
                        c = lo;
                    } else {
                        c = min((uint32_t)(x * (float)G), G - 1);
                    }
                    clu[k] = c;
                }
                __syncwarp();
                if (lane == 0) {
                    uint32_t n = 0;
                    for (uint32_t k = 0; k < K; ++k) {
                        const uint32_t c = clu[k];
                        if (n > 0 && clu[n - 1] == c) {
                            cw[n - 1] += 1.f;
                        } else {
                            clu[n] = c;
                            cw[n] = 1.f;
                            ++n;
                        }
                    }
                    for (uint32_t j = 0; j < n; ++j) {
                        const uint32_t c = clu[j];
                        const float pc = cdf ? cdf[c] - (c > 0 ? cdf[c - 1] : 0.f) : 1.f / (float)G;
                        cw[j] = pc > 0.f ? cw[j] / ((float)K * pc) : 0.f;
                    }
                    ncl = n;
                }
            }
            __syncthreads();
            nitems = ncl * p.smp.cluster_side * p.smp.cluster_side;
            s_clu = clu;
            s_cw = cw;
        }
    }
    const uint32_t nchunks = (nitems + CH - 1) / CH;

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
                    // Point `inner` of the j-th chosen cluster (outside the grid
                    // for a ragged edge cluster: skipped).
                    const uint32_t cs = p.smp.cluster_side, cpr = (p.smp.n_side + cs - 1) / cs;
                    const uint32_t j = item / (cs * cs), inner = item - j * (cs * cs);
                    const uint32_t cl = s_clu[j];
                    const uint32_t ix = (cl % cpr) * cs + inner % cs, iz = (cl / cpr) * cs + inner / cs;
                    l = (ix < p.smp.n_side && iz < p.smp.n_side) ? iz * p.smp.n_side + ix : 0xFFFFFFFFu;
                    pl = 0.f;
                    wgt = s_cw[j];
                }
                if (p.smp.mode != SAMPLE_CLUSTERS) wgt = pl > 0.f ? 1.f / ((float)nitems * pl) : 0.f;
            }
            float4 g = make_float4(0.f, 0.f, 0.f, 0.f);
            int cnt = 0, src = 0, near = 0, a = 0;
            bool skip = true;
            // A point of a ragged edge cluster that lies outside the scan grid:
            // planned with scan point 0's geometry (finite paths and weights)
            // and read from the zero slot.
            const bool ragged = item < nitems && l >= p.L;
            if (item < nitems) {
                g = p.scan[ragged ? 0u : l];
                // Nearest and farthest voxel-centre distance of the tile.
                const float cx = fminf(fmaxf(g.x, bx0), bx1), cy = fminf(fmaxf(g.y, by0), by1),
                            cz = fminf(fmaxf(g.z, bz0), bz1);
                const float dmin = sqrtf((g.x - cx) * (g.x - cx) + (g.y - cy) * (g.y - cy) + (g.z - cz) * (g.z - cz));
                const float fx = fmaxf(fabsf(g.x - bx0), fabsf(g.x - bx1)), fy = fmaxf(fabsf(g.y - by0), fabsf(g.y - by1)),
                            fz = fmaxf(fabsf(g.z - bz0), fabsf(g.z - bz1));
                const float dmax = sqrtf(fx * fx + fy * fy + fz * fz);
                const float bnc = BOUNCE ? g.w : 0.f;
                float pmin = 2.f * dmin + neg_t0 + bnc, pmax = 2.f * dmax + neg_t0 + bnc;
                if (is_scatter(PATH)) {
                    // The bins of dist -/+ ext, read one step past dist + ext;
                    // a walk clipped at 0 reads up to max(step, 2 ext).
                    pmin = fmaxf(0.f, pmin - 1.01f * scat_ext);
                    pmax = fmaxf(pmax + 1.01f * scat_ext, 2.02f * scat_ext) + scat_step;
                }
                // Paths this short make dist^2 <= EPS possible: use safeRCP's
                // branch.  Paths this long (or NaN) could take the batched
                // reciprocal's products out of the FP32 range: also per voxel.
                // The unconditional scattering walk also wants paths under
                // 64 m (its rounding bound) and dist - ext > 0 (pmin above).
                near = pmin < 0.0035f || !(pmax < (scatter_free(PATH) ? 64.f : 1.0e4f));
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
                if (ragged) {
                    skip = true;
                    cnt = 0;
                    wgt = 0.f;
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
            if (item >= nitems) {
                // Beyond the last scan point: x + 0 < 2^23 lands on the sentinel
                // (CLAMP) or, unclamped, reads the zero slot at index 0.
                bias = PATH == PATH_EXACT ? 0x40000000 : 0;
                saddr = sbase + (uint32_t)slots_off + (zero_slot << SH);
                if (!CLAMP && PATH != PATH_EXACT) saddr -= (__float_as_uint(0.f) << SH);
                g = make_float4(3.0e18f, 3.0e18f, 3.0e18f, 0.f);  // far away: x is huge
                wgt = 0.f;
            }
            s_geo[buf * CHMAX + tid] = g;
            {
                ulonglong2* g2 = s_geo2 + (buf * CHMAX + tid) * PG;
                const float bf = __int_as_float(bias);
                g2[0] = make_ulonglong2(pack2(g.x, g.x), pack2(g.y, g.y));
                g2[1] = make_ulonglong2(pack2(g.z, g.z), pack2(bf, bf));
                g2[2] = make_ulonglong2(pack2(g.w, g.w), pack2(wgt, wgt));
            }
            s_meta[buf * CHMAX + tid] = make_int2(bias, (int)saddr);
            s_cnt[buf * CHMAX + tid] = cnt;
            s_src[buf * CHMAX + tid] = src;
            s_row[buf * CHMAX + tid] = ragged ? 0 : (int)l;
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

    // Compensated sums: in registers, or (16 voxels per thread) in shared
    // memory behind the zero slot, [2 KV][NT] so a warp's accesses are
    // consecutive words.
    constexpr bool KSMEM = kahan_smem_bytes(KV, NT) > 0;
    float* s_kahan = reinterpret_cast<float*>(
        smem_raw + ((slots_off + (size_t)(zero_slot + slot_stride) * sizeof(S) + 15) & ~size_t(15)));
    float acc[KV], ksum[KSMEM ? 1 : KV], kcomp[KSMEM ? 1 : KV];
#pragma unroll
    for (int k = 0; k < KV; ++k) acc[k] = 0.f;
    if constexpr (KSMEM) {
#pragma unroll
        for (int k = 0; k < 2 * KV; ++k) s_kahan[k * NT + tid] = 0.f;
    } else {
#pragma unroll
        for (int k = 0; k < KV; ++k) ksum[k] = kcomp[k] = 0.f;
    }

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
        const ulonglong2* geo2 = s_geo2 + buf * CHMAX * PG;
        const int2* meta = s_meta + buf * CHMAX;
        const float* wts = s_w + buf * CHMAX;
        const bool safe = s_flag[buf] != 0 || p.exact_weights;
        const int nl = (int)min((uint32_t)CH, nitems - c * CH);
        float scale = 1.f;
        if (!safe) {
            confocal_stage<S, KV, PATH, BOUNCE, CLAMP, false, SAMPLED>(geo, geo2, meta, wts, nl, px, py, pz, neg_t0, rcp_dt,
                                                                        p.slot_w, acc, scat_ext, scat_step,
                                                                        !p.scat_exact);
            if (PATH == PATH_2D) scale = 0.25f;  // w was rcp(d^2) = 4 rcp(dist^2)
        } else {
            confocal_stage<S, KV, PATH, BOUNCE, CLAMP, true, SAMPLED>(geo, geo2, meta, wts, nl, px, py, pz, neg_t0, rcp_dt,
                                                                       p.slot_w, acc, scat_ext, scat_step);
        }

        // Compensated (Kahan) fold of this stage's partial sums.
#pragma unroll
        for (int k = 0; k < KV; ++k) {
            const float sk = KSMEM ? s_kahan[(2 * k) * NT + tid] : ksum[k];
            const float ck = KSMEM ? s_kahan[(2 * k + 1) * NT + tid] : kcomp[k];
            const float y = sub_rn(mul_rn(acc[k], scale), ck);
            const float t = add_rn(sk, y);
            const float c = sub_rn(sub_rn(t, sk), y);
            if constexpr (KSMEM) {
                s_kahan[(2 * k) * NT + tid] = t;
                s_kahan[(2 * k + 1) * NT + tid] = c;
            } else {
                kcomp[k] = c;
                ksum[k] = t;
            }
            acc[k] = 0.f;
        }
    }

    if (row_ok) {
        float* out = p.volume + ((size_t)vz * p.Vy + vy) * p.Vx + tx0;
#pragma unroll
        for (int k = 0; k < KV; ++k)
            if (tx0 + k < p.Vx) out[k] = KSMEM ? s_kahan[(2 * k) * NT + tid] : ksum[k];
    }
}

template <typename S, int KV, int WY, int WZ, int PATH, bool BOUNCE, bool SAMPLED, bool CLAMP>
__global__ void __launch_bounds__(32 * WY * WZ)
confocal_gather_kernel(ConfocalGatherParams p) {
    const unsigned long long tile_id =
        ((unsigned long long)blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x;
    confocal_tile<S, KV, WY, WZ, PATH, BOUNCE, SAMPLED, CLAMP>(p, blockIdx.x, blockIdx.y, blockIdx.z, tile_id);
}

// Persistent form for a batch of captures: CTAs pull (capture, tile) work items
// from an atomic counter until the list is exhausted.  Items are sorted by
// decreasing cost on the host, so the long tiles start first.
struct BatchItem {
    uint32_t capture, bx, by, bz;
};

template <typename S, int KV, int WY, int WZ, int PATH, bool BOUNCE, bool CLAMP>
__global__ void __launch_bounds__(32 * WY * WZ)
confocal_batch_kernel(const ConfocalGatherParams* __restrict__ caps, const BatchItem* __restrict__ items,
                      uint32_t nitems, unsigned int* __restrict__ counter) {
    __shared__ uint32_t s_item;
    for (;;) {
        __syncthreads();  // the previous tile is done with shared memory and s_item
        if (threadIdx.x == 0) s_item = atomicAdd(counter, 1u);
        __syncthreads();
        const uint32_t it = s_item;
        if (it >= nitems) break;
        const BatchItem w = items[it];
        confocal_tile<S, KV, WY, WZ, PATH, BOUNCE, false, CLAMP>(caps[w.capture], w.bx, w.by, w.bz, it);
    }
}

}  // namespace fbp
