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
    const void* rows;  // [L*S][row_pitch]
    uint32_t Vx, Vy, Vz, L, S, T;
    float t0, dt;
    uint32_t row_pitch, slot_w;
    int ch;

    __host__ __device__ static constexpr size_t meta_bytes(int ch) {
        return ((size_t)2 * ch * (2 * sizeof(float4) + sizeof(float) + 4 * sizeof(int)) + 2 * sizeof(int) + 15) &
               ~size_t(15);
    }
};

// LB = 4: pairs are walked as (laser block of 4, SPAD, laser in block), so
// the SPAD-to-voxel distance is computed once per SPAD for 4 lasers (the 4
// laser distances are kept per block); requires L % 4 == 0 and ch % 4 == 0.
// LB = 1: pairs in (laser, SPAD) order.
template <typename S, int KV, int WY, int WZ, bool BOUNCE, bool EXACT_TRUNC, int LB>
__global__ void __launch_bounds__(32 * WY * WZ)
exhaustive_gather_kernel(ExhaustiveGatherParams p) {
    constexpr int NT = 32 * WY * WZ;
    constexpr int CHMAX = 32;  // scan points (pairs) per stage, upper bound
    const int CH = p.ch;
    constexpr int ALIGN = 16 / sizeof(S);
    constexpr int TY = 8 * WY, TZ = 4 * WZ;

    extern __shared__ __align__(16) unsigned char smem_raw[];
    const uint32_t slot_stride = p.slot_w + ALIGN;
    float4* s_lg = reinterpret_cast<float4*>(smem_raw);  // [2][CHMAX]
    float4* s_sg = s_lg + 2 * CHMAX;                     // [2][CHMAX]
    float* s_cl = reinterpret_cast<float*>(s_sg + 2 * CHMAX);
    int* s_cnt = reinterpret_cast<int*>(s_cl + 2 * CHMAX);
    int* s_src = s_cnt + 2 * CHMAX;
    int* s_lid = s_src + 2 * CHMAX;
    int* s_row = s_lid + 2 * CHMAX;
    int* s_flag = s_row + 2 * CHMAX;
    S* s_slots = reinterpret_cast<S*>(smem_raw + ExhaustiveGatherParams::meta_bytes(CHMAX));

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
    float px[KV];
#pragma unroll
    for (int k = 0; k < KV; ++k) px[k] = p.xs[min(tx0 + k, p.Vx - 1)];

    const float rcp_dt = rcp_approx(p.dt);
    const uint64_t npairs = (uint64_t)p.L * p.S;
    const uint64_t nchunks = (npairs + CH - 1) / CH;

    for (int i = tid; i < 2 * CH * ALIGN; i += NT) {
        const int slot = i / ALIGN, e = i % ALIGN;
        s_slots[(size_t)slot * slot_stride + p.slot_w + e] = from_f32<S>(0.f);
    }

    auto box_range = [&](const float4& g, float& dmin, float& dmax) {
        const float cx = fminf(fmaxf(g.x, bx0), bx1), cy = fminf(fmaxf(g.y, by0), by1), cz = fminf(fmaxf(g.z, bz0), bz1);
        dmin = sqrtf((g.x - cx) * (g.x - cx) + (g.y - cy) * (g.y - cy) + (g.z - cz) * (g.z - cz));
        const float fx = fmaxf(fabsf(g.x - bx0), fabsf(g.x - bx1)), fy = fmaxf(fabsf(g.y - by0), fabsf(g.y - by1)),
                    fz = fmaxf(fabsf(g.z - bz0), fabsf(g.z - bz1));
        dmax = sqrtf(fx * fx + fy * fy + fz * fz);
    };

    auto plan_chunk = [&](uint64_t c, int buf) {
        if (tid < CH) {
            const uint64_t ls = c * CH + tid;
            float4 lg = make_float4(0.f, 0.f, 0.f, 0.f), sg = lg;
            float cl = 0.f;
            int cnt = 0, src = 0, near = 0, lid = -1, row = 0;
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
                const float bnc = BOUNCE ? lg.w + sg.w : 0.f;
                const float pmin = dl0 + ds0 - p.t0 + bnc, pmax = dl1 + ds1 - p.t0 + bnc;
                near = pmin < 0.0035f;
                int blo = (int)fmaxf(fminf(floorf(pmin * rcp_dt), 1.0e9f), -1.0e9f) - 2;
                int bhi = (int)fmaxf(fminf(floorf(pmax * rcp_dt), 1.0e9f), -1.0e9f) + 2;
                int a = max(blo, 0) & ~(ALIGN - 1);
                a = min(a, (int)(p.row_pitch - p.slot_w));
                const int hi = min(bhi + 1, (int)p.row_pitch);
                cnt = hi - a;
                if (cnt < 0) cnt = 0;
                cnt = (cnt + ALIGN - 1) & ~(ALIGN - 1);
                // A window capped at slot_w still covers every valid bin as long
                // as the bins below T it needs fit; bins past the copy map to the
                // zero sentinel.
                if (min(bhi + 1, (int)p.T) - a > (int)p.slot_w) {
                    atomicExch(p.status, (int)FBP_ERR_DEVICE);  // window too small: should not happen
                }
                if (cnt > (int)p.slot_w) {
                    cnt = (int)p.slot_w;
                }
                src = a;
                cl = EXACT_TRUNC ? __int_as_float(a) : (float)(8388608 - a);
            }
            s_lg[buf * CHMAX + tid] = lg;
            s_sg[buf * CHMAX + tid] = sg;
            s_cl[buf * CHMAX + tid] = cl;
            s_cnt[buf * CHMAX + tid] = cnt;
            s_src[buf * CHMAX + tid] = src;
            s_lid[buf * CHMAX + tid] = lid;
            s_row[buf * CHMAX + tid] = row;
            const unsigned any_near = __ballot_sync(CH >= 32 ? 0xffffffffu : ((1u << CH) - 1u), near);
            if (tid == 0) s_flag[buf] = any_near != 0;
        }
    };

    auto copy_chunk = [&](uint64_t c, int buf) {
        const uint32_t vecs = p.slot_w / ALIGN;
        for (uint32_t i = tid; i < CH * vecs; i += NT) {
            const uint32_t s = i / vecs, j = i - s * vecs;
            if ((int)(j * ALIGN) < s_cnt[buf * CHMAX + s]) {
                const uint64_t row = (uint32_t)s_row[buf * CHMAX + s];
                const S* src = static_cast<const S*>(p.rows) + row * p.row_pitch + s_src[buf * CHMAX + s] + j * ALIGN;
                cp_async_16(s_slots + (size_t)(buf * CH + s) * slot_stride + j * ALIGN, src);
            }
        }
        cp_async_commit();
    };

    float acc[KV], ksum[KV], kcomp[KV], dl[LB][KV];
#pragma unroll
    for (int k = 0; k < KV; ++k) acc[k] = ksum[k] = kcomp[k] = 0.f;
#pragma unroll
    for (int li = 0; li < LB; ++li)
#pragma unroll
        for (int k = 0; k < KV; ++k) dl[li][k] = 0.f;
    int cur_l = -1;
    int buf_cur = 0;  // buffer of the stage being accumulated

    // Triples of pair i of the stage in buffer buf with the laser distances
    // dl[li] and the SPAD distances ds (transient_reconstruction.cuh:155-162).
    auto pair_terms = [&](int i, int li, const float (&ds)[KV], bool safe) {
        const float4 lg = s_lg[buf_cur * CHMAX + i];
        const float4 sg = s_sg[buf_cur * CHMAX + i];
        const float cl = s_cl[buf_cur * CHMAX + i];
        const S* slot = s_slots + (size_t)(buf_cur * CH + i) * slot_stride;
        const float bnc = BOUNCE ? add_rn(lg.w, sg.w) : 0.f;
        if constexpr (!EXACT_TRUNC && KV % 2 == 0) {
            if (!safe) {
                // Voxel pairs in packed FP32 pairs, the scalar loop's operations.
                const f32x2_t t0p = pack2(p.t0, p.t0), rdp = pack2(rcp_dt, rcp_dt), clp = pack2(cl, cl);
                const f32x2_t bncp = pack2(bnc, bnc);
#pragma unroll
                for (int j = 0; j < KV / 2; ++j) {
                    f32x2_t dist = sub_rn2(add_rn2(pack2(dl[li][2 * j], dl[li][2 * j + 1]),
                                                   pack2(ds[2 * j], ds[2 * j + 1])), t0p);
                    if (BOUNCE) dist = add_rn2(dist, bncp);
                    float b0, b1;
                    unpack2(add_rz2(mul_rn2(dist, rdp), clp), b0, b1);
                    const uint32_t i0 = min(__float_as_uint(b0) - 0x4B000000u, p.slot_w);
                    const uint32_t i1 = min(__float_as_uint(b1) - 0x4B000000u, p.slot_w);
                    const f32x2_t I = pack2(to_f32(slot[i0]), to_f32(slot[i1]));
                    float s0, s1;
                    unpack2(mul_rn2(dist, dist), s0, s1);
                    const f32x2_t a = fmaf2(I, pack2(rcp_approx(s0), rcp_approx(s1)),
                                            pack2(acc[2 * j], acc[2 * j + 1]));
                    unpack2(a, acc[2 * j], acc[2 * j + 1]);
                }
                return;
            }
        }
#pragma unroll
        for (int k = 0; k < KV; ++k) {
            float dist = sub_rn(add_rn(dl[li][k], ds[k]), p.t0);
            if (BOUNCE) dist = add_rn(dist, bnc);
            const float x = ref_bin_ratio(dist, rcp_dt);
            uint32_t idx;
            if (EXACT_TRUNC) {
                idx = min((uint32_t)(__float2int_rz(x) - __float_as_int(cl)), p.slot_w);
            } else {
                idx = min(__float_as_uint(add_rz(x, cl)) - 0x4B000000u, p.slot_w);
            }
            const float I = to_f32(slot[idx]);
            const float dd = mul_rn(dist, dist);
            const float w = safe ? ref_safe_rcp(dd) : rcp_approx(dd);
            acc[k] = fmaf(I, w, acc[k]);
        }
    };
    auto point_dist = [&](const float4& g, float (&d)[KV]) {
        const float ddy = sub_rn(py, g.y), ddz = sub_rn(pz, g.z);
        const float ddy2 = mul_rn(ddy, ddy);
        if constexpr (KV % 2 == 0) {
            const f32x2_t gxp = pack2(g.x, g.x), ddzp = pack2(ddz, ddz), ddy2p = pack2(ddy2, ddy2);
#pragma unroll
            for (int j = 0; j < KV / 2; ++j) {
                const f32x2_t dx = sub_rn2(pack2(px[2 * j], px[2 * j + 1]), gxp);
                float q0, q1;
                unpack2(fma_rn2(ddzp, ddzp, fma_rn2(dx, dx, ddy2p)), q0, q1);
                d[2 * j] = sqrt_approx(q0);
                d[2 * j + 1] = sqrt_approx(q1);
            }
        } else {
#pragma unroll
            for (int k = 0; k < KV; ++k) {
                const float dx = sub_rn(px[k], g.x);
                d[k] = sqrt_approx(fma_rn(ddz, ddz, fma_rn(dx, dx, ddy2)));
            }
        }
    };

    if (nchunks > 0) {
        plan_chunk(0, 0);
        __syncthreads();
        copy_chunk(0, 0);
    }
    for (uint64_t c = 0; c < nchunks; ++c) {
        const int buf = (int)(c & 1);
        buf_cur = buf;
        __syncthreads();  // every thread is done with chunk c-1, whose buffer plan(c+1) reuses
        if (c + 1 < nchunks) plan_chunk(c + 1, buf ^ 1);
        __syncthreads();  // plan(c+1) visible to the copy loop
        if (c + 1 < nchunks) {
            copy_chunk(c + 1, buf ^ 1);
            cp_async_wait<1>();
        } else {
            cp_async_wait<0>();
        }
        __syncthreads();

        const bool safe = s_flag[buf] != 0;
        const int np = (int)min((uint64_t)CH, npairs - c * CH);
        if (LB == 1) {
            for (int i = 0; i < np; ++i) {
                const int lid = s_lid[buf * CHMAX + i];
                if (lid != cur_l) {  // uniform across the CTA
                    cur_l = lid;
                    point_dist(s_lg[buf * CHMAX + i], dl[0]);
                }
                float ds[KV];
                point_dist(s_sg[buf * CHMAX + i], ds);
                pair_terms(i, 0, ds, safe);
            }
        } else {
            for (int g = 0; g < np; g += LB) {
                const int lb = s_lid[buf * CHMAX + g] / LB;
                if (lb != cur_l) {  // a new block of LB lasers (uniform across the CTA)
                    cur_l = lb;
#pragma unroll
                    for (int li = 0; li < LB; ++li) point_dist(s_lg[buf * CHMAX + g + li], dl[li]);
                }
                float ds[KV];
                point_dist(s_sg[buf * CHMAX + g], ds);  // the group's SPAD
#pragma unroll
                for (int li = 0; li < LB; ++li) pair_terms(g + li, li, ds, safe);
            }
        }
#pragma unroll
        for (int k = 0; k < KV; ++k) {
            const float y = sub_rn(acc[k], kcomp[k]);
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

namespace {

constexpr int kKV = 8, kWY = 2, kWZ = 4;

template <typename S>
__global__ void pair_rows_kernel(S* __restrict__ rows, const S* __restrict__ cube, uint64_t npairs, uint32_t T,
                                 uint32_t pitch) {
    const uint64_t n = npairs * pitch;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t r = i / pitch;
        const uint32_t t = (uint32_t)(i % pitch);
        S v = from_f32<S>(0.f);
        if (t < T) {
            const S c = cube[r * T + t];
            if (to_f32(c) > FBP_EPS) v = c;
        }
        rows[i] = v;
    }
}

template <typename S>
fbp_status launch_exhaustive(fbp_context* ctx, const fbp_recon_info& in, const void* cube, const float* laser_xyz,
                             const float* sensor_xyz, float* volume, cudaStream_t stream) {
    const uint32_t L = in.num_laser_targets, Sn = in.num_sensor_targets, T = in.num_time_bins;
    const uint32_t Vx = in.voxel_res[0], Vy = in.voxel_res[1], Vz = in.voxel_res[2];
    constexpr int ALIGN = 16 / sizeof(S);
    const double ex = (double)std::min<uint32_t>(kKV, Vx) * std::fabs(in.voxel_size[0]);
    const double ey = (double)std::min<uint32_t>(4 * kWZ, Vz) * std::fabs(in.voxel_size[1]);
    const double ez = (double)std::min<uint32_t>(8 * kWY, Vy) * std::fabs(in.voxel_size[2]);
    WindowPlan wp;
    FBP_TRY(plan_window(ctx, ex, ey, ez, in.time_step, T, ALIGN, sizeof(S), ExhaustiveGatherParams::meta_bytes(32), &wp,
                        "fbp_backproject_exhaustive"));
    const uint32_t slot_w = wp.slot_w, pitch = wp.pitch;
    const uint64_t npairs = (uint64_t)L * Sn;

    void* rows = nullptr;
    FBP_TRY(workspace(ctx, WS_CUBE_ROWS, npairs * pitch * sizeof(S), stream, &rows));
    {
        const uint64_t n = npairs * pitch;
        const unsigned blocks = (unsigned)std::min<uint64_t>(cdiv(n, 256), (uint64_t)ctx->sm_count * 16);
        pair_rows_kernel<S><<<blocks, 256, 0, stream>>>(static_cast<S*>(rows), static_cast<const S*>(cube), npairs, T,
                                                        pitch);
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
    p.rows = rows;
    p.Vx = Vx; p.Vy = Vy; p.Vz = Vz; p.L = L; p.S = Sn; p.T = T;
    p.t0 = in.time_offset;
    p.dt = in.time_step;
    p.row_pitch = pitch;
    p.slot_w = slot_w;
    p.ch = wp.ch;
    const size_t smem = wp.smem;
    dim3 grid(cdiv(Vx, kKV), cdiv(Vy, 8 * kWY), cdiv(Vz, 4 * kWZ));
    const bool bounce = in.discard_first_last_bounces == 0;
    const bool exact = in.time_offset > 0.f;
    auto go = [&](auto kernel) -> fbp_status {
        FBP_TRY_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        kernel<<<grid, 32 * kWY * kWZ, smem, stream>>>(p);
        FBP_CHECK_LAUNCH(ctx, "exhaustive_gather_kernel");
        return FBP_OK;
    };
    if (L % 4 == 0 && wp.ch % 4 == 0) {
        if (bounce) {
            if (exact) return go(exhaustive_gather_kernel<S, kKV, kWY, kWZ, true, true, 4>);
            return go(exhaustive_gather_kernel<S, kKV, kWY, kWZ, true, false, 4>);
        }
        if (exact) return go(exhaustive_gather_kernel<S, kKV, kWY, kWZ, false, true, 4>);
        return go(exhaustive_gather_kernel<S, kKV, kWY, kWZ, false, false, 4>);
    }
    if (bounce) {
        if (exact) return go(exhaustive_gather_kernel<S, kKV, kWY, kWZ, true, true, 1>);
        return go(exhaustive_gather_kernel<S, kKV, kWY, kWZ, true, false, 1>);
    }
    if (exact) return go(exhaustive_gather_kernel<S, kKV, kWY, kWZ, false, true, 1>);
    return go(exhaustive_gather_kernel<S, kKV, kWY, kWZ, false, false, 1>);
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
