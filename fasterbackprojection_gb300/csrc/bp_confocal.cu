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

// The main kernel.  Template parameters:
//   S        storage type of the rows (float, bf16, half)
//   KV       voxels per thread, consecutive along x (they share dy, dz)
//   WY, WZ   warps per CTA along the tile's y (voxel rows) and z (depth) axes;
//            a warp covers 8 rows x 4 depth slices
//   CH       scan points staged per pipeline stage
//   BOUNCE   add the per-scan-point bounce term
//   EXACT_TRUNC  bin = int(x) with a conversion (needed when time_offset > 0
//            makes negative paths possible); otherwise the truncation uses a
//            round-toward-zero add, valid because every path is >= 0.
template <typename S, int KV, int WY, int WZ, bool BOUNCE, bool EXACT_TRUNC>
__global__ void __launch_bounds__(32 * WY * WZ)
confocal_gather_kernel(ConfocalGatherParams p) {
    constexpr int NT = 32 * WY * WZ;
    constexpr int CHMAX = 32;  // scan points (pairs) per stage, upper bound
    const int CH = p.ch;
    constexpr int ALIGN = 16 / sizeof(S);  // elements per 16-byte copy
    constexpr int TY = 8 * WY, TZ = 4 * WZ;

    extern __shared__ __align__(16) unsigned char smem_raw[];
    const uint32_t slot_stride = p.slot_w + ALIGN;  // zero element(s) at slot_w
    float4* s_geo = reinterpret_cast<float4*>(smem_raw);                  // [2][CHMAX]
    float* s_cl = reinterpret_cast<float*>(s_geo + 2 * CHMAX);           // [2][CHMAX]
    int* s_cnt = reinterpret_cast<int*>(s_cl + 2 * CHMAX);               // [2][CHMAX]
    int* s_src = s_cnt + 2 * CHMAX;                                      // [2][CHMAX]
    int* s_flag = s_src + 2 * CHMAX;                                     // [2]
    S* s_slots = reinterpret_cast<S*>(smem_raw + ConfocalGatherParams::meta_bytes(CHMAX));  // [2][CH][slot_stride]

    const int tid = threadIdx.x;
    const int lane = tid & 31, warp = tid >> 5;
    const int wy = warp % WY, wz = warp / WY;

    // Tile origin.
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

    // Zero the sentinel element(s) of every slot once.
    for (int i = tid; i < 2 * CH * ALIGN; i += NT) {
        const int slot = i / ALIGN, e = i % ALIGN;
        s_slots[(size_t)slot * slot_stride + p.slot_w + e] = from_f32<S>(0.f);
    }

    const uint32_t nchunks = (p.L + CH - 1) / CH;

    // Stage-1 of a chunk: window bounds for each scan point (threads < CH).
    auto plan_chunk = [&](uint32_t c, int buf) {
        if (tid < CH) {
            const uint32_t l = c * CH + tid;
            float4 g = make_float4(0.f, 0.f, 0.f, 0.f);
            float cl = 0.f;  // x + 0 < 2^23 -> always the zero sentinel
            int cnt = 0, src = 0, near = 0;
            if (l < p.L) {
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
                // Paths this close make dist^2 <= EPS possible: use safeRCP's branch.
                near = pmin < 0.0035f;
                const float xlo = pmin * rcp_dt, xhi = pmax * rcp_dt;
                // Conservative bin range with a 2-bin margin for rounding.
                int blo = (int)fmaxf(fminf(floorf(xlo), 1.0e9f), -1.0e9f) - 2;
                int bhi = (int)fmaxf(fminf(floorf(xhi), 1.0e9f), -1.0e9f) + 2;
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
            s_geo[buf * CHMAX + tid] = g;
            s_cl[buf * CHMAX + tid] = cl;
            s_cnt[buf * CHMAX + tid] = cnt;
            s_src[buf * CHMAX + tid] = src;
            // Warp 0 holds every planning thread (CH <= 32): vote the flag.
            const unsigned any_near = __ballot_sync(CH >= 32 ? 0xffffffffu : ((1u << CH) - 1u), near);
            if (tid == 0) s_flag[buf] = any_near != 0;
        }
    };

    // Stage-2 of a chunk: issue the window copies (all threads).
    auto copy_chunk = [&](uint32_t c, int buf) {
        const uint32_t vecs_per_slot = p.slot_w / ALIGN;
        for (uint32_t i = tid; i < CH * vecs_per_slot; i += NT) {
            const uint32_t s = i / vecs_per_slot, j = i - s * vecs_per_slot;
            if ((int)(j * ALIGN) < s_cnt[buf * CHMAX + s]) {
                const uint32_t l = c * CH + s;
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
        copy_chunk(0, 0);
    }

    for (uint32_t c = 0; c < nchunks; ++c) {
        const int buf = c & 1;
        __syncthreads();  // every thread is done with chunk c-1, whose buffer plan(c+1) reuses
        if (c + 1 < nchunks) plan_chunk(c + 1, buf ^ 1);
        __syncthreads();  // plan(c+1) visible to the copy loop
        if (c + 1 < nchunks) {
            copy_chunk(c + 1, buf ^ 1);
            cp_async_wait<1>();
        } else {
            cp_async_wait<0>();
        }
        __syncthreads();  // chunk c's windows visible

        const float4* geo = s_geo + buf * CHMAX;
        const float* clv = s_cl + buf * CHMAX;
        const S* slots = s_slots + (size_t)buf * CH * slot_stride;
        const bool safe = s_flag[buf] != 0;
        const int nl = (int)min((uint32_t)CH, p.L - c * CH);

        if (!safe) {
            confocal_chunk<S, KV, BOUNCE, EXACT_TRUNC, false>(geo, clv, slots, slot_stride, p.slot_w, nl, px, py, pz,
                                                              neg_t0, rcp_dt, acc);
        } else {
            confocal_chunk<S, KV, BOUNCE, EXACT_TRUNC, true>(geo, clv, slots, slot_stride, p.slot_w, nl, px, py, pz,
                                                             neg_t0, rcp_dt, acc);
        }

        // Compensated (Kahan) fold of this chunk's partial sums.
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

template <typename S>
fbp_status launch_confocal(fbp_context* ctx, const fbp_recon_info& in, const void* cube, int layout,
                           const float* laser_xyz, float* volume, cudaStream_t stream) {
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
    const uint32_t slot_w = wp.slot_w, pitch = wp.pitch;

    S* rows = nullptr;
    FBP_TRY(prepare_rows<S>(ctx, cube, layout, L, T, pitch, stream, &rows));

    ConfocalGatherParams p{};
    FBP_TRY(build_tables(ctx, in, laser_xyz, stream, &p.scan, &p.xs, &p.ys, &p.zs));
    p.rows = rows;
    p.volume = volume;
    p.status = ctx->status_dev;
    p.Vx = Vx; p.Vy = Vy; p.Vz = Vz; p.L = L; p.T = T;
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
        FBP_CHECK_LAUNCH(ctx, "confocal_gather_kernel");
        return FBP_OK;
    };
    if (bounce) {
        if (exact) return go(confocal_gather_kernel<S, kKV, kWY, kWZ, true, true>);
        return go(confocal_gather_kernel<S, kKV, kWY, kWZ, true, false>);
    }
    if (exact) return go(confocal_gather_kernel<S, kKV, kWY, kWZ, false, true>);
    return go(confocal_gather_kernel<S, kKV, kWY, kWZ, false, false>);
}

}  // namespace

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
    out->pitch = t_round + slot_w;
    const size_t per_stage = (size_t)2 * (slot_w + align) * elem_bytes;  // double-buffered, per scan point
    int ch = 32;
    while (ch > 1 && meta_bytes + (size_t)ch * per_stage > (size_t)ctx->smem_optin) ch >>= 1;
    if (meta_bytes + (size_t)ch * per_stage > (size_t)ctx->smem_optin)
        return set_error(FBP_ERR_UNSUPPORTED, std::string(who) + ": time-bin window too large for shared memory");
    out->ch = ch;
    out->smem = meta_bytes + (size_t)ch * per_stage;
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
    cudaStream_t s = (cudaStream_t)stream;
    switch (dtype) {
        case FBP_F32: return launch_confocal<float>(ctx, *info, cube, layout, laser_xyz, volume, s);
        case FBP_BF16: return launch_confocal<__nv_bfloat16>(ctx, *info, cube, layout, laser_xyz, volume, s);
        case FBP_F16: return launch_confocal<__half>(ctx, *info, cube, layout, laser_xyz, volume, s);
        default: return set_error(FBP_ERR_INVALID_ARG, "fbp_backproject_confocal: unknown dtype");
    }
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
