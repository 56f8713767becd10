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
//   rows   [L][row_pitch] FP32: one padded row per scan point, time
//          innermost, values <= 1e-5 already replaced by 0 (the reference
//          skips them), zeros in [T, row_pitch).  BF16 / FP16 captures are
//          widened here (exactly), so the pair loop reads FP32 with no
//          per-pair conversion; the gather is bound by instruction issue, not
//          by the bytes of its windows.
//   scan   [L] float4 (x, y, z, bounce)   bounce = |l-laser|+|l-sensor| or 0
//   axes   xs[Vx], ys[Vz], zs[Vy]         voxel-centre coordinates
#include "fbp_internal.cuh"
#include "bp_common.cuh"
#include "bp_gather.cuh"

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

// Rows from a time-innermost cube: copy (widened to FP32), threshold, pad.
template <typename S>
__global__ void rows_from_time_inner_kernel(float* __restrict__ rows, const S* __restrict__ cube, uint32_t L,
                                            uint32_t T, uint32_t pitch) {
    const uint64_t n = (uint64_t)L * pitch;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t l = (uint32_t)(i / pitch), t = (uint32_t)(i % pitch);
        float v = 0.f;
        if (t < T) {
            const float c = to_f32(cube[(uint64_t)l * T + t]);
            if (c > FBP_EPS) v = c;
        }
        rows[i] = v;
    }
}

// Rows from a time-major cube (cube[t*L + l]): tiled transpose through shared
// memory so both the read and the write are coalesced.
template <typename S>
__global__ void rows_from_time_major_kernel(float* __restrict__ rows, const S* __restrict__ cube, uint32_t L,
                                            uint32_t T, uint32_t pitch) {
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
        if (l < L && t < pitch) rows[(uint64_t)l * pitch + t] = tile[threadIdx.x][j];
    }
}

// Zero the padding columns [roundup(T,32), pitch) the transpose grid does not cover.
__global__ void rows_zero_tail_kernel(float* __restrict__ rows, uint32_t L, uint32_t from, uint32_t pitch) {
    const uint32_t w = pitch - from;
    const uint64_t n = (uint64_t)L * w;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        rows[(i / w) * pitch + from + (i % w)] = 0.f;
}

// ------------------------------------------------------------ host driver --

template <typename S>
fbp_status prepare_rows_into(fbp_context* ctx, const void* cube, int layout, uint32_t L, uint32_t T, uint32_t pitch,
                             float* r, cudaStream_t stream) {
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
            rows_zero_tail_kernel<<<blocks, 256, 0, stream>>>(r, L, tcover, pitch);
            FBP_CHECK_LAUNCH(ctx, "rows_zero_tail_kernel");
        }
    }
    return FBP_OK;
}
template fbp_status prepare_rows_into<float>(fbp_context*, const void*, int, uint32_t, uint32_t, uint32_t, float*,
                                             cudaStream_t);
template fbp_status prepare_rows_into<__nv_bfloat16>(fbp_context*, const void*, int, uint32_t, uint32_t, uint32_t,
                                                     float*, cudaStream_t);
template fbp_status prepare_rows_into<__half>(fbp_context*, const void*, int, uint32_t, uint32_t, uint32_t, float*,
                                              cudaStream_t);

namespace {

template <typename S>
fbp_status prepare_rows(fbp_context* ctx, const void* cube, int layout, uint32_t L, uint32_t T, uint32_t pitch,
                        cudaStream_t stream, float** rows_out) {
    void* rows = nullptr;
    FBP_TRY(workspace(ctx, WS_CUBE_ROWS, (size_t)L * pitch * sizeof(float), stream, &rows));
    *rows_out = static_cast<float*>(rows);
    return prepare_rows_into<S>(ctx, cube, layout, L, T, pitch, *rows_out, stream);
}

// Voxels per thread along x: 16 for the full gather (the scan point's
// geometry and the stage's bookkeeping amortised over more pairs: 2.67e12 ->
// 2.74e12 pairs/s at 256^3), 8 for the sampled gather (its tiles are the MIS
// sampling tiles) and the voxel-scattering walk.
constexpr int kKV = 8, kKVFull = 16, kWY = 2, kWZ = 4;

template <typename S, int PATH, bool BOUNCE, bool SAMPLED, bool CLAMP, int KV = SAMPLED ? kKV : kKVFull>
fbp_status go_confocal(fbp_context* ctx, const ConfocalGatherParams& p, dim3 grid, size_t smem, cudaStream_t stream) {
    auto kernel = confocal_gather_kernel<S, KV, kWY, kWZ, PATH, BOUNCE, SAMPLED, CLAMP>;
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

// The voxel-scattering walk with unconditional unrolled steps (prefix sp),
// clamped window index only where the window is the whole row.
fbp_status dispatch_scatter_free(fbp_context* ctx, const ConfocalGatherParams& p, dim3 grid, size_t smem,
                                 cudaStream_t stream, int sp, bool bounce, bool capped) {
    constexpr int F = PATH_SCATTER + kScatterForms;
    switch ((sp - 2) + (bounce ? 4 : 0) + (capped ? 8 : 0)) {
        case 0: return go_confocal<float, F, false, false, false, kKV>(ctx, p, grid, smem, stream);
        case 1: return go_confocal<float, F + 1, false, false, false, kKV>(ctx, p, grid, smem, stream);
        case 2: return go_confocal<float, F + 2, false, false, false, kKV>(ctx, p, grid, smem, stream);
        case 4: return go_confocal<float, F, true, false, false, kKV>(ctx, p, grid, smem, stream);
        case 5: return go_confocal<float, F + 1, true, false, false, kKV>(ctx, p, grid, smem, stream);
        case 6: return go_confocal<float, F + 2, true, false, false, kKV>(ctx, p, grid, smem, stream);
        case 8: return go_confocal<float, F, false, false, true, kKV>(ctx, p, grid, smem, stream);
        case 9: return go_confocal<float, F + 1, false, false, true, kKV>(ctx, p, grid, smem, stream);
        case 10: return go_confocal<float, F + 2, false, false, true, kKV>(ctx, p, grid, smem, stream);
        case 12: return go_confocal<float, F, true, false, true, kKV>(ctx, p, grid, smem, stream);
        case 13: return go_confocal<float, F + 1, true, false, true, kKV>(ctx, p, grid, smem, stream);
        case 14: return go_confocal<float, F + 2, true, false, true, kKV>(ctx, p, grid, smem, stream);
        default: return set_error(FBP_ERR_INTERNAL, "voxel scattering: no kernel for this step prefix");
    }
}

// Depth slices [z_begin, z_end) of the volume (the whole volume by default)
// into `volume` ([z_end - z_begin][Vy][Vx]).  The window plan and the voxel
// tables are those of the whole volume, so with z_begin a multiple of the
// tile depth a slab is bitwise the same rows of the full result.
template <typename S>
fbp_status launch_confocal(fbp_context* ctx, const fbp_recon_info& in, const void* cube, int layout,
                           const float* laser_xyz, float* volume, cudaStream_t stream, const SampleParams* smp,
                           uint32_t z_begin = 0, uint32_t z_end = 0xFFFFFFFFu, bool scatter = false) {
    const uint32_t L = in.num_laser_targets, T = in.num_time_bins;
    const uint32_t Vx = in.voxel_res[0], Vy = in.voxel_res[1], Vz = in.voxel_res[2];
    if (z_end > Vz) z_end = Vz;
    if (z_begin >= z_end) return FBP_OK;
    constexpr int ALIGN = 4;  // FP32 rows

    // World extents of the largest tile (clamped to the volume).
    const uint32_t kv = (smp || scatter) ? kKV : kKVFull;
    const double ex = (double)std::min<uint32_t>(kv, Vx) * std::fabs(in.voxel_size[0]);
    const double ey = (double)std::min<uint32_t>(4 * kWZ, Vz) * std::fabs(in.voxel_size[1]);
    const double ez = (double)std::min<uint32_t>(8 * kWY, Vy) * std::fabs(in.voxel_size[2]);
    WindowPlan wp;
    // The sampled kernel also holds its cluster list in static shared memory.
    // The voxel-scattering variant reads every bin of dist -/+ half the voxel
    // diagonal, one step past the end (up to max(step, diagonal) from 0 where
    // a walk is clipped at 0).
    const double vdiag = std::sqrt((double)in.voxel_size[0] * in.voxel_size[0] +
                                   (double)in.voxel_size[1] * in.voxel_size[1] +
                                   (double)in.voxel_size[2] * in.voxel_size[2]);
    const double extra = scatter ? 1.52 * vdiag + 2.0 * std::fabs((double)in.time_step) : 0.0;
    FBP_TRY(plan_window(ctx, ex, ey, ez, in.time_step, T, ALIGN, sizeof(float),
                        ConfocalGatherParams::meta_bytes(32) + (smp ? kSampledStaticSmem : 0) +
                            kahan_smem_bytes((int)kv, 32 * kWY * kWZ) + 16,
                        &wp, "fbp_backproject_confocal", extra));
    if (smp) wp.smem -= kSampledStaticSmem;

    float* rows = nullptr;
    FBP_TRY(prepare_rows<S>(ctx, cube, layout, L, T, wp.pitch, stream, &rows));

    ConfocalGatherParams p{};
    FBP_TRY(build_tables(ctx, in, laser_xyz, stream, &p.scan, &p.xs, &p.ys, &p.zs));
    p.rows = rows;
    p.volume = volume;
    p.status = ctx->status_dev;
    p.ys += z_begin;
    p.Vx = Vx; p.Vy = Vy; p.Vz = z_end - z_begin; p.L = L; p.T = T;
    p.t0 = in.time_offset;
    p.dt = in.time_step;
    p.row_pitch = wp.pitch;
    p.slot_w = wp.slot_w;
    p.ch = wp.ch;
    for (int k = 0; k < 3; ++k) p.vs[k] = in.voxel_size[k];
    p.exact_weights = ctx->weight_mode == FBP_WEIGHTS_REFERENCE;
    if (smp) p.smp = *smp;
    dim3 grid(cdiv(Vx, kv), cdiv(Vy, 8 * kWY), cdiv(z_end - z_begin, 4 * kWZ));
    const bool bounce = in.discard_first_last_bounces == 0;
    if (scatter) {
        // Steps per (voxel, scan point): at most ceil(diagonal / (dt + EPS)),
        // one more where rounding lands on the end; the kernel unrolls 2..4
        // of them and loops over the rest.  Where even the shortest walk
        // takes all the unrolled steps (a 1e-4 m margin over the rounding of
        // the path arithmetic below 64 m) they need no end test, and the
        // unclamped window index of the other paths applies.
        const double step = (double)in.time_step + (double)FBP_EPS;
        const double steps = std::ceil(vdiag / step);
        const int sp = (int)std::min(std::max(steps, 2.0), (double)kScatterMaxPrefix);
        const bool free_walk = (sp - 1) * step + 1e-4 < vdiag;
        // ... and where none takes more (sp steps already pass the far end).
        p.scat_exact = free_walk && sp * step > vdiag + 1e-4;
        switch ((sp - 2) + (free_walk ? kScatterForms : 0) + (bounce ? 8 : 0)) {
            case 0: return go_confocal<float, PATH_SCATTER, false, false, true, kKV>(ctx, p, grid, wp.smem, stream);
            case 1: return go_confocal<float, PATH_SCATTER + 1, false, false, true, kKV>(ctx, p, grid, wp.smem, stream);
            case 2: return go_confocal<float, PATH_SCATTER + 2, false, false, true, kKV>(ctx, p, grid, wp.smem, stream);
            case 8: return go_confocal<float, PATH_SCATTER, true, false, true, kKV>(ctx, p, grid, wp.smem, stream);
            case 9: return go_confocal<float, PATH_SCATTER + 1, true, false, true, kKV>(ctx, p, grid, wp.smem, stream);
            case 10: return go_confocal<float, PATH_SCATTER + 2, true, false, true, kKV>(ctx, p, grid, wp.smem, stream);
            default: break;
        }
        return dispatch_scatter_free(ctx, p, grid, wp.smem, stream, sp, bounce, wp.capped);
    }
    if (smp) return dispatch_confocal<float, true>(ctx, p, grid, wp.smem, stream, bounce, in.time_offset, wp.capped);
    return dispatch_confocal<float, false>(ctx, p, grid, wp.smem, stream, bounce, in.time_offset, wp.capped);
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

fbp_status confocal_gather_scatter(fbp_context* ctx, const fbp_recon_info& in, const void* cube, int dtype,
                                   int layout, const float* laser_xyz, float* volume, cudaStream_t s) {
    const uint32_t all = 0xFFFFFFFFu;
    switch (dtype) {
        case FBP_F32: return launch_confocal<float>(ctx, in, cube, layout, laser_xyz, volume, s, nullptr, 0, all, true);
        case FBP_BF16:
            return launch_confocal<__nv_bfloat16>(ctx, in, cube, layout, laser_xyz, volume, s, nullptr, 0, all, true);
        case FBP_F16: return launch_confocal<__half>(ctx, in, cube, layout, laser_xyz, volume, s, nullptr, 0, all, true);
        default: return set_error(FBP_ERR_INVALID_ARG, "unknown dtype");
    }
}

fbp_status confocal_gather_slab(fbp_context* ctx, const fbp_recon_info& in, const void* cube, int dtype, int layout,
                                const float* laser_xyz, uint32_t z_begin, uint32_t z_end, float* volume,
                                cudaStream_t s) {
    switch (dtype) {
        case FBP_F32: return launch_confocal<float>(ctx, in, cube, layout, laser_xyz, volume, s, nullptr, z_begin, z_end);
        case FBP_BF16:
            return launch_confocal<__nv_bfloat16>(ctx, in, cube, layout, laser_xyz, volume, s, nullptr, z_begin, z_end);
        case FBP_F16: return launch_confocal<__half>(ctx, in, cube, layout, laser_xyz, volume, s, nullptr, z_begin, z_end);
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
                       size_t elem_bytes, size_t meta_bytes, WindowPlan* out, const char* who, double extra_path) {
    const double diag = std::sqrt(ex * ex + ey * ey + ez * ez);
    // Round trip across the tile (plus any extra path range), a 2-bin margin
    // on each side, alignment slack.
    const double span = (2.0 * diag + extra_path) / std::fabs(time_step) + 8.0 + align;
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

extern "C" fbp_status fbp_backproject_confocal_scatter(fbp_context* ctx, const fbp_recon_info* info,
                                                       const void* cube, int dtype, int layout,
                                                       const float* laser_xyz, float* volume, void* stream) {
    return guarded("fbp_backproject_confocal_scatter", [&]() -> fbp_status {
        clear_error();
        FBP_TRY(check_ctx(ctx));
        FBP_TRY(validate_info(info, false, "fbp_backproject_confocal_scatter"));
        if (!cube || !laser_xyz || !volume)
            return set_error(FBP_ERR_INVALID_ARG, "fbp_backproject_confocal_scatter: null buffer");
        if (layout != FBP_LAYOUT_TIME_MAJOR && layout != FBP_LAYOUT_TIME_INNER)
            return set_error(FBP_ERR_INVALID_ARG, "fbp_backproject_confocal_scatter: unknown layout");
        if (!(info->time_step > 1e-4f))
            return set_error(FBP_ERR_UNSUPPORTED, "fbp_backproject_confocal_scatter: time_step must exceed 0.1 mm");
        return confocal_gather_scatter(ctx, *info, cube, dtype, layout, laser_xyz, volume, (cudaStream_t)stream);
    });
}

extern "C" fbp_status fbp_backproject_confocal(fbp_context* ctx, const fbp_recon_info* info, const void* cube,
                                               int dtype, int layout, const float* laser_xyz, float* volume,
                                               void* stream) {
    return guarded("fbp_backproject_confocal", [&]() -> fbp_status {
        clear_error();
        FBP_TRY(check_ctx(ctx));
        FBP_TRY(validate_info(info, false, "fbp_backproject_confocal"));
        if (!cube || !laser_xyz || !volume) return set_error(FBP_ERR_INVALID_ARG, "fbp_backproject_confocal: null buffer");
        if (layout != FBP_LAYOUT_TIME_MAJOR && layout != FBP_LAYOUT_TIME_INNER)
            return set_error(FBP_ERR_INVALID_ARG, "fbp_backproject_confocal: unknown layout");
        if (dtype != FBP_F32 && dtype != FBP_BF16 && dtype != FBP_F16)
            return set_error(FBP_ERR_INVALID_ARG, "fbp_backproject_confocal: unknown dtype");
        return confocal_gather(ctx, *info, cube, dtype, layout, laser_xyz, volume, (cudaStream_t)stream, nullptr);
    });
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

// The path (dist) of each pair in the gathers' FP32 expression, and the two
// per-call constants of the scattering walk: rcp.approx(timeStep) and half the
// voxel diagonal.
__global__ void debug_confocal_paths_kernel(fbp_recon_info in, const float4* __restrict__ scan,
                                            const int64_t* __restrict__ vidx, uint64_t nv, float* __restrict__ paths,
                                            float* __restrict__ consts) {
    const uint64_t L = in.num_laser_targets;
    const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i == 0 && consts) {
        consts[0] = rcp_approx(in.time_step);
        consts[1] = mul_rn(0.5f, sqrt_approx(ref_dot3(in.voxel_size[0], in.voxel_size[1], in.voxel_size[2])));
    }
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
    paths[i] = dist;
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
    return guarded("fbp_debug_confocal_bins", [&]() -> fbp_status {
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
    });
}

extern "C" fbp_status fbp_debug_confocal_paths(fbp_context* ctx, const fbp_recon_info* info, const float* laser_xyz,
                                               const int64_t* voxel_idx, uint64_t num_voxels, float* paths,
                                               float* consts, void* stream) {
    return guarded("fbp_debug_confocal_paths", [&]() -> fbp_status {
        clear_error();
        FBP_TRY(check_ctx(ctx));
        FBP_TRY(validate_info(info, false, "fbp_debug_confocal_paths"));
        if (!laser_xyz || !voxel_idx || !paths || !consts)
            return set_error(FBP_ERR_INVALID_ARG, "fbp_debug_confocal_paths: null buffer");
        cudaStream_t s = (cudaStream_t)stream;
        const float4* scan;
        const float *xs, *ys, *zs;
        FBP_TRY(build_tables(ctx, *info, laser_xyz, s, &scan, &xs, &ys, &zs));
        const uint64_t n = std::max<uint64_t>(num_voxels * info->num_laser_targets, 1);
        debug_confocal_paths_kernel<<<cdiv(n, 256), 256, 0, s>>>(*info, scan, voxel_idx, num_voxels, paths, consts);
        FBP_CHECK_LAUNCH(ctx, "debug_confocal_paths_kernel");
        return FBP_OK;
    });
}

extern "C" fbp_status fbp_debug_exhaustive_bins(fbp_context* ctx, const fbp_recon_info* info, const float* laser_xyz,
                                                const float* sensor_xyz, const int64_t* voxel_idx, uint64_t num_voxels,
                                                int32_t* bins, void* stream) {
    return guarded("fbp_debug_exhaustive_bins", [&]() -> fbp_status {
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
    });
}
