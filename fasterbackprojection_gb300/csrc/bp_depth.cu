// Depth-plane backprojection (the reference's non-AABB mode).
//
// Replaces Laser::reconstructDepthConfocal / reconstructDepthExhaustive
// (Laser.cu:379-480) and backprojectConfocal / backprojectExhaustive
// (transient_reconstruction.cuh:41-91).  Test points are
//   laser_xyz[c] + wall_normal * float(depths[d])
// and contributions are unweighted.  One thread owns one test point and sums
// over every scan point (or laser/SPAD pair) from the padded rows in a fixed
// order (FP32 per block of 64, Kahan across blocks), instead of one atomic per
// pair.  Time bins follow the reference's FP32 expression exactly.
#include "fbp_internal.cuh"
#include "bp_common.cuh"

#include <algorithm>

namespace fbp {

template <typename S>
__global__ void depth_confocal_kernel(const S* __restrict__ rows, uint32_t pitch, const float4* __restrict__ scan,
                                      const float* __restrict__ laser_xyz, const double* __restrict__ depths,
                                      uint32_t L, uint32_t D, uint32_t T, float nx, float ny, float nz, float t0,
                                      float dt, int bounce, float* __restrict__ act) {
    const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i >= (uint64_t)L * D) return;
    const uint32_t c = (uint32_t)(i / D), d = (uint32_t)(i % D);
    const float df = (float)depths[d];
    // transient_reconstruction.cuh:51
    const float px = fma_rn(nx, df, laser_xyz[3 * (size_t)c]);
    const float py = fma_rn(ny, df, laser_xyz[3 * (size_t)c + 1]);
    const float pz = fma_rn(nz, df, laser_xyz[3 * (size_t)c + 2]);
    const float rcp_dt = rcp_approx(dt);
    float ksum = 0.f, kcomp = 0.f;
    for (uint32_t l0 = 0; l0 < L; l0 += 64) {
        const uint32_t l1 = min(L, l0 + 64);
        float acc = 0.f;
        for (uint32_t l = l0; l < l1; ++l) {
            const float4 g = scan[l];
            const float dist0 = sqrt_approx(ref_dot3(sub_rn(px, g.x), sub_rn(py, g.y), sub_rn(pz, g.z)));
            float dist = fma_rn(dist0, 2.f, -t0);
            if (bounce) dist = add_rn(dist, g.w);
            const int b = __float2int_rz(ref_bin_ratio(dist, rcp_dt));
            if (b < 0 || b >= (int)T) continue;
            acc += to_f32(rows[(size_t)l * pitch + b]);
        }
        const float y = sub_rn(acc, kcomp);
        const float t = add_rn(ksum, y);
        kcomp = sub_rn(sub_rn(t, ksum), y);
        ksum = t;
    }
    act[i] = ksum;
}

template <typename S>
__global__ void depth_exhaustive_kernel(const S* __restrict__ rows, uint32_t pitch, const float4* __restrict__ lscan,
                                        const float4* __restrict__ sscan, const float* __restrict__ laser_xyz,
                                        const double* __restrict__ depths, uint32_t L, uint32_t Sn, uint32_t D,
                                        uint32_t T, float nx, float ny, float nz, float t0, float dt, int bounce,
                                        float* __restrict__ act) {
    const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i >= (uint64_t)L * D) return;
    const uint32_t c = (uint32_t)(i / D), d = (uint32_t)(i % D);
    const float df = (float)depths[d];
    // transient_reconstruction.cuh:78
    const float px = fma_rn(nx, df, laser_xyz[3 * (size_t)c]);
    const float py = fma_rn(ny, df, laser_xyz[3 * (size_t)c + 1]);
    const float pz = fma_rn(nz, df, laser_xyz[3 * (size_t)c + 2]);
    const float rcp_dt = rcp_approx(dt);
    float ksum = 0.f, kcomp = 0.f;
    for (uint32_t l = 0; l < L; ++l) {
        const float4 lg = lscan[l];
        const float dl = sqrt_approx(ref_dot3(sub_rn(px, lg.x), sub_rn(py, lg.y), sub_rn(pz, lg.z)));
        for (uint32_t s0 = 0; s0 < Sn; s0 += 64) {
            const uint32_t s1 = min(Sn, s0 + 64);
            float acc = 0.f;
            for (uint32_t s = s0; s < s1; ++s) {
                const float4 sg = sscan[s];
                const float ds = sqrt_approx(ref_dot3(sub_rn(sg.x, px), sub_rn(sg.y, py), sub_rn(sg.z, pz)));
                // transient_reconstruction.cuh:80-82
                float dist = sub_rn(add_rn(dl, ds), t0);
                if (bounce) dist = add_rn(dist, add_rn(lg.w, sg.w));
                const int b = __float2int_rz(ref_bin_ratio(dist, rcp_dt));
                if (b < 0 || b >= (int)T) continue;
                acc += to_f32(rows[((size_t)l * Sn + s) * pitch + b]);
            }
            const float y = sub_rn(acc, kcomp);
            const float t = add_rn(ksum, y);
            kcomp = sub_rn(sub_rn(t, ksum), y);
            ksum = t;
        }
    }
    act[i] = ksum;
}

// Thresholded copy into [R][pitch] rows (time innermost).  Confocal
// time-major cubes are transposed.
template <typename S>
__global__ void depth_rows_kernel(S* __restrict__ rows, const S* __restrict__ cube, uint64_t R, uint32_t T,
                                  uint32_t pitch, int time_major) {
    const uint64_t n = R * pitch;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t r = i / pitch;
        const uint32_t t = (uint32_t)(i % pitch);
        S v = from_f32<S>(0.f);
        if (t < T) {
            const S c = time_major ? cube[(uint64_t)t * R + r] : cube[r * T + t];
            if (to_f32(c) > FBP_EPS) v = c;
        }
        rows[i] = v;
    }
}

template <typename S>
fbp_status launch_depths(fbp_context* ctx, const fbp_recon_info& in, const void* cube, int layout,
                         const float* laser_xyz, const float* sensor_xyz, const double* depths, uint32_t D,
                         float* act, cudaStream_t stream) {
    const bool exhaustive = in.capture_system == FBP_EXHAUSTIVE;
    const uint32_t L = in.num_laser_targets, Sn = exhaustive ? in.num_sensor_targets : 1, T = in.num_time_bins;
    const uint32_t pitch = (T + 7) / 8 * 8;
    const uint64_t R = (uint64_t)L * Sn;
    void* rows = nullptr;
    FBP_TRY(workspace(ctx, WS_CUBE_ROWS, R * pitch * sizeof(S), stream, &rows));
    {
        const uint64_t n = R * pitch;
        const unsigned blocks = (unsigned)std::min<uint64_t>(cdiv(n, 256), (uint64_t)ctx->sm_count * 16);
        depth_rows_kernel<S><<<blocks, 256, 0, stream>>>(static_cast<S*>(rows), static_cast<const S*>(cube), R, T,
                                                         pitch, !exhaustive && layout == FBP_LAYOUT_TIME_MAJOR);
        FBP_CHECK_LAUNCH(ctx, "depth_rows_kernel");
    }
    const int bounce = in.discard_first_last_bounces == 0;
    const uint64_t npts = (uint64_t)L * D;
    if (!exhaustive) {
        void* sp = nullptr;
        FBP_TRY(workspace(ctx, WS_SCAN_TABLE, (size_t)L * sizeof(float4), stream, &sp));
        scan_table_kernel<<<cdiv(L, 256), 256, 0, stream>>>(static_cast<float4*>(sp), laser_xyz, L,
                                                           (int)in.discard_first_last_bounces, in.laser_position[0],
                                                           in.laser_position[1], in.laser_position[2],
                                                           in.sensor_position[0], in.sensor_position[1],
                                                           in.sensor_position[2], 1);
        FBP_CHECK_LAUNCH(ctx, "scan_table_kernel");
        depth_confocal_kernel<S><<<cdiv(npts, 128), 128, 0, stream>>>(
            static_cast<const S*>(rows), pitch, static_cast<const float4*>(sp), laser_xyz, depths, L, D, T,
            in.wall_normal[0], in.wall_normal[1], in.wall_normal[2], in.time_offset, in.time_step, bounce, act);
        FBP_CHECK_LAUNCH(ctx, "depth_confocal_kernel");
        return FBP_OK;
    }
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
    depth_exhaustive_kernel<S><<<cdiv(npts, 128), 128, 0, stream>>>(
        static_cast<const S*>(rows), pitch, static_cast<const float4*>(lp), static_cast<const float4*>(sp), laser_xyz,
        depths, L, Sn, D, T, in.wall_normal[0], in.wall_normal[1], in.wall_normal[2], in.time_offset, in.time_step,
        bounce, act);
    FBP_CHECK_LAUNCH(ctx, "depth_exhaustive_kernel");
    return FBP_OK;
}

}  // namespace fbp

using namespace fbp;

extern "C" fbp_status fbp_backproject_depths(fbp_context* ctx, const fbp_recon_info* info, const void* cube, int dtype,
                                             int layout, const float* laser_xyz, const float* sensor_xyz,
                                             const double* depths, uint32_t num_depths, float* activation,
                                             void* stream) {
    return guarded("fbp_backproject_depths", [&]() -> fbp_status {
        clear_error();
        FBP_TRY(check_ctx(ctx));
        if (!info) return set_error(FBP_ERR_INVALID_ARG, "fbp_backproject_depths: null info");
        const bool exhaustive = info->capture_system == FBP_EXHAUSTIVE;
        if (info->capture_system != FBP_CONFOCAL && !exhaustive)
            return set_error(FBP_ERR_INVALID_ARG, "fbp_backproject_depths: unknown capture system");
        if (info->num_laser_targets == 0 || info->num_time_bins == 0 || (exhaustive && info->num_sensor_targets == 0))
            return set_error(FBP_ERR_INVALID_ARG, "fbp_backproject_depths: empty capture");
        if (!(info->time_step > 0.f)) return set_error(FBP_ERR_INVALID_ARG, "fbp_backproject_depths: time_step must be > 0");
        if (!cube || !laser_xyz || !depths || !activation || (exhaustive && !sensor_xyz))
            return set_error(FBP_ERR_INVALID_ARG, "fbp_backproject_depths: null buffer");
        if (num_depths == 0) return set_error(FBP_ERR_INVALID_ARG, "fbp_backproject_depths: num_depths == 0");
        if (layout != FBP_LAYOUT_TIME_MAJOR && layout != FBP_LAYOUT_TIME_INNER)
            return set_error(FBP_ERR_INVALID_ARG, "fbp_backproject_depths: unknown layout");
        cudaStream_t s = (cudaStream_t)stream;
        switch (dtype) {
            case FBP_F32:
                return launch_depths<float>(ctx, *info, cube, layout, laser_xyz, sensor_xyz, depths, num_depths, activation, s);
            case FBP_BF16:
                return launch_depths<__nv_bfloat16>(ctx, *info, cube, layout, laser_xyz, sensor_xyz, depths, num_depths,
                                                    activation, s);
            case FBP_F16:
                return launch_depths<__half>(ctx, *info, cube, layout, laser_xyz, sensor_xyz, depths, num_depths, activation, s);
            default: return set_error(FBP_ERR_INVALID_ARG, "fbp_backproject_depths: unknown dtype");
        }
    });
}
