// End-to-end reconstruction from host buffers.
//
// Replaces Laser::reconstructShape in its default AABB mode (Laser.cu:40-67,
// 341-363): filter_H on the capture (reference: on the host copy, with a
// round trip through the device), upload (NLosData::toGpu, NLosData.cpp:131-159),
// backprojection, the configured post-filter, min-max normalisation, and the
// download that saveReconstructedAABB performs (Laser.cu:518-524).  Here the
// filter runs on the device copy and every step stays on one stream.
#include "fbp_internal.cuh"

namespace fbp {
fbp_status normalize_device(fbp_context* ctx, float* v, uint64_t n, cudaStream_t stream);
fbp_status filter_h_device(fbp_context* ctx, float* data, uint64_t nseries, uint32_t T, float delta_t, float wl_mean,
                           float wl_sigma, int border, cudaStream_t stream);

template <typename S>
__global__ void widen_kernel(float* __restrict__ out, const S* __restrict__ in, uint64_t n) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        out[i] = to_f32(in[i]);
}
}  // namespace fbp

using namespace fbp;

extern "C" fbp_status fbp_reconstruct_shape_host(fbp_context* ctx, const fbp_recon_info* info, const void* cube_host,
                                                 int dtype, const float* laser_xyz_host, const float* sensor_xyz_host,
                                                 const fbp_shape_params* params, float* volume_host, void* stream) {
    return guarded("fbp_reconstruct_shape_host", [&]() -> fbp_status {
        clear_error();
        FBP_TRY(check_ctx(ctx));
        if (!info || !cube_host || !laser_xyz_host || !params || !volume_host)
            return set_error(FBP_ERR_INVALID_ARG, "fbp_reconstruct_shape_host: null argument");
        if (dtype != FBP_F32 && dtype != FBP_BF16 && dtype != FBP_F16)
            return set_error(FBP_ERR_INVALID_ARG, "fbp_reconstruct_shape_host: unknown dtype");
        const bool exhaustive = info->capture_system == FBP_EXHAUSTIVE;
        if (exhaustive && !sensor_xyz_host)
            return set_error(FBP_ERR_INVALID_ARG, "fbp_reconstruct_shape_host: exhaustive capture needs sensor positions");
        cudaStream_t s = (cudaStream_t)stream;
        const uint64_t L = info->num_laser_targets, Sn = exhaustive ? info->num_sensor_targets : 1, T = info->num_time_bins;
        const uint64_t nel = L * Sn * T;
        const uint64_t V = (uint64_t)info->voxel_res[0] * info->voxel_res[1] * info->voxel_res[2];
        if (nel == 0 || V == 0) return set_error(FBP_ERR_INVALID_ARG, "fbp_reconstruct_shape_host: empty capture or volume");

        void *dcube = nullptr, *dgeo = nullptr, *dvol = nullptr, *dtmp = nullptr;
        FBP_TRY(workspace(ctx, WS_HOST_STAGING_IN, nel * dtype_size(dtype), s, &dcube));
        FBP_TRY(workspace(ctx, WS_HOST_STAGING_AUX, (size_t)(L + (exhaustive ? Sn : 0)) * 3 * sizeof(float), s, &dgeo));
        FBP_TRY(workspace(ctx, WS_HOST_STAGING_OUT, V * sizeof(float), s, &dvol));
        float* dlaser = static_cast<float*>(dgeo);
        float* dsensor = exhaustive ? dlaser + 3 * L : nullptr;
        FBP_TRY_CUDA(cudaMemcpyAsync(dcube, cube_host, nel * dtype_size(dtype), cudaMemcpyHostToDevice, s));
        FBP_TRY_CUDA(cudaMemcpyAsync(dlaser, laser_xyz_host, L * 3 * sizeof(float), cudaMemcpyHostToDevice, s));
        if (exhaustive)
            FBP_TRY_CUDA(cudaMemcpyAsync(dsensor, sensor_xyz_host, Sn * 3 * sizeof(float), cudaMemcpyHostToDevice, s));

        const void* bp_cube = dcube;
        int bp_dtype = dtype;
        if (params->use_fourier_filter) {
            float* f32 = static_cast<float*>(dcube);
            if (dtype != FBP_F32) {
                // The filter is defined on float data: widen the 16-bit capture first.
                void* w = nullptr;
                FBP_TRY(workspace(ctx, WS_HOST_STAGING_AUX2, nel * sizeof(float), s, &w));
                f32 = static_cast<float*>(w);
                const unsigned blocks = (unsigned)std::min<uint64_t>(cdiv(nel, 256), (uint64_t)ctx->sm_count * 16);
                if (dtype == FBP_BF16)
                    widen_kernel<__nv_bfloat16><<<blocks, 256, 0, s>>>(f32, static_cast<const __nv_bfloat16*>(dcube), nel);
                else
                    widen_kernel<__half><<<blocks, 256, 0, s>>>(f32, static_cast<const __half*>(dcube), nel);
                FBP_CHECK_LAUNCH(ctx, "widen_kernel");
            }
            // Laser.cu:46-47: wl_mean = 10 * deltaT, sigma chosen by filter_H.
            FBP_TRY(filter_h_device(ctx, f32, L * Sn, (uint32_t)T, info->time_step, info->time_step * 10.0f, 0.0f,
                                    FBP_BORDER_ZERO, s));
            bp_cube = f32;
            bp_dtype = FBP_F32;
        }

        float* vol = static_cast<float*>(dvol);
        fbp_status st = exhaustive
                            ? fbp_backproject_exhaustive(ctx, info, bp_cube, bp_dtype, dlaser, dsensor, vol, stream)
                            : fbp_backproject_confocal(ctx, info, bp_cube, bp_dtype, FBP_LAYOUT_TIME_INNER, dlaser, vol, stream);
        if (st != FBP_OK) return st;

        if (params->postfilter != FBP_FILTER_NONE) {
            FBP_TRY(workspace(ctx, WS_FILTER, V * sizeof(float), s, &dtmp));
            st = fbp_postfilter(ctx, params->postfilter, params->kernel_size, params->sigma, vol, static_cast<float*>(dtmp),
                                info->voxel_res[0], info->voxel_res[1], info->voxel_res[2], stream);
            if (st != FBP_OK) return st;
            vol = static_cast<float*>(dtmp);
        }
        if (params->normalize) FBP_TRY(normalize_device(ctx, vol, V, s));
        FBP_TRY_CUDA(cudaMemcpyAsync(volume_host, vol, V * sizeof(float), cudaMemcpyDeviceToHost, s));
        FBP_TRY_CUDA(cudaStreamSynchronize(s));
        return fbp_check_device_status(ctx, stream);
    });
}
