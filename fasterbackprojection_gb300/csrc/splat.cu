// Scatter-form backprojection: the rasterised ellipsoid splat of the
// reference's OpenGL path (DrawEllipsoids.cpp:12-114, 332-440, shaders
// backprojection-vs/fs.glsl), as CUDA kernels.
//
// The reference draws, for every scan point l and bin t < 700 with intensity
// above FLT_EPSILON, a half ellipsoid (sphere) centred on the scan point with
// radius half the bin's path length, t * deltaT + t0 minus the first and last
// bounces (DrawEllipsoids.cpp:39-49), rasterised under an orthographic
// projection of the hidden volume; every fragment adds the intensity into the
// voxel it falls in with imageAtomicAdd (backprojection-fs.glsl:17-23).
//
// Here the projection is onto the relay wall's plane (x, z) with an explicit
// grid of grid_w x grid_h pixel centres over the volume's x/z extent (the
// reference inherits its viewport from the window); the surface is the exact
// hemisphere towards the hidden side (-y) rather than a 100 x 100
// tessellation.  A pixel (px, pz) inside the disk of an instance contributes
// at y = c.y - sqrt(r^2 - (px - c.x)^2 - (pz - c.z)^2).  Voxel indices are
// computed in FP32 with IEEE operations (same results as the NumPy oracle);
// sums are FP32 atomics like the reference's.  The first and last bounces are
// subtracted only when discard_first_last_bounces == 0, the convention of the
// backprojection kernels.
#include "fbp_internal.cuh"
#include "bp_common.cuh"

#include <algorithm>

namespace fbp {
namespace {

struct SplatInstance {
    float cx, cy, cz, r;
    float intensity;
};

// Instances of every (scan point, bin < nbins) with intensity > FLT_EPSILON.
template <typename S>
__global__ void splat_instances_kernel(const S* __restrict__ cube, int time_major, uint32_t L, uint32_t T,
                                       uint32_t nbins, const float4* __restrict__ scan, float dt, float t0,
                                       int bounce, SplatInstance* __restrict__ out, unsigned int* __restrict__ count,
                                       uint32_t cap) {
    const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i >= (uint64_t)L * nbins) return;
    const uint32_t l = (uint32_t)(i / nbins), t = (uint32_t)(i % nbins);
    const float v = to_f32(time_major ? cube[(uint64_t)t * L + l] : cube[(uint64_t)l * T + t]);
    if (!(v > 1.1920929e-7f)) return;
    const float4 g = scan[l];
    float path = __fadd_rn(__fmul_rn((float)t, dt), t0);
    if (bounce) path = __fsub_rn(path, g.w);
    const float r = __fmul_rn(0.5f, path);
    if (!(r > 0.f)) return;
    const unsigned int k = atomicAdd(count, 1u);
    if (k < cap) out[k] = SplatInstance{g.x, g.y, g.z, r, v};
}

struct SplatGrid {
    float x0, z0, px, pz;       // first pixel centre, pixel pitch
    uint32_t w, h;
    float hx, hy, hz;           // hidden volume minimum
    float vsx, vsy, vsz;        // voxel size
    uint32_t Vx, Vy, Vz;
};

// Pixel-centre coordinates and voxel indices of the grid's columns (x) and
// rows (z), computed once per call with the per-pixel expressions: x = x0 +
// ix * px, vx = (uint)((x - hx) / vsx), or -1 outside the volume.
__global__ void splat_axes_kernel(SplatGrid gd, float* __restrict__ xs, int* __restrict__ vxs, float* __restrict__ zs,
                                  int* __restrict__ vys) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < gd.w) {
        const float x = __fadd_rn(gd.x0, __fmul_rn((float)i, gd.px));
        const float fx = __fdiv_rn(__fsub_rn(x, gd.hx), gd.vsx);
        xs[i] = x;
        vxs[i] = (fx >= 0.f && (uint32_t)fx < gd.Vx) ? (int)(uint32_t)fx : -1;
    }
    if (i < gd.h) {
        const float z = __fadd_rn(gd.z0, __fmul_rn((float)i, gd.pz));
        const float fz = __fdiv_rn(__fsub_rn(z, gd.hz), gd.vsz);
        zs[i] = z;
        vys[i] = (fz >= 0.f && (uint32_t)fz < gd.Vy) ? (int)(uint32_t)fz : -1;  // volume vy <- world z
    }
}

// One CTA per instance: 32 x 8 threads walk the rows and columns of the
// disk's bounding box.
__global__ void __launch_bounds__(256) splat_kernel(const SplatInstance* __restrict__ inst,
                                                    const unsigned int* __restrict__ count, uint32_t cap,
                                                    SplatGrid gd, const float* __restrict__ xs,
                                                    const int* __restrict__ vxs, const float* __restrict__ zs,
                                                    const int* __restrict__ vys, float* __restrict__ vol) {
    const uint32_t n = min(*count, cap);
    for (uint32_t k = blockIdx.x; k < n; k += gridDim.x) {
        const SplatInstance s = inst[k];
        // Pixel ranges covering [c - r, c + r], one pixel of slack on each side
        // (the disk test below decides).
        const float fx0 = floorf(__fdiv_rn(__fsub_rn(__fsub_rn(s.cx, s.r), gd.x0), gd.px)) - 1.f;
        const float fx1 = ceilf(__fdiv_rn(__fsub_rn(__fadd_rn(s.cx, s.r), gd.x0), gd.px)) + 1.f;
        const float fz0 = floorf(__fdiv_rn(__fsub_rn(__fsub_rn(s.cz, s.r), gd.z0), gd.pz)) - 1.f;
        const float fz1 = ceilf(__fdiv_rn(__fsub_rn(__fadd_rn(s.cz, s.r), gd.z0), gd.pz)) + 1.f;
        const int ix0 = (int)fmaxf(fx0, 0.f), ix1 = (int)fminf(fx1, (float)gd.w - 1.f);
        const int iz0 = (int)fmaxf(fz0, 0.f), iz1 = (int)fminf(fz1, (float)gd.h - 1.f);
        if (ix1 < ix0 || iz1 < iz0) continue;
        const float r2 = __fmul_rn(s.r, s.r);
        for (int iz = iz0 + (int)threadIdx.y; iz <= iz1; iz += 8) {
            const int vy = vys[iz];
            if (vy < 0) continue;
            const float dz = __fsub_rn(zs[iz], s.cz);
            const float dz2 = __fmul_rn(dz, dz);
            float* col = vol + (uint64_t)vy * gd.Vx;
            for (int ix = ix0 + (int)threadIdx.x; ix <= ix1; ix += 32) {
                const float dx = __fsub_rn(xs[ix], s.cx);
                const float h2 = __fsub_rn(__fsub_rn(r2, __fmul_rn(dx, dx)), dz2);
                const int vx = vxs[ix];
                if (h2 < 0.f || vx < 0) continue;
                const float y = __fsub_rn(s.cy, __fsqrt_rn(h2));
                const float fy = __fdiv_rn(__fsub_rn(y, gd.hy), gd.vsy);
                if (!(fy >= 0.f)) continue;
                const uint32_t vz = (uint32_t)fy;  // volume vz <- world y
                if (vz >= gd.Vz) continue;
                atomicAdd(col + (uint64_t)vz * gd.Vy * gd.Vx + vx, s.intensity);
            }
        }
    }
}

template <typename S>
fbp_status splat_typed(fbp_context* ctx, const fbp_recon_info& in, const void* cube, int layout,
                       const float* laser_xyz, uint32_t nbins, uint32_t grid_w, uint32_t grid_h, float* volume,
                       cudaStream_t s) {
    const uint32_t L = in.num_laser_targets, T = in.num_time_bins;
    const float4* scan;
    const float *xs, *ys, *zs;
    FBP_TRY(build_tables(ctx, in, laser_xyz, s, &scan, &xs, &ys, &zs));
    const uint64_t cap64 = (uint64_t)L * nbins;
    if (cap64 > 0x7FFFFFFFull) return set_error(FBP_ERR_UNSUPPORTED, "fbp_splat_backproject: too many (scan point, bin) pairs");
    const uint32_t cap = (uint32_t)cap64;
    // Workspace: count, the axis tables (x, vx per column; z, vy per row), the instances.
    const size_t axes = ((size_t)2 * (grid_w + grid_h) * 4 + 255) & ~size_t(255);
    void* ws = nullptr;
    FBP_TRY(workspace(ctx, WS_MISC, 256 + axes + (size_t)cap * sizeof(SplatInstance), s, &ws));
    unsigned int* count = static_cast<unsigned int*>(ws);
    float* ax_x = reinterpret_cast<float*>(static_cast<char*>(ws) + 256);
    int* ax_vx = reinterpret_cast<int*>(ax_x + grid_w);
    float* ax_z = reinterpret_cast<float*>(ax_vx + grid_w);
    int* ax_vy = reinterpret_cast<int*>(ax_z + grid_h);
    SplatInstance* inst = reinterpret_cast<SplatInstance*>(static_cast<char*>(ws) + 256 + axes);
    const uint64_t V = (uint64_t)in.voxel_res[0] * in.voxel_res[1] * in.voxel_res[2];
    FBP_TRY_CUDA(cudaMemsetAsync(count, 0, sizeof(unsigned int), s));
    FBP_TRY_CUDA(cudaMemsetAsync(volume, 0, V * sizeof(float), s));
    splat_instances_kernel<S><<<cdiv(cap64, 256), 256, 0, s>>>(
        static_cast<const S*>(cube), layout == FBP_LAYOUT_TIME_MAJOR, L, T, nbins, scan, in.time_step,
        in.time_offset, in.discard_first_last_bounces == 0, inst, count, cap);
    FBP_CHECK_LAUNCH(ctx, "splat_instances_kernel");
    SplatGrid gd{};
    const float wx = in.voxel_size[0] * (float)in.voxel_res[0], wz = in.voxel_size[2] * (float)in.voxel_res[1];
    gd.px = wx / (float)grid_w;
    gd.pz = wz / (float)grid_h;
    gd.x0 = in.hidden_min[0] + 0.5f * gd.px;
    gd.z0 = in.hidden_min[2] + 0.5f * gd.pz;
    gd.w = grid_w;
    gd.h = grid_h;
    gd.hx = in.hidden_min[0];
    gd.hy = in.hidden_min[1];
    gd.hz = in.hidden_min[2];
    gd.vsx = in.voxel_size[0];
    gd.vsy = in.voxel_size[1];
    gd.vsz = in.voxel_size[2];
    gd.Vx = in.voxel_res[0];
    gd.Vy = in.voxel_res[1];
    gd.Vz = in.voxel_res[2];
    splat_axes_kernel<<<cdiv(std::max(grid_w, grid_h), 256), 256, 0, s>>>(gd, ax_x, ax_vx, ax_z, ax_vy);
    FBP_CHECK_LAUNCH(ctx, "splat_axes_kernel");
    const unsigned blocks = (unsigned)std::min<uint64_t>(cap, (uint64_t)ctx->sm_count * 64);
    splat_kernel<<<std::max(1u, blocks), dim3(32, 8), 0, s>>>(inst, count, cap, gd, ax_x, ax_vx, ax_z, ax_vy, volume);
    FBP_CHECK_LAUNCH(ctx, "splat_kernel");
    return FBP_OK;
}

}  // namespace
}  // namespace fbp

using namespace fbp;

extern "C" fbp_status fbp_splat_backproject(fbp_context* ctx, const fbp_recon_info* info, const void* cube, int dtype,
                                            int layout, const float* laser_xyz, uint32_t max_bins, uint32_t grid_w,
                                            uint32_t grid_h, float* volume, void* stream) {
    return guarded("fbp_splat_backproject", [&]() -> fbp_status {
        clear_error();
        FBP_TRY(check_ctx(ctx));
        FBP_TRY(validate_info(info, false, "fbp_splat_backproject"));
        if (!cube || !laser_xyz || !volume) return set_error(FBP_ERR_INVALID_ARG, "fbp_splat_backproject: null buffer");
        if (layout != FBP_LAYOUT_TIME_MAJOR && layout != FBP_LAYOUT_TIME_INNER)
            return set_error(FBP_ERR_INVALID_ARG, "fbp_splat_backproject: unknown layout");
        if (grid_w == 0 || grid_h == 0 || grid_w > 65536 || grid_h > 65536)
            return set_error(FBP_ERR_INVALID_ARG, "fbp_splat_backproject: grid sides must be in 1..65536");
        const uint32_t nbins = std::min(info->num_time_bins, max_bins ? max_bins : info->num_time_bins);
        cudaStream_t s = (cudaStream_t)stream;
        switch (dtype) {
            case FBP_F32: return splat_typed<float>(ctx, *info, cube, layout, laser_xyz, nbins, grid_w, grid_h, volume, s);
            case FBP_BF16:
                return splat_typed<__nv_bfloat16>(ctx, *info, cube, layout, laser_xyz, nbins, grid_w, grid_h, volume, s);
            case FBP_F16: return splat_typed<__half>(ctx, *info, cube, layout, laser_xyz, nbins, grid_w, grid_h, volume, s);
            default: return set_error(FBP_ERR_INVALID_ARG, "fbp_splat_backproject: unknown dtype");
        }
    });
}
