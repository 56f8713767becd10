// Depth-slab partition of a confocal reconstruction across ranks.
//
// Voxels are independent, so N GPUs can each reconstruct a contiguous range
// of depth slices of the same capture with no collective on the data path
// (the slabs are gathered afterwards).  A rank needs only the time bins its
// slab can reach: fbp_slab_bin_window bounds them, so a rank copies that bin
// range of the capture to its GPU (the rest of its cube stays zero and is
// never read).  The reference has no multi-GPU path.
#include "fbp_internal.cuh"
#include "bp_common.cuh"

#include <algorithm>
#include <cmath>

namespace fbp {
namespace {

constexpr uint32_t kSlabAlign = 16;  // the gather's tile depth

// Distance from p to the nearest and farthest points of the box [lo, hi].
void box_dist(const double p[3], const double lo[3], const double hi[3], double* dmin, double* dmax) {
    double n2 = 0.0, f2 = 0.0;
    for (int k = 0; k < 3; ++k) {
        const double c = std::min(std::max(p[k], lo[k]), hi[k]);
        n2 += (p[k] - c) * (p[k] - c);
        const double f = std::max(std::fabs(p[k] - lo[k]), std::fabs(p[k] - hi[k]));
        f2 += f * f;
    }
    *dmin = std::sqrt(n2);
    *dmax = std::sqrt(f2);
}

}  // namespace
}  // namespace fbp

using namespace fbp;

extern "C" fbp_status fbp_plan_slabs(const fbp_recon_info* info, uint32_t nranks, uint32_t* z_bounds) {
    return guarded("fbp_plan_slabs", [&]() -> fbp_status {
        clear_error();
        if (!info || !z_bounds || nranks == 0) return set_error(FBP_ERR_INVALID_ARG, "fbp_plan_slabs: bad arguments");
        const uint32_t Vz = info->voxel_res[2];
        const uint32_t tiles = (Vz + kSlabAlign - 1) / kSlabAlign;
        // Balanced by tile rows; ranks past the last tile row get empty slabs.
        for (uint32_t r = 0; r <= nranks; ++r) {
            const uint64_t t = ((uint64_t)tiles * r) / nranks;
            z_bounds[r] = (uint32_t)std::min<uint64_t>(t * kSlabAlign, Vz);
        }
        return FBP_OK;
    });
}

extern "C" fbp_status fbp_slab_bin_window(const fbp_recon_info* info, const float* laser_xyz, uint32_t z_begin,
                                          uint32_t z_end, uint32_t* bin_lo, uint32_t* bin_hi) {
    return guarded("fbp_slab_bin_window", [&]() -> fbp_status {
        clear_error();
        if (!info || !laser_xyz || !bin_lo || !bin_hi) return set_error(FBP_ERR_INVALID_ARG, "fbp_slab_bin_window: null argument");
        const fbp_recon_info& in = *info;
        if (z_end > in.voxel_res[2] || z_begin >= z_end || in.voxel_res[0] == 0 || in.voxel_res[1] == 0)
            return set_error(FBP_ERR_INVALID_ARG, "fbp_slab_bin_window: empty or out-of-range slab");
        if (!(in.time_step > 0.f)) return set_error(FBP_ERR_INVALID_ARG, "fbp_slab_bin_window: time_step must be > 0");
        // Voxel-centre box of the slab: world (x, y, z) <- (vx, vz, vy).
        const double c0[3] = {in.hidden_min[0] + 0.5 * in.voxel_size[0],
                              in.hidden_min[1] + (z_begin + 0.5) * (double)in.voxel_size[1],
                              in.hidden_min[2] + 0.5 * in.voxel_size[2]};
        const double c1[3] = {in.hidden_min[0] + (in.voxel_res[0] - 0.5) * (double)in.voxel_size[0],
                              in.hidden_min[1] + (z_end - 0.5) * (double)in.voxel_size[1],
                              in.hidden_min[2] + (in.voxel_res[1] - 0.5) * (double)in.voxel_size[2]};
        double lo[3], hi[3];
        for (int k = 0; k < 3; ++k) {
            lo[k] = std::min(c0[k], c1[k]);
            hi[k] = std::max(c0[k], c1[k]);
        }
        const double dt = in.time_step, T = in.num_time_bins;
        double pmin = 1e300, pmax = -1e300;
        for (uint32_t l = 0; l < in.num_laser_targets; ++l) {
            const double p[3] = {laser_xyz[3 * l], laser_xyz[3 * l + 1], laser_xyz[3 * l + 2]};
            double dmin, dmax;
            box_dist(p, lo, hi, &dmin, &dmax);
            double bounce = 0.0;
            if (in.discard_first_last_bounces == 0) {
                double a = 0.0, b = 0.0;
                for (int k = 0; k < 3; ++k) {
                    a += (in.laser_position[k] - p[k]) * (in.laser_position[k] - p[k]);
                    b += (in.sensor_position[k] - p[k]) * (in.sensor_position[k] - p[k]);
                }
                bounce = std::sqrt(a) + std::sqrt(b);
            }
            pmin = std::min(pmin, 2.0 * dmin - in.time_offset + bounce);
            pmax = std::max(pmax, 2.0 * dmax - in.time_offset + bounce);
        }
        // Two bins of margin for the FP32 bin arithmetic of the gathers.
        const double blo = std::floor(pmin / dt) - 2.0, bhi = std::floor(pmax / dt) + 2.0;
        if (bhi < 0.0 || blo > T - 1.0) {  // the slab reaches no bin
            *bin_lo = 1;
            *bin_hi = 0;
            return FBP_OK;
        }
        *bin_lo = (uint32_t)std::max(0.0, blo);
        *bin_hi = (uint32_t)std::min(T - 1.0, bhi);
        return FBP_OK;
    });
}

extern "C" fbp_status fbp_backproject_confocal_slab(fbp_context* ctx, const fbp_recon_info* info, const void* cube,
                                                    int dtype, int layout, const float* laser_xyz, uint32_t z_begin,
                                                    uint32_t z_end, float* volume_slab, void* stream) {
    return guarded("fbp_backproject_confocal_slab", [&]() -> fbp_status {
        clear_error();
        FBP_TRY(check_ctx(ctx));
        FBP_TRY(validate_info(info, false, "fbp_backproject_confocal_slab"));
        if (!cube || !laser_xyz || !volume_slab)
            return set_error(FBP_ERR_INVALID_ARG, "fbp_backproject_confocal_slab: null buffer");
        if (layout != FBP_LAYOUT_TIME_MAJOR && layout != FBP_LAYOUT_TIME_INNER)
            return set_error(FBP_ERR_INVALID_ARG, "fbp_backproject_confocal_slab: unknown layout");
        if (z_begin >= z_end || z_end > info->voxel_res[2])
            return set_error(FBP_ERR_INVALID_ARG, "fbp_backproject_confocal_slab: empty or out-of-range slab");
        return confocal_gather_slab(ctx, *info, cube, dtype, layout, laser_xyz, z_begin, z_end, volume_slab,
                                    (cudaStream_t)stream);
    });
}
