/* CPU oracle for the reconstruction hot path — TEST INFRASTRUCTURE ONLY.
 *
 * Plain C restatements of the reference's kernels and host-side weight
 * builders, accumulating in FP64.  Only tests/, __graft_entry__.smoke() and
 * bench.py's cpu_baseline / --impl reference legs may load this library, and
 * only as a checker or as the timed CPU baseline; the product path never
 * calls it.
 *
 * Pinning: the backprojection restatements are checked on the GPU against the
 * reference's own kernels compiled from its sources (oracle/ref_harness), and
 * on the CPU against hand-derived known-answer cases.  The reference ships no
 * golden vectors or tests of its own for these kernels.
 */
#ifndef FBP_ORACLE_H
#define FBP_ORACLE_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Same field order and packing as the reference's ReconstructionInfo
 * (FasterBackprojection/GpuStructs.cuh:8-38): glm::vec3 is three packed floats. */
typedef struct {
    float sensor_position[3];
    uint32_t capture_system;
    float laser_position[3];
    float time_offset;
    uint32_t num_laser_targets;
    uint32_t num_sensor_targets;
    uint32_t num_time_bins;
    float time_step;
    float hidden_min[3];
    uint32_t discard_first_last_bounces;
    float hidden_max[3];
    float hidden_size[3];
    float voxel_size[3];
    float wall_min[3];
    float wall_size[3];
    float wall_normal[3];
    uint32_t voxel_res[3];
} oracle_info;

enum { ORACLE_LAYOUT_TIME_MAJOR = 0, ORACLE_LAYOUT_TIME_INNER = 1 };
enum { ORACLE_BINS_F64 = 0, ORACLE_BINS_GIVEN = 1 };

size_t oracle_info_size(void);

/* backprojectConfocalVoxel (transient_reconstruction.cuh:93-136), FP64.
 * vol[Vx*Vy*vz + vy*Vx + vx] = sum_l I(l, bin) / dist^2 over I > 1e-5.
 * bins_mode ORACLE_BINS_GIVEN reads int32 bins[v*L + l] instead of computing them. */
int oracle_confocal_voxel(const oracle_info* info, const float* cube, int layout, const float* laser_xyz,
                          int bins_mode, const int32_t* bins, double* vol);

/* Same, restricted to an explicit list of voxel linear indices (for sampled
 * checks at full size).  out[i] is the value of voxel idx[i]. */
int oracle_confocal_voxel_subset(const oracle_info* info, const float* cube, int layout, const float* laser_xyz,
                                 const int64_t* idx, int64_t n, double* out);

/* Same subset with given bins: bins[i*L + l] for voxel idx[i] (isolates the
 * accumulation from the bin arithmetic at full size). */
int oracle_confocal_voxel_subset_bins(const oracle_info* info, const float* cube, int layout, const float* laser_xyz,
                                      const int64_t* idx, int64_t n, const int32_t* bins, double* out);

/* The ACCUMULATE_VOXEL_SCATTERING build of backprojectConfocalVoxel
 * (transient_reconstruction.cuh:112-126), FP64: per (voxel, scan point) every
 * bin of the path d = max(0, dist - ext) .. dist + ext (exclusive) stepped by
 * timeStep + EPS, ext = |voxelSize| / 2, ending at the first bin outside
 * [0, T); each I > 1e-5 adds I / dist^2. */
int oracle_confocal_scatter_voxel(const oracle_info* info, const float* cube, int layout, const float* laser_xyz,
                                  double* vol);

/* FP32 restatement of the same kernel (reference arithmetic in float, IEEE
 * sqrt/div, one thread per voxel instead of per pair): the timed CPU baseline. */
int oracle_confocal_voxel_f32_subset(const oracle_info* info, const float* cube, int layout, const float* laser_xyz,
                                     const int64_t* idx, int64_t n, float* out, int threads);

/* backprojectExhaustiveVoxel (transient_reconstruction.cuh:138-166) with the
 * laser/SPAD index split l = ls / S, s = ls % S. cube[l][s][t]. */
int oracle_exhaustive_voxel(const oracle_info* info, const float* cube, const float* laser_xyz,
                            const float* sensor_xyz, int bins_mode, const int32_t* bins, double* vol);
int oracle_exhaustive_voxel_subset(const oracle_info* info, const float* cube, const float* laser_xyz,
                                   const float* sensor_xyz, const int64_t* idx, int64_t n, double* out);
/* The same with given bins: bins[(i*L + l)*S + s] for voxel idx[i] (NULL: FP64 bins). */
int oracle_exhaustive_voxel_subset_bins(const oracle_info* info, const float* cube, const float* laser_xyz,
                                        const float* sensor_xyz, const int64_t* idx, int64_t n, const int32_t* bins,
                                        double* out);

/* backprojectConfocal / backprojectExhaustive depth planes
 * (transient_reconstruction.cuh:41-91): act[c*D + d], unweighted. */
int oracle_depth_confocal(const oracle_info* info, const float* cube, int layout, const float* laser_xyz,
                          const double* depths, uint32_t num_depths, double* act);
int oracle_depth_exhaustive(const oracle_info* info, const float* cube, const float* laser_xyz,
                            const float* sensor_xyz, const double* depths, uint32_t num_depths, double* act);

/* LoG::calculateLaplacianKernel (PostprocessingFilters.cu:102-175), float. */
int oracle_log_weights(int size, float sigma, float* w);
/* LoGFilter (transient_postprocessing.cuh:52-83), clamp-to-edge, FP64 sums. */
int oracle_log_filter(const float* in, double* out, uint32_t nx, uint32_t ny, uint32_t nz, const float* w, int size);
/* laplacianFilter (transient_postprocessing.cuh:21-50), zero padding, FP64. */
int oracle_laplacian_filter(const float* in, double* out, uint32_t nx, uint32_t ny, uint32_t nz, int size);
/* Laser::normalizeMatrix + normalizeReconstruction (Laser.cu:317-339,
 * transient_postprocessing.cuh:10-17), FP64. */
int oracle_normalize(double* v, int64_t n);

/* Laser::buildAliasTables (Laser.cu:253-315): Vose alias tables in float from
 * a CDF.  Returns 0, or 1 on a negative probability, 2 when the
 * probabilities do not sum to 1 within 1e-5 (the reference throws). */
int oracle_build_alias(const float* cdf, uint32_t n, uint32_t* alias, float* prob);

#ifdef __cplusplus
}
#endif
#endif
