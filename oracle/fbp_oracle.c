/* CPU oracle for the reconstruction hot path — TEST INFRASTRUCTURE ONLY.
 * See fbp_oracle.h for the contract.  Every function cites the reference
 * code it restates (paths relative to the reference's FasterBackprojection/). */
#include "fbp_oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* math.cuh:11 — EPS is a float literal; comparisons in the reference are in float. */
#define ORACLE_EPS 0.00001f

size_t oracle_info_size(void) { return sizeof(oracle_info); }

/* math.cuh:23-29 safeRCP, evaluated in double with the float threshold. */
static double safe_rcp_d(double x) {
    if (x > (double)ORACLE_EPS || x < -(double)ORACLE_EPS) return 1.0 / x;
    return x >= 0 ? (double)FLT_MAX : -(double)FLT_MAX;
}

static double dist3(const double a[3], const double b[3]) {
    const double dx = b[0] - a[0], dy = b[1] - a[1], dz = b[2] - a[2];
    return sqrt(dx * dx + dy * dy + dz * dz);
}

static void load3(const float* p, double out[3]) {
    out[0] = p[0];
    out[1] = p[1];
    out[2] = p[2];
}

/* World position of voxel (vx, vy, vz): transient_reconstruction.cuh:106,
 *   hiddenMin + vec3(vx, voxelZ, vy) * voxelSize + 0.5 * voxelSize
 * The depth index vz drives the world y axis and vy the world z axis. */
static void voxel_center(const oracle_info* in, uint32_t vx, uint32_t vy, uint32_t vz, double p[3]) {
    p[0] = (double)in->hidden_min[0] + (double)vx * in->voxel_size[0] + 0.5 * in->voxel_size[0];
    p[1] = (double)in->hidden_min[1] + (double)vz * in->voxel_size[1] + 0.5 * in->voxel_size[1];
    p[2] = (double)in->hidden_min[2] + (double)vy * in->voxel_size[2] + 0.5 * in->voxel_size[2];
}

/* static_cast<int>(dist / timeStep) with the 0 <= bin < T test
 * (transient_reconstruction.cuh:128-130); -1 when out of range. */
static int32_t bin_of(double dist, double dt, uint32_t T) {
    const double x = dist / dt;
    if (!(x > -1.0) || !(x < (double)T)) return -1; /* also rejects NaN */
    return (int32_t)x; /* truncation toward zero, like the C++ cast */
}

/* transient_utils.cuh:6-9 (time-major, what the kernels read) and the
 * loader's time-innermost order (NLosData.cpp:241, 264). */
static size_t confocal_index(int layout, uint32_t l, uint32_t t, uint32_t L, uint32_t T) {
    return layout == ORACLE_LAYOUT_TIME_MAJOR ? (size_t)t * L + l : (size_t)l * T + t;
}

/* Per-scan-point bounce term, transient_reconstruction.cuh:109-110. */
static double confocal_bounce(const oracle_info* in, const double l[3]) {
    if (in->discard_first_last_bounces != 0) return 0.0;
    double lp[3], sp[3];
    load3(in->laser_position, lp);
    load3(in->sensor_position, sp);
    return dist3(l, lp) + dist3(l, sp);
}

static double confocal_voxel_value(const oracle_info* in, const float* cube, int layout, const float* laser_xyz,
                                   const double* bounce, int64_t v, int bins_mode, const int32_t* vbins) {
    const uint32_t Vx = in->voxel_res[0], Vy = in->voxel_res[1];
    const uint32_t L = in->num_laser_targets, T = in->num_time_bins;
    const uint32_t slice = Vx * Vy;
    const uint32_t vz = (uint32_t)(v / slice), rem = (uint32_t)(v % slice);
    const uint32_t vy = rem / Vx, vx = rem % Vx;
    double p[3];
    voxel_center(in, vx, vy, vz, p);
    double acc = 0.0;
    for (uint32_t l = 0; l < L; ++l) {
        double lp[3];
        load3(laser_xyz + 3 * (size_t)l, lp);
        const double dist = dist3(lp, p) * 2.0 - (double)in->time_offset + bounce[l];
        const int32_t b = bins_mode == ORACLE_BINS_GIVEN ? vbins[l] : bin_of(dist, in->time_step, T);
        if (b < 0 || (uint32_t)b >= T) continue;
        const float I = cube[confocal_index(layout, l, (uint32_t)b, L, T)];
        if (I > ORACLE_EPS) acc += (double)I * safe_rcp_d(dist * dist);
    }
    return acc;
}

static double* confocal_bounces(const oracle_info* in, const float* laser_xyz) {
    const uint32_t L = in->num_laser_targets;
    double* b = (double*)malloc(sizeof(double) * (L ? L : 1));
    if (!b) return NULL;
    for (uint32_t l = 0; l < L; ++l) {
        double lp[3];
        load3(laser_xyz + 3 * (size_t)l, lp);
        b[l] = confocal_bounce(in, lp);
    }
    return b;
}

int oracle_confocal_voxel(const oracle_info* in, const float* cube, int layout, const float* laser_xyz,
                          int bins_mode, const int32_t* bins, double* vol) {
    const int64_t V = (int64_t)in->voxel_res[0] * in->voxel_res[1] * in->voxel_res[2];
    double* bounce = confocal_bounces(in, laser_xyz);
    if (!bounce) return 1;
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t v = 0; v < V; ++v)
        vol[v] = confocal_voxel_value(in, cube, layout, laser_xyz, bounce, v, bins_mode,
                                      bins_mode == ORACLE_BINS_GIVEN ? bins + (size_t)v * in->num_laser_targets : NULL);
    free(bounce);
    return 0;
}

int oracle_confocal_voxel_subset(const oracle_info* in, const float* cube, int layout, const float* laser_xyz,
                                 const int64_t* idx, int64_t n, double* out) {
    double* bounce = confocal_bounces(in, laser_xyz);
    if (!bounce) return 1;
#pragma omp parallel for schedule(dynamic, 8)
    for (int64_t i = 0; i < n; ++i)
        out[i] = confocal_voxel_value(in, cube, layout, laser_xyz, bounce, idx[i], ORACLE_BINS_F64, NULL);
    free(bounce);
    return 0;
}

int oracle_confocal_voxel_subset_bins(const oracle_info* in, const float* cube, int layout, const float* laser_xyz,
                                      const int64_t* idx, int64_t n, const int32_t* bins, double* out) {
    const uint32_t L = in->num_laser_targets;
    double* bounce = confocal_bounces(in, laser_xyz);
    if (!bounce) return 1;
#pragma omp parallel for schedule(dynamic, 8)
    for (int64_t i = 0; i < n; ++i)
        out[i] = confocal_voxel_value(in, cube, layout, laser_xyz, bounce, idx[i], ORACLE_BINS_GIVEN,
                                      bins + (size_t)i * L);
    free(bounce);
    return 0;
}

/* transient_reconstruction.cuh:112-126 (ACCUMULATE_VOXEL_SCATTERING): the walk
 * over [max(0, dist - ext), dist + ext) in steps of timeStep + EPS; the
 * reference's thread returns at the first bin outside [0, T). */
static double scatter_voxel_value(const oracle_info* in, const float* cube, int layout, const float* laser_xyz,
                                  const double* bounce, int64_t v) {
    const uint32_t Vx = in->voxel_res[0], Vy = in->voxel_res[1];
    const uint32_t L = in->num_laser_targets, T = in->num_time_bins;
    const uint32_t slice = Vx * Vy;
    const uint32_t vz = (uint32_t)(v / slice), rem = (uint32_t)(v % slice);
    const uint32_t vy = rem / Vx, vx = rem % Vx;
    const double vs0 = in->voxel_size[0], vs1 = in->voxel_size[1], vs2 = in->voxel_size[2];
    const double ext = 0.5 * sqrt(vs0 * vs0 + vs1 * vs1 + vs2 * vs2);
    const double dt = in->time_step, step = dt + (double)ORACLE_EPS;
    double p[3];
    voxel_center(in, vx, vy, vz, p);
    double acc = 0.0;
    for (uint32_t l = 0; l < L; ++l) {
        double lp[3];
        load3(laser_xyz + 3 * (size_t)l, lp);
        const double dist = dist3(lp, p) * 2.0 - (double)in->time_offset + bounce[l];
        const double w = safe_rcp_d(dist * dist);
        const double dmax = dist + ext;
        for (double d = dist - ext > 0.0 ? dist - ext : 0.0; d < dmax; d += step) {
            const int32_t b = bin_of(d, dt, T);
            if (b < 0) break;
            const float I = cube[confocal_index(layout, l, (uint32_t)b, L, T)];
            if (I > ORACLE_EPS) acc += (double)I * w;
        }
    }
    return acc;
}

int oracle_confocal_scatter_voxel(const oracle_info* in, const float* cube, int layout, const float* laser_xyz,
                                  double* vol) {
    if (!(in->time_step > 0.f)) return 2; /* the walk needs a positive step */
    const int64_t V = (int64_t)in->voxel_res[0] * in->voxel_res[1] * in->voxel_res[2];
    double* bounce = confocal_bounces(in, laser_xyz);
    if (!bounce) return 1;
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t v = 0; v < V; ++v) vol[v] = scatter_voxel_value(in, cube, layout, laser_xyz, bounce, v);
    free(bounce);
    return 0;
}

/* FP32 restatement of backprojectConfocalVoxel: the reference arithmetic in
 * float (IEEE sqrt and divide), one task per voxel summing over all scan
 * points.  Used as the timed CPU baseline. */
int oracle_confocal_voxel_f32_subset(const oracle_info* in, const float* cube, int layout, const float* laser_xyz,
                                     const int64_t* idx, int64_t n, float* out, int threads) {
    const uint32_t Vx = in->voxel_res[0], Vy = in->voxel_res[1];
    const uint32_t L = in->num_laser_targets, T = in->num_time_bins;
    const uint32_t slice = Vx * Vy;
    const float dt = in->time_step, t0 = in->time_offset;
    float* bounce = (float*)malloc(sizeof(float) * (L ? L : 1));
    if (!bounce) return 1;
    for (uint32_t l = 0; l < L; ++l) {
        const float* q = laser_xyz + 3 * (size_t)l;
        float b = 0.f;
        if (in->discard_first_last_bounces == 0) {
            const float ax = in->laser_position[0] - q[0], ay = in->laser_position[1] - q[1], az = in->laser_position[2] - q[2];
            const float sx = in->sensor_position[0] - q[0], sy = in->sensor_position[1] - q[1], sz = in->sensor_position[2] - q[2];
            b = sqrtf(ax * ax + ay * ay + az * az) + sqrtf(sx * sx + sy * sy + sz * sz);
        }
        bounce[l] = b;
    }
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#else
    (void)threads;
#endif
#pragma omp parallel for schedule(dynamic, 4)
    for (int64_t i = 0; i < n; ++i) {
        const int64_t v = idx[i];
        const uint32_t vz = (uint32_t)(v / slice), rem = (uint32_t)(v % slice);
        const uint32_t vy = rem / Vx, vx = rem % Vx;
        const float px = in->hidden_min[0] + (float)vx * in->voxel_size[0] + 0.5f * in->voxel_size[0];
        const float py = in->hidden_min[1] + (float)vz * in->voxel_size[1] + 0.5f * in->voxel_size[1];
        const float pz = in->hidden_min[2] + (float)vy * in->voxel_size[2] + 0.5f * in->voxel_size[2];
        float acc = 0.f;
        for (uint32_t l = 0; l < L; ++l) {
            const float* q = laser_xyz + 3 * (size_t)l;
            const float dx = px - q[0], dy = py - q[1], dz = pz - q[2];
            float dist = sqrtf(dx * dx + dy * dy + dz * dz) * 2.0f - t0;
            dist += bounce[l];
            const float x = dist / dt;
            if (!(x > -1.0f) || !(x < (float)T)) continue;
            const int b = (int)x;
            const float I = cube[confocal_index(layout, l, (uint32_t)b, L, T)];
            if (I > ORACLE_EPS) {
                const float d2 = dist * dist;
                const float w = (d2 > ORACLE_EPS || d2 < -ORACLE_EPS) ? 1.0f / d2 : (d2 >= 0 ? FLT_MAX : -FLT_MAX);
                acc += I * w;
            }
        }
        out[i] = acc;
    }
    free(bounce);
    return 0;
}

/* vbins: this voxel's bins [l*S + s] (ORACLE_BINS_GIVEN) or NULL. */
static double exhaustive_voxel_value(const oracle_info* in, const float* cube, const float* laser_xyz,
                                     const float* sensor_xyz, const double* bl, const double* bs, int64_t v,
                                     int bins_mode, const int32_t* vbins) {
    const uint32_t Vx = in->voxel_res[0], Vy = in->voxel_res[1];
    const uint32_t L = in->num_laser_targets, S = in->num_sensor_targets, T = in->num_time_bins;
    const uint32_t slice = Vx * Vy;
    const uint32_t vz = (uint32_t)(v / slice), rem = (uint32_t)(v % slice);
    const uint32_t vy = rem / Vx, vx = rem % Vx;
    double p[3];
    voxel_center(in, vx, vy, vz, p);
    double acc = 0.0;
    for (uint32_t l = 0; l < L; ++l) {
        double lp[3];
        load3(laser_xyz + 3 * (size_t)l, lp);
        const double dl = dist3(lp, p);
        for (uint32_t s = 0; s < S; ++s) {
            double sp[3];
            load3(sensor_xyz + 3 * (size_t)s, sp);
            const double dist = dl + dist3(sp, p) - (double)in->time_offset + bl[l] + bs[s];
            const size_t pair = (size_t)l * S + s;
            const int32_t b = bins_mode == ORACLE_BINS_GIVEN ? vbins[pair] : bin_of(dist, in->time_step, T);
            if (b < 0 || (uint32_t)b >= T) continue;
            /* transient_utils.cuh:11-14 */
            const float I = cube[pair * T + (uint32_t)b];
            if (I > ORACLE_EPS) acc += (double)I * safe_rcp_d(dist * dist);
        }
    }
    return acc;
}

static int exhaustive_bounces(const oracle_info* in, const float* laser_xyz, const float* sensor_xyz, double** bl,
                              double** bs) {
    const uint32_t L = in->num_laser_targets, S = in->num_sensor_targets;
    *bl = (double*)malloc(sizeof(double) * (L ? L : 1));
    *bs = (double*)malloc(sizeof(double) * (S ? S : 1));
    if (!*bl || !*bs) { free(*bl); free(*bs); return 1; }
    double lp0[3], sp0[3];
    load3(in->laser_position, lp0);
    load3(in->sensor_position, sp0);
    /* transient_reconstruction.cuh:156-157: |l - laserPos| + |s - sensorPos|. */
    for (uint32_t l = 0; l < L; ++l) {
        double q[3];
        load3(laser_xyz + 3 * (size_t)l, q);
        (*bl)[l] = in->discard_first_last_bounces == 0 ? dist3(q, lp0) : 0.0;
    }
    for (uint32_t s = 0; s < S; ++s) {
        double q[3];
        load3(sensor_xyz + 3 * (size_t)s, q);
        (*bs)[s] = in->discard_first_last_bounces == 0 ? dist3(q, sp0) : 0.0;
    }
    return 0;
}

int oracle_exhaustive_voxel(const oracle_info* in, const float* cube, const float* laser_xyz,
                            const float* sensor_xyz, int bins_mode, const int32_t* bins, double* vol) {
    const int64_t V = (int64_t)in->voxel_res[0] * in->voxel_res[1] * in->voxel_res[2];
    double *bl, *bs;
    if (exhaustive_bounces(in, laser_xyz, sensor_xyz, &bl, &bs)) return 1;
#pragma omp parallel for schedule(dynamic, 16)
    for (int64_t v = 0; v < V; ++v)
        vol[v] = exhaustive_voxel_value(in, cube, laser_xyz, sensor_xyz, bl, bs, v, bins_mode,
                                        bins_mode == ORACLE_BINS_GIVEN
                                            ? bins + (size_t)v * in->num_laser_targets * in->num_sensor_targets
                                            : NULL);
    free(bl);
    free(bs);
    return 0;
}

int oracle_exhaustive_voxel_subset(const oracle_info* in, const float* cube, const float* laser_xyz,
                                   const float* sensor_xyz, const int64_t* idx, int64_t n, double* out) {
    return oracle_exhaustive_voxel_subset_bins(in, cube, laser_xyz, sensor_xyz, idx, n, NULL, out);
}

/* bins: NULL (FP64 bins) or the GPU's bins of voxel idx[i] at
 * bins[(i*L + l)*S + s] (fbp_debug_exhaustive_bins' order). */
int oracle_exhaustive_voxel_subset_bins(const oracle_info* in, const float* cube, const float* laser_xyz,
                                        const float* sensor_xyz, const int64_t* idx, int64_t n, const int32_t* bins,
                                        double* out) {
    const size_t LS = (size_t)in->num_laser_targets * in->num_sensor_targets;
    double *bl, *bs;
    if (exhaustive_bounces(in, laser_xyz, sensor_xyz, &bl, &bs)) return 1;
#pragma omp parallel for schedule(dynamic, 4)
    for (int64_t i = 0; i < n; ++i)
        out[i] = exhaustive_voxel_value(in, cube, laser_xyz, sensor_xyz, bl, bs, idx[i],
                                        bins ? ORACLE_BINS_GIVEN : ORACLE_BINS_F64,
                                        bins ? bins + (size_t)i * LS : NULL);
    free(bl);
    free(bs);
    return 0;
}

/* Depth-plane test point: transient_reconstruction.cuh:51 / :78,
 *   laserTargets[c] + relayWallNormal * float(depths[d]). */
static void plane_point(const oracle_info* in, const float* laser_xyz, uint32_t c, double depth, double p[3]) {
    const double d = (double)(float)depth;
    for (int k = 0; k < 3; ++k) p[k] = (double)laser_xyz[3 * (size_t)c + k] + (double)in->wall_normal[k] * d;
}

int oracle_depth_confocal(const oracle_info* in, const float* cube, int layout, const float* laser_xyz,
                          const double* depths, uint32_t D, double* act) {
    const uint32_t L = in->num_laser_targets, T = in->num_time_bins;
    double* bounce = confocal_bounces(in, laser_xyz);
    if (!bounce) return 1;
#pragma omp parallel for schedule(dynamic, 4)
    for (int64_t cd = 0; cd < (int64_t)L * D; ++cd) {
        const uint32_t c = (uint32_t)(cd / D), d = (uint32_t)(cd % D);
        double p[3];
        plane_point(in, laser_xyz, c, depths[d], p);
        double acc = 0.0;
        for (uint32_t l = 0; l < L; ++l) {
            double lp[3];
            load3(laser_xyz + 3 * (size_t)l, lp);
            const double dist = dist3(lp, p) * 2.0 - (double)in->time_offset + bounce[l];
            const int32_t b = bin_of(dist, in->time_step, T);
            if (b < 0) continue;
            const float I = cube[confocal_index(layout, l, (uint32_t)b, L, T)];
            if (I > ORACLE_EPS) acc += (double)I;
        }
        act[(size_t)c * D + d] = acc;
    }
    free(bounce);
    return 0;
}

int oracle_depth_exhaustive(const oracle_info* in, const float* cube, const float* laser_xyz,
                            const float* sensor_xyz, const double* depths, uint32_t D, double* act) {
    const uint32_t L = in->num_laser_targets, S = in->num_sensor_targets, T = in->num_time_bins;
    double *bl, *bs;
    if (exhaustive_bounces(in, laser_xyz, sensor_xyz, &bl, &bs)) return 1;
#pragma omp parallel for schedule(dynamic, 4)
    for (int64_t cd = 0; cd < (int64_t)L * D; ++cd) {
        const uint32_t c = (uint32_t)(cd / D), d = (uint32_t)(cd % D);
        double p[3];
        plane_point(in, laser_xyz, c, depths[d], p);
        double acc = 0.0;
        /* transient_reconstruction.cuh:75-76: l = ls % L, s = ls / L. */
        for (uint32_t l = 0; l < L; ++l) {
            double lp[3];
            load3(laser_xyz + 3 * (size_t)l, lp);
            const double dl = dist3(lp, p);
            for (uint32_t s = 0; s < S; ++s) {
                double sp[3];
                load3(sensor_xyz + 3 * (size_t)s, sp);
                const double dist = dl + dist3(p, sp) - (double)in->time_offset + bl[l] + bs[s];
                const int32_t b = bin_of(dist, in->time_step, T);
                if (b < 0) continue;
                const float I = cube[((size_t)l * S + s) * T + (uint32_t)b];
                if (I > ORACLE_EPS) acc += (double)I;
            }
        }
        act[(size_t)c * D + d] = acc;
    }
    free(bl);
    free(bs);
    return 0;
}

/* PostprocessingFilters.cu:102-175, in float with the reference's step order:
 * Gaussian, threshold at FLT_EPSILON * max, normalise, multiply by
 * (r^2 - 3 sigma^2) / sigma^4, subtract the mean. */
int oracle_log_weights(int size, float std1, float* w_final) {
    if (size <= 0) return 1;
    const int lim = (size - 1) / 2;
    const float std2 = std1 * std1;
    const int n = size * size * size;
    float* w = (float*)malloc(sizeof(float) * n);
    float* r2 = (float*)malloc(sizeof(float) * n);
    if (!w || !r2) { free(w); free(r2); return 1; }
    float maxw = 0.0f;
    for (int kz = 0; kz < size; ++kz)
        for (int ky = 0; ky < size; ++ky)
            for (int kx = 0; kx < size; ++kx) {
                const float x = (float)(kx - lim), y = (float)(ky - lim), z = (float)(kz - lim);
                const int i = kz * size * size + ky * size + kx;
                r2[i] = x * x + y * y + z * z;
                w[i] = expf(-(x * x + y * y + z * z) / (2.0f * std2));
                if (w[i] > maxw) maxw = w[i];
            }
    const float threshold = FLT_EPSILON * maxw;
    float sum_w = 0.0f;
    for (int i = 0; i < n; ++i) {
        if (w[i] < threshold) w[i] = 0.0f;
        sum_w += w[i];
    }
    if (sum_w != 0.0f)
        for (int i = 0; i < n; ++i) w[i] /= sum_w;
    float sum_w1 = 0.0f;
    for (int i = 0; i < n; ++i) {
        w[i] = w[i] * (r2[i] - 3.0f * std2) / (std2 * std2);
        sum_w1 += w[i];
    }
    const float adjustment = sum_w1 / (float)n;
    for (int i = 0; i < n; ++i) w_final[i] = w[i] - adjustment;
    free(w);
    free(r2);
    return 0;
}

static int64_t clampi(int64_t v, int64_t lo, int64_t hi) { return v < lo ? lo : (v > hi ? hi : v); }

int oracle_log_filter(const float* in, double* out, uint32_t nx, uint32_t ny, uint32_t nz, const float* w, int size) {
    const int h = (size - 1) / 2;
#pragma omp parallel for schedule(static)
    for (int64_t z = 0; z < nz; ++z)
        for (int64_t y = 0; y < ny; ++y)
            for (int64_t x = 0; x < nx; ++x) {
                double acc = 0.0;
                for (int kz = -h; kz <= h; ++kz)
                    for (int ky = -h; ky <= h; ++ky)
                        for (int kx = -h; kx <= h; ++kx) {
                            const int64_t ix = clampi(x + kx, 0, nx - 1), iy = clampi(y + ky, 0, ny - 1),
                                          iz = clampi(z + kz, 0, nz - 1);
                            acc += (double)in[(iz * ny + iy) * nx + ix] *
                                   (double)w[(kz + h) * size * size + (ky + h) * size + (kx + h)];
                        }
                out[(z * ny + y) * nx + x] = acc;
            }
    return 0;
}

int oracle_laplacian_filter(const float* in, double* out, uint32_t nx, uint32_t ny, uint32_t nz, int size) {
    const int h = (int)floor((double)size / 2.0);
    const double k3 = (double)size * size * size;
#pragma omp parallel for schedule(static)
    for (int64_t z = 0; z < nz; ++z)
        for (int64_t y = 0; y < ny; ++y)
            for (int64_t x = 0; x < nx; ++x) {
                double acc = 0.0;
                for (int dx = -h; dx <= h; ++dx)
                    for (int dy = -h; dy <= h; ++dy)
                        for (int dz = -h; dz <= h; ++dz) {
                            const int64_t ix = x + dx, iy = y + dy, iz = z + dz;
                            if (ix < 0 || ix >= nx || iy < 0 || iy >= ny || iz < 0 || iz >= nz) continue;
                            acc += in[(iz * ny + iy) * nx + ix];
                        }
                out[(z * ny + y) * nx + x] = k3 * in[(z * ny + y) * nx + x] - acc;
            }
    return 0;
}

int oracle_normalize(double* v, int64_t n) {
    if (n <= 0) return 0;
    double mn = v[0], mx = v[0];
    for (int64_t i = 1; i < n; ++i) {
        if (v[i] < mn) mn = v[i];
        if (v[i] > mx) mx = v[i];
    }
    const double r = safe_rcp_d(mx - mn);
    for (int64_t i = 0; i < n; ++i) v[i] = (v[i] - mn) * r;
    return 0;
}

int oracle_build_alias(const float* cdf, uint32_t n, uint32_t* alias, float* prob) {
    if (n == 0) return 1;
    float* p = (float*)malloc(sizeof(float) * n);
    uint32_t* small = (uint32_t*)malloc(sizeof(uint32_t) * n);
    uint32_t* large = (uint32_t*)malloc(sizeof(uint32_t) * n);
    if (!p || !small || !large) { free(p); free(small); free(large); return 3; }
    p[0] = cdf[0];
    for (uint32_t i = 1; i < n; ++i) p[i] = cdf[i] - cdf[i - 1];
    uint32_t ns = 0, nl = 0;
    float sum = 0.0f;
    int rc = 0;
    for (uint32_t i = 0; i < n; ++i) {
        alias[i] = 0;
        if (p[i] < 0.0f) { rc = 1; goto done; }
        prob[i] = p[i] * (float)n;
        sum += p[i];
        if (prob[i] < 1.0f) small[ns++] = i;
        else large[nl++] = i;
    }
    if (fabsf(sum - 1.0f) > 1e-5f) { rc = 2; goto done; }
    while (ns > 0 && nl > 0) {
        const uint32_t s = small[--ns];
        const uint32_t l = large[--nl];
        alias[s] = l;
        prob[l] += prob[s] - 1.0f;
        if (prob[l] < 1.0f) small[ns++] = l;
        else large[nl++] = l;
    }
    while (ns > 0) prob[small[--ns]] = 1.0f;
    while (nl > 0) prob[large[--nl]] = 1.0f;
done:
    free(p);
    free(small);
    free(large);
    return rc;
}
