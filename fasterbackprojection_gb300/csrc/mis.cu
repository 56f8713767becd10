// Sampled (MIS) confocal backprojection.
//
// Replaces Laser::reconstructAABBConfocalMIS (Laser.cu:526-611), its alias
// tables (buildAliasTables, Laser.cu:253-315) and backprojectConfocalVoxelMIS
// (transient_reconstruction.cuh:194-260).
//
// FBP_MIS_REFERENCE reproduces the reference kernel's arithmetic: per voxel and
// sample, a 50/50 choice between the spatial alias table and a uniform scan
// point, the noise-buffer RNG (transient_utils.cuh:18-22), balance weight
// pdf / (pdf_alias + 1/L), no 1/(pdf K) factor.  The spatial CDF is built from
// the capture (the reference scans the still-zero volume instead, Laser.cu:550,
// which makes buildAliasTables throw) and min-max normalised as the reference
// does (Laser.cu:574).  Samples are summed in order per voxel (the reference's
// non-atomic += races).
//
// FBP_MIS_UNIFORM / _SPATIAL are unbiased: each voxel tile draws K scan points
// from the proposal and the staged gather weights every pair by 1/(K p(l)).
// FBP_MIS_LEARNED draws K clusters of scan points per tile by systematic
// sampling from the tile's cluster distribution (uniform without one) and
// gathers each chosen cluster whole, weighted by hits / (K p_c): unbiased, as
// the expected number of hits of cluster c is exactly K p_c.
#include "fbp_internal.cuh"
#include "bp_common.cuh"

#include <algorithm>
#include <cmath>
#include <random>
#include <vector>

namespace fbp {

// Per scan point: sum of raw values and of values above EPS.
template <typename S>
__global__ void scan_totals_kernel(const S* __restrict__ cube, uint32_t L, uint32_t T, int time_major,
                                   double* __restrict__ raw, double* __restrict__ thr) {
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (!time_major) {
        if (warp >= L) return;
        double a = 0.0, b = 0.0;
        for (uint32_t t = lane; t < T; t += 32) {
            const float v = to_f32(cube[(uint64_t)warp * T + t]);
            a += v;
            if (v > FBP_EPS) b += v;
        }
        for (int o = 16; o > 0; o >>= 1) {
            a += __shfl_xor_sync(0xffffffffu, a, o);
            b += __shfl_xor_sync(0xffffffffu, b, o);
        }
        if (lane == 0) {
            raw[warp] = a;
            thr[warp] = b;
        }
    } else {
        const uint32_t l = blockIdx.x * blockDim.x + threadIdx.x;
        if (l >= L) return;
        double a = 0.0, b = 0.0;
        for (uint32_t t = 0; t < T; ++t) {
            const float v = to_f32(cube[(uint64_t)t * L + l]);
            a += v;
            if (v > FBP_EPS) b += v;
        }
        raw[l] = a;
        thr[l] = b;
    }
}

// backprojectConfocalVoxelMIS arithmetic, one thread per voxel.
struct MisRefParams {
    const void* rows;
    uint32_t pitch;
    const float4* scan;
    const float* xs;
    const float* ys;
    const float* zs;
    const float* noise;
    uint32_t noise_size;
    const float* spatial;  // normalised CDF over scan points
    const uint32_t* alias;
    const float* prob;
    uint32_t Vx, Vy, Vz, L, T, samples;
    float t0, dt;
    int bounce;
    float* volume;
    float vs[3];  // voxel size: the scattering walk's extent |vs| / 2
};

__device__ __forceinline__ float noise_next(const float* noise, uint32_t n, uint32_t& state) {
    state = state * 747796405u + 2891336453u;  // transient_utils.cuh:20
    return noise[state % n];
}

// Sample s of voxel v starts its generator at state v + s
// (transient_reconstruction.cuh:209), so everything a sample draws (proposal,
// scan point, balance weight) depends on v + s alone: a block of kMisVoxels
// consecutive voxels needs kMisVoxels + C - 1 states per chunk of C samples,
// not kMisVoxels * C.  The block draws them once into shared memory; then
// thread t takes its samples in the rotated order j = (k - t) mod C, so at
// step k a warp's lanes share one or two states: one scan point, and
// neighbouring voxels, so the cube reads coalesce.  Each sample's term is the
// one-sample kernel's; the per-voxel sum runs in the rotated order.
constexpr uint32_t kMisVoxels = 256, kMisChunk = 256;

__device__ __forceinline__ void mis_draw(const MisRefParams& p, uint32_t state, float invL, uint32_t& l, float& a) {
    float pdf, gpdf;
    if (noise_next(p.noise, p.noise_size, state) < 0.5f) {
        const float r1 = noise_next(p.noise, p.noise_size, state);
        const float r2 = noise_next(p.noise, p.noise_size, state);
        const uint32_t k = min((uint32_t)(r1 * (float)p.L), p.L - 1);
        l = r2 < p.prob[k] ? k : p.alias[k];
        pdf = l > 0 ? p.spatial[l] - p.spatial[l - 1] : p.spatial[l];
        gpdf = pdf + 1.0f * invL;
    } else {
        l = min((uint32_t)(noise_next(p.noise, p.noise_size, state) * (float)p.L), p.L - 1);
        pdf = 1.0f * invL;
        gpdf = pdf + (l > 0 ? p.spatial[l] - p.spatial[l - 1] : p.spatial[l]);
    }
    a = pdf * ref_safe_rcp(gpdf);  // the balance weight
}

// SCATTER: the reference's ACCUMULATE_VOXEL_SCATTERING build of the kernel
// (transient_reconstruction.cuh:235-250): each sample adds
// (weight * I) * safeRCP(dist^2) for every bin of d = max(0, dist - e),
// d += timeStep + EPS while d < dist + e (e half the voxel diagonal), and
// stops at the first bin outside [0, T); the reference adds each term with an
// atomic, one rounding per add, so the terms are added (not fused) in order.
template <typename S, bool SCATTER>
__global__ void __launch_bounds__(kMisVoxels) mis_reference_kernel(MisRefParams p) {
    __shared__ float4 s_scan[kMisVoxels + kMisChunk - 1];
    __shared__ float2 s_draw[kMisVoxels + kMisChunk - 1];  // (weight, scan point index bits)
    const uint32_t t = threadIdx.x;
    const uint64_t slice = (uint64_t)p.Vx * p.Vy;
    const uint64_t v0 = (uint64_t)blockIdx.x * kMisVoxels, v = v0 + t;
    const bool live = v < slice * p.Vz;
    float px = 0.f, py = 0.f, pz = 0.f;
    if (live) {
        const uint32_t vz = (uint32_t)(v / slice), vs = (uint32_t)(v % slice);
        px = p.xs[vs % p.Vx];
        py = p.ys[vz];
        pz = p.zs[vs / p.Vx];
    }
    const float rcp_dt = rcp_approx(p.dt);
    const float invL = ref_safe_rcp((float)p.L);
    const S* rows = static_cast<const S*>(p.rows);
    float ksum = 0.f, kcomp = 0.f, acc = 0.f;
    // length(voxelSize) / 2 and the step timeStep + EPS in the reference's FP32.
    const float ext = SCATTER ? mul_rn(0.5f, sqrt_approx(ref_dot3(p.vs[0], p.vs[1], p.vs[2]))) : 0.f;
    const float step = SCATTER ? add_rn(p.dt, FBP_EPS) : 0.f;
    // A bound on the walk's steps (only a path so long that adding the step
    // no longer changes it could exceed it; such a path reaches no bin).
    const int max_it = SCATTER ? (int)(2.f * ext / step) + 4 : 0;
    for (uint32_t s0 = 0; s0 < p.samples; s0 += kMisChunk) {
        const uint32_t ce = min(kMisChunk, p.samples - s0), ntab = kMisVoxels + ce - 1;
        __syncthreads();  // the previous chunk's table is no longer read
        for (uint32_t i = t; i < ntab; i += kMisVoxels) {
            uint32_t l;
            float a;
            mis_draw(p, (uint32_t)(v0 + s0 + i), invL, l, a);
            s_scan[i] = p.scan[l];
            s_draw[i] = make_float2(a, __uint_as_float(l));
        }
        __syncthreads();
        if (!live) continue;
        const uint32_t r = t % ce;
        if constexpr (SCATTER) {
            for (uint32_t k = 0; k < ce; ++k) {
                const uint32_t e = t + (k >= r ? k - r : k + ce - r);
                const float4 g = s_scan[e];
                const float2 d = s_draw[e];
                float dist = fma_rn(sqrt_approx(ref_dot3(sub_rn(px, g.x), sub_rn(py, g.y), sub_rn(pz, g.z))), 2.f,
                                    -p.t0);
                if (p.bounce) dist = add_rn(dist, g.w);
                const float w = ref_safe_rcp(mul_rn(dist, dist));
                const S* row = rows + (uint64_t)__float_as_uint(d.y) * p.pitch;
                float dd = fmaxf(0.f, sub_rn(dist, ext));
                const float dmax = add_rn(dist, ext);
                for (int it = 0; dd < dmax && it < max_it; ++it) {
                    const int b = __float2int_rz(ref_bin_ratio(dd, rcp_dt));
                    if (b < 0 || b >= (int)p.T) break;
                    const float I = to_f32(row[b]);
                    if (I > FBP_EPS) acc = add_rn(acc, mul_rn(mul_rn(d.x, I), w));
                    dd = add_rn(dd, step);
                }
                const uint32_t n = s0 + k;
                if ((n & 63) == 63 || n + 1 == p.samples) {
                    const float y = sub_rn(acc, kcomp);
                    const float tt = add_rn(ksum, y);
                    kcomp = sub_rn(sub_rn(tt, ksum), y);
                    ksum = tt;
                    acc = 0.f;
                }
            }
            continue;
        }
        // U steps at a time: their cube reads are in flight together; the
        // terms are added in step order.
        constexpr int U = 4;
        for (uint32_t k0 = 0; k0 < ce; k0 += U) {
            float A[U], W[U], I[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                A[u] = 0.f;
                W[u] = 0.f;
                I[u] = 0.f;
                const uint32_t k = k0 + u;
                if (k >= ce) continue;
                const uint32_t e = t + (k >= r ? k - r : k + ce - r);
                const float4 g = s_scan[e];
                const float2 d = s_draw[e];
                float dist = fma_rn(sqrt_approx(ref_dot3(sub_rn(px, g.x), sub_rn(py, g.y), sub_rn(pz, g.z))), 2.f,
                                    -p.t0);
                if (p.bounce) dist = add_rn(dist, g.w);
                A[u] = d.x;
                const int b = __float2int_rz(ref_bin_ratio(dist, rcp_dt));
                if (b >= 0 && b < (int)p.T) {
                    I[u] = to_f32(rows[(uint64_t)__float_as_uint(d.y) * p.pitch + b]);
                    W[u] = ref_safe_rcp(mul_rn(dist, dist));
                }
            }
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const uint32_t n = s0 + k0 + u;  // samples taken so far, this one included: n + 1
                if (k0 + u >= ce) break;
                if (I[u] > FBP_EPS) acc = fmaf(A[u] * I[u], W[u], acc);
                if ((n & 63) == 63 || n + 1 == p.samples) {
                    const float y = sub_rn(acc, kcomp);
                    const float tt = add_rn(ksum, y);
                    kcomp = sub_rn(sub_rn(tt, ksum), y);
                    ksum = tt;
                    acc = 0.f;
                }
            }
        }
    }
    if (live) p.volume[v] = ksum;
}

template <typename S>
__global__ void mis_rows_kernel(S* __restrict__ rows, const S* __restrict__ cube, uint32_t L, uint32_t T, uint32_t pitch,
                                int time_major) {
    const uint64_t n = (uint64_t)L * pitch;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t l = (uint32_t)(i / pitch), t = (uint32_t)(i % pitch);
        S v = from_f32<S>(0.f);
        if (t < T) {
            const S c = time_major ? cube[(uint64_t)t * L + l] : cube[(uint64_t)l * T + t];
            if (to_f32(c) > FBP_EPS) v = c;
        }
        rows[i] = v;
    }
}

// Laser::buildAliasTables (Laser.cu:253-315) in float, same pairing order.
// Returns 0, 1 (negative probability) or 2 (does not sum to 1 within 1e-5).
int build_alias_reference(const std::vector<float>& cdf, std::vector<uint32_t>& alias, std::vector<float>& prob) {
    const uint32_t N = (uint32_t)cdf.size();
    std::vector<float> p(N);
    p[0] = cdf[0];
    for (uint32_t i = 1; i < N; ++i) p[i] = cdf[i] - cdf[i - 1];
    alias.assign(N, 0);
    prob.assign(N, 0.f);
    std::vector<uint32_t> small, large;
    float sum = 0.f;
    for (uint32_t i = 0; i < N; ++i) {
        if (p[i] < 0.f) return 1;
        prob[i] = p[i] * N;
        sum += p[i];
        (prob[i] < 1.f ? small : large).push_back(i);
    }
    if (std::fabs(sum - 1.f) > 1e-5f) return 2;
    while (!small.empty() && !large.empty()) {
        const uint32_t s = small.back();
        small.pop_back();
        const uint32_t l = large.back();
        large.pop_back();
        alias[s] = l;
        prob[l] += prob[s] - 1.f;
        (prob[l] < 1.f ? small : large).push_back(l);
    }
    while (!small.empty()) {
        prob[small.back()] = 1.f;
        small.pop_back();
    }
    while (!large.empty()) {
        prob[large.back()] = 1.f;
        large.pop_back();
    }
    return 0;
}

// Vose alias tables of p (double, sums to 1) for the unbiased spatial proposal.
static void build_alias_double(const std::vector<double>& p, std::vector<uint32_t>& alias, std::vector<float>& prob) {
    const size_t N = p.size();
    std::vector<double> q(N);
    alias.assign(N, 0);
    prob.assign(N, 1.f);
    std::vector<uint32_t> small, large;
    for (size_t i = 0; i < N; ++i) {
        q[i] = p[i] * (double)N;
        (q[i] < 1.0 ? small : large).push_back((uint32_t)i);
    }
    while (!small.empty() && !large.empty()) {
        const uint32_t s = small.back();
        small.pop_back();
        const uint32_t l = large.back();
        large.pop_back();
        alias[s] = l;
        prob[s] = (float)q[s];
        q[l] += q[s] - 1.0;
        (q[l] < 1.0 ? small : large).push_back(l);
    }
    for (uint32_t s : small) prob[s] = 1.f;
    for (uint32_t l : large) prob[l] = 1.f;
}

// Spatial CDF = running sum of the capture over scan points (what the
// reference's inclusive scan + spatioTemporalPrefixSum produce when applied to
// the capture), min-max normalised (Laser.cu:574), then buildAliasTables.
static fbp_status reference_tables(const std::vector<double>& raw, std::vector<float>& cdf,
                                   std::vector<uint32_t>& alias, std::vector<float>& prob) {
    const size_t L = raw.size();
    cdf.resize(L);
    double run = 0.0;
    for (size_t l = 0; l < L; ++l) cdf[l] = (float)(run += raw[l]);
    const float mn = *std::min_element(cdf.begin(), cdf.end()), mx = *std::max_element(cdf.begin(), cdf.end());
    const float d = mx - mn;
    const float r = (d > FBP_EPS || d < -FBP_EPS) ? 1.0f / d : 3.402823466e+38f;
    for (float& c : cdf) c = (c - mn) * r;
    const int rc = build_alias_reference(cdf, alias, prob);
    if (rc == 1) return set_error(FBP_ERR_INVALID_ARG, "MIS: negative scan-point probability");
    if (rc == 2) return set_error(FBP_ERR_INVALID_ARG, "MIS: scan-point probabilities do not sum to 1");
    return FBP_OK;
}

// Per-scan-point raw and thresholded totals, copied to the host.
template <typename S>
static fbp_status scan_totals(fbp_context* ctx, const void* cube, uint32_t L, uint32_t T, int tmaj, cudaStream_t s,
                              std::vector<double>& raw, std::vector<double>& thr, double** d_raw_out) {
    void* ws = nullptr;
    const size_t tot_bytes = (size_t)2 * L * sizeof(double);
    const size_t tab_bytes = (size_t)L * (3 * sizeof(float) + sizeof(uint32_t)) + 64;
    FBP_TRY(workspace(ctx, WS_MISC, tot_bytes + tab_bytes, s, &ws));
    double* d_raw = static_cast<double*>(ws);
    double* d_thr = d_raw + L;
    const unsigned tb = tmaj ? cdiv(L, 256) : cdiv((uint64_t)L * 32, 256);
    scan_totals_kernel<S><<<tb, 256, 0, s>>>(static_cast<const S*>(cube), L, T, tmaj, d_raw, d_thr);
    FBP_CHECK_LAUNCH(ctx, "scan_totals_kernel");
    raw.resize(L);
    thr.resize(L);
    FBP_TRY_CUDA(cudaMemcpyAsync(raw.data(), d_raw, L * sizeof(double), cudaMemcpyDeviceToHost, s));
    FBP_TRY_CUDA(cudaMemcpyAsync(thr.data(), d_thr, L * sizeof(double), cudaMemcpyDeviceToHost, s));
    FBP_TRY_CUDA(cudaStreamSynchronize(s));
    *d_raw_out = d_raw;
    return FBP_OK;
}

template <typename T>
static fbp_status upload(fbp_context* ctx, int slot, const std::vector<T>& h, cudaStream_t s, T** d, size_t offset = 0) {
    (void)ctx;
    (void)slot;
    (void)offset;
    FBP_TRY_CUDA(cudaMemcpyAsync(*d, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, s));
    return FBP_OK;
}

// Control variate of the cluster estimator: the capture summed over cv x cv
// blocks of scan points (values above EPS only, as the gathers skip the
// rest), one "virtual" scan point per block at the block's mean position.
// vcube is time innermost [Gv][T] FP32.  Grid (Gv, ceil(T / 256)).
template <typename S>
__global__ void virtual_capture_kernel(const S* __restrict__ cube, int time_major, uint32_t L, uint32_t T,
                                       uint32_t n_side, uint32_t cv, const float* __restrict__ lxyz,
                                       float* __restrict__ vcube, float* __restrict__ vxyz) {
    const uint32_t m = n_side / cv;
    const uint32_t g = blockIdx.x, gx = g % m, gz = g / m;
    const uint32_t t = blockIdx.y * blockDim.x + threadIdx.x;
    if (t < T) {
        float acc = 0.f;
        for (uint32_t iz = 0; iz < cv; ++iz)
            for (uint32_t ix = 0; ix < cv; ++ix) {
                const uint64_t l = (uint64_t)(gz * cv + iz) * n_side + gx * cv + ix;
                const float v = to_f32(time_major ? cube[(uint64_t)t * L + l] : cube[l * T + t]);
                if (v > FBP_EPS) acc += v;
            }
        vcube[(uint64_t)g * T + t] = acc;
    }
    if (blockIdx.y == 0 && threadIdx.x == 0) {
        float sx = 0.f, sy = 0.f, sz = 0.f;
        for (uint32_t iz = 0; iz < cv; ++iz)
            for (uint32_t ix = 0; ix < cv; ++ix) {
                const uint64_t l = (uint64_t)(gz * cv + iz) * n_side + gx * cv + ix;
                sx += lxyz[3 * l];
                sy += lxyz[3 * l + 1];
                sz += lxyz[3 * l + 2];
            }
        const float inv = 1.f / (float)(cv * cv);
        vxyz[3 * g] = sx * inv;
        vxyz[3 * g + 1] = sy * inv;
        vxyz[3 * g + 2] = sz * inv;
    }
}

// volume = volume + a - b
__global__ void cv_combine_kernel(float* __restrict__ vol, const float* __restrict__ a, const float* __restrict__ b,
                                  uint64_t n) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        vol[i] = (vol[i] + a[i]) - b[i];
}

// FBP_MIS_LEARNED: whole clusters per tile; with cv_side, the estimator is
// BP(virtual capture) + sum over the chosen clusters of (real - virtual)
// contributions, weighted hits / (K p_c): unbiased for the full
// backprojection, with the variance of the residual only.
template <typename S>
static fbp_status mis_clusters(fbp_context* ctx, const fbp_recon_info& in, const void* cube, int layout,
                               const float* laser_xyz, const fbp_mis_params& prm, float* volume, cudaStream_t s) {
    const uint32_t L = in.num_laser_targets, T = in.num_time_bins;
    if (prm.cluster_side == 0 || prm.scan_side == 0 || (uint64_t)prm.scan_side * prm.scan_side != L)
        return set_error(FBP_ERR_INVALID_ARG, "fbp_mis_backproject: cluster sampling needs a square scan grid");
    if (prm.samples == 0) return set_error(FBP_ERR_INVALID_ARG, "fbp_mis_backproject: samples must be > 0");
    if (prm.samples > kMaxClusterSamples)
        return set_error(FBP_ERR_UNSUPPORTED, "fbp_mis_backproject: at most 256 cluster samples per tile");
    const uint32_t cpr = (prm.scan_side + prm.cluster_side - 1) / prm.cluster_side;
    SampleParams smp{};
    smp.mode = SAMPLE_CLUSTERS;
    smp.K = prm.samples;
    smp.seed = prm.seed;
    smp.tile_cdf = prm.tile_cluster_cdf;
    smp.G = cpr * cpr;
    smp.cluster_side = prm.cluster_side;
    smp.n_side = prm.scan_side;
    if (prm.cv_side == 0) return confocal_gather(ctx, in, cube, dtype_of<S>(), layout, laser_xyz, volume, s, &smp);

    const uint32_t cv = prm.cv_side;
    if (prm.scan_side % cv != 0 || prm.cluster_side % cv != 0)
        return set_error(FBP_ERR_INVALID_ARG, "fbp_mis_backproject: cv_side must divide scan_side and cluster_side");
    const uint32_t m = prm.scan_side / cv, Gv = m * m;
    const uint64_t V = (uint64_t)in.voxel_res[0] * in.voxel_res[1] * in.voxel_res[2];
    const size_t vc_bytes = ((size_t)Gv * T * sizeof(float) + 255) & ~size_t(255);
    const size_t vx_bytes = ((size_t)Gv * 3 * sizeof(float) + 255) & ~size_t(255);
    const size_t vol_bytes = ((size_t)V * sizeof(float) + 255) & ~size_t(255);
    void* ws = nullptr;
    FBP_TRY(workspace(ctx, WS_MIS_VIRTUAL, vc_bytes + vx_bytes + 2 * vol_bytes, s, &ws));
    float* vcube = static_cast<float*>(ws);
    float* vxyz = reinterpret_cast<float*>(static_cast<char*>(ws) + vc_bytes);
    float* tmp_a = reinterpret_cast<float*>(static_cast<char*>(ws) + vc_bytes + vx_bytes);
    float* tmp_b = reinterpret_cast<float*>(static_cast<char*>(ws) + vc_bytes + vx_bytes + vol_bytes);
    virtual_capture_kernel<S><<<dim3(Gv, cdiv(T, 256)), 256, 0, s>>>(static_cast<const S*>(cube),
                                                                    layout == FBP_LAYOUT_TIME_MAJOR, L, T,
                                                                    prm.scan_side, cv, laser_xyz, vcube, vxyz);
    FBP_CHECK_LAUNCH(ctx, "virtual_capture_kernel");
    fbp_recon_info vin = in;
    vin.num_laser_targets = Gv;
    vin.num_sensor_targets = Gv;
    FBP_TRY(confocal_gather(ctx, vin, vcube, FBP_F32, FBP_LAYOUT_TIME_INNER, vxyz, volume, s, nullptr));
    FBP_TRY(confocal_gather(ctx, in, cube, dtype_of<S>(), layout, laser_xyz, tmp_a, s, &smp));
    SampleParams vs = smp;  // the same clusters (same seed, tiles, CDF) of the virtual grid
    vs.cluster_side = prm.cluster_side / cv;
    vs.n_side = m;
    FBP_TRY(confocal_gather(ctx, vin, vcube, FBP_F32, FBP_LAYOUT_TIME_INNER, vxyz, tmp_b, s, &vs));
    cv_combine_kernel<<<std::min<uint64_t>(cdiv(V, 256), (uint64_t)ctx->sm_count * 8), 256, 0, s>>>(volume, tmp_a,
                                                                                                     tmp_b, V);
    FBP_CHECK_LAUNCH(ctx, "cv_combine_kernel");
    return FBP_OK;
}

template <typename S>
static fbp_status mis_run(fbp_context* ctx, const fbp_recon_info& in, const void* cube, int layout,
                          const float* laser_xyz, const fbp_mis_params& prm, float* volume, cudaStream_t s) {
    if (prm.proposal == FBP_MIS_LEARNED) return mis_clusters<S>(ctx, in, cube, layout, laser_xyz, prm, volume, s);
    const uint32_t L = in.num_laser_targets, T = in.num_time_bins;
    const int tmaj = layout == FBP_LAYOUT_TIME_MAJOR;
    // Per-scan-point totals (device -> host): the proposal is built on the host
    // like the reference's alias tables.
    std::vector<double> raw, thr;
    double* d_raw = nullptr;
    FBP_TRY(scan_totals<S>(ctx, cube, L, T, tmaj, s, raw, thr, &d_raw));
    double* d_thr = d_raw + L;
    char* tab = reinterpret_cast<char*>(d_thr + L);
    float* d_prob = reinterpret_cast<float*>(tab);
    float* d_pl = d_prob + L;
    float* d_spatial = d_pl + L;
    uint32_t* d_alias = reinterpret_cast<uint32_t*>(d_spatial + L);

    if (prm.proposal == FBP_MIS_REFERENCE || prm.proposal == FBP_MIS_REFERENCE_SCATTER) {
        std::vector<float> cdf, prob;
        std::vector<uint32_t> alias;
        FBP_TRY(reference_tables(raw, cdf, alias, prob));
        FBP_TRY(upload(ctx, 0, prob, s, &d_prob));
        FBP_TRY(upload(ctx, 0, cdf, s, &d_spatial));
        FBP_TRY(upload(ctx, 0, alias, s, &d_alias));
        FBP_TRY_CUDA(cudaStreamSynchronize(s));  // host tables are temporaries
        // Noise buffer (Laser.cu:541-545): caller's, or numVoxels uniforms from
        // a default-seeded std::mt19937 (libstdc++'s uniform_real_distribution).
        const uint64_t V = (uint64_t)in.voxel_res[0] * in.voxel_res[1] * in.voxel_res[2];
        const float* noise = prm.noise;
        uint64_t nn = prm.noise_size;
        if (!noise) {
            nn = V;
            void* nb = nullptr;
            FBP_TRY(workspace(ctx, WS_FILTER, nn * sizeof(float), s, &nb));
            std::vector<float> h(nn);
            std::mt19937 gen;
            std::uniform_real_distribution<float> dist(0.f, 1.f);
            for (auto& x : h) x = dist(gen);
            FBP_TRY_CUDA(cudaMemcpyAsync(nb, h.data(), nn * sizeof(float), cudaMemcpyHostToDevice, s));
            FBP_TRY_CUDA(cudaStreamSynchronize(s));
            noise = static_cast<const float*>(nb);
        }
        if (nn == 0 || nn > 0xffffffffull) return set_error(FBP_ERR_INVALID_ARG, "fbp_mis_backproject: bad noise size");
        const uint32_t pitch = (T + 7) / 8 * 8;
        void* rows = nullptr;
        FBP_TRY(workspace(ctx, WS_CUBE_ROWS, (size_t)L * pitch * sizeof(S), s, &rows));
        const uint64_t n = (uint64_t)L * pitch;
        mis_rows_kernel<S><<<(unsigned)std::min<uint64_t>(cdiv(n, 256), (uint64_t)ctx->sm_count * 16), 256, 0, s>>>(
            static_cast<S*>(rows), static_cast<const S*>(cube), L, T, pitch, tmaj);
        FBP_CHECK_LAUNCH(ctx, "mis_rows_kernel");
        MisRefParams p{};
        FBP_TRY(build_tables(ctx, in, laser_xyz, s, &p.scan, &p.xs, &p.ys, &p.zs));
        p.rows = rows;
        p.pitch = pitch;
        p.noise = noise;
        p.noise_size = (uint32_t)nn;
        p.spatial = d_spatial;
        p.alias = d_alias;
        p.prob = d_prob;
        p.Vx = in.voxel_res[0]; p.Vy = in.voxel_res[1]; p.Vz = in.voxel_res[2];
        p.L = L; p.T = T;
        p.samples = prm.samples ? prm.samples : L / 4;  // Laser.cu:590
        p.t0 = in.time_offset;
        p.dt = in.time_step;
        p.bounce = in.discard_first_last_bounces == 0;
        p.volume = volume;
        for (int k = 0; k < 3; ++k) p.vs[k] = in.voxel_size[k];
        if (prm.proposal == FBP_MIS_REFERENCE_SCATTER) {
            if (!(in.time_step > 1e-4f))
                return set_error(FBP_ERR_UNSUPPORTED, "fbp_mis_backproject: the scattering walk needs time_step > 0.1 mm");
            mis_reference_kernel<S, true><<<cdiv(V, kMisVoxels), kMisVoxels, 0, s>>>(p);
        } else {
            mis_reference_kernel<S, false><<<cdiv(V, kMisVoxels), kMisVoxels, 0, s>>>(p);
        }
        FBP_CHECK_LAUNCH(ctx, "mis_reference_kernel");
        return FBP_OK;
    }

    SampleParams smp{};
    smp.K = prm.samples;
    smp.seed = prm.seed;
    if (smp.K == 0) return set_error(FBP_ERR_INVALID_ARG, "fbp_mis_backproject: samples must be > 0");
    if (prm.proposal == FBP_MIS_UNIFORM) {
        smp.mode = SAMPLE_UNIFORM;
    } else if (prm.proposal == FBP_MIS_SPATIAL) {
        double sum = 0.0;
        for (double t : thr) sum += t;
        if (!(sum > 0.0)) {  // empty capture: the estimate is zero everywhere
            FBP_TRY_CUDA(cudaMemsetAsync(volume, 0, (size_t)in.voxel_res[0] * in.voxel_res[1] * in.voxel_res[2] * 4, s));
            return FBP_OK;
        }
        std::vector<double> pd(L);
        std::vector<float> pl(L);
        for (uint32_t l = 0; l < L; ++l) {
            pd[l] = thr[l] / sum;
            pl[l] = (float)pd[l];
        }
        std::vector<uint32_t> alias;
        std::vector<float> prob;
        build_alias_double(pd, alias, prob);
        FBP_TRY(upload(ctx, 0, prob, s, &d_prob));
        FBP_TRY(upload(ctx, 0, pl, s, &d_pl));
        FBP_TRY(upload(ctx, 0, alias, s, &d_alias));
        smp.mode = SAMPLE_ALIAS;
        smp.prob = d_prob;
        smp.alias = d_alias;
        smp.pl = d_pl;
        FBP_TRY_CUDA(cudaStreamSynchronize(s));  // host tables are temporaries
    } else {
        return set_error(FBP_ERR_INVALID_ARG, "fbp_mis_backproject: unknown proposal");
    }
    return confocal_gather(ctx, in, cube, dtype_of<S>(), layout, laser_xyz, volume, s, &smp);
}

}  // namespace fbp

using namespace fbp;

template <typename S>
static fbp_status tables_run(fbp_context* ctx, const fbp_recon_info& in, const void* cube, int layout, float* spatial,
                             uint32_t* alias, float* prob, cudaStream_t s) {
    std::vector<double> raw, thr;
    double* d_raw = nullptr;
    FBP_TRY(scan_totals<S>(ctx, cube, in.num_laser_targets, in.num_time_bins, layout == FBP_LAYOUT_TIME_MAJOR, s, raw,
                           thr, &d_raw));
    std::vector<float> c, p;
    std::vector<uint32_t> a;
    FBP_TRY(reference_tables(raw, c, a, p));
    std::copy(c.begin(), c.end(), spatial);
    std::copy(a.begin(), a.end(), alias);
    std::copy(p.begin(), p.end(), prob);
    return FBP_OK;
}

extern "C" fbp_status fbp_mis_reference_tables(fbp_context* ctx, const fbp_recon_info* info, const void* cube,
                                               int dtype, int layout, float* spatial_cdf, uint32_t* alias, float* prob,
                                               void* stream) {
    return guarded("fbp_mis_reference_tables", [&]() -> fbp_status {
        clear_error();
        FBP_TRY(check_ctx(ctx));
        FBP_TRY(validate_info(info, false, "fbp_mis_reference_tables"));
        if (!cube || !spatial_cdf || !alias || !prob)
            return set_error(FBP_ERR_INVALID_ARG, "fbp_mis_reference_tables: null argument");
        cudaStream_t s = (cudaStream_t)stream;
        switch (dtype) {
            case FBP_F32: return tables_run<float>(ctx, *info, cube, layout, spatial_cdf, alias, prob, s);
            case FBP_BF16: return tables_run<__nv_bfloat16>(ctx, *info, cube, layout, spatial_cdf, alias, prob, s);
            case FBP_F16: return tables_run<__half>(ctx, *info, cube, layout, spatial_cdf, alias, prob, s);
            default: return set_error(FBP_ERR_INVALID_ARG, "fbp_mis_reference_tables: unknown dtype");
        }
    });
}

extern "C" fbp_status fbp_mis_tile_grid(const fbp_recon_info* info, uint32_t tiles[3]) {
    return guarded("fbp_mis_tile_grid", [&]() -> fbp_status {
        clear_error();
        if (!info || !tiles) return set_error(FBP_ERR_INVALID_ARG, "fbp_mis_tile_grid: null argument");
        confocal_tile_grid(*info, tiles);
        return FBP_OK;
    });
}

extern "C" fbp_status fbp_mis_backproject(fbp_context* ctx, const fbp_recon_info* info, const void* cube, int dtype,
                                          int layout, const float* laser_xyz, const fbp_mis_params* params,
                                          float* volume, void* stream) {
    return guarded("fbp_mis_backproject", [&]() -> fbp_status {
        clear_error();
        FBP_TRY(check_ctx(ctx));
        FBP_TRY(validate_info(info, false, "fbp_mis_backproject"));
        if (!cube || !laser_xyz || !params || !volume)
            return set_error(FBP_ERR_INVALID_ARG, "fbp_mis_backproject: null argument");
        if (layout != FBP_LAYOUT_TIME_MAJOR && layout != FBP_LAYOUT_TIME_INNER)
            return set_error(FBP_ERR_INVALID_ARG, "fbp_mis_backproject: unknown layout");
        cudaStream_t s = (cudaStream_t)stream;
        switch (dtype) {
            case FBP_F32: return mis_run<float>(ctx, *info, cube, layout, laser_xyz, *params, volume, s);
            case FBP_BF16: return mis_run<__nv_bfloat16>(ctx, *info, cube, layout, laser_xyz, *params, volume, s);
            case FBP_F16: return mis_run<__half>(ctx, *info, cube, layout, laser_xyz, *params, volume, s);
            default: return set_error(FBP_ERR_INVALID_ARG, "fbp_mis_backproject: unknown dtype");
        }
    });
}
