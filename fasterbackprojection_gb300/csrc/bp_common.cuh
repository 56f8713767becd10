// Pieces shared by the backprojection gathers.
#pragma once

#include "fbp_internal.cuh"

namespace fbp {

// ------------------------------------------------------------- cp.async --

__device__ __forceinline__ void cp_async_16(void* smem_dst, const void* gmem_src) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem_dst);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem_src) : "memory");
}
// One FP32 element of shared memory at a shared-state-space byte address.
__device__ __forceinline__ float lds_f32(uint32_t addr) {
    float v;
    asm volatile("ld.shared.f32 %0, [%1];" : "=f"(v) : "r"(addr));
    return v;
}

__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// ------------------------------------------------------ confocal gather --

// Scan-point sampling for the unbiased MIS estimator: each voxel tile draws
// K scan points i.i.d. from a proposal p(l | tile) and weights each pair by
// 1 / (K p(l | tile)), so sum_k f(v, l_k) / (K p(l_k)) is an unbiased estimate
// of the full backprojection sum at every voxel of the tile.
enum SampleMode { SAMPLE_UNIFORM = 0, SAMPLE_ALIAS = 1, SAMPLE_CLUSTERS = 2 };
// Cluster samples per tile (SAMPLE_CLUSTERS) and the static shared memory the
// sampled gather keeps for them.
constexpr uint32_t kMaxClusterSamples = 256;
constexpr size_t kSampledStaticSmem = kMaxClusterSamples * 8 + 64;
struct SampleParams {
    int mode;
    uint32_t K;              // samples per tile
    unsigned long long seed;
    const float* prob;       // SAMPLE_ALIAS: Vose tables over scan points
    const uint32_t* alias;
    const float* pl;         // SAMPLE_ALIAS: p(l)
    const float* tile_cdf;   // SAMPLE_CLUSTERS: [tiles][G] inclusive CDF over clusters (null: uniform)
    uint32_t G;              // clusters
    uint32_t cluster_side;   // scan points per cluster side
    uint32_t n_side;         // scan grid side (scan point l = iz * n_side + ix)
};

// Counter-based uniforms in [0, 1): a 64-bit mix of (seed, tile, k, stream).
__device__ __forceinline__ float hash_uniform(unsigned long long seed, unsigned long long tile, unsigned k, unsigned s) {
    unsigned long long x = seed ^ (tile * 0x9E3779B97F4A7C15ull) ^ ((unsigned long long)k << 32 | s) * 0xD1B54A32D192ED03ull;
    x ^= x >> 31;
    x *= 0x7FB5D329728EA185ull;
    x ^= x >> 27;
    x *= 0x81DADEF4BC2DD44Dull;
    x ^= x >> 33;
    return (float)(x >> 40) * (1.0f / 16777216.0f);
}

struct ConfocalGatherParams {
    const float4* scan;
    const float* xs;
    const float* ys;
    const float* zs;
    float* volume;
    int* status;
    uint32_t Vx, Vy, Vz, L, T;
    float t0, dt;
    uint32_t row_pitch;  // elements per padded row
    uint32_t slot_w;     // window width in elements (the sentinel zero sits at slot_w)
    int ch;              // scan points per pipeline stage (<= 32)
    const void* rows;    // [L][row_pitch] FP32
    SampleParams smp;    // used by the sampled (MIS) variant only
    float vs[3];         // voxel size (the voxel-scattering variant's extent)
    int exact_weights;   // 1: every weight by its own rcp.approx (FBP_WEIGHTS_REFERENCE)
    int scat_exact;      // voxel scattering: every walk is exactly the unrolled steps long (no tail loop)

    // Per scan point of a stage, in shared memory: (x, y, z, bounce), (bias,
    // slot address), the sample weight, three planning ints, and the packed
    // broadcast copies the pair loop reads as 64-bit register pairs:
    // (x, x, y, y), (z, z, bias, bias), (bounce, bounce, weight, weight).
    static constexpr int kPackedGeo = 3;
    // Bytes of per-chunk metadata in front of the window slots (16-byte aligned).
    __host__ __device__ static constexpr size_t meta_bytes(int ch) {
        return ((size_t)2 * ch * (sizeof(float4) * (1 + kPackedGeo) + sizeof(int2) + sizeof(float) + 3 * sizeof(int)) +
                2 * sizeof(int) + 15) &
               ~size_t(15);
    }
};

// Shared memory holding the compensated (Kahan) sums of a CTA's voxels when a
// thread owns 16 of them (sum and compensation per voxel, [2 KV][threads]):
// kept there instead of in 64 registers, so three CTAs fit per SM.
__host__ __device__ constexpr size_t kahan_smem_bytes(int kv, int threads) {
    return kv >= 16 ? (size_t)2 * kv * threads * sizeof(float) : 0;
}

// Window geometry shared by the gathers: the widest bin span a tile of the
// given world extents can need, capped at the whole row (T bins plus one
// alignment step), the padded row pitch, and the stage size that fits the
// shared-memory budget.
struct WindowPlan {
    uint32_t slot_w, pitch;
    int ch;
    bool capped;  // slot_w is the whole row: bins past a window must be clamped
    size_t smem;
};
fbp_status plan_window(const fbp_context* ctx, double ex, double ey, double ez, double time_step, uint32_t T, int align,
                       size_t elem_bytes, size_t meta_bytes, WindowPlan* out, const char* who,
                       double extra_path = 0.0);

// The confocal gather over all scan points (smp == nullptr) or over K sampled
// scan points per tile (the unbiased MIS estimator).
fbp_status confocal_gather_scatter(fbp_context* ctx, const fbp_recon_info& in, const void* cube, int dtype,
                                   int layout, const float* laser_xyz, float* volume, cudaStream_t s);
fbp_status confocal_gather_slab(fbp_context* ctx, const fbp_recon_info& in, const void* cube, int dtype, int layout,
                                const float* laser_xyz, uint32_t z_begin, uint32_t z_end, float* volume,
                                cudaStream_t s);
fbp_status confocal_gather(fbp_context* ctx, const fbp_recon_info& in, const void* cube, int dtype, int layout,
                           const float* laser_xyz, float* volume, cudaStream_t s, const SampleParams* smp);
void confocal_tile_grid(const fbp_recon_info& in, uint32_t out[3]);

// Padded, thresholded FP32 rows [L][pitch] of a confocal cube of storage type
// S (16-bit values widened exactly), written to dst.
template <typename S>
fbp_status prepare_rows_into(fbp_context* ctx, const void* cube, int layout, uint32_t L, uint32_t T, uint32_t pitch,
                             float* dst, cudaStream_t stream);

__global__ void axis_tables_kernel(float* __restrict__ xs, float* __restrict__ ys, float* __restrict__ zs,
                                   uint32_t Vx, uint32_t Vy, uint32_t Vz, float mnx, float mny, float mnz, float sx,
                                   float sy, float sz);

// Shared host helpers.
fbp_status build_tables(fbp_context* ctx, const fbp_recon_info& in, const float* laser_xyz, cudaStream_t stream,
                        const float4** scan, const float** xs, const float** ys, const float** zs);
fbp_status validate_info(const fbp_recon_info* info, bool need_sensors, const char* who);

__global__ void scan_table_kernel(float4* __restrict__ out, const float* __restrict__ xyz, uint32_t n, int discard,
                                  float ax, float ay, float az, float bx, float by, float bz, int confocal_pair);

}  // namespace fbp
