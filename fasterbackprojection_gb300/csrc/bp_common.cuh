// Pieces shared by the backprojection gathers.
#pragma once

#include "fbp_internal.cuh"

namespace fbp {

// ------------------------------------------------------------- cp.async --

__device__ __forceinline__ void cp_async_16(void* smem_dst, const void* gmem_src) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem_dst);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem_src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// ------------------------------------------------------ confocal gather --

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
    const void* rows;    // [L][row_pitch] of the storage type

    // Bytes of per-chunk metadata in front of the window slots (16-byte aligned).
    __host__ __device__ static constexpr size_t meta_bytes(int ch) {
        return ((size_t)2 * ch * (sizeof(float4) + sizeof(float) + 2 * sizeof(int)) + 2 * sizeof(int) + 15) & ~size_t(15);
    }
};

// One staged chunk of scan points against a thread's KV voxels (consecutive
// along x, sharing the y/z offsets).  The per-pair sequence reproduces the
// reference's time-bin arithmetic exactly (see fbp_internal.cuh); the bin then
// indexes the scan point's staged window, whose element slot_w is zero.
template <typename S, int KV, bool BOUNCE, bool EXACT_TRUNC, bool SAFE>
__device__ __forceinline__ void confocal_chunk(const float4* __restrict__ geo, const float* __restrict__ clv,
                                               const S* __restrict__ slots, uint32_t slot_stride, uint32_t slot_w,
                                               int nl, const float (&px)[KV], float py, float pz, float neg_t0,
                                               float rcp_dt, float (&acc)[KV]) {
#pragma unroll 2
    for (int i = 0; i < nl; ++i) {
        const float4 g = geo[i];
        const float c = clv[i];
        const S* slot = slots + (size_t)i * slot_stride;
        const float dy = sub_rn(py, g.y), dz = sub_rn(pz, g.z);
        const float dy2 = mul_rn(dy, dy);
#pragma unroll
        for (int k = 0; k < KV; ++k) {
            const float dx = sub_rn(px[k], g.x);
            const float q = fma_rn(dz, dz, fma_rn(dx, dx, dy2));
            const float d = sqrt_approx(q);
            float dist = fma_rn(d, 2.f, neg_t0);
            if (BOUNCE) dist = add_rn(dist, g.w);
            const float x = ref_bin_ratio(dist, rcp_dt);
            uint32_t idx;
            if (EXACT_TRUNC) {
                const int b = __float2int_rz(x);  // static_cast<int>, like the reference
                idx = min((uint32_t)(b - __float_as_int(c)), slot_w);
            } else {
                // x >= 0 here: round-toward-zero add of 2^23 - a leaves
                // floor(x) - a in the low mantissa bits.
                const float y = add_rz(x, c);
                idx = min(__float_as_uint(y) - 0x4B000000u, slot_w);
            }
            const float I = to_f32(slot[idx]);
            const float dd = mul_rn(dist, dist);
            const float w = SAFE ? ref_safe_rcp(dd) : rcp_approx(dd);
            acc[k] = fmaf(I, w, acc[k]);
        }
    }
}

// Window geometry shared by the gathers: the widest bin span a tile of the
// given world extents can need, capped at the whole row (T bins plus one
// alignment step), the padded row pitch, and the stage size that fits the
// shared-memory budget.
struct WindowPlan {
    uint32_t slot_w, pitch;
    int ch;
    size_t smem;
};
fbp_status plan_window(const fbp_context* ctx, double ex, double ey, double ez, double time_step, uint32_t T, int align,
                       size_t elem_bytes, size_t meta_bytes, WindowPlan* out, const char* who);

// Shared host helpers.
fbp_status build_tables(fbp_context* ctx, const fbp_recon_info& in, const float* laser_xyz, cudaStream_t stream,
                        const float4** scan, const float** xs, const float** ys, const float** zs);
fbp_status validate_info(const fbp_recon_info* info, bool need_sensors, const char* who);

__global__ void scan_table_kernel(float4* __restrict__ out, const float* __restrict__ xyz, uint32_t n, int discard,
                                  float ax, float ay, float az, float bx, float by, float bz, int confocal_pair);

}  // namespace fbp
