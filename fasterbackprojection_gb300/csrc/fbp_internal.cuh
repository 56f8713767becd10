// Internal declarations shared by the libfbp translation units.
#pragma once

#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cstdint>
#include <cstddef>
#include <exception>
#include <new>
#include <string>

#include "../../include/fbp.h"

namespace fbp {

// ---------------------------------------------------------------- errors --

// Records `msg` as this thread's last error and returns `st`.
fbp_status set_error(fbp_status st, const std::string& msg);
fbp_status cuda_error(cudaError_t e, const char* what);
void clear_error();

// The body of a C entry point: no C++ exception may cross the C ABI.  A host
// allocation failure becomes FBP_ERR_OOM, anything else FBP_ERR_INTERNAL,
// with the message in fbp_last_error() (when there is memory left to keep it).
fbp_status fail_quietly(fbp_status st, const char* who, const char* what) noexcept;
// check_ctx makes the context's device current for the call; this puts the
// caller's device back (a no-op when check_ctx did not switch).
void restore_device() noexcept;
template <typename Body>
fbp_status guarded(const char* who, Body&& body) noexcept {
    fbp_status st;
    try {
        st = body();
    } catch (const std::bad_alloc&) {
        st = fail_quietly(FBP_ERR_OOM, who, "host allocation failed");
    } catch (const std::exception& e) {
        st = fail_quietly(FBP_ERR_INTERNAL, who, e.what());
    } catch (...) {
        st = fail_quietly(FBP_ERR_INTERNAL, who, "unknown exception");
    }
    restore_device();
    return st;
}

#define FBP_TRY_CUDA(expr)                                               \
    do {                                                                 \
        cudaError_t e_ = (expr);                                         \
        if (e_ != cudaSuccess) return ::fbp::cuda_error(e_, #expr);      \
    } while (0)

#define FBP_TRY(expr)                          \
    do {                                       \
        fbp_status s_ = (expr);                \
        if (s_ != FBP_OK) return s_;           \
    } while (0)

#define FBP_CHECK_LAUNCH(ctx, name)                                      \
    do {                                                                 \
        cudaError_t e_ = cudaGetLastError();                             \
        if (e_ != cudaSuccess) return ::fbp::cuda_error(e_, name);       \
        (ctx)->launches++;                                               \
    } while (0)

// --------------------------------------------------------------- context --

// Grow-only device scratch.  Slots are independent so one entry point can hold
// several buffers at once; growing synchronises the stream first so no
// in-flight kernel still reads the old allocation.
enum WorkspaceSlot {
    WS_CUBE_ROWS = 0,   // padded, thresholded scan-point rows for the gathers
    WS_SCAN_TABLE,      // per scan point (x, y, z, bounce)
    WS_SENSOR_TABLE,    // per SPAD point (x, y, z, bounce)
    WS_AXIS_TABLES,     // voxel-centre coordinates per axis
    WS_POINTS,          // explicit point sets (depth planes)
    WS_PARTIALS,        // per-block partial results (reductions)
    WS_FILTER,          // post-filter / temporal-filter temporaries
    WS_FFT_A,
    WS_FFT_B,
    WS_FFT_C,
    WS_LCT_OPERATOR,    // resampling operator CSR (mtx and its transpose)
    WS_MISC,
    WS_HOST_STAGING_IN, // device copies for the host-buffer entry points
    WS_HOST_STAGING_OUT,
    WS_HOST_STAGING_AUX,
    WS_HOST_STAGING_AUX2,
    WS_MLP_PROFILES,    // learned proposal: pooled cluster profiles, centres, scale
    WS_MLP_PARTIALS,    // learned proposal: per-CTA gradient partials
    WS_MIS_VIRTUAL,     // cluster MIS control variate: virtual capture + two partial volumes
    WS_NUM_SLOTS
};

}  // namespace fbp

struct fbp_context {
    int device = 0;
    int sm_count = 0;
    int smem_optin = 0;
    void* ws[fbp::WS_NUM_SLOTS] = {};
    size_t ws_bytes[fbp::WS_NUM_SLOTS] = {};
    int* status_dev = nullptr;  // device status word: 0 ok, else an fbp_status
    int weight_mode = FBP_WEIGHTS_BATCHED;  // fbp_weight_mode of the gathers
    uint64_t launches = 0;
    // FFT twiddle tables, one per power-of-two length (index log2 n): the
    // half table exp(-2 pi i k / n) and the per-pass tables of the LCT kernels.
    void* twiddles[16] = {};
    void* stage_twiddles[16] = {};
    // Cached LCT plan: Wiener filter of the PSF and the resampling operator
    // for the last (N, M, slope, snr) seen; valid while lct_key_valid.
    bool lct_key_valid = false;
    uint32_t lct_N = 0, lct_M = 0;
    double lct_slope = 0.0, lct_snr = 0.0;
    size_t lct_nnz = 0;
};

namespace fbp {

// Makes ctx's device (or `device`) current for the rest of the call; the
// guard of the entry point (guarded) restores the caller's device afterwards.
fbp_status check_ctx(fbp_context* ctx);
fbp_status use_device(int device);
// Returns a device buffer of at least `bytes` in slot `slot`.
fbp_status workspace(fbp_context* ctx, int slot, size_t bytes, cudaStream_t stream, void** out);

inline unsigned cdiv(uint64_t a, uint64_t b) { return (unsigned)((a + b - 1) / b); }

// ---------------------------------------------------- element conversion --

template <typename T> __device__ __forceinline__ float to_f32(T v);
template <> __device__ __forceinline__ float to_f32<float>(float v) { return v; }
template <> __device__ __forceinline__ float to_f32<__nv_bfloat16>(__nv_bfloat16 v) { return __bfloat162float(v); }
template <> __device__ __forceinline__ float to_f32<__half>(__half v) { return __half2float(v); }

template <typename T> __device__ __forceinline__ T from_f32(float v);
template <> __device__ __forceinline__ float from_f32<float>(float v) { return v; }
template <> __device__ __forceinline__ __nv_bfloat16 from_f32<__nv_bfloat16>(float v) { return __float2bfloat16_rn(v); }
template <> __device__ __forceinline__ __half from_f32<__half>(float v) { return __float2half_rn(v); }

inline size_t dtype_size(int dtype) { return dtype == FBP_F32 ? 4 : 2; }
template <typename T> constexpr int dtype_of();
template <> constexpr int dtype_of<float>() { return FBP_F32; }
template <> constexpr int dtype_of<__nv_bfloat16>() { return FBP_BF16; }
template <> constexpr int dtype_of<__half>() { return FBP_F16; }

// ---------------------------------------------------- reference arithmetic --
//
// The reference kernels are built with fast math and FMA contraction
// (FasterBackprojection.vcxproj:66, 96).  The time-bin index
//     int(dist / timeStep),  dist = 2 * distance(l, p) - t0 (+ bounces)
// must be reproduced bit for bit, so the operations below pin each
// instruction explicitly instead of leaving the rounding sequence to the
// compiler: the square root, the division, and the FMA nesting of the dot
// product.  The sequence was matched black-box against the reference kernels
// compiled from the reference sources (bitwise-equal volumes on single-scan
// runs), see tests/test_ref_parity_gpu.py.

#define FBP_EPS 0.00001f  // math.cuh:11

__device__ __forceinline__ float sqrt_approx(float x) {
    float r;
    asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ float rcp_approx(float x) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ float div_full(float a, float b) {
    float r;
    asm("div.full.ftz.f32 %0, %1, %2;" : "=f"(r) : "f"(a), "f"(b));
    return r;
}
__device__ __forceinline__ float fma_rn(float a, float b, float c) {
    float r;
    asm("fma.rn.ftz.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
}
__device__ __forceinline__ float mul_rn(float a, float b) {
    float r;
    asm("mul.rn.ftz.f32 %0, %1, %2;" : "=f"(r) : "f"(a), "f"(b));
    return r;
}
__device__ __forceinline__ float add_rn(float a, float b) {
    float r;
    asm("add.rn.ftz.f32 %0, %1, %2;" : "=f"(r) : "f"(a), "f"(b));
    return r;
}
__device__ __forceinline__ float sub_rn(float a, float b) {
    float r;
    asm("sub.rn.ftz.f32 %0, %1, %2;" : "=f"(r) : "f"(a), "f"(b));
    return r;
}
// a + p (round to nearest) where x < y, else a unchanged: one compare and a
// predicated add.
__device__ __forceinline__ float add_rn_if_lt(float a, float p, float x, float y) {
    asm("{\n\t.reg .pred q;\n\tsetp.lt.f32 q, %2, %3;\n\t@q add.rn.ftz.f32 %0, %0, %1;\n\t}"
        : "+f"(a)
        : "f"(p), "f"(x), "f"(y));
    return a;
}
// add with round-toward-zero: used for the float->bin truncation trick.
__device__ __forceinline__ float add_rz(float a, float b) {
    float r;
    asm("add.rz.ftz.f32 %0, %1, %2;" : "=f"(r) : "f"(a), "f"(b));
    return r;
}

// Packed FP32 pairs (the f32x2 instructions of sm_100 and later): one
// instruction applies the scalar operation above to both halves, with the
// same rounding, so results are bitwise those of two scalar operations.
typedef unsigned long long f32x2_t;
__device__ __forceinline__ f32x2_t pack2(float lo, float hi) {
    f32x2_t r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
    return r;
}
__device__ __forceinline__ void unpack2(f32x2_t v, float& lo, float& hi) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
}
__device__ __forceinline__ f32x2_t sub_rn2(f32x2_t a, f32x2_t b) {
    f32x2_t r;
    asm("sub.rn.ftz.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ f32x2_t add_rn2(f32x2_t a, f32x2_t b) {
    f32x2_t r;
    asm("add.rn.ftz.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ f32x2_t mul_rn2(f32x2_t a, f32x2_t b) {
    f32x2_t r;
    asm("mul.rn.ftz.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ f32x2_t fma_rn2(f32x2_t a, f32x2_t b, f32x2_t c) {
    f32x2_t r;
    asm("fma.rn.ftz.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
    return r;
}
__device__ __forceinline__ f32x2_t add_rz2(f32x2_t a, f32x2_t b) {
    f32x2_t r;
    asm("add.rz.ftz.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
// a * b and fmaf (no flush to zero) on both halves.
__device__ __forceinline__ f32x2_t mulf2(f32x2_t a, f32x2_t b) {
    f32x2_t r;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ f32x2_t fmaf2(f32x2_t a, f32x2_t b, f32x2_t c) {
    f32x2_t r;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
    return r;
}

// |d|^2 of the difference vector with the reference's rounding sequence:
// the y product is rounded first, then x and z are fused in.
__device__ __forceinline__ float ref_dot3(float dx, float dy, float dz) {
    return fma_rn(dz, dz, fma_rn(dx, dx, mul_rn(dy, dy)));
}

// distance(a, b) as compiled in the reference.
__device__ __forceinline__ float ref_distance(float ax, float ay, float az, float bx, float by, float bz) {
    return sqrt_approx(ref_dot3(sub_rn(bx, ax), sub_rn(by, ay), sub_rn(bz, az)));
}

// One coordinate of a voxel centre: min + i * size + 0.5 * size
// (transient_reconstruction.cuh:106, contracted into two FMAs).
__device__ __forceinline__ float ref_voxel_coord(uint32_t i, float size, float mn) {
    return fma_rn(0.5f, size, fma_rn((float)i, size, mn));
}

// x = dist / timeStep as the reference's fast-math division computes it: the
// division equals dist * rcp.approx(timeStep), so the reciprocal is hoisted
// and passed in precomputed (rcp_dt = rcp_approx(timeStep)).
__device__ __forceinline__ float ref_bin_ratio(float dist, float rcp_dt) { return mul_rn(dist, rcp_dt); }

// safeRCP(x) (math.cuh:23-29) with the fast-math reciprocal.
__device__ __forceinline__ float ref_safe_rcp(float x) {
    if (x > FBP_EPS || x < -FBP_EPS) return rcp_approx(x);
    return x >= 0.f ? 3.402823466e+38f : -3.402823466e+38f;
}

}  // namespace fbp
