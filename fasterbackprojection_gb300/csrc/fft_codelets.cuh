// Complex arithmetic, small DFT codelets and the padded shared-memory line
// layout shared by the FFT kernels (fft.cu, lct_fused.cu).
#pragma once

#include <cuda_runtime.h>

namespace fbp {

__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// Complex add and subtract as one packed-pair instruction each (add / sub
// .rn.f32x2, sm_100 and later): the same round-to-nearest results as two
// scalar operations, half the instructions in the DFT codelets.
__device__ __forceinline__ float2 cadd(float2 a, float2 b) {
    float2 d;
    asm("{\n\t.reg .b64 pa, pb, pd;\n\t"
        "mov.b64 pa, {%2, %3};\n\tmov.b64 pb, {%4, %5};\n\t"
        "add.rn.f32x2 pd, pa, pb;\n\tmov.b64 {%0, %1}, pd;\n\t}"
        : "=f"(d.x), "=f"(d.y) : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return d;
}
__device__ __forceinline__ float2 csub(float2 a, float2 b) {
    float2 d;
    asm("{\n\t.reg .b64 pa, pb, pd;\n\t"
        "mov.b64 pa, {%2, %3};\n\tmov.b64 pb, {%4, %5};\n\t"
        "sub.rn.f32x2 pd, pa, pb;\n\tmov.b64 {%0, %1}, pd;\n\t}"
        : "=f"(d.x), "=f"(d.y) : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return d;
}
// a * (-i) forward, a * (+i) inverse
template <bool INV>
__device__ __forceinline__ float2 rot_mi(float2 a) { return INV ? make_float2(-a.y, a.x) : make_float2(a.y, -a.x); }

template <bool INV>
__device__ __forceinline__ void dft2(float2& a, float2& b) {
    const float2 t = a;
    a = cadd(t, b);
    b = csub(t, b);
}

template <bool INV>
__device__ __forceinline__ void dft4(float2& a, float2& b, float2& c, float2& d) {
    const float2 s0 = cadd(a, c), d0 = csub(a, c), s1 = cadd(b, d), d1 = rot_mi<INV>(csub(b, d));
    a = cadd(s0, s1);
    c = csub(s0, s1);
    b = cadd(d0, d1);
    d = csub(d0, d1);
}

template <bool INV>
__device__ __forceinline__ void dft8(float2* v) {
    // Even and odd halves, then the radix-2 combination with w8^k.
    dft4<INV>(v[0], v[2], v[4], v[6]);
    dft4<INV>(v[1], v[3], v[5], v[7]);
    constexpr float h = 0.70710678118654752f;  // sqrt(2) / 2
    const float2 o1 = INV ? make_float2(h * (v[3].x - v[3].y), h * (v[3].x + v[3].y))
                          : make_float2(h * (v[3].x + v[3].y), h * (v[3].y - v[3].x));
    const float2 o2 = rot_mi<INV>(v[5]);
    const float2 o3 = INV ? make_float2(-h * (v[7].x + v[7].y), h * (v[7].x - v[7].y))
                          : make_float2(h * (v[7].y - v[7].x), -h * (v[7].x + v[7].y));
    const float2 e0 = v[0], e1 = v[2], e2 = v[4], e3 = v[6], o0 = v[1];
    v[0] = cadd(e0, o0);
    v[4] = csub(e0, o0);
    v[1] = cadd(e1, o1);
    v[5] = csub(e1, o1);
    v[2] = cadd(e2, o2);
    v[6] = csub(e2, o2);
    v[3] = cadd(e3, o3);
    v[7] = csub(e3, o3);
}

// 16-point DFT as 4 x 4: n = n1 + 4 n2, k = k2 + 4 k1; DFT4 over n2 for
// every n1, twiddles w16^(n1 k2), DFT4 over n1 for every k2, then the
// transposition back to natural order.
template <bool INV>
__device__ __forceinline__ float2 cmul_const(float2 a, float c, float s) {  // a * (c + i s)
    return make_float2(a.x * c - a.y * s, a.x * s + a.y * c);
}
template <bool INV>
__device__ __forceinline__ void dft16(float2* v) {
#pragma unroll
    for (int n1 = 0; n1 < 4; ++n1) dft4<INV>(v[n1], v[n1 + 4], v[n1 + 8], v[n1 + 12]);
    constexpr float c1 = 0.92387953251128674f, s1 = 0.38268343236508977f, h = 0.70710678118654752f;
    constexpr float sg = INV ? 1.f : -1.f;  // sign of the imaginary parts of w16^k
    v[5] = cmul_const<INV>(v[5], c1, sg * s1);     // n1 = 1, k2 = 1: w^1
    v[9] = cmul_const<INV>(v[9], h, sg * h);       // n1 = 1, k2 = 2: w^2
    v[13] = cmul_const<INV>(v[13], s1, sg * c1);   // n1 = 1, k2 = 3: w^3
    v[6] = cmul_const<INV>(v[6], h, sg * h);       // n1 = 2, k2 = 1: w^2
    v[10] = rot_mi<INV>(v[10]);                     // n1 = 2, k2 = 2: w^4
    v[14] = cmul_const<INV>(v[14], -h, sg * h);    // n1 = 2, k2 = 3: w^6
    v[7] = cmul_const<INV>(v[7], s1, sg * c1);     // n1 = 3, k2 = 1: w^3
    v[11] = cmul_const<INV>(v[11], -h, sg * h);    // n1 = 3, k2 = 2: w^6
    v[15] = cmul_const<INV>(v[15], -c1, -sg * s1); // n1 = 3, k2 = 3: w^9
#pragma unroll
    for (int k2 = 0; k2 < 4; ++k2) dft4<INV>(v[4 * k2], v[4 * k2 + 1], v[4 * k2 + 2], v[4 * k2 + 3]);
    // v[k1 + 4 k2] holds X[k2 + 4 k1].
    float2 t[16];
#pragma unroll
    for (int i = 0; i < 16; ++i) t[i] = v[i];
#pragma unroll
    for (int k1 = 0; k1 < 4; ++k1)
#pragma unroll
        for (int k2 = 0; k2 < 4; ++k2) v[k2 + 4 * k1] = t[k1 + 4 * k2];
}

// Shared-memory layout of a line: element j at pidx(j) = j + j/16 (one pad
// slot per 128 bytes breaks the power-of-two strides of the Stockham writes
// into different banks); lines are line_stride(n) = n + n/16 + 1 apart so the
// C lines of a strided-axis load land in different banks too.
__device__ __forceinline__ int pidx(int j) { return j + (j >> 4); }
__host__ __device__ constexpr int line_stride(int n) { return n + (n >> 4) + 1; }


// buildLoGKernel3D (transient_postprocessing.cuh:116-148) at full-grid index (x, y, z).
__device__ __forceinline__ float log_response(int x, int y, int z, int nx, int ny, int nz, float sigma) {
    const float fx = (x <= nx / 2) ? (float)x : (float)(x - nx);
    const float fy = (y <= ny / 2) ? (float)y : (float)(y - ny);
    const float fz = (z <= nz / 2) ? (float)z : (float)(z - nz);
    const float fxn = fx / nx, fyn = fy / ny, fzn = fz / nz;
    const float k2 = fxn * fxn + fyn * fyn + fzn * fzn;
    const float pi = 3.14159265358979323846f;
    return -4.0f * pi * pi * k2 * expf(-2.0f * pi * pi * sigma * sigma * k2);
}

}  // namespace fbp
