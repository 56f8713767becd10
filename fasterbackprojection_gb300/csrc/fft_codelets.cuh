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

// Shared-memory layout of a line: element j at pidx(j) = j + j/16 (one pad
// slot per 128 bytes breaks the power-of-two strides of the Stockham writes
// into different banks); lines are line_stride(n) = n + n/16 + 1 apart so the
// C lines of a strided-axis load land in different banks too.
__device__ __forceinline__ int pidx(int j) { return j + (j >> 4); }
__host__ __device__ constexpr int line_stride(int n) { return n + (n >> 4) + 1; }


}  // namespace fbp
