// Minimal vector-math subset used to compile the reference's CUDA kernel
// headers for the oracle harness.  Written for this project from the
// documented semantics of the types and functions the reference calls; no
// third-party source is reproduced.
//
// The one convention that matters numerically is the evaluation order of the
// geometric functions, which the harness treats as the definition:
//   dot(a, b)      = (a.x*b.x + a.y*b.y) + a.z*b.z   (products first, summed
//                    left to right, as a component-wise product then a sum)
//   length(v)      = sqrt(dot(v, v))
//   distance(p, q) = length(q - p)
// The upstream library is not vendored by the reference and no version is
// pinned, so this order is an assumption of the harness.
#pragma once

#include <cmath>
#include <cfloat>
#include <cstdint>

#if defined(__CUDACC__)
#define FBPH_QUAL __host__ __device__ __forceinline__
#else
#define FBPH_QUAL inline
#endif

namespace glm {

typedef unsigned int uint;

struct uvec3;
struct ivec3;

struct vec2 {
    float x, y;
    vec2() = default;
    FBPH_QUAL explicit vec2(float s) : x(s), y(s) {}
    FBPH_QUAL vec2(float a, float b) : x(a), y(b) {}
    FBPH_QUAL float& operator[](int i) { return i == 0 ? x : y; }
    FBPH_QUAL const float& operator[](int i) const { return i == 0 ? x : y; }
};

struct vec3 {
    float x, y, z;
    vec3() = default;  // trivial, so __constant__ objects of these types need no dynamic initialisation
    FBPH_QUAL explicit vec3(float s) : x(s), y(s), z(s) {}
    FBPH_QUAL vec3(float a, float b, float c) : x(a), y(b), z(c) {}
    // Mixed scalar constructor (e.g. three unsigned voxel indices): each
    // component converts on its own.
    template <typename A, typename B, typename C>
    FBPH_QUAL vec3(A a, B b, C c) : x(static_cast<float>(a)), y(static_cast<float>(b)), z(static_cast<float>(c)) {}
    FBPH_QUAL explicit vec3(const uvec3& u);
    FBPH_QUAL float& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
    FBPH_QUAL const float& operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
    FBPH_QUAL vec3& operator+=(const vec3& o) { x += o.x; y += o.y; z += o.z; return *this; }
    FBPH_QUAL vec3& operator-=(const vec3& o) { x -= o.x; y -= o.y; z -= o.z; return *this; }
    FBPH_QUAL vec3& operator*=(float s) { x *= s; y *= s; z *= s; return *this; }
    FBPH_QUAL vec3& operator/=(float s) { x /= s; y /= s; z /= s; return *this; }
};

struct uvec3 {
    uint x, y, z;
    uvec3() = default;
    FBPH_QUAL uvec3(uint s) : x(s), y(s), z(s) {}
    FBPH_QUAL uvec3(uint a, uint b, uint c) : x(a), y(b), z(c) {}
    FBPH_QUAL uint& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
    FBPH_QUAL const uint& operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};

struct ivec3 {
    int x, y, z;
    ivec3() = default;
    FBPH_QUAL ivec3(int a, int b, int c) : x(a), y(b), z(c) {}
};

struct uvec2 {
    uint x, y;
    uvec2() = default;
    FBPH_QUAL explicit uvec2(uint s) : x(s), y(s) {}
    FBPH_QUAL uvec2(uint a, uint b) : x(a), y(b) {}
};

struct vec4 {
    union { float x, r; };
    union { float y, g; };
    union { float z, b; };
    union { float w, a; };
    vec4() = default;
    FBPH_QUAL vec4(float p, float q, float s, float t) : x(p), y(q), z(s), w(t) {}
};

struct uvec4 {
    uint x, y, z, w;
    uvec4() = default;
    FBPH_QUAL uvec4(uint a, uint b, uint c, uint d) : x(a), y(b), z(c), w(d) {}
};

FBPH_QUAL bool operator==(const uvec2& a, const uvec2& b) { return a.x == b.x && a.y == b.y; }
FBPH_QUAL bool operator!=(const uvec2& a, const uvec2& b) { return !(a == b); }

FBPH_QUAL vec3::vec3(const uvec3& u) : x(static_cast<float>(u.x)), y(static_cast<float>(u.y)), z(static_cast<float>(u.z)) {}

// Component-wise arithmetic.
FBPH_QUAL vec3 operator+(const vec3& a, const vec3& b) { return vec3(a.x + b.x, a.y + b.y, a.z + b.z); }
FBPH_QUAL vec3 operator-(const vec3& a, const vec3& b) { return vec3(a.x - b.x, a.y - b.y, a.z - b.z); }
FBPH_QUAL vec3 operator*(const vec3& a, const vec3& b) { return vec3(a.x * b.x, a.y * b.y, a.z * b.z); }
FBPH_QUAL vec3 operator/(const vec3& a, const vec3& b) { return vec3(a.x / b.x, a.y / b.y, a.z / b.z); }
FBPH_QUAL vec3 operator*(float s, const vec3& a) { return vec3(s * a.x, s * a.y, s * a.z); }
FBPH_QUAL vec3 operator*(const vec3& a, float s) { return vec3(a.x * s, a.y * s, a.z * s); }
FBPH_QUAL vec3 operator/(const vec3& a, float s) { return vec3(a.x / s, a.y / s, a.z / s); }
FBPH_QUAL vec3 operator+(const vec3& a, float s) { return vec3(a.x + s, a.y + s, a.z + s); }
FBPH_QUAL vec3 operator-(const vec3& a, float s) { return vec3(a.x - s, a.y - s, a.z - s); }
FBPH_QUAL vec3 operator-(const vec3& a) { return vec3(-a.x, -a.y, -a.z); }
FBPH_QUAL vec2 operator*(const vec2& a, float s) { return vec2(a.x * s, a.y * s); }
FBPH_QUAL uvec2 operator*(const uvec2& a, uint s) { return uvec2(a.x * s, a.y * s); }

// Geometry: the evaluation order documented at the top of this file.
FBPH_QUAL float dot(const vec3& a, const vec3& b) {
    const vec3 t = a * b;
    return t.x + t.y + t.z;
}
FBPH_QUAL float length(const vec3& v) { return sqrtf(dot(v, v)); }
FBPH_QUAL float distance(const vec3& p0, const vec3& p1) { return length(p1 - p0); }
FBPH_QUAL vec3 normalize(const vec3& v) { return v * (1.0f / length(v)); }

template <typename T> FBPH_QUAL T max(T a, T b) { return a < b ? b : a; }
template <typename T> FBPH_QUAL T min(T a, T b) { return b < a ? b : a; }
template <typename T> FBPH_QUAL T clamp(T v, T lo, T hi) { return min(max(v, lo), hi); }
FBPH_QUAL float abs(float a) { return a < 0.f ? -a : a; }
FBPH_QUAL float sqrt(float a) { return sqrtf(a); }
FBPH_QUAL uint sqrt(uint a) { return static_cast<uint>(sqrtf(static_cast<float>(a))); }

template <typename T> FBPH_QUAL T pi() { return static_cast<T>(3.14159265358979323846264338327950288); }
template <typename T> FBPH_QUAL T epsilon() { return static_cast<T>(FLT_EPSILON); }
FBPH_QUAL bool epsilonEqual(float a, float b, float eps) { return abs(a - b) < eps; }

}  // namespace glm
