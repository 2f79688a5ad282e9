// devmath.cuh — FP32 vector / quaternion / 3x3 helpers for the device path.
// The formulas are those of the reference's Math library (Math/src/Vec3.h,
// Quaternion.h, Mat3.h) evaluated in FP32.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>

namespace cpgpu {

struct f3 { float x, y, z; };
struct M33 { float m[9]; };  // row-major

__device__ __forceinline__ f3 mk(float x, float y, float z) { return f3{x, y, z}; }
__device__ __forceinline__ f3 mk(float4 v) { return f3{v.x, v.y, v.z}; }
__device__ __forceinline__ f3 operator+(f3 a, f3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ f3 operator-(f3 a, f3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ f3 operator-(f3 a) { return mk(-a.x, -a.y, -a.z); }
__device__ __forceinline__ f3 operator*(f3 a, float d) { return mk(a.x * d, a.y * d, a.z * d); }
__device__ __forceinline__ f3 operator*(float d, f3 a) { return mk(a.x * d, a.y * d, a.z * d); }
__device__ __forceinline__ float dot(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ f3 cross(f3 a, f3 b) { return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
__device__ __forceinline__ float mag2(f3 a) { return a.x * a.x + a.y * a.y + a.z * a.z; }
__device__ __forceinline__ float mag(f3 a) { return sqrtf(a.x * a.x + a.y * a.y + a.z * a.z); }
__device__ __forceinline__ f3 normalize(f3 a) {
    float m = mag(a);
    return m == 0.f ? mk(0.f, 0.f, 0.f) : mk(a.x / m, a.y / m, a.z / m);
}
// Vec3::getPerpendicularBasis (Math/src/Vec3.h:53-57)
__device__ __forceinline__ void basis(f3 n, f3* u, f3* w) {
    f3 a1 = mk(1.f, 0.f, 0.f), a2 = mk(0.f, 1.f, 0.f);
    *u = (fabsf(dot(n, a1)) < fabsf(dot(n, a2))) ? normalize(cross(n, a1)) : normalize(cross(n, a2));
    *w = normalize(cross(n, *u));
}

__device__ __forceinline__ M33 quatRot(float4 q) {
    float r = q.x, i = q.y, j = q.z, k = q.w;
    M33 o;
    o.m[0] = r * r + i * i - j * j - k * k; o.m[1] = 2 * i * j - 2 * r * k;         o.m[2] = 2 * i * k + 2 * r * j;
    o.m[3] = 2 * i * j + 2 * r * k;         o.m[4] = r * r - i * i + j * j - k * k; o.m[5] = 2 * j * k - 2 * r * i;
    o.m[6] = 2 * i * k - 2 * r * j;         o.m[7] = 2 * j * k + 2 * r * i;         o.m[8] = r * r - i * i - j * j + k * k;
    return o;
}
__device__ __forceinline__ float4 qconj(float4 q) { return make_float4(q.x, -q.y, -q.z, -q.w); }
__device__ __forceinline__ float4 qmul(float4 a, float4 b) {
    return make_float4(a.x * b.x - a.y * b.y - a.z * b.z - a.w * b.w,
                       a.x * b.y + a.y * b.x + a.z * b.w - a.w * b.z,
                       a.x * b.z - a.y * b.w + a.z * b.x + a.w * b.y,
                       a.x * b.w + a.y * b.z - a.z * b.y + a.w * b.x);
}
__device__ __forceinline__ float4 qnormalize(float4 q) {
    float m = sqrtf(q.x * q.x + q.y * q.y + q.z * q.z + q.w * q.w);
    return make_float4(q.x / m, q.y / m, q.z / m, q.w / m);
}
// Quaternion(theta, axis) (Math/src/Quaternion.h:26-33)
__device__ __forceinline__ float4 qaxis(float theta, f3 axis) {
    axis = normalize(axis);
    float s, c;
    sincosf(theta / 2.0f, &s, &c);
    return make_float4(c, axis.x * s, axis.y * s, axis.z * s);
}
__device__ __forceinline__ f3 mul(const M33& a, f3 v) {
    return mk(a.m[0] * v.x + a.m[1] * v.y + a.m[2] * v.z,
              a.m[3] * v.x + a.m[4] * v.y + a.m[5] * v.z,
              a.m[6] * v.x + a.m[7] * v.y + a.m[8] * v.z);
}
__device__ __forceinline__ M33 mul(const M33& a, const M33& b) {
    M33 o;
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++) o.m[3 * i + j] = a.m[3 * i] * b.m[j] + a.m[3 * i + 1] * b.m[3 + j] + a.m[3 * i + 2] * b.m[6 + j];
    return o;
}
__device__ __forceinline__ M33 transpose(const M33& a) {
    M33 o;
    o.m[0] = a.m[0]; o.m[1] = a.m[3]; o.m[2] = a.m[6];
    o.m[3] = a.m[1]; o.m[4] = a.m[4]; o.m[5] = a.m[7];
    o.m[6] = a.m[2]; o.m[7] = a.m[5]; o.m[8] = a.m[8];
    return o;
}
__device__ __forceinline__ float det(const M33& a) {
    return a.m[0] * (a.m[4] * a.m[8] - a.m[5] * a.m[7]) - a.m[1] * (a.m[3] * a.m[8] - a.m[5] * a.m[6]) +
           a.m[2] * (a.m[3] * a.m[7] - a.m[4] * a.m[6]);
}
__device__ __forceinline__ M33 inverse(const M33& s) {
    float a = s.m[0], b = s.m[1], c = s.m[2], d = s.m[3], e = s.m[4], f = s.m[5], g = s.m[6], h = s.m[7], i = s.m[8];
    float dt = a * (e * i - f * h) - b * (d * i - f * g) + c * (d * h - e * g);
    M33 o;
    o.m[0] = (e * i - f * h) / dt; o.m[1] = (c * h - b * i) / dt; o.m[2] = (b * f - c * e) / dt;
    o.m[3] = (f * g - d * i) / dt; o.m[4] = (a * i - c * g) / dt; o.m[5] = (c * d - a * f) / dt;
    o.m[6] = (d * h - e * g) / dt; o.m[7] = (b * g - a * h) / dt; o.m[8] = (a * e - b * d) / dt;
    return o;
}
__device__ __forceinline__ M33 load9(const float* p) { M33 o; for (int i = 0; i < 9; i++) o.m[i] = p[i]; return o; }
__device__ __forceinline__ void store9(float* p, const M33& a) { for (int i = 0; i < 9; i++) p[i] = a.m[i]; }

}  // namespace cpgpu
