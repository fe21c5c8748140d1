// Small float3/float4 helpers shared by the wavefront kernels.
// Host+device so the host-side scene preparation can use the same types.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#define VV_HD __host__ __device__ __forceinline__

VV_HD float3 f3(float x, float y, float z) { return make_float3(x, y, z); }
VV_HD float3 f3(float s) { return make_float3(s, s, s); }
VV_HD float3 f3(const float4 &v) { return make_float3(v.x, v.y, v.z); }
VV_HD float4 f4(const float3 &v, float w) { return make_float4(v.x, v.y, v.z, w); }

VV_HD float3 operator+(const float3 &a, const float3 &b) { return f3(a.x + b.x, a.y + b.y, a.z + b.z); }
VV_HD float3 operator-(const float3 &a, const float3 &b) { return f3(a.x - b.x, a.y - b.y, a.z - b.z); }
VV_HD float3 operator*(const float3 &a, const float3 &b) { return f3(a.x * b.x, a.y * b.y, a.z * b.z); }
VV_HD float3 operator/(const float3 &a, const float3 &b) { return f3(a.x / b.x, a.y / b.y, a.z / b.z); }
VV_HD float3 operator*(const float3 &a, float s) { return f3(a.x * s, a.y * s, a.z * s); }
VV_HD float3 operator*(float s, const float3 &a) { return f3(s * a.x, s * a.y, s * a.z); }
VV_HD float3 operator/(const float3 &a, float s) { return f3(a.x / s, a.y / s, a.z / s); }
VV_HD float3 operator-(const float3 &a) { return f3(-a.x, -a.y, -a.z); }
VV_HD float3 &operator+=(float3 &a, const float3 &b) { a = a + b; return a; }
VV_HD float3 &operator*=(float3 &a, const float3 &b) { a = a * b; return a; }
VV_HD float3 &operator*=(float3 &a, float s) { a = a * s; return a; }

VV_HD float dot3(const float3 &a, const float3 &b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
VV_HD float3 cross3(const float3 &a, const float3 &b)
{
    return f3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
VV_HD float length3(const float3 &a) { return sqrtf(dot3(a, a)); }
VV_HD float3 normalize3(const float3 &a) { return a * (1.0f / sqrtf(dot3(a, a))); }
VV_HD float max3f(const float3 &a) { return fmaxf(fmaxf(a.x, a.y), a.z); }
VV_HD float3 fmax3(const float3 &a, float s) { return f3(fmaxf(a.x, s), fmaxf(a.y, s), fmaxf(a.z, s)); }
VV_HD float3 clamp3(const float3 &a, float lo, float hi)
{
    return f3(fminf(fmaxf(a.x, lo), hi), fminf(fmaxf(a.y, lo), hi), fminf(fmaxf(a.z, lo), hi));
}
VV_HD float3 mix3(const float3 &a, const float3 &b, float t) { return a * (1.0f - t) + b * t; }
VV_HD float mixf(float a, float b, float t) { return a * (1.0f - t) + b * t; }
VV_HD bool is_black(const float3 &c) { return c.x == 0.0f && c.y == 0.0f && c.z == 0.0f; }
VV_HD bool is_black_eps(const float3 &c, float e)
{
    return fabsf(c.x) <= e && fabsf(c.y) <= e && fabsf(c.z) <= e;
}
VV_HD float comp(const float3 &v, int i) { return i == 0 ? v.x : (i == 1 ? v.y : v.z); }

// 3x4 affine transform stored as three rows (row-major, as VkTransformMatrixKHR).
struct Affine34 {
    float4 r0, r1, r2;
};
VV_HD float3 xform_point(const Affine34 &m, const float3 &p)
{
    return f3(m.r0.x * p.x + m.r0.y * p.y + m.r0.z * p.z + m.r0.w,
              m.r1.x * p.x + m.r1.y * p.y + m.r1.z * p.z + m.r1.w,
              m.r2.x * p.x + m.r2.y * p.y + m.r2.z * p.z + m.r2.w);
}
VV_HD float3 xform_vector(const Affine34 &m, const float3 &v)
{
    return f3(m.r0.x * v.x + m.r0.y * v.y + m.r0.z * v.z,
              m.r1.x * v.x + m.r1.y * v.y + m.r1.z * v.z,
              m.r2.x * v.x + m.r2.y * v.y + m.r2.z * v.z);
}
// v * M for the 3x3 part (row vector times matrix): transforms a normal by
// the transpose of M. With M = world-to-object this is the normal transform
// `localNormal * gl_WorldToObjectEXT` of shaders/pt/construct_frame.glsl:9.
VV_HD float3 xform_normal_transposed(const Affine34 &m, const float3 &n)
{
    return f3(n.x * m.r0.x + n.y * m.r1.x + n.z * m.r2.x,
              n.x * m.r0.y + n.y * m.r1.y + n.z * m.r2.y,
              n.x * m.r0.z + n.y * m.r1.z + n.z * m.r2.z);
}
