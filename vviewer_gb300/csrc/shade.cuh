// Device-side shading building blocks of the path tracer. Each function
// restates one function of the reference's GLSL includes (file:line given in
// the comment above it) with the same operation order and constants.
#pragma once
#include "scene_gpu.h"
#include "vmath.cuh"

namespace vvpt {

// shaders/include/constants.glsl:1-9
constexpr float kEps = 0.000001f;
constexpr float kPi = 3.14159265358979323846f;
constexpr float kInvPi = 0.31830988618379067154f;
constexpr float kInv4Pi = 0.079577472f;
constexpr float kPiOver2 = 1.57079632679489661923f;
constexpr float kPiOver4 = 0.78539816339744830961f;
// shaders/pt/defines_pt.glsl:9
constexpr uint32_t kRussianRouletteDepth = 3;

// ---- RNG: shaders/include/rng/rng_def.glsl:4-36 (Ray Tracing Gems II ch. 14)

__device__ __forceinline__ float rng_to_float(uint32_t x) { return __uint_as_float(0x3f800000u | (x >> 9)) - 1.0f; }
__device__ __forceinline__ uint32_t xorshift32(uint32_t &s)
{
    s ^= s << 13;
    s ^= s >> 17;
    s ^= s << 5;
    return s;
}
__device__ __forceinline__ float rand1(uint32_t &s) { return rng_to_float(xorshift32(s)); }
__host__ __device__ __forceinline__ uint32_t jenkins_hash(uint32_t x)
{
    x += x << 10;
    x ^= x >> 6;
    x += x << 3;
    x ^= x >> 11;
    x += x << 15;
    return x;
}
// pixelIdx = pixel.x * resolution.x + pixel.y, kept as in rng_def.glsl:33
__host__ __device__ __forceinline__ uint32_t init_rng(uint32_t px, uint32_t py, uint32_t resx, uint32_t frame)
{
    uint32_t pixel_idx = px * resx + py;
    return jenkins_hash(pixel_idx ^ jenkins_hash(frame));
}

// ---- Sampling warps: shaders/include/sampling.glsl:3-67

__device__ __forceinline__ float3 cosine_sample_hemisphere(float u0, float u1, float &pdf)
{
    float rx = 2.0f * u0 - 1.0f;
    float ry = 2.0f * u1 - 1.0f;
    float3 dir = f3(0.0f);
    if (rx != 0.0f || ry != 0.0f) {
        // one sine and one cosine for both wedges (shorter inlined code)
        const bool xw = fabsf(rx) > fabsf(ry);
        const float r = xw ? rx : ry;
        const float phi = xw ? kPiOver4 * (ry / rx) : kPiOver2 - kPiOver4 * (rx / ry);
        dir.x = r * cosf(phi);
        dir.z = r * sinf(phi);
    }
    dir.y = sqrtf(fmaxf(0.0f, 1.0f - dir.x * dir.x - dir.z * dir.z));
    pdf = kInvPi * dir.y;
    pdf = fmaxf(pdf, kEps);
    return dir;
}
__device__ __forceinline__ float cosine_hemisphere_pdf(float cos_theta) { return cos_theta * kInvPi; }
__device__ __forceinline__ float2 uniform_sample_triangle(float u0, float u1)
{
    const float a = sqrtf(1.0f - u0);
    return make_float2(1.0f - a, a * u1);
}
__device__ __forceinline__ float2 concentric_sample_disk(float u0, float u1)
{
    float ox = 2.0f * u0 - 1.0f, oy = 2.0f * u1 - 1.0f;
    if (ox == 0.0f && oy == 0.0f)
        return make_float2(0.0f, 0.0f);
    float theta, r;
    if (fabsf(ox) > fabsf(oy)) {
        r = ox;
        theta = kPiOver4 * (oy / ox);
    } else {
        r = oy;
        theta = kPiOver2 - kPiOver4 * (ox / oy);
    }
    return make_float2(r * cosf(theta), r * sinf(theta));
}

// ---- Frames: shaders/include/frame.glsl:7-88

struct Frame {
    float3 n, t, b;
};
// returns `flipped`
__device__ __forceinline__ bool fix_frame(Frame &f, const float3 &ray)
{
    bool flipped = false;
    if (dot3(f.n, ray) > 0.0f) {
        f.n = -f.n;
        f.t = -f.t;
        flipped = true;
    }
    f.n = normalize3(f.n);
    f.t = normalize3(f.t);
    if (fabsf(dot3(f.n, f.t)) > 0.999f) {
        f.b = fabsf(f.n.z) < 0.999f ? f3(0.0f, 0.0f, 1.0f) : f3(1.0f, 0.0f, 0.0f);
        f.t = cross3(f.b, f.n);
        f.b = cross3(f.n, f.t);
    } else {
        f.b = cross3(f.n, f.t);
        f.t = cross3(f.b, f.n);
    }
    return flipped;
}
__device__ __forceinline__ float3 local_to_world(const Frame &f, const float3 &v) { return f.t * v.x + f.n * v.y + f.b * v.z; }
__device__ __forceinline__ float3 world_to_local(const Frame &f, const float3 &v)
{
    return f3(dot3(v, f.t), dot3(v, f.n), dot3(v, f.b));
}
__device__ __forceinline__ void apply_normal_to_frame(Frame &f, const float3 &local_normal)
{
    float3 nw = local_to_world(f, local_normal);
    f.n = nw;
    f.t = cross3(f.n, f.b);
    f.b = cross3(f.t, f.n);
}
__device__ __forceinline__ void create_coordinate_system(const float3 &v1, float3 &v2, float3 &v3)
{
    if (fabsf(v1.x) > fabsf(v1.y))
        v2 = f3(-v1.z, 0.0f, v1.x) / sqrtf(v1.x * v1.x + v1.z * v1.z);
    else
        v2 = f3(0.0f, v1.z, -v1.y) / sqrtf(v1.y * v1.y + v1.z * v1.z);
    v3 = cross3(v1, v2);
}
// shaders/include/utils.glsl:10-14
__device__ __forceinline__ float3 normal_from_normal_map(const float3 &c)
{
    float3 N = c * 2.0f - f3(1.0f);
    return normalize3(f3(N.x, N.z, -N.y));
}

// ---- BRDFs: shaders/include/brdfs/common.glsl:3-49, pbrStandard.glsl:1-165

struct PBR {
    float3 albedo;
    float metallic;
    float roughness;
};
__device__ __forceinline__ float schlick_weight(float cos_theta)
{
    float m = fminf(fmaxf(1.0f - cos_theta, 0.0f), 1.0f);
    return (m * m) * (m * m) * m;
}
__device__ __forceinline__ float gtr2(float ndoth, float a)
{
    float a2 = a * a;
    float t = 1.0f + (a2 - 1.0f) * ndoth * ndoth;
    return a2 / (kPi * t * t);
}
__device__ __forceinline__ float smith_g_ggx(float ndotv, float alpha_g)
{
    float a = alpha_g * alpha_g;
    float b = ndotv * ndotv;
    return 1.0f / (fabsf(ndotv) + fmaxf(sqrtf(a + b - a * b), kEps));
}
__device__ __forceinline__ float3 eval_disney_diffuse(float ndotl, float ndotv, float ldoth, const PBR &p)
{
    float FL = schlick_weight(ndotl);
    float FV = schlick_weight(ndotv);
    float Fd90 = 0.5f + 2.0f * ldoth * ldoth * p.roughness;
    float Fd = mixf(1.0f, Fd90, FL) * mixf(1.0f, Fd90, FV);
    return (1.0f / kPi) * Fd * p.albedo;
}
__device__ __forceinline__ float3 eval_disney_microfacet(float ndotl, float ndotv, float ndoth, float ldoth, const PBR &p)
{
    float cdlum = 0.3f * p.albedo.x + 0.6f * p.albedo.y + 0.1f * p.albedo.z;
    float3 ctint = cdlum > 0.0f ? p.albedo / cdlum : f3(1.0f);
    const float specular = 0.5f, specular_tint = 0.0f;
    float3 cspec0 = mix3(specular * 0.08f * mix3(f3(1.0f), ctint, specular_tint), p.albedo, p.metallic);
    float a = fmaxf(0.001f, p.roughness * p.roughness);
    float Ds = gtr2(ndoth, a);
    float FH = schlick_weight(ldoth);
    float3 Fs = mix3(cspec0, f3(1.0f), FH);
    float Gs = smith_g_ggx(ndotl, a);
    Gs *= smith_g_ggx(ndotv, a);
    return Gs * Fs * Ds;
}
__device__ __forceinline__ float pdf_disney_microfacet(const float3 &wi, const float3 &wo, const PBR &p)
{
    if (!(wo.y > 0.0f))
        return 0.0f;
    if (!(wi.y > 0.0f))
        return 0.0f;
    float3 wh = normalize3(wo + wi);
    float ndoth = fmaxf(wh.y, kEps);
    float alpha2 = p.roughness * p.roughness;
    alpha2 *= alpha2;
    float cos2 = ndoth * ndoth;
    float denom = cos2 * (alpha2 - 1.0f) + 1.0f;
    if (denom == 0.0f)
        return 0.0f;
    float pdf_distribution = alpha2 * ndoth / (kPi * denom * denom);
    return pdf_distribution / (4.0f * dot3(wo, wh));
}
__device__ __forceinline__ float diffuse_sampling_ratio(const PBR &p)
{
    float d = fmaxf(1.0f - p.metallic, 0.1f);
    float g = fmaxf(1.0f - p.roughness, 0.1f);
    return d / (d + g);
}
__device__ __forceinline__ float3 eval_pbr(const PBR &p, const float3 &wi, const float3 &wo, const float3 &H)
{
    float ndotl = wi.y, ndotv = wo.y;
    if (ndotl < 0.0f || ndotv < 0.0f)
        return f3(0.0f);
    float ndoth = H.y;
    float ldoth = dot3(wi, H);
    float3 diffuse = eval_disney_diffuse(ndotl, ndotv, ldoth, p);
    float3 glossy = eval_disney_microfacet(ndotl, ndotv, ndoth, ldoth, p);
    return (diffuse * (1.0f - p.metallic) + glossy) * ndotl;
}
__device__ __forceinline__ float pdf_pbr(const float3 &wi, const float3 &wo, const PBR &p)
{
    float cos_theta = wi.y;
    if (cos_theta < 0.0f)
        return 0.0f;
    float pd = cosine_hemisphere_pdf(cos_theta);
    float pm = pdf_disney_microfacet(wi, wo, p);
    float r = diffuse_sampling_ratio(p);
    return pd * r + pm * (1.0f - r);
}
// samplePBRStandard (pbrStandard.glsl:188-214): draws u0,u1 then rnd
// The specular lobe's direction: a GGX half vector, mirrored.
__device__ __forceinline__ float3 ggx_sample_reflect(const float3 &wo, const PBR &p, float u0, float u1)
{
    float phi = (2.0f * kPi) * u1;
    float alpha = p.roughness * p.roughness;
    float tan2 = alpha * alpha * u0 / (1.0f - u0);
    float cos_theta = 1.0f / sqrtf(1.0f + tan2);
    float sin_theta = sqrtf(fmaxf(kEps, 1.0f - cos_theta * cos_theta));
    float3 wh = f3(sin_theta * cosf(phi), cos_theta, sin_theta * sinf(phi));
    if (!(wh.y > 0.0f))
        wh = wh * -1.0f;
    // reflect(-wo, wh) = -wo - 2 dot(wh, -wo) wh
    float3 I = -wo;
    return I - 2.0f * dot3(wh, I) * wh;
}

// The reference's sampling of the metallic/roughness BSDF: the diffuse lobe
// with probability diffuse_sampling_ratio, else the specular lobe; the
// returned pdf is the two-lobe pdf and F the BSDF (zero when the pdf is
// below kEps). The shading kernel draws the same numbers and makes the same
// choice with its surface code shared between Lambert and PBR surfaces.
__device__ __forceinline__ float3 sample_pbr(float3 &wi, const float3 &wo, float &pdf, const PBR &p, float u0, float u1,
                                             float rnd)
{
    pdf = 0.0f;
    wi = f3(0.0f);
    float r = diffuse_sampling_ratio(p);
    if (rnd <= r)
        wi = cosine_sample_hemisphere(u0, u1, pdf);
    else
        wi = ggx_sample_reflect(wo, p, u0, u1);
    float3 F = eval_pbr(p, wi, wo, normalize3(wi + wo));
    pdf = pdf_pbr(wi, wo, p);
    if (pdf < kEps)
        return f3(0.0f);
    return F;
}

// ---- MIS: shaders/pt/MIS.glsl:5-10
// When a square overflows (a light sample grazing the emitter's own plane,
// whose pdf carries d^2 / cos with cos near zero) the quotient would be
// inf / inf; the weight is then taken from the ratio of the pdfs, its limit.
// Finite squares give the reference's formula and rounding unchanged.
__device__ __forceinline__ float power_heuristic(float fpdf, float gpdf)
{
    float f = fpdf, g = gpdf;
    const float ff = f * f, gg = g * g;
    if (isinf(ff) || isinf(gg)) {
        if (isinf(f) || isinf(g))
            return isinf(g) ? (isinf(f) ? 0.5f : 0.0f) : 1.0f;
        const float r = g / f;
        return 1.0f / (1.0f + r * r);
    }
    return ff / (ff + gg);
}

// ---- Phase function: shaders/include/phaseFunctions.glsl:1-31
__device__ __forceinline__ float henyey_greenstein(float cos_theta, float g)
{
    float denom = 1.0f + g * g + 2.0f * g * cos_theta;
    return kInv4Pi * (1.0f - g * g) / (denom * sqrtf(denom));
}
__device__ __forceinline__ float hg_sample(const float3 &wo, float3 &wi, float u0, float u1, float g)
{
    float cos_theta;
    if (fabsf(g) < 1e-3f) {
        cos_theta = 1.0f - 2.0f * u0;
    } else {
        float sqr = (1.0f - g * g) / (1.0f + g - 2.0f * g * u0);
        cos_theta = -(1.0f + g * g - sqr * sqr) / (2.0f * g);
    }
    float sin_theta = sqrtf(fmaxf(0.0f, 1.0f - cos_theta * cos_theta));
    float phi = 2.0f * kPi * u1;
    float3 v1, v2;
    create_coordinate_system(wo, v1, v2);
    wi = sin_theta * cosf(phi) * v1 + sin_theta * sinf(phi) * v2 + cos_theta * wo;
    return henyey_greenstein(cos_theta, g);
}

// ---- Textures: bilinear, repeat addressing, LOD 0 (sampler of
// src/lib/vengine/vulkan/resources/VulkanTexture.cpp:219-230)

__device__ __forceinline__ float srgb_to_linear(float c)
{
    return c <= 0.04045f ? c / 12.92f : powf((c + 0.055f) / 1.055f, 2.4f);
}
// srgb_to_linear(k / 255) for the 256 values of an 8-bit channel, written by
// k_init_slots at the start of every render (the same expression, so the
// same bits as evaluating it per texel). A table read instead of three powf
// per texel keeps the shading kernels' code short: every texture lookup is
// inlined and fetches up to five texels.
// (VVPT_SRGB_LUT = 0 evaluates it per texel, for comparison.)
#ifndef VVPT_SRGB_LUT
#define VVPT_SRGB_LUT 1
#endif
__device__ float vvpt_srgb_lut[256];
__device__ __forceinline__ float4 texel(const SceneView &s, const DevTexture &t, int x, int y)
{
    size_t i = (size_t)y * t.width + (size_t)x;
    if (t.format == 2) {
        return __ldg(reinterpret_cast<const float4 *>(s.texels + t.offset) + i);
    }
    uchar4 c = __ldg(reinterpret_cast<const uchar4 *>(s.texels + t.offset) + i);
#if VVPT_SRGB_LUT
    if (t.format == 1)
        return make_float4(vvpt_srgb_lut[c.x], vvpt_srgb_lut[c.y], vvpt_srgb_lut[c.z], c.w / 255.0f);
    return make_float4(c.x / 255.0f, c.y / 255.0f, c.z / 255.0f, c.w / 255.0f);
#else
    float4 v = make_float4(c.x / 255.0f, c.y / 255.0f, c.z / 255.0f, c.w / 255.0f);
    if (t.format == 1) {
        v.x = srgb_to_linear(v.x);
        v.y = srgb_to_linear(v.y);
        v.z = srgb_to_linear(v.z);
    }
    return v;
#endif
}
__device__ __forceinline__ int wrap_repeat(int i, int n)
{
    int m = i % n;
    return m < 0 ? m + n : m;
}
__device__ __forceinline__ float4 tex2d(const SceneView &s, uint32_t index, float u, float v, bool clamp_v = false)
{
    if (index >= s.num_textures)
        return make_float4(1.0f, 1.0f, 1.0f, 1.0f);
    const DevTexture t = s.textures[index];
    if (t.width == 1 && t.height == 1)
        return texel(s, t, 0, 0);
    float x = u * (float)t.width - 0.5f;
    float y = v * (float)t.height - 0.5f;
    float fx = floorf(x), fy = floorf(y);
    float ax = x - fx, ay = y - fy;
    int x0 = (int)fx, y0 = (int)fy;
    int x1 = x0 + 1, y1 = y0 + 1;
    x0 = wrap_repeat(x0, (int)t.width);
    x1 = wrap_repeat(x1, (int)t.width);
    if (clamp_v) {
        y0 = min(max(y0, 0), (int)t.height - 1);
        y1 = min(max(y1, 0), (int)t.height - 1);
    } else {
        y0 = wrap_repeat(y0, (int)t.height);
        y1 = wrap_repeat(y1, (int)t.height);
    }
    float4 c00 = texel(s, t, x0, y0), c10 = texel(s, t, x1, y0);
    float4 c01 = texel(s, t, x0, y1), c11 = texel(s, t, x1, y1);
    float w00 = (1.0f - ax) * (1.0f - ay), w10 = ax * (1.0f - ay), w01 = (1.0f - ax) * ay, w11 = ax * ay;
    return make_float4(c00.x * w00 + c10.x * w10 + c01.x * w01 + c11.x * w11,
                       c00.y * w00 + c10.y * w10 + c01.y * w01 + c11.y * w11,
                       c00.z * w00 + c10.z * w10 + c01.z * w01 + c11.z * w11,
                       c00.w * w00 + c10.w * w10 + c01.w * w01 + c11.w * w11);
}

// Environment lookup: equirect mapping of shaders/include/environmentMap.glsl:3-10
// (the mapping the reference uses to fill its cubemap), read directly.
// VVPT_ENV_OUTLINE = 1 (a build option, measured, not kept) compiles it out
// of line, one copy for the four places that call it: the same speed on the
// 1080p medium scene, 1 % slower on the 4K sky scene, which calls it most.
#ifndef VVPT_ENV_OUTLINE
#define VVPT_ENV_OUTLINE 0
#endif
#if VVPT_ENV_OUTLINE
__device__ __noinline__ float3 env_lookup(const SceneView &s, const float3 dir)
#else
__device__ __forceinline__ float3 env_lookup(const SceneView &s, const float3 dir)
#endif
{
    if (s.env_texture < 0)
        return f3(0.0f);
    float3 v = normalize3(dir);
    float u = atan2f(v.z, v.x) * 0.1591f + 0.5f;
    float w = asinf(fminf(fmaxf(v.y, -1.0f), 1.0f)) * 0.3183f + 0.5f;
    float x = u + 0.25f;
    u = x - floorf(x);
    float4 c = tex2d(s, (uint32_t)s.env_texture, u, w, true);
    return f3(c.x, c.y, c.z);
}

// ---- environment importance sampling (an estimator addition: the
// reference never light-samples the environment, lightSampling.glsl:101-106)
//
// Directions map to the texture like env_lookup: u = atan2(z, x) * 0.1591 +
// 0.75 (wrapped), w = asin(y) * 0.3183 + 0.5, so a solid-angle density is the
// (u, w) density times 0.1591 * 0.3183 / cos(latitude).
constexpr float kEnvJacobian = 0.1591f * 0.3183f;

// Density (solid angle) of sample_env producing `dir`.
__device__ __forceinline__ float env_pdf(const SceneView &s, const float3 &dir)
{
    if (s.env_func_int <= 0.0f)
        return 0.0f;
    const float3 v = normalize3(dir);
    const float y = fminf(fmaxf(v.y, -1.0f), 1.0f);
    float u = atan2f(v.z, v.x) * 0.1591f + 0.5f;
    const float w = asinf(y) * 0.3183f + 0.5f;
    const float x = u + 0.25f;
    u = x - floorf(x);
    const float cosl = sqrtf(fmaxf(0.0f, 1.0f - y * y));
    if (cosl < 1e-6f)
        return 0.0f;
    const uint32_t col = min((uint32_t)(u * (float)s.env_w), s.env_w - 1);
    const uint32_t row = min((uint32_t)(w * (float)s.env_h), s.env_h - 1);
    return s.env_func[(size_t)row * s.env_w + col] / s.env_func_int * kEnvJacobian / cosl;
}

// Last index i in [0, n) with cdf[i] <= x (cdf ascending, cdf[0] = 0): skips
// zero-probability cells.
__device__ __forceinline__ uint32_t cdf_find(const float *cdf, uint32_t n, float x)
{
    uint32_t lo = 0, hi = n;
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (cdf[mid] <= x)
            lo = mid;
        else
            hi = mid;
    }
    return lo;
}

// Direction with density proportional to env_func (PBRT's piecewise-constant
// 2D distribution: marginal over rows from u_row, conditional over the row's
// columns from u_col). pdf = 0 when the cell maps outside the lookup's range.
__device__ __forceinline__ float3 sample_env(const SceneView &s, float u_row, float u_col, float &pdf)
{
    pdf = 0.0f;
    const uint32_t W = s.env_w, H = s.env_h;
    const uint32_t r = cdf_find(s.env_marg_cdf, H, u_row);
    const float m0 = s.env_marg_cdf[r], m1 = s.env_marg_cdf[r + 1];
    const float dv = m1 > m0 ? (u_row - m0) / (m1 - m0) : 0.0f;
    const float *cc = s.env_cond_cdf + (size_t)r * (W + 1);
    const uint32_t c = cdf_find(cc, W, u_col);
    const float c0 = cc[c], c1 = cc[c + 1];
    const float du = c1 > c0 ? (u_col - c0) / (c1 - c0) : 0.0f;
    const float u = ((float)c + du) / (float)W;
    const float w = ((float)r + dv) / (float)H;
    float x = u - 0.25f;
    if (x < 0.0f)
        x += 1.0f;
    const float lon = (x - 0.5f) / 0.1591f;
    if (fabsf(lon) > kPi)
        return f3(0.0f, 1.0f, 0.0f);
    const float lat = fminf(fmaxf((w - 0.5f) / 0.3183f, -0.5f * kPi), 0.5f * kPi);
    const float cosl = cosf(lat);
    if (cosl < 1e-6f)
        return f3(0.0f, 1.0f, 0.0f);
    pdf = s.env_func[(size_t)r * W + c] / s.env_func_int * kEnvJacobian / cosl;
    return f3(cosl * cosf(lon), sinf(lat), cosl * sinf(lon));
}

}  // namespace vvpt
