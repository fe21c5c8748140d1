// Closest-hit traversal of the two-level BVH (instance TLAS over per-mesh BLAS)
// with a watertight ray/triangle test.
//
// Semantics replaced: traceRayEXT against a TLAS whose instances have culling
// disabled (src/lib/vengine/vulkan/VulkanScene.cpp:375) and an any-hit shader
// that accepts every candidate (shaders/pt/rayPrimary.rahit.glsl:32-71), i.e.
// plain closest hit over [tmin, tmax]. Ties in t are broken by the smallest
// (instance slot, primitive index) so the result does not depend on BVH
// layout; the CPU oracle applies the same rule.
//
// The triangle test is the watertight algorithm of Woop, Benthin and Wald,
// "Watertight Ray/Triangle Intersection", JCGT 2(1), 2013, written with
// explicitly rounded operations (no FMA contraction) so that it gives the same
// bits as a plain IEEE float evaluation on the host.
#pragma once
#include "scene_gpu.h"
#include "vmath.cuh"

namespace vvpt {

// Traversal step counter hook (node visits, triangle tests, instance
// entries) for host builds that measure BVH quality; empty otherwise.
#ifndef VVPT_TRAVERSAL_STAT
#define VVPT_TRAVERSAL_STAT(kind)
#endif

constexpr uint32_t kNoHit = 0xFFFFFFFFu;
// device status word bits
constexpr uint32_t kErrStackOverflow = 1u;
constexpr uint32_t kErrLoopCap = 2u;

struct Hit {
    float t, u, v;
    uint32_t inst, prim;
};

// Per-ray constants of the watertight test.
struct WatertightRay {
    float3 org;
    int kx, ky, kz;
    float Sx, Sy, Sz;
};

__device__ __forceinline__ WatertightRay wt_setup(const float3 &o, const float3 &d)
{
    WatertightRay r;
    r.org = o;
    float ax = fabsf(d.x), ay = fabsf(d.y), az = fabsf(d.z);
    int kz = (ax > ay) ? (ax > az ? 0 : 2) : (ay > az ? 1 : 2);
    int kx = kz + 1 == 3 ? 0 : kz + 1;
    int ky = kx + 1 == 3 ? 0 : kx + 1;
    float dz = comp(d, kz);
    if (dz < 0.0f) {
        int t = kx;
        kx = ky;
        ky = t;
    }
    r.kx = kx;
    r.ky = ky;
    r.kz = kz;
    r.Sx = __fdiv_rn(comp(d, kx), dz);
    r.Sy = __fdiv_rn(comp(d, ky), dz);
    r.Sz = __fdiv_rn(1.0f, dz);
    return r;
}

__device__ __forceinline__ float sel(const float4 &v, int k) { return k == 0 ? v.x : (k == 1 ? v.y : v.z); }
__device__ __forceinline__ float sel3(const float3 &v, int k) { return k == 0 ? v.x : (k == 1 ? v.y : v.z); }

// Returns true and writes t/u/v when the triangle is hit with t in
// [tmin, best_t]; u, v are the barycentric weights of v1 and v2.
__device__ __forceinline__ bool wt_intersect(const WatertightRay &r, const float4 &p0, const float4 &p1,
                                             const float4 &p2, float tmin, float best_t, float &t_out,
                                             float &u_out, float &v_out)
{
    const float ox = sel3(r.org, r.kx), oy = sel3(r.org, r.ky), oz = sel3(r.org, r.kz);
    const float Ax = __fsub_rn(sel(p0, r.kx), ox), Ay = __fsub_rn(sel(p0, r.ky), oy), Az0 = __fsub_rn(sel(p0, r.kz), oz);
    const float Bx = __fsub_rn(sel(p1, r.kx), ox), By = __fsub_rn(sel(p1, r.ky), oy), Bz0 = __fsub_rn(sel(p1, r.kz), oz);
    const float Cx = __fsub_rn(sel(p2, r.kx), ox), Cy = __fsub_rn(sel(p2, r.ky), oy), Cz0 = __fsub_rn(sel(p2, r.kz), oz);
    const float ax = __fsub_rn(Ax, __fmul_rn(r.Sx, Az0)), ay = __fsub_rn(Ay, __fmul_rn(r.Sy, Az0));
    const float bx = __fsub_rn(Bx, __fmul_rn(r.Sx, Bz0)), by = __fsub_rn(By, __fmul_rn(r.Sy, Bz0));
    const float cx = __fsub_rn(Cx, __fmul_rn(r.Sx, Cz0)), cy = __fsub_rn(Cy, __fmul_rn(r.Sy, Cz0));
    float U = __fsub_rn(__fmul_rn(cx, by), __fmul_rn(cy, bx));
    float V = __fsub_rn(__fmul_rn(ax, cy), __fmul_rn(ay, cx));
    float W = __fsub_rn(__fmul_rn(bx, ay), __fmul_rn(by, ax));
    if (U == 0.0f || V == 0.0f || W == 0.0f) {
        // edge case: redo the 2D edge tests in double precision
        double cxby = __dmul_rn((double)cx, (double)by), cybx = __dmul_rn((double)cy, (double)bx);
        U = (float)__dsub_rn(cxby, cybx);
        double axcy = __dmul_rn((double)ax, (double)cy), aycx = __dmul_rn((double)ay, (double)cx);
        V = (float)__dsub_rn(axcy, aycx);
        double bxay = __dmul_rn((double)bx, (double)ay), byax = __dmul_rn((double)by, (double)ax);
        W = (float)__dsub_rn(bxay, byax);
    }
    if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f))
        return false;
    const float det = __fadd_rn(__fadd_rn(U, V), W);
    if (det == 0.0f)
        return false;
    const float az = __fmul_rn(r.Sz, Az0), bz = __fmul_rn(r.Sz, Bz0), cz = __fmul_rn(r.Sz, Cz0);
    const float T = __fadd_rn(__fadd_rn(__fmul_rn(U, az), __fmul_rn(V, bz)), __fmul_rn(W, cz));
    const float rcp = __fdiv_rn(1.0f, det);
    const float t = __fmul_rn(T, rcp);
    if (!(t >= tmin) || !(t <= best_t))
        return false;
    t_out = t;
    u_out = __fmul_rn(V, rcp);
    v_out = __fmul_rn(W, rcp);
    return true;
}

// Strictly after `a` in (t, instance, primitive) order; a.inst == kNoHit
// means no constraint. Used to walk any-hit candidates nearest first.
__device__ __forceinline__ bool is_after(float t, uint32_t inst, uint32_t prim, const Hit &a)
{
    if (a.inst == kNoHit)
        return true;
    if (t != a.t)
        return t > a.t;
    if (inst != a.inst)
        return inst > a.inst;
    return prim > a.prim;
}

__device__ __forceinline__ bool better(float t, uint32_t inst, uint32_t prim, const Hit &h)
{
    if (t != h.t)
        return t < h.t;
    if (inst != h.inst)
        return inst < h.inst;
    return prim < h.prim;
}

// Conservative slab test (Pharr, Jakob, Humphreys, PBRT 3rd ed. sec. 3.9.2:
// (lo - o) * invd with tfar scaled by 1 + 2*gamma(3)). Returns both children's
// entry distances; a child is missed when its entry is +inf.
__device__ __forceinline__ void box2(const BVHNode &n, const float3 &o, const float3 &invd, float tmin, float tmax,
                                     float &tl, float &tr)
{
    const float kScale = 1.0f + 2.0f * 3.5762793e-07f; // 1 + 2*gamma(3), gamma(3) = 3u/(1-3u), u = 2^-24
    float lx0 = __fmul_rn(__fsub_rn(n.lxy.x, o.x), invd.x), lx1 = __fmul_rn(__fsub_rn(n.lxy.y, o.x), invd.x);
    float ly0 = __fmul_rn(__fsub_rn(n.lxy.z, o.y), invd.y), ly1 = __fmul_rn(__fsub_rn(n.lxy.w, o.y), invd.y);
    float lz0 = __fmul_rn(__fsub_rn(n.lrz.x, o.z), invd.z), lz1 = __fmul_rn(__fsub_rn(n.lrz.y, o.z), invd.z);
    float rx0 = __fmul_rn(__fsub_rn(n.rxy.x, o.x), invd.x), rx1 = __fmul_rn(__fsub_rn(n.rxy.y, o.x), invd.x);
    float ry0 = __fmul_rn(__fsub_rn(n.rxy.z, o.y), invd.y), ry1 = __fmul_rn(__fsub_rn(n.rxy.w, o.y), invd.y);
    float rz0 = __fmul_rn(__fsub_rn(n.lrz.z, o.z), invd.z), rz1 = __fmul_rn(__fsub_rn(n.lrz.w, o.z), invd.z);
    float lnear = fmaxf(fmaxf(fminf(lx0, lx1), fminf(ly0, ly1)), fmaxf(fminf(lz0, lz1), tmin));
    float lfar = fminf(fminf(fmaxf(lx0, lx1), fmaxf(ly0, ly1)), fminf(fmaxf(lz0, lz1), tmax)) * kScale;
    float rnear = fmaxf(fmaxf(fminf(rx0, rx1), fminf(ry0, ry1)), fmaxf(fminf(rz0, rz1), tmin));
    float rfar = fminf(fminf(fmaxf(rx0, rx1), fmaxf(ry0, ry1)), fminf(fmaxf(rz0, rz1), tmax)) * kScale;
    // empty boxes (lo > hi) give near > far
    tl = (lnear <= lfar && n.lxy.x <= n.lxy.y) ? lnear : __int_as_float(0x7f800000);
    tr = (rnear <= rfar && n.rxy.x <= n.rxy.y) ? rnear : __int_as_float(0x7f800000);
}

// Culling bounds with slack. A node is skipped when its entry distance lies
// beyond the current best hit. The slab distances and the triangle test's t
// carry independent rounding errors, so for a triangle on a node's face
// (coplanar geometry, axis-aligned walls) the computed entry can exceed the
// computed hit t. Two margins keep such nodes (and equal-t ties, which the
// (instance, primitive) order resolves) in the search: 1e-5 relative to t, and
// an absolute one for hits close to the ray origin, where the triangle's t is
// a difference of coordinates far larger than t itself and its error is about
// machine epsilon times those coordinates over |d| (cull_slack).
__device__ __forceinline__ float cull_far(float best_t, float slack)
{
    return best_t * (1.0f + 1e-5f) + slack + 1e-30f;
}
__device__ __forceinline__ float cull_near(float tmin, float slack) { return tmin - fabsf(tmin) * 1e-5f - slack; }
// Absolute culling margin of one ray: 1e-5 (about 160 ulps) times the largest
// object-space coordinate magnitude a triangle test of this scene can see,
// bounded per instance on the host (SceneView::cull_o, cull_r), over |d|.
__device__ __forceinline__ float cull_slack(const SceneView &s, const float3 &o, const float3 &d)
{
    const float om = fmaxf(fmaxf(fabsf(o.x), fabsf(o.y)), fabsf(o.z));
    const float dm = fmaxf(fmaxf(fabsf(d.x), fabsf(d.y)), fabsf(d.z));
    return dm > 0.0f ? 1e-5f * (s.cull_o * om + s.cull_r) / dm : 0.0f;
}

// Loads of BVH nodes and triangles. With VVPT_SCENE_L2_KEEP = 1 (a build
// option) they carry an L2 evict-last policy, so that the scene's lines,
// re-read by every traversal kernel, outlive the path state and queues that
// stream through L2. Measured on the 1080p medium scene: no gain (137.3
// against 140.3 M paths/s without it, within run-to-run spread), so off.
#ifndef VVPT_SCENE_L2_KEEP
#define VVPT_SCENE_L2_KEEP 0
#endif
#if defined(__CUDA_ARCH__) && VVPT_SCENE_L2_KEEP
__device__ __forceinline__ uint64_t scene_l2_policy()
{
    uint64_t pol;
    asm("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(pol));
    return pol;
}
__device__ __forceinline__ float4 ldg_scene(const float4 *p)
{
    float4 v;
    asm("ld.global.nc.L2::cache_hint.v4.f32 {%0, %1, %2, %3}, [%4], %5;"
        : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
        : "l"(p), "l"(scene_l2_policy()));
    return v;
}
#else
__device__ __forceinline__ float4 ldg_scene(const float4 *p) { return __ldg(p); }
#endif

__device__ __forceinline__ BVHNode load_node(const BVHNode *nodes, int idx)
{
    const float4 *p = reinterpret_cast<const float4 *>(nodes + idx);
    BVHNode n;
    n.lxy = ldg_scene(p + 0);
    n.rxy = ldg_scene(p + 1);
    n.lrz = ldg_scene(p + 2);
    float4 c = ldg_scene(p + 3);
    n.c = make_int4(__float_as_int(c.x), __float_as_int(c.y), __float_as_int(c.z), __float_as_int(c.w));
    return n;
}

__device__ __forceinline__ float3 safe_inv(const float3 &d)
{
    return f3(__fdiv_rn(1.0f, d.x), __fdiv_rn(1.0f, d.y), __fdiv_rn(1.0f, d.z));
}

// Object-space ray of an instance, with explicitly rounded arithmetic so the
// host oracle reproduces it exactly: ((m0*x + m1*y) + m2*z) + m3.
__device__ __forceinline__ float3 wt_xform_point(const float4 *rows, const float3 &p)
{
    float3 r;
    r.x = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(rows[0].x, p.x), __fmul_rn(rows[0].y, p.y)), __fmul_rn(rows[0].z, p.z)), rows[0].w);
    r.y = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(rows[1].x, p.x), __fmul_rn(rows[1].y, p.y)), __fmul_rn(rows[1].z, p.z)), rows[1].w);
    r.z = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(rows[2].x, p.x), __fmul_rn(rows[2].y, p.y)), __fmul_rn(rows[2].z, p.z)), rows[2].w);
    return r;
}
__device__ __forceinline__ float3 wt_xform_vector(const float4 *rows, const float3 &v)
{
    float3 r;
    r.x = __fadd_rn(__fadd_rn(__fmul_rn(rows[0].x, v.x), __fmul_rn(rows[0].y, v.y)), __fmul_rn(rows[0].z, v.z));
    r.y = __fadd_rn(__fadd_rn(__fmul_rn(rows[1].x, v.x), __fmul_rn(rows[1].y, v.y)), __fmul_rn(rows[1].z, v.z));
    r.z = __fadd_rn(__fadd_rn(__fmul_rn(rows[2].x, v.x), __fmul_rn(rows[2].y, v.y)), __fmul_rn(rows[2].z, v.z));
    return r;
}

#if VVPT_BLAS_WIDE
// Byte k of w as an exact float: 0x4B0000bb is the float 2^23 + bb.
__device__ __forceinline__ float byte_as_float(uint32_t w, int k)
{
    return __fsub_rn(__uint_as_float(__byte_perm(w, 0x4B000000u, 0x7440u | (uint32_t)k)), 8388608.0f);
}

// Ray against the 8 child boxes of a wide node (five 128-bit words `w`).
// Per axis the node gives the slab distance of a plane q as one multiply-add,
// q * A + B with A = scale * invd and B = (p - o) * invd, near and far planes
// chosen by the sign of the inverse direction. That form rounds relative to
// |B| + 255 |A| rather than to the distance itself (the two terms cancel near
// the plane), so each axis carries its own margin, 8 ulps of |B| + 255 |A|
// (several times the worst-case error of the four roundings), folded into B:
// near distances move down and far ones up, and no child the ray touches is
// missed (a zero direction component gives infinities or NaN there, and NaN
// leaves that axis unconstrained). Outputs: the internal-child hits at bit
// (slot ^ oct), the node's imask and child_base, and the hit leaf children's
// triangles as a mask over tri_base + 0..31.
__device__ __forceinline__ void wide_visit(const float4 (&w)[5], const float3 &o, const float3 &invd, uint32_t oct,
                                           float tmin, float tmax, uint32_t &node_bits, uint32_t &imask,
                                           uint32_t &child_base, uint32_t &tri_base, uint32_t &tri_bits)
{
    const uint32_t eim = __float_as_uint(w[0].w);
    const float ax = __fmul_rn(__uint_as_float((eim & 0xffu) << 23), invd.x);
    const float ay = __fmul_rn(__uint_as_float(((eim >> 8) & 0xffu) << 23), invd.y);
    const float az = __fmul_rn(__uint_as_float(((eim >> 16) & 0xffu) << 23), invd.z);
    const float bx = __fmul_rn(__fsub_rn(w[0].x, o.x), invd.x);
    const float by = __fmul_rn(__fsub_rn(w[0].y, o.y), invd.y);
    const float bz = __fmul_rn(__fsub_rn(w[0].z, o.z), invd.z);
    const float kUlps = 8.0f * 5.9604645e-08f; // 8 x 2^-24
    const float mx = __fmul_rn(kUlps, __fmaf_rn(255.0f, fabsf(ax), fabsf(bx)));
    const float my = __fmul_rn(kUlps, __fmaf_rn(255.0f, fabsf(ay), fabsf(by)));
    const float mz = __fmul_rn(kUlps, __fmaf_rn(255.0f, fabsf(az), fabsf(bz)));
    const float bnx = __fsub_rn(bx, mx), bfx = __fadd_rn(bx, mx);
    const float bny = __fsub_rn(by, my), bfy = __fadd_rn(by, my);
    const float bnz = __fsub_rn(bz, mz), bfz = __fadd_rn(bz, mz);
    imask = eim >> 24;
    child_base = __float_as_uint(w[1].x);
    tri_base = __float_as_uint(w[1].y);
    const uint32_t meta[2] = {__float_as_uint(w[1].z), __float_as_uint(w[1].w)};
    const bool nx = (oct & 1u) != 0, ny = (oct & 2u) != 0, nz = (oct & 4u) != 0;
    // near / far plane words per axis: lo (w2.xy, w2.zw, w3.xy), hi (w3.zw, w4.xy, w4.zw)
    const uint32_t nxw[2] = {__float_as_uint(nx ? w[3].z : w[2].x), __float_as_uint(nx ? w[3].w : w[2].y)};
    const uint32_t fxw[2] = {__float_as_uint(nx ? w[2].x : w[3].z), __float_as_uint(nx ? w[2].y : w[3].w)};
    const uint32_t nyw[2] = {__float_as_uint(ny ? w[4].x : w[2].z), __float_as_uint(ny ? w[4].y : w[2].w)};
    const uint32_t fyw[2] = {__float_as_uint(ny ? w[2].z : w[4].x), __float_as_uint(ny ? w[2].w : w[4].y)};
    const uint32_t nzw[2] = {__float_as_uint(nz ? w[4].z : w[3].x), __float_as_uint(nz ? w[4].w : w[3].y)};
    const uint32_t fzw[2] = {__float_as_uint(nz ? w[3].x : w[4].z), __float_as_uint(nz ? w[3].y : w[4].w)};
    node_bits = 0;
    tri_bits = 0;
#pragma unroll 2
    for (int i = 0; i < 8; i++) {
        const int h = i >> 2, k = i & 3;
        const float tnx = __fmaf_rn(byte_as_float(nxw[h], k), ax, bnx);
        const float tfx = __fmaf_rn(byte_as_float(fxw[h], k), ax, bfx);
        const float tny = __fmaf_rn(byte_as_float(nyw[h], k), ay, bny);
        const float tfy = __fmaf_rn(byte_as_float(fyw[h], k), ay, bfy);
        const float tnz = __fmaf_rn(byte_as_float(nzw[h], k), az, bnz);
        const float tfz = __fmaf_rn(byte_as_float(fzw[h], k), az, bfz);
        const float tn = fmaxf(fmaxf(tnx, tny), fmaxf(tnz, tmin));
        const float tf = fminf(fminf(tfx, tfy), fminf(tfz, tmax));
        if (tn <= tf) {
            const uint32_t m = (meta[h] >> (8 * k)) & 0xffu;
            if ((imask >> i) & 1u)
                node_bits |= 1u << (i ^ (int)oct);
            else if (m)
                tri_bits |= ((1u << (m >> 5)) - 1u) << (m & 31u);
        }
    }
}

__device__ __forceinline__ void load_wide(const WideNode *nodes, uint32_t idx, float4 (&w)[5])
{
    const float4 *p = reinterpret_cast<const float4 *>(nodes + idx);
#pragma unroll
    for (int k = 0; k < 5; k++)
        w[k] = __ldg(p + k);
}
#endif

// Top of the TLAS staged in shared memory: a traversal kernel fills it at its
// start with the first kTlasCacheNodes nodes of one live scene (the scene of
// its block's first queue entry; launched with kTlasCacheBytes of dynamic
// shared memory), and trace_after reads TLAS nodes of that scene from it.
// Kernels that do not fill it clear it (tlas_cache_none).
constexpr int kTlasCacheNodes = 128;
constexpr int kTlasCacheBytes = kTlasCacheNodes * (int)sizeof(BVHNode);
extern __shared__ __align__(16) float4 vvpt_tlas_cache[];
__shared__ const BVHNode *vvpt_tlas_cache_src;
__shared__ int vvpt_tlas_cache_count;

#ifdef __CUDACC__
__device__ __forceinline__ void tlas_cache_fill(const SceneView &s)
{
    const BVHNode *src = s.nodes + s.tlas_root;
    const int cnt = min((int)s.tlas_count, kTlasCacheNodes);
    const float4 *f = reinterpret_cast<const float4 *>(src);
    for (int i = threadIdx.x; i < 4 * cnt; i += blockDim.x)
        vvpt_tlas_cache[i] = __ldg(f + i);
    if (threadIdx.x == 0) {
        vvpt_tlas_cache_src = src;
        vvpt_tlas_cache_count = cnt;
    }
    __syncthreads();
}

__device__ __forceinline__ void tlas_cache_none()
{
    if (threadIdx.x == 0) {
        vvpt_tlas_cache_src = nullptr;
        vvpt_tlas_cache_count = 0;
    }
    __syncthreads();
}
#endif

__device__ __forceinline__ BVHNode load_node_cached(int idx)
{
    const float4 *p = vvpt_tlas_cache + 4 * idx;
    BVHNode n;
    n.lxy = p[0];
    n.rxy = p[1];
    n.lrz = p[2];
    const float4 c = p[3];
    n.c = make_int4(__float_as_int(c.x), __float_as_int(c.y), __float_as_int(c.z), __float_as_int(c.w));
    return n;
}

// Closest hit over all TLAS instances among candidates strictly after
// `after`, as one flat loop over a single stack. Every loop step is one of:
// a triangle test, a node visit (both children's boxes), or a stack
// transition (enter an instance: transform the ray into its object space and
// push a return marker; pop the marker: back to the world-space ray). Keeping
// the two levels in one loop keeps a warp's lanes in step: a lane inside an
// instance never holds lanes that are still in the TLAS, as nested per-level
// loops would. The loop's state lives in a TraceState and one step is
// trace_step, so that a kernel can also run the steps of several rays on one
// lane, one after the other (trace_after is the one-ray loop). `err` receives
// status bits.
constexpr int kTagNode = 0, kTagLeaf = 1, kTagInst = 2, kTagReturn = 3, kTagWide = 4;

struct TraceState {
    float3 o, d;        // world-space ray
    float3 winvd;       // its inverse direction
    float tmin, slack, box_tmin;
    // current level: the TLAS (world ray) or one instance's BLAS (object
    // ray); wr.org is the level's origin (the watertight constants are only
    // read in a BLAS)
    WatertightRay wr;
    float3 cinvd;
    Hit best;
    uint32_t inst_id, node_base, tri_base;
    bool in_blas;
    int node;                    // inner node to visit (local index), -1 none
    int leaf_first, leaf_count;  // triangles still to test (local indices)
    int cached;                  // TLAS nodes below this index come from shared memory
#if VVPT_BLAS_WIDE
    // BLAS level: the group of wide children still to visit (hits at bit
    // slot ^ oct, imask, first child) and the triangles still to test (mask
    // over t_base + 0..31); oct = sign bits of the object-space direction
    uint32_t w_base, w_bits, w_imask, t_base, t_bits, oct;
#endif
    int sp;                      // entries on the traversal stack
};
// The traversal stack, kept apart from the scalar state so that the scalars
// stay in registers.
typedef int2 TraceStack[kTraversalStack];

__device__ __forceinline__ void trace_begin(TraceState &st, const SceneView &s, const float3 &o, const float3 &d,
                                            float tmin, float tmax, const Hit &after)
{
    st.o = o;
    st.d = d;
    st.tmin = tmin;
    st.best.t = tmax;
    st.best.u = st.best.v = 0.0f;
    st.best.inst = kNoHit;
    st.best.prim = kNoHit;
    st.slack = cull_slack(s, o, d);
    st.box_tmin = cull_near(after.inst == kNoHit ? tmin : fmaxf(tmin, after.t), st.slack);
    st.winvd = safe_inv(d);
    st.cinvd = st.winvd;
    st.wr = wt_setup(o, d);
    st.inst_id = kNoHit;
    st.node_base = s.tlas_root;
    st.tri_base = 0;
    st.in_blas = false;
    st.node = 0;
    st.leaf_first = st.leaf_count = 0;
    st.cached = vvpt_tlas_cache_src == s.nodes + s.tlas_root ? vvpt_tlas_cache_count : 0;
#if VVPT_BLAS_WIDE
    st.w_base = st.w_bits = st.w_imask = st.t_base = st.t_bits = st.oct = 0;
#endif
    st.sp = 0;
}

__device__ __forceinline__ void trace_push(TraceState &st, TraceStack &stack, int value, int tag, int count,
                                           uint32_t &err)
{
    if (st.sp < kTraversalStack)
        stack[st.sp++] = make_int2(value, (tag << 28) | count);
    else
        err |= kErrStackOverflow;
}

// Tests one triangle of the current BLAS against the ray and keeps it when it
// is the best candidate after `after`.
__device__ __forceinline__ void trace_triangle(TraceState &st, const SceneView &s, uint32_t local, const Hit &after)
{
    const float4 *tp = reinterpret_cast<const float4 *>(s.tris + st.tri_base + local);
    const float4 p0 = ldg_scene(tp), p1 = ldg_scene(tp + 1), p2 = ldg_scene(tp + 2);
    const uint32_t prim = __float_as_uint(p0.w);
    const uint32_t tag = __float_as_uint(p1.w);
    const uint32_t hinst = tag ? tag - 1u : st.inst_id; // baked triangles name their instance
    float t, u, v;
    if (wt_intersect(st.wr, p0, p1, p2, st.tmin, st.best.t, t, u, v) && better(t, hinst, prim, st.best) &&
        is_after(t, hinst, prim, after)) {
        st.best.t = t;
        st.best.u = u;
        st.best.v = v;
        st.best.inst = hinst;
        st.best.prim = prim;
    }
}

// One loop step; false when the traversal is over (st.best holds the result).
__device__ __forceinline__ bool trace_step(TraceState &st, TraceStack &stack, const SceneView &s, const Hit &after,
                                           uint32_t &err)
{
#if VVPT_BLAS_WIDE
    if (st.t_bits) {
        const int b = __ffs((int)st.t_bits) - 1;
        st.t_bits &= st.t_bits - 1u;
        trace_triangle(st, s, st.t_base + (uint32_t)b, after);
        return true;
    }
    if (st.w_bits) {
        // nearest remaining child of the group (octant order)
        const int b = __ffs((int)st.w_bits) - 1;
        st.w_bits &= st.w_bits - 1u;
        const uint32_t slot = (uint32_t)b ^ st.oct;
        const uint32_t child = st.w_base + (uint32_t)__popc(st.w_imask & ((1u << slot) - 1u));
        if (st.w_bits)
            trace_push(st, stack, (int)st.w_base, kTagWide, (int)((st.w_bits << 8) | st.w_imask), err);
        float4 wn[5];
        load_wide(s.wnodes, st.node_base + child, wn);
        wide_visit(wn, st.wr.org, st.cinvd, st.oct, st.box_tmin, cull_far(st.best.t, st.slack), st.w_bits,
                   st.w_imask, st.w_base, st.t_base, st.t_bits);
        return true;
    }
#endif
    if (st.leaf_count > 0) {
        VVPT_TRAVERSAL_STAT(1);
        trace_triangle(st, s, (uint32_t)st.leaf_first, after);
        st.leaf_first++;
        st.leaf_count--;
        return true;
    }
    if (st.node >= 0) {
        VVPT_TRAVERSAL_STAT(st.in_blas ? 0 : 3);
        const BVHNode n = (!st.in_blas && st.node < st.cached) ? load_node_cached(st.node)
                                                                : load_node(s.nodes, (int)st.node_base + st.node);
        float tl, tr;
        const float far_t = cull_far(st.best.t, st.slack);
        box2(n, st.wr.org, st.cinvd, st.box_tmin, far_t, tl, tr);
        const bool hl = tl <= far_t && n.c.x >= 0;
        const bool hr = tr <= far_t && n.c.y >= 0;
        // near child first
        const bool swap = hl && hr && tr < tl;
        int next = -1;
#pragma unroll
        for (int k = 0; k < 2; k++) {
            const bool right = (k == 0) == swap;
            const bool h = right ? hr : hl;
            if (!h)
                continue;
            const int idx = right ? n.c.y : n.c.x;
            const int cnt = right ? n.c.w : n.c.z;
            if (cnt == 0) {
                if (next < 0)
                    next = idx;
                else
                    trace_push(st, stack, idx, kTagNode, 0, err);
            } else if (st.in_blas) {
                if (st.leaf_count == 0) {
                    st.leaf_first = idx;
                    st.leaf_count = cnt;
                } else {
                    trace_push(st, stack, idx, kTagLeaf, cnt, err);
                }
            } else {
                trace_push(st, stack, idx, kTagInst, cnt, err);
            }
        }
        st.node = next;
        return true;
    }
    if (st.sp == 0)
        return false;
    const int2 e = stack[--st.sp];
    const int tag = (int)((unsigned)e.y >> 28);
    const int cnt = e.y & 0x0FFFFFFF;
    if (tag == kTagNode) {
        st.node = e.x;
#if VVPT_BLAS_WIDE
    } else if (tag == kTagWide) {
        st.w_base = (uint32_t)e.x;
        st.w_bits = ((uint32_t)cnt >> 8) & 0xffu;
        st.w_imask = (uint32_t)cnt & 0xffu;
#endif
    } else if (tag == kTagLeaf) {
        st.leaf_first = e.x;
        st.leaf_count = cnt;
    } else if (tag == kTagInst) {
        VVPT_TRAVERSAL_STAT(2);
        if (cnt > 1)
            trace_push(st, stack, e.x + 1, kTagInst, cnt - 1, err);
        st.inst_id = __ldg(s.tlas_order + e.x);
        const DevInstance &inst = s.instances[st.inst_id];
        const float4 rows[3] = {inst.w2o[0], inst.w2o[1], inst.w2o[2]};
        const float3 co = wt_xform_point(rows, st.o);
        const float3 cd = wt_xform_vector(rows, st.d);
        st.cinvd = safe_inv(cd);
        st.wr = wt_setup(co, cd);
        st.node_base = inst.node_offset;
        st.tri_base = inst.tri_offset;
        st.in_blas = true;
        trace_push(st, stack, 0, kTagReturn, 0, err);
#if VVPT_BLAS_WIDE
        // the BLAS root as a one-child group
        st.oct = (__float_as_uint(cd.x) >> 31) | ((__float_as_uint(cd.y) >> 31) << 1) |
                 ((__float_as_uint(cd.z) >> 31) << 2);
        st.w_base = 0;
        st.w_imask = 1u;
        st.w_bits = 1u << st.oct;
#else
        st.node = 0;
#endif
    } else {
        // back to the TLAS
        st.wr.org = st.o;
        st.cinvd = st.winvd;
        st.node_base = s.tlas_root;
        st.in_blas = false;
        st.inst_id = kNoHit;
    }
    return true;
}

// VVPT_TRACE_TURNS: the lanes that run this loop together take triangle
// tests and the other kinds of step in separate steps (as the extension
// kernel's refill loop does), triangle tests when at least
// VVPT_TRACE_TURN_PCT % of them have one pending.
#ifndef VVPT_TRACE_TURNS
#define VVPT_TRACE_TURNS 0
#endif
#ifndef VVPT_TRACE_TURN_PCT
#define VVPT_TRACE_TURN_PCT 33
#endif
__device__ __forceinline__ Hit trace_after(const SceneView &s, const float3 &o, const float3 &d, float tmin, float tmax,
                                           const Hit &after, uint32_t &err)
{
    TraceState st;
    TraceStack stack;
    trace_begin(st, s, o, d, tmin, tmax, after);
#if VVPT_TRACE_TURNS && defined(__CUDA_ARCH__)
    for (;;) {
        const uint32_t act = __activemask();
        const bool tri = st.leaf_count > 0;
        const bool turn = 100 * __popc(__ballot_sync(act, tri)) >= VVPT_TRACE_TURN_PCT * __popc(act);
        if (tri == turn && !trace_step(st, stack, s, after, err))
            break;
    }
#else
    while (trace_step(st, stack, s, after, err)) {
    }
#endif
    return st.best;
}

#if VVPT_BLAS_WIDE && VVPT_GROUP_TRAVERSAL && defined(__CUDACC__)
// ---------------------------------------------------------------------------
// Cooperative traversal: eight consecutive lanes of a warp (a lane group)
// trace one ray together. Every lane holds the same traversal state (ray,
// best hit, stack) and takes the same branches; the two steps that carry the
// work are spread over the lanes: a wide BLAS node visit tests one child slot
// per lane, and a triangle step tests up to eight of the pending triangles at
// once, the nearest (t, primitive) winning through a group reduction. A warp
// holds four groups, so a warp instruction serves up to four rays' node or
// triangle work with eight lanes each, where the one-ray-per-lane loop above
// ran at about six active lanes per instruction under divergence. The result
// is the same closest hit: candidate order does not matter to the
// (t, instance, primitive) minimum, and the node tests keep their margins.
struct LaneGroup {
    uint32_t mask; // the group's eight lanes
    int gl;        // this lane's index in the group (0..7)
};

__device__ __forceinline__ LaneGroup lane_group()
{
    LaneGroup g;
    const int lane = (int)(threadIdx.x & 31u);
    g.gl = lane & 7;
    g.mask = 0xFFu << (lane & 24);
    return g;
}

__device__ __forceinline__ float fmin3f(float a, float b, float c)
{
    float d;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
    return d;
}
__device__ __forceinline__ float fmax3f(float a, float b, float c)
{
    float d;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
    return d;
}

// wide_visit with lane gl testing child slot gl ^ oct: the ballot bit of lane
// gl is then the node-group bit of that slot (bit = slot ^ oct). Same plane
// reconstruction and margins as wide_visit.
__device__ __forceinline__ void wide_visit_group(const float4 (&w)[5], const float3 &o, const float3 &invd,
                                                 uint32_t oct, float tmin, float tmax, const LaneGroup &g,
                                                 uint32_t &node_bits, uint32_t &imask, uint32_t &child_base,
                                                 uint32_t &tri_base, uint32_t &tri_bits)
{
    const uint32_t eim = __float_as_uint(w[0].w);
    const float ax = __fmul_rn(__uint_as_float((eim & 0xffu) << 23), invd.x);
    const float ay = __fmul_rn(__uint_as_float(((eim >> 8) & 0xffu) << 23), invd.y);
    const float az = __fmul_rn(__uint_as_float(((eim >> 16) & 0xffu) << 23), invd.z);
    const float bx = __fmul_rn(__fsub_rn(w[0].x, o.x), invd.x);
    const float by = __fmul_rn(__fsub_rn(w[0].y, o.y), invd.y);
    const float bz = __fmul_rn(__fsub_rn(w[0].z, o.z), invd.z);
    const float kUlps = 8.0f * 5.9604645e-08f; // 8 x 2^-24
    const float mx = __fmul_rn(kUlps, __fmaf_rn(255.0f, fabsf(ax), fabsf(bx)));
    const float my = __fmul_rn(kUlps, __fmaf_rn(255.0f, fabsf(ay), fabsf(by)));
    const float mz = __fmul_rn(kUlps, __fmaf_rn(255.0f, fabsf(az), fabsf(bz)));
    imask = eim >> 24;
    child_base = __float_as_uint(w[1].x);
    tri_base = __float_as_uint(w[1].y);
    const uint32_t slot = (uint32_t)g.gl ^ oct;
    const int h = (int)(slot >> 2), k = (int)(slot & 3u);
    const bool nx = (oct & 1u) != 0, ny = (oct & 2u) != 0, nz = (oct & 4u) != 0;
    // this slot's near / far plane words per axis: lo (w2.xy, w2.zw, w3.xy), hi (w3.zw, w4.xy, w4.zw)
    const uint32_t lox = __float_as_uint(h ? w[2].y : w[2].x), hix = __float_as_uint(h ? w[3].w : w[3].z);
    const uint32_t loy = __float_as_uint(h ? w[2].w : w[2].z), hiy = __float_as_uint(h ? w[4].y : w[4].x);
    const uint32_t loz = __float_as_uint(h ? w[3].y : w[3].x), hiz = __float_as_uint(h ? w[4].w : w[4].z);
    const float tnx = __fmaf_rn(byte_as_float(nx ? hix : lox, k), ax, __fsub_rn(bx, mx));
    const float tfx = __fmaf_rn(byte_as_float(nx ? lox : hix, k), ax, __fadd_rn(bx, mx));
    const float tny = __fmaf_rn(byte_as_float(ny ? hiy : loy, k), ay, __fsub_rn(by, my));
    const float tfy = __fmaf_rn(byte_as_float(ny ? loy : hiy, k), ay, __fadd_rn(by, my));
    const float tnz = __fmaf_rn(byte_as_float(nz ? hiz : loz, k), az, __fsub_rn(bz, mz));
    const float tfz = __fmaf_rn(byte_as_float(nz ? loz : hiz, k), az, __fadd_rn(bz, mz));
    const float tn = fmaxf(fmax3f(tnx, tny, tnz), tmin);
    const float tf = fminf(fmin3f(tfx, tfy, tfz), tmax);
    const bool hit = tn <= tf;
    const bool internal = ((imask >> slot) & 1u) != 0;
    const uint32_t m = (__float_as_uint(h ? w[1].w : w[1].z) >> (8 * k)) & 0xffu;
    const uint32_t lane0 = threadIdx.x & 24u;
    node_bits = (__ballot_sync(g.mask, hit && internal) >> lane0) & 0xffu;
    const uint32_t mine = (hit && !internal && m) ? ((1u << (m >> 5)) - 1u) << (m & 31u) : 0u;
    tri_bits = __reduce_or_sync(g.mask, mine);
}

// trace_after for a lane group (see above). All eight lanes call it with the
// same arguments and get the same result.
__device__ __forceinline__ Hit trace_after_group(const SceneView &s, const float3 &o, const float3 &d, float tmin,
                                                 float tmax, const Hit &after, uint32_t &err, const LaneGroup &g)
{
    Hit best;
    best.t = tmax;
    best.u = best.v = 0.0f;
    best.inst = kNoHit;
    best.prim = kNoHit;
    const float slack = cull_slack(s, o, d);
    const float box_tmin = cull_near(after.inst == kNoHit ? tmin : fmaxf(tmin, after.t), slack);
    const float3 winvd = safe_inv(d);
    float3 co = o, cinvd = winvd;
    WatertightRay wr = wt_setup(o, d);
    uint32_t inst_id = kNoHit;
    uint32_t node_base = s.tlas_root, tri_base = 0;
    bool in_blas = false;
    int node = 0; // TLAS node to visit, -1 none
    uint32_t w_base = 0, w_bits = 0, w_imask = 0, t_base = 0, t_bits = 0, oct = 0;
    int2 stack[kTraversalStack];
    int sp = 0;
    const int cached = vvpt_tlas_cache_src == s.nodes + s.tlas_root ? vvpt_tlas_cache_count : 0;
    auto push = [&](int value, int tag, int count) {
        if (sp < kTraversalStack)
            stack[sp++] = make_int2(value, (tag << 28) | count);
        else
            err |= kErrStackOverflow;
    };
    for (;;) {
        if (t_bits) {
            // up to eight pending triangles, one per lane
            const int cnt = __popc(t_bits);
            float ct = INFINITY, cu = 0.0f, cv = 0.0f;
            uint32_t cp = kNoHit, ci = kNoHit;
            if (g.gl < cnt) {
                const int b = (int)__fns(t_bits, 0, g.gl + 1);
                const float4 *tp = reinterpret_cast<const float4 *>(s.tris + tri_base + t_base + (uint32_t)b);
                const float4 p0 = __ldg(tp), p1 = __ldg(tp + 1), p2 = __ldg(tp + 2);
                const uint32_t prim = __float_as_uint(p0.w);
                const uint32_t tag = __float_as_uint(p1.w);
                const uint32_t hinst = tag ? tag - 1u : inst_id;
                float t, u, v;
                if (wt_intersect(wr, p0, p1, p2, tmin, best.t, t, u, v) && better(t, hinst, prim, best) &&
                    is_after(t, hinst, prim, after)) {
                    ct = t;
                    cu = u;
                    cv = v;
                    cp = prim;
                    ci = hinst;
                }
            }
            if (cnt <= 8) {
                t_bits = 0;
            } else {
                const uint32_t b8 = __fns(t_bits, 0, 8); // the eighth set bit
                t_bits &= ~((2u << b8) - 1u);
            }
            // group minimum of (t, instance, primitive)
            float mt = ct;
            uint32_t mi = ci, mp = cp;
#pragma unroll
            for (int sh = 1; sh < 8; sh <<= 1) {
                const float ot = __shfl_xor_sync(g.mask, mt, sh);
                const uint32_t oi = __shfl_xor_sync(g.mask, mi, sh);
                const uint32_t op = __shfl_xor_sync(g.mask, mp, sh);
                if (ot < mt || (ot == mt && (oi < mi || (oi == mi && op < mp)))) {
                    mt = ot;
                    mi = oi;
                    mp = op;
                }
            }
            if (mp != kNoHit) {
                const uint32_t owner = __ffs(__ballot_sync(g.mask, cp == mp && ci == mi && ct == mt)) - 1;
                best.u = __shfl_sync(g.mask, cu, (int)owner);
                best.v = __shfl_sync(g.mask, cv, (int)owner);
                best.t = mt;
                best.inst = mi;
                best.prim = mp;
            }
            continue;
        }
        if (w_bits) {
            const int b = __ffs((int)w_bits) - 1;
            w_bits &= w_bits - 1u;
            const uint32_t slot = (uint32_t)b ^ oct;
            const uint32_t child = w_base + (uint32_t)__popc(w_imask & ((1u << slot) - 1u));
            if (w_bits)
                push((int)w_base, kTagWide, (int)((w_bits << 8) | w_imask));
            float4 wn[5];
            load_wide(s.wnodes, node_base + child, wn);
            wide_visit_group(wn, co, cinvd, oct, box_tmin, cull_far(best.t, slack), g, w_bits, w_imask, w_base,
                             t_base, t_bits);
            continue;
        }
        if (node >= 0) {
            // TLAS (binary nodes): every lane tests both children
            const BVHNode n = node < cached ? load_node_cached(node) : load_node(s.nodes, (int)node_base + node);
            float tl, tr;
            const float far_t = cull_far(best.t, slack);
            box2(n, co, cinvd, box_tmin, far_t, tl, tr);
            const bool hl = tl <= far_t && n.c.x >= 0;
            const bool hr = tr <= far_t && n.c.y >= 0;
            const bool swap = hl && hr && tr < tl;
            int next = -1;
#pragma unroll
            for (int k = 0; k < 2; k++) {
                const bool right = (k == 0) == swap;
                const bool h = right ? hr : hl;
                if (!h)
                    continue;
                const int idx = right ? n.c.y : n.c.x;
                const int cnt = right ? n.c.w : n.c.z;
                if (cnt == 0) {
                    if (next < 0)
                        next = idx;
                    else
                        push(idx, kTagNode, 0);
                } else {
                    push(idx, kTagInst, cnt);
                }
            }
            node = next;
            continue;
        }
        if (sp == 0)
            break;
        const int2 e = stack[--sp];
        const int tag = (int)((unsigned)e.y >> 28);
        const int cnt = e.y & 0x0FFFFFFF;
        if (tag == kTagNode) {
            node = e.x;
        } else if (tag == kTagWide) {
            w_base = (uint32_t)e.x;
            w_bits = ((uint32_t)cnt >> 8) & 0xffu;
            w_imask = (uint32_t)cnt & 0xffu;
        } else if (tag == kTagInst) {
            if (cnt > 1)
                push(e.x + 1, kTagInst, cnt - 1);
            inst_id = __ldg(s.tlas_order + e.x);
            const DevInstance &inst = s.instances[inst_id];
            const float4 rows[3] = {inst.w2o[0], inst.w2o[1], inst.w2o[2]};
            co = wt_xform_point(rows, o);
            const float3 cd = wt_xform_vector(rows, d);
            cinvd = safe_inv(cd);
            wr = wt_setup(co, cd);
            node_base = inst.node_offset;
            tri_base = inst.tri_offset;
            in_blas = true;
            push(0, kTagReturn, 0);
            oct = (__float_as_uint(cd.x) >> 31) | ((__float_as_uint(cd.y) >> 31) << 1) |
                  ((__float_as_uint(cd.z) >> 31) << 2);
            w_base = 0;
            w_imask = 1u;
            w_bits = 1u << oct;
        } else {
            co = o;
            cinvd = winvd;
            node_base = s.tlas_root;
            in_blas = false;
            inst_id = kNoHit;
        }
    }
    (void)in_blas;
    return best;
}
#endif

__device__ __forceinline__ Hit no_hit()
{
    Hit h;
    h.t = -1.0f;
    h.u = h.v = 0.0f;
    h.inst = kNoHit;
    h.prim = kNoHit;
    return h;
}

__device__ __forceinline__ Hit trace_closest(const SceneView &s, const float3 &o, const float3 &d, float tmin, float tmax,
                                             uint32_t &err)
{
    return trace_after(s, o, d, tmin, tmax, no_hit(), err);
}

// A BSDF-direction emitter ray adds radiance only at an emissive surface,
// and its candidate walk keeps the direction and moves the origin along the
// line, so it can contribute only if the half-line from `o` along `d` meets
// one of the scene's emissive boxes. The slab interval of each axis is
// widened by 1e-5 of its ends (far above float rounding) and the boxes are
// padded, so a ray that reaches an emitter is never rejected.
__device__ __forceinline__ bool may_reach_emitter(const SceneView &s, const float3 &o, const float3 &d)
{
    const float big = 3.402823466e38f; // NaN and infinities fail |x| <= big
    if (!(fabsf(o.x) <= big && fabsf(o.y) <= big && fabsf(o.z) <= big && fabsf(d.x) <= big && fabsf(d.y) <= big &&
          fabsf(d.z) <= big))
        return true;
    for (uint32_t k = 0; k < s.num_emit_boxes; k++) {
        const float4 lo = __ldg(&s.emit_boxes[2 * k]), hi = __ldg(&s.emit_boxes[2 * k + 1]);
        float t0 = 0.0f, t1 = INFINITY;
        bool out = false;
#pragma unroll
        for (int a = 0; a < 3; a++) {
            const float oa = a == 0 ? o.x : (a == 1 ? o.y : o.z);
            const float da = a == 0 ? d.x : (a == 1 ? d.y : d.z);
            const float la = a == 0 ? lo.x : (a == 1 ? lo.y : lo.z);
            const float ha = a == 0 ? hi.x : (a == 1 ? hi.y : hi.z);
            if (da == 0.0f) {
                out |= oa < la || oa > ha;
            } else {
                const float ta = (la - oa) / da, tb = (ha - oa) / da;
                float tn = fminf(ta, tb), tf = fmaxf(ta, tb);
                tn -= 1e-5f * fabsf(tn);
                tf += 1e-5f * fabsf(tf);
                t0 = fmaxf(t0, tn);
                t1 = fminf(t1, tf);
            }
        }
        if (!out && t0 <= t1)
            return true;
    }
    return false;
}

}  // namespace vvpt
