// ORACLE — test infrastructure only. CPU restatement of vviewer's path-traced
// renderer (the GLSL shaders of src/lib/vengine/shaders/pt and
// src/lib/vengine/shaders/include), used by tests/, the smoke check and the
// CPU-baseline leg of bench.py as the checker. It is never part of the
// product path.
//
// It follows the reference's own control structure — raygen loop around a
// trace, closest-hit / miss bodies with the shadow and BSDF-direction emitter
// rays traced inside them — rather than the GPU build's wavefront, so a
// reordering bug in the wavefront shows up as a difference.
//
// Pinning: the reference's images come from its Vulkan ray-tracing pipeline,
// which cannot run on these machines, so the oracle is pinned against the 12
// golden RGBE images of src/bin/unittests/RenderTests.cpp that can be rebuilt
// from assets present in the reference tree (statistically: per-pixel error
// normalised by the Monte Carlo standard error, and the reference's own MSE).
//
// Conventions shared with the GPU build where bit-exact closest-hit results
// are required: the Woop-Benthin-Wald watertight triangle test evaluated in
// IEEE float without contraction (build with -ffp-contract=off), the
// object-space ray computed as ((m0*x + m1*y) + m2*z) + m3, and ties in t
// broken by the smallest (instance slot, primitive index).
#include <algorithm>
#include <array>
#include <atomic>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

#include "../include/vvpt.h"

namespace {

// ------------------------------------------------------------------ vectors
struct V3 {
    float x, y, z;
};
inline V3 v3(float x, float y, float z) { return {x, y, z}; }
inline V3 v3s(float s) { return {s, s, s}; }
inline V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 operator*(V3 a, V3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
inline V3 operator/(V3 a, V3 b) { return {a.x / b.x, a.y / b.y, a.z / b.z}; }
inline V3 operator*(V3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
inline V3 operator*(float s, V3 a) { return {s * a.x, s * a.y, s * a.z}; }
inline V3 operator/(V3 a, float s) { return {a.x / s, a.y / s, a.z / s}; }
inline V3 operator-(V3 a) { return {-a.x, -a.y, -a.z}; }
inline float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 cross(V3 a, V3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
inline float length(V3 a) { return std::sqrt(dot(a, a)); }
inline V3 normalize(V3 a) { return a * (1.0f / std::sqrt(dot(a, a))); }
inline float comp(V3 a, int i) { return i == 0 ? a.x : (i == 1 ? a.y : a.z); }
inline bool isBlack(V3 c) { return c.x == 0.0f && c.y == 0.0f && c.z == 0.0f; }
inline bool isBlackEps(V3 c, float e) { return std::fabs(c.x) <= e && std::fabs(c.y) <= e && std::fabs(c.z) <= e; }
inline float max3(V3 v) { return std::max(std::max(v.x, v.y), v.z); }
inline V3 vexp(V3 v) { return {std::exp(v.x), std::exp(v.y), std::exp(v.z)}; }
inline V3 vmix(V3 a, V3 b, float t) { return a * (1.0f - t) + b * t; }
inline float fmix(float a, float b, float t) { return a * (1.0f - t) + b * t; }

// shaders/include/constants.glsl:1-9
const float EPSILON = 0.000001f;
const float PI = 3.14159265358979323846f;
const float INV_PI = 0.31830988618379067154f;
const float INV_4PI = 0.079577472f;
const float PI_OVER_TWO = 1.57079632679489661923f;
const float PI_OVER_FOUR = 0.78539816339744830961f;
const uint32_t RUSSIAN_ROULETTE_DEPTH = 3;  // shaders/pt/defines_pt.glsl:9

struct Rows {
    float m[3][4];
};
inline V3 xpoint(const Rows &r, V3 p)
{
    return {r.m[0][0] * p.x + r.m[0][1] * p.y + r.m[0][2] * p.z + r.m[0][3],
            r.m[1][0] * p.x + r.m[1][1] * p.y + r.m[1][2] * p.z + r.m[1][3],
            r.m[2][0] * p.x + r.m[2][1] * p.y + r.m[2][2] * p.z + r.m[2][3]};
}
inline V3 xvector(const Rows &r, V3 v)
{
    return {r.m[0][0] * v.x + r.m[0][1] * v.y + r.m[0][2] * v.z, r.m[1][0] * v.x + r.m[1][1] * v.y + r.m[1][2] * v.z,
            r.m[2][0] * v.x + r.m[2][1] * v.y + r.m[2][2] * v.z};
}
// v * M (row vector): construct_frame.glsl:9 `localNormal * gl_WorldToObjectEXT`
inline V3 xnormalT(const Rows &r, V3 n)
{
    return {n.x * r.m[0][0] + n.y * r.m[1][0] + n.z * r.m[2][0], n.x * r.m[0][1] + n.y * r.m[1][1] + n.z * r.m[2][1],
            n.x * r.m[0][2] + n.y * r.m[1][2] + n.z * r.m[2][2]};
}

bool invert_rows(const float m[16], Rows &out)
{
    double a[3][3], t[3];
    for (int r = 0; r < 3; r++) {
        for (int c = 0; c < 3; c++)
            a[r][c] = m[c * 4 + r];
        t[r] = m[12 + r];
    }
    double det = a[0][0] * (a[1][1] * a[2][2] - a[1][2] * a[2][1]) - a[0][1] * (a[1][0] * a[2][2] - a[1][2] * a[2][0]) +
                 a[0][2] * (a[1][0] * a[2][1] - a[1][1] * a[2][0]);
    if (!(std::fabs(det) > 0.0))
        return false;
    double inv[3][3];
    inv[0][0] = (a[1][1] * a[2][2] - a[1][2] * a[2][1]) / det;
    inv[0][1] = (a[0][2] * a[2][1] - a[0][1] * a[2][2]) / det;
    inv[0][2] = (a[0][1] * a[1][2] - a[0][2] * a[1][1]) / det;
    inv[1][0] = (a[1][2] * a[2][0] - a[1][0] * a[2][2]) / det;
    inv[1][1] = (a[0][0] * a[2][2] - a[0][2] * a[2][0]) / det;
    inv[1][2] = (a[0][2] * a[1][0] - a[0][0] * a[1][2]) / det;
    inv[2][0] = (a[1][0] * a[2][1] - a[1][1] * a[2][0]) / det;
    inv[2][1] = (a[0][1] * a[2][0] - a[0][0] * a[2][1]) / det;
    inv[2][2] = (a[0][0] * a[1][1] - a[0][1] * a[1][0]) / det;
    for (int r = 0; r < 3; r++) {
        for (int c = 0; c < 3; c++)
            out.m[r][c] = (float)inv[r][c];
        out.m[r][3] = (float)(-(inv[r][0] * t[0] + inv[r][1] * t[1] + inv[r][2] * t[2]));
    }
    return true;
}

// ------------------------------------------------------------------ RNG: shaders/include/rng/rng_def.glsl:4-36
inline float uintToFloat(uint32_t x)
{
    uint32_t b = 0x3f800000u | (x >> 9);
    float f;
    std::memcpy(&f, &b, 4);
    return f - 1.0f;
}
inline uint32_t xorshift(uint32_t &s)
{
    s ^= s << 13;
    s ^= s >> 17;
    s ^= s << 5;
    return s;
}
inline uint32_t jenkinsHash(uint32_t x)
{
    x += x << 10;
    x ^= x >> 6;
    x += x << 3;
    x ^= x >> 11;
    x += x << 15;
    return x;
}
inline uint32_t initRNG(uint32_t px, uint32_t py, uint32_t resx, uint32_t frame)
{
    uint32_t pixelIdx = px * resx + py;
    uint32_t state = pixelIdx ^ jenkinsHash(frame);
    return jenkinsHash(state);
}

// ------------------------------------------------------------------ scene
struct Tri {
    V3 p0, p1, p2;
    uint32_t prim;
    uint32_t inst = 0xFFFFFFFFu; // baked small-instance triangles: their instance
};
struct Node {
    float lo[3], hi[3];
    int left = -1, right = -1; // internal children
    int first = 0, count = 0;  // leaf range
};
struct BVH {
    std::vector<Node> nodes;
    std::vector<uint32_t> order;
};

void build_bvh(const std::vector<std::array<float, 6>> &boxes, BVH &bvh)
{
    const int n = (int)boxes.size();
    bvh.order.resize(n);
    for (int i = 0; i < n; i++)
        bvh.order[i] = i;
    bvh.nodes.clear();
    struct Task {
        int node, begin, end;
    };
    bvh.nodes.push_back(Node());
    std::vector<Task> stack{{0, 0, n}};
    while (!stack.empty()) {
        Task t = stack.back();
        stack.pop_back();
        Node nd;
        for (int a = 0; a < 3; a++) {
            nd.lo[a] = FLT_MAX;
            nd.hi[a] = -FLT_MAX;
        }
        float clo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, chi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
        for (int i = t.begin; i < t.end; i++) {
            const auto &b = boxes[bvh.order[i]];
            for (int a = 0; a < 3; a++) {
                nd.lo[a] = std::min(nd.lo[a], b[a]);
                nd.hi[a] = std::max(nd.hi[a], b[3 + a]);
                float c = 0.5f * (b[a] + b[3 + a]);
                clo[a] = std::min(clo[a], c);
                chi[a] = std::max(chi[a], c);
            }
        }
        int cnt = t.end - t.begin;
        int axis = 0;
        float ext = chi[0] - clo[0];
        for (int a = 1; a < 3; a++)
            if (chi[a] - clo[a] > ext) {
                ext = chi[a] - clo[a];
                axis = a;
            }
        if (cnt <= 4 || !(ext > 0.0f)) {
            nd.first = t.begin;
            nd.count = cnt;
            bvh.nodes[t.node] = nd;
            continue;
        }
        int mid = t.begin + cnt / 2;
        std::nth_element(bvh.order.begin() + t.begin, bvh.order.begin() + mid, bvh.order.begin() + t.end,
                         [&](uint32_t x, uint32_t y) {
                             return boxes[x][axis] + boxes[x][3 + axis] < boxes[y][axis] + boxes[y][3 + axis];
                         });
        nd.left = (int)bvh.nodes.size();
        nd.right = nd.left + 1;
        bvh.nodes.push_back(Node());
        bvh.nodes.push_back(Node());
        bvh.nodes[t.node] = nd;
        stack.push_back({nd.left, t.begin, mid});
        stack.push_back({nd.right, mid, t.end});
    }
}

struct Mesh {
    const vvpt_vertex *v = nullptr;
    const uint32_t *idx = nullptr;
    uint32_t ntri = 0;
    std::vector<Tri> tris; // BVH leaf order
    BVH bvh;
    float lo[3], hi[3];
};
struct Inst {
    Rows o2w, w2o;
    const vvpt_instance *src = nullptr;
    int mesh = -1;
    bool in_tlas = false;
};
struct Tex {
    uint32_t w, h, fmt;
    const uint8_t *data;
};

struct Scene {
    std::vector<Mesh> meshes;
    std::vector<Inst> inst;
    std::vector<uint32_t> tlas_ids;
    BVH tlas;
    const vvpt_material *mats = nullptr;
    uint32_t nmats = 0;
    const vvpt_light_instance *lights = nullptr;
    uint32_t nlights = 0;
    const vvpt_light_data *ldata = nullptr;
    std::vector<Tex> tex;
    int env = -1;
    float cull_o = 0.0f, cull_r = 0.0f;
    // environment importance sampling (VVPT_RENDER_ENV_IS): piecewise
    // constant over the equirect texels
    std::vector<float> envFunc, envCond, envMarg;
    uint32_t envW = 0, envH = 0;
    float envInt = 0.0f;
};

// ------------------------------------------------------------------ closest hit
struct Hit {
    float t = 0, u = 0, v = 0;
    uint32_t inst = 0xFFFFFFFFu, prim = 0xFFFFFFFFu;
};
const uint32_t NOHIT = 0xFFFFFFFFu;

inline bool hit_better(float t, uint32_t i, uint32_t p, const Hit &h)
{
    if (t != h.t)
        return t < h.t;
    if (i != h.inst)
        return i < h.inst;
    return p < h.prim;
}
inline bool hit_after(float t, uint32_t i, uint32_t p, const Hit &a)
{
    if (a.inst == NOHIT)
        return true;
    if (t != a.t)
        return t > a.t;
    if (i != a.inst)
        return i > a.inst;
    return p > a.prim;
}

// Woop, Benthin, Wald, "Watertight Ray/Triangle Intersection", JCGT 2013.
struct WRay {
    V3 o;
    int kx, ky, kz;
    float Sx, Sy, Sz;
};
WRay wsetup(V3 o, V3 d)
{
    WRay r;
    r.o = o;
    float ax = std::fabs(d.x), ay = std::fabs(d.y), az = std::fabs(d.z);
    int kz = (ax > ay) ? (ax > az ? 0 : 2) : (ay > az ? 1 : 2);
    int kx = (kz + 1) % 3, ky = (kx + 1) % 3;
    float dz = comp(d, kz);
    if (dz < 0.0f)
        std::swap(kx, ky);
    r.kx = kx;
    r.ky = ky;
    r.kz = kz;
    r.Sx = comp(d, kx) / dz;
    r.Sy = comp(d, ky) / dz;
    r.Sz = 1.0f / dz;
    return r;
}
bool wtest(const WRay &r, const Tri &tr, float tmin, float tmax, float &t, float &u, float &v)
{
    float ox = comp(r.o, r.kx), oy = comp(r.o, r.ky), oz = comp(r.o, r.kz);
    float Ax = comp(tr.p0, r.kx) - ox, Ay = comp(tr.p0, r.ky) - oy, Az0 = comp(tr.p0, r.kz) - oz;
    float Bx = comp(tr.p1, r.kx) - ox, By = comp(tr.p1, r.ky) - oy, Bz0 = comp(tr.p1, r.kz) - oz;
    float Cx = comp(tr.p2, r.kx) - ox, Cy = comp(tr.p2, r.ky) - oy, Cz0 = comp(tr.p2, r.kz) - oz;
    float ax = Ax - r.Sx * Az0, ay = Ay - r.Sy * Az0;
    float bx = Bx - r.Sx * Bz0, by = By - r.Sy * Bz0;
    float cx = Cx - r.Sx * Cz0, cy = Cy - r.Sy * Cz0;
    float U = cx * by - cy * bx;
    float V = ax * cy - ay * cx;
    float W = bx * ay - by * ax;
    if (U == 0.0f || V == 0.0f || W == 0.0f) {
        U = (float)((double)cx * (double)by - (double)cy * (double)bx);
        V = (float)((double)ax * (double)cy - (double)ay * (double)cx);
        W = (float)((double)bx * (double)ay - (double)by * (double)ax);
    }
    if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f))
        return false;
    float det = (U + V) + W;
    if (det == 0.0f)
        return false;
    float az = r.Sz * Az0, bz = r.Sz * Bz0, cz = r.Sz * Cz0;
    float T = (U * az + V * bz) + W * cz;
    float rcp = 1.0f / det;
    float tt = T * rcp;
    if (!(tt >= tmin) || !(tt <= tmax))
        return false;
    t = tt;
    u = V * rcp;
    v = W * rcp;
    return true;
}

// Culling margins: a node is kept unless its entry lies clearly beyond the
// best hit, so rounding in the slab and triangle distances never drops a
// candidate, in particular equal-t ties on coplanar geometry that the
// (instance, primitive) order must see. Relative slack 1e-5, plus an absolute
// one per ray for hits near the origin, where the triangle's t carries an
// error of about epsilon times the object-space coordinates over |d|:
// 1e-5 * (cull_o * |o| + cull_r) / |d| (max-norms; cull_o, cull_r bound the
// object-space coordinate growth over the TLAS instances).
inline float cull_far(float best_t, float slack) { return best_t * (1.0f + 1e-5f) + slack + 1e-30f; }
inline float cull_near(float tmin, float slack) { return tmin - std::fabs(tmin) * 1e-5f - slack; }

// box test widened generously: culling only needs to be conservative
inline bool box_hit(const Node &n, V3 o, V3 inv, float tmin, float tmax)
{
    float t0 = tmin, t1 = tmax;
    for (int a = 0; a < 3; a++) {
        float oa = comp(o, a), ia = comp(inv, a);
        float lo = n.lo[a], hi = n.hi[a];
        float pad = 1e-5f * (std::fabs(lo) + std::fabs(hi) + 1e-3f);
        float ta = (lo - pad - oa) * ia, tb = (hi + pad - oa) * ia;
        if (std::isnan(ta) || std::isnan(tb))
            continue; // ray parallel and on the slab boundary: treat as inside
        if (ta > tb)
            std::swap(ta, tb);
        t0 = std::max(t0, ta);
        t1 = std::min(t1, tb * 1.00001f + 1e-7f);
        if (t0 > t1)
            return false;
    }
    return true;
}

void trace_mesh(const Scene &s, uint32_t inst_id, V3 o, V3 d, float tmin, float slack, const Hit &after, Hit &best)
{
    const Inst &in = s.inst[inst_id];
    const Mesh &m = s.meshes[in.mesh];
    if (m.bvh.nodes.empty())
        return;
    // object-space ray: ((m0*x + m1*y) + m2*z) + m3 with no contraction
    V3 oo = xpoint(in.w2o, o);
    V3 od = xvector(in.w2o, d);
    V3 inv = {1.0f / od.x, 1.0f / od.y, 1.0f / od.z};
    WRay wr = wsetup(oo, od);
    float box_tmin = cull_near(after.inst == NOHIT ? tmin : std::max(tmin, after.t), slack);
    int stack[128];
    int sp = 0;
    stack[sp++] = 0;
    while (sp) {
        const Node &n = m.bvh.nodes[stack[--sp]];
        if (!box_hit(n, oo, inv, box_tmin, cull_far(best.t, slack)))
            continue;
        if (n.left < 0) {
            for (int k = n.first; k < n.first + n.count; k++) {
                const Tri &tr = m.tris[k];
                float t, u, v;
                const uint32_t hinst = tr.inst != 0xFFFFFFFFu ? tr.inst : inst_id;
                if (wtest(wr, tr, tmin, best.t, t, u, v) && hit_better(t, hinst, tr.prim, best) &&
                    hit_after(t, hinst, tr.prim, after)) {
                    best.t = t;
                    best.u = u;
                    best.v = v;
                    best.inst = hinst;
                    best.prim = tr.prim;
                }
            }
        } else {
            if (sp + 2 > 128)
                continue;
            stack[sp++] = n.left;
            stack[sp++] = n.right;
        }
    }
}

Hit trace_after(const Scene &s, V3 o, V3 d, float tmin, float tmax, const Hit &after)
{
    Hit best;
    best.t = tmax;
    if (s.tlas.nodes.empty())
        return best;
    V3 inv = {1.0f / d.x, 1.0f / d.y, 1.0f / d.z};
    int stack[128];
    int sp = 0;
    stack[sp++] = 0;
    const float om = std::max(std::max(std::fabs(o.x), std::fabs(o.y)), std::fabs(o.z));
    const float dm = std::max(std::max(std::fabs(d.x), std::fabs(d.y)), std::fabs(d.z));
    const float slack = dm > 0.0f ? 1e-5f * (s.cull_o * om + s.cull_r) / dm : 0.0f;
    float box_tmin = cull_near(after.inst == NOHIT ? tmin : std::max(tmin, after.t), slack);
    while (sp) {
        const Node &n = s.tlas.nodes[stack[--sp]];
        if (!box_hit(n, o, inv, box_tmin, cull_far(best.t, slack)))
            continue;
        if (n.left < 0) {
            for (int k = n.first; k < n.first + n.count; k++)
                trace_mesh(s, s.tlas_ids[s.tlas.order[k]], o, d, tmin, slack, after, best);
        } else {
            if (sp + 2 > 128)
                continue;
            stack[sp++] = n.left;
            stack[sp++] = n.right;
        }
    }
    if (best.inst == NOHIT)
        best.t = tmax;
    return best;
}
Hit trace_closest(const Scene &s, V3 o, V3 d, float tmin, float tmax)
{
    Hit none;
    return trace_after(s, o, d, tmin, tmax, none);
}

// ------------------------------------------------------------------ textures
inline float srgb_to_linear(float c) { return c <= 0.04045f ? c / 12.92f : std::pow((c + 0.055f) / 1.055f, 2.4f); }
struct C4 {
    float r, g, b, a;
};
C4 texel(const Tex &t, int x, int y)
{
    size_t i = (size_t)y * t.w + x;
    if (t.fmt == VVPT_TEXTURE_RGBA32F) {
        const float *p = reinterpret_cast<const float *>(t.data) + 4 * i;
        return {p[0], p[1], p[2], p[3]};
    }
    const uint8_t *p = t.data + 4 * i;
    C4 c = {p[0] / 255.0f, p[1] / 255.0f, p[2] / 255.0f, p[3] / 255.0f};
    if (t.fmt == VVPT_TEXTURE_RGBA8_SRGB) {
        c.r = srgb_to_linear(c.r);
        c.g = srgb_to_linear(c.g);
        c.b = srgb_to_linear(c.b);
    }
    return c;
}
inline int wrapi(int i, int n)
{
    int m = i % n;
    return m < 0 ? m + n : m;
}
// texture(sampler2D, uv) with linear filtering, repeat, LOD 0
C4 texture(const Scene &s, uint32_t idx, float u, float v, bool clampv = false)
{
    if (idx >= s.tex.size())
        return {1, 1, 1, 1};
    const Tex &t = s.tex[idx];
    if (t.w == 1 && t.h == 1)
        return texel(t, 0, 0);
    float x = u * (float)t.w - 0.5f, y = v * (float)t.h - 0.5f;
    float fx = std::floor(x), fy = std::floor(y);
    float ax = x - fx, ay = y - fy;
    int x0 = (int)fx, y0 = (int)fy, x1 = x0 + 1, y1 = y0 + 1;
    x0 = wrapi(x0, t.w);
    x1 = wrapi(x1, t.w);
    if (clampv) {
        y0 = std::min(std::max(y0, 0), (int)t.h - 1);
        y1 = std::min(std::max(y1, 0), (int)t.h - 1);
    } else {
        y0 = wrapi(y0, t.h);
        y1 = wrapi(y1, t.h);
    }
    C4 a = texel(t, x0, y0), b = texel(t, x1, y0), c = texel(t, x0, y1), d = texel(t, x1, y1);
    float w00 = (1 - ax) * (1 - ay), w10 = ax * (1 - ay), w01 = (1 - ax) * ay, w11 = ax * ay;
    return {a.r * w00 + b.r * w10 + c.r * w01 + d.r * w11, a.g * w00 + b.g * w10 + c.g * w01 + d.g * w11,
            a.b * w00 + b.b * w10 + c.b * w01 + d.b * w11, a.a * w00 + b.a * w10 + c.a * w01 + d.a * w11};
}
inline V3 rgb(C4 c) { return {c.r, c.g, c.b}; }
// shaders/include/environmentMap.glsl:3-10
V3 env_sample(const Scene &s, V3 dir)
{
    if (s.env < 0)
        return v3s(0.0f);
    V3 v = normalize(dir);
    float u = std::atan2(v.z, v.x) * 0.1591f + 0.5f;
    float w = std::asin(std::min(std::max(v.y, -1.0f), 1.0f)) * 0.3183f + 0.5f;
    float x = u + 0.25f;
    u = x - std::floor(x);
    return rgb(texture(s, (uint32_t)s.env, u, w, true));
}

// Environment sampling tables: function = texel luminance maximised over the
// 3x3 neighbourhood (columns wrap, rows clamp) times the cosine of the row
// centre's latitude; per-row and marginal CDFs summed in double.
void build_env_tables(Scene &s, const float *rgba, uint32_t w, uint32_t h)
{
    s.envW = w;
    s.envH = h;
    std::vector<double> lum((size_t)w * h), f((size_t)w * h);
    for (size_t i = 0; i < lum.size(); i++) {
        double y = 0.2126 * rgba[4 * i] + 0.7152 * rgba[4 * i + 1] + 0.0722 * rgba[4 * i + 2];
        lum[i] = (y > 0.0 && std::isfinite(y)) ? y : 0.0;
    }
    for (uint32_t r = 0; r < h; r++) {
        double lat = (((double)r + 0.5) / (double)h - 0.5) / (double)0.3183f;
        lat = std::min(std::max(lat, -0.5 * M_PI), 0.5 * M_PI);
        double cl = std::max(0.0, std::cos(lat));
        for (uint32_t c = 0; c < w; c++) {
            double mx = 0.0;
            for (int a = -1; a <= 1; a++) {
                long rr = std::min<long>(std::max<long>((long)r + a, 0), (long)h - 1);
                for (int b = -1; b <= 1; b++)
                    mx = std::max(mx, lum[(size_t)rr * w + (c + w + b) % w]);
            }
            f[(size_t)r * w + c] = mx * cl;
        }
    }
    s.envFunc.resize((size_t)w * h);
    s.envCond.resize((size_t)h * (w + 1));
    s.envMarg.resize(h + 1);
    std::vector<double> rowInt(h);
    for (uint32_t r = 0; r < h; r++) {
        double sum = 0.0;
        for (uint32_t c = 0; c < w; c++)
            sum += f[(size_t)r * w + c];
        rowInt[r] = sum / (double)w;
        double run = 0.0;
        float *cdf = &s.envCond[(size_t)r * (w + 1)];
        cdf[0] = 0.0f;
        for (uint32_t c = 0; c < w; c++) {
            run += f[(size_t)r * w + c];
            cdf[c + 1] = sum > 0.0 ? (float)(run / sum) : (float)((double)(c + 1) / (double)w);
            s.envFunc[(size_t)r * w + c] = (float)f[(size_t)r * w + c];
        }
        cdf[w] = 1.0f;
    }
    double total = 0.0;
    for (uint32_t r = 0; r < h; r++)
        total += rowInt[r];
    double run = 0.0;
    s.envMarg[0] = 0.0f;
    for (uint32_t r = 0; r < h; r++) {
        run += rowInt[r];
        s.envMarg[r + 1] = total > 0.0 ? (float)(run / total) : (float)((double)(r + 1) / (double)h);
    }
    s.envMarg[h] = 1.0f;
    s.envInt = (float)(total / (double)h);
}

// density in solid angle of envSampleDir producing `dir` (lookup mapping of
// env_sample: du dv = 0.1591 * 0.3183 * dw / cos(latitude))
float envPdf(const Scene &s, V3 dir)
{
    if (s.envInt <= 0.0f)
        return 0.0f;
    V3 v = normalize(dir);
    float y = std::min(std::max(v.y, -1.0f), 1.0f);
    float u = std::atan2(v.z, v.x) * 0.1591f + 0.5f;
    float w = std::asin(y) * 0.3183f + 0.5f;
    float x = u + 0.25f;
    u = x - std::floor(x);
    float cl = std::sqrt(std::max(0.0f, 1.0f - y * y));
    if (cl < 1e-6f)
        return 0.0f;
    uint32_t col = std::min((uint32_t)(u * (float)s.envW), s.envW - 1);
    uint32_t row = std::min((uint32_t)(w * (float)s.envH), s.envH - 1);
    return s.envFunc[(size_t)row * s.envW + col] / s.envInt * (0.1591f * 0.3183f) / cl;
}

// last index in [0, n) whose CDF value is <= x
uint32_t cdfIndex(const float *cdf, uint32_t n, float x)
{
    uint32_t lo = 0, hi = n;
    while (hi - lo > 1) {
        uint32_t mid = (lo + hi) / 2;
        if (cdf[mid] <= x)
            lo = mid;
        else
            hi = mid;
    }
    return lo;
}

// PBRT-style 2D piecewise-constant sample: row from the marginal, column
// from that row's conditional, continuous offsets inside the cells.
V3 envSampleDir(const Scene &s, float uRow, float uCol, float &pdf)
{
    pdf = 0.0f;
    uint32_t r = cdfIndex(s.envMarg.data(), s.envH, uRow);
    float m0 = s.envMarg[r], m1 = s.envMarg[r + 1];
    float dv = m1 > m0 ? (uRow - m0) / (m1 - m0) : 0.0f;
    const float *cdf = &s.envCond[(size_t)r * (s.envW + 1)];
    uint32_t c = cdfIndex(cdf, s.envW, uCol);
    float c0 = cdf[c], c1 = cdf[c + 1];
    float du = c1 > c0 ? (uCol - c0) / (c1 - c0) : 0.0f;
    float u = ((float)c + du) / (float)s.envW;
    float w = ((float)r + dv) / (float)s.envH;
    float x = u - 0.25f;
    if (x < 0.0f)
        x += 1.0f;
    float lon = (x - 0.5f) / 0.1591f;
    if (std::fabs(lon) > PI)
        return v3(0.0f, 1.0f, 0.0f);
    float lat = std::min(std::max((w - 0.5f) / 0.3183f, -0.5f * PI), 0.5f * PI);
    float cl = std::cos(lat);
    if (cl < 1e-6f)
        return v3(0.0f, 1.0f, 0.0f);
    pdf = s.envFunc[(size_t)r * s.envW + c] / s.envInt * (0.1591f * 0.3183f) / cl;
    return v3(cl * std::cos(lon), std::sin(lat), cl * std::sin(lon));
}

// ------------------------------------------------------------------ shader math (GLSL includes)

// sampling.glsl:3-40
V3 cosineSampleHemisphere(float r0, float r1, float &pdf)
{
    float rx = 2.0f * r0 - 1.0f, ry = 2.0f * r1 - 1.0f;
    V3 dir = v3s(0.0f);
    if (rx == 0 && ry == 0) {
        dir.x = 0;
        dir.z = 0;
    } else if (std::fabs(rx) > std::fabs(ry)) {
        float r = rx, phi = PI_OVER_FOUR * (ry / rx);
        dir.x = r * std::cos(phi);
        dir.z = r * std::sin(phi);
    } else {
        float r = ry, phi = PI_OVER_TWO - PI_OVER_FOUR * (rx / ry);
        dir.x = r * std::cos(phi);
        dir.z = r * std::sin(phi);
    }
    dir.y = std::sqrt(std::max(0.0f, 1.0f - dir.x * dir.x - dir.z * dir.z));
    pdf = INV_PI * dir.y;
    pdf = std::max(pdf, EPSILON);
    return dir;
}
float cosineSampleHemispherePdf(float c) { return c * INV_PI; }
// sampling.glsl:42-46
void uniformSampleTriangle(float r0, float r1, float &bx, float &by)
{
    float a = std::sqrt(1.0f - r0);
    bx = 1 - a;
    by = a * r1;
}
// sampling.glsl:48-67
void concentricSampleDisk(float r0, float r1, float &x, float &y)
{
    float ux = 2.0f * r0 - 1.0f, uy = 2.0f * r1 - 1.0f;
    if (ux == 0 && uy == 0) {
        x = y = 0;
        return;
    }
    float theta, r;
    if (std::fabs(ux) > std::fabs(uy)) {
        r = ux;
        theta = PI_OVER_FOUR * (uy / ux);
    } else {
        r = uy;
        theta = PI_OVER_TWO - PI_OVER_FOUR * (ux / uy);
    }
    x = r * std::cos(theta);
    y = r * std::sin(theta);
}

// frame.glsl:1-88
struct Frame {
    V3 normal, tangent, bitangent;
};
bool fixFrame(V3 &normal, V3 &tangent, V3 &bitangent, V3 ray)
{
    bool flipped = false;
    if (dot(normal, ray) > 0) {
        normal = -normal;
        tangent = -tangent;
        flipped = true;
    }
    normal = normalize(normal);
    tangent = normalize(tangent);
    bitangent = normalize(bitangent);
    if (std::fabs(dot(normal, tangent)) > 0.999f) {
        bitangent = std::fabs(normal.z) < 0.999f ? v3(0, 0, 1) : v3(1, 0, 0);
        tangent = cross(bitangent, normal);
        bitangent = cross(normal, tangent);
    } else {
        bitangent = cross(normal, tangent);
        tangent = cross(bitangent, normal);
    }
    return flipped;
}
V3 localToWorld(const Frame &f, V3 l) { return f.tangent * l.x + f.normal * l.y + f.bitangent * l.z; }
V3 worldToLocal(const Frame &f, V3 w) { return {dot(w, f.tangent), dot(w, f.normal), dot(w, f.bitangent)}; }
void applyNormalToFrame(Frame &f, V3 n)
{
    V3 nw = localToWorld(f, n);
    f.normal = nw;
    f.tangent = cross(f.normal, f.bitangent);
    f.bitangent = cross(f.tangent, f.normal);
}
void createCoordinateSystem(V3 v1, V3 &v2, V3 &v3_)
{
    if (std::fabs(v1.x) > std::fabs(v1.y))
        v2 = v3(-v1.z, 0, v1.x) / std::sqrt(v1.x * v1.x + v1.z * v1.z);
    else
        v2 = v3(0, v1.z, -v1.y) / std::sqrt(v1.y * v1.y + v1.z * v1.z);
    v3_ = cross(v1, v2);
}
// utils.glsl:10-14
V3 processNormalFromNormalMap(V3 c)
{
    V3 N = c * 2.0f - v3s(1.0f);
    return normalize(v3(N.x, N.z, -N.y));
}

// brdfs/common.glsl:3-49
float schlickWeight(float c)
{
    float m = std::min(std::max(1.0f - c, 0.0f), 1.0f);
    return (m * m) * (m * m) * m;
}
float GTR2(float NdotH, float a)
{
    float a2 = a * a;
    float t = 1.0f + (a2 - 1.0f) * NdotH * NdotH;
    return a2 / (PI * t * t);
}
float smithG_GGX(float NdotV, float alphaG)
{
    float a = alphaG * alphaG, b = NdotV * NdotV;
    return 1.0f / (std::fabs(NdotV) + std::max(std::sqrt(a + b - a * b), EPSILON));
}
// brdfs/pbrStandard.glsl:3-214
struct PBR {
    V3 albedo;
    float metallic, roughness;
};
V3 evalDisneyDiffuse(float NdotL, float NdotV, float LdotH, const PBR &p)
{
    float FL = schlickWeight(NdotL), FV = schlickWeight(NdotV);
    float Fd90 = 0.5f + 2.0f * LdotH * LdotH * p.roughness;
    float Fd = fmix(1.0f, Fd90, FL) * fmix(1.0f, Fd90, FV);
    return (1.0f / PI) * Fd * p.albedo;
}
V3 evalDisneyMicrofacetIsotropic(float NdotL, float NdotV, float NdotH, float LdotH, const PBR &p)
{
    float Cdlum = 0.3f * p.albedo.x + 0.6f * p.albedo.y + 0.1f * p.albedo.z;
    V3 Ctint = Cdlum > 0.0f ? p.albedo / Cdlum : v3s(1.0f);
    float specular = 0.5f, specularTint = 0.0f;
    V3 Cspec0 = vmix(specular * 0.08f * vmix(v3s(1.0f), Ctint, specularTint), p.albedo, p.metallic);
    float a = std::max(0.001f, p.roughness * p.roughness);
    float Ds = GTR2(NdotH, a);
    float FH = schlickWeight(LdotH);
    V3 Fs = vmix(Cspec0, v3s(1.0f), FH);
    float Gs = smithG_GGX(NdotL, a);
    Gs *= smithG_GGX(NdotV, a);
    return Gs * Fs * Ds;
}
float pdfDisneyMicrofacetIsotropic(V3 wi, V3 wo, const PBR &p)
{
    if (!(wo.y > 0))
        return 0.0f;
    if (!(wi.y > 0))
        return 0.0f;
    V3 wh = normalize(wo + wi);
    float NdotH = std::max(wh.y, EPSILON);
    float alpha2 = p.roughness * p.roughness;
    alpha2 *= alpha2;
    float cos2Theta = NdotH * NdotH;
    float denom = cos2Theta * (alpha2 - 1.0f) + 1.0f;
    if (denom == 0.0f)
        return 0.0f;
    float pdfDistribution = alpha2 * NdotH / (PI * denom * denom);
    return pdfDistribution / (4.0f * dot(wo, wh));
}
void sampleDisneyMicrofacetIsotropic(V3 &wi, V3 wo, float &pdf, float u0, float u1, const PBR &p)
{
    float phi = (2.0f * PI) * u1;
    float alpha = p.roughness * p.roughness;
    float tanTheta2 = alpha * alpha * u0 / (1.0f - u0);
    float cosTheta = 1.0f / std::sqrt(1.0f + tanTheta2);
    float sinTheta = std::sqrt(std::max(EPSILON, 1.0f - cosTheta * cosTheta));
    V3 wh = v3(sinTheta * std::cos(phi), cosTheta, sinTheta * std::sin(phi));
    if (!(wh.y > 0))
        wh = wh * -1.0f;
    V3 I = -wo;
    wi = I - 2.0f * dot(wh, I) * wh; // reflect(-wo, wh)
    pdf = pdfDisneyMicrofacetIsotropic(wi, wo, p);
}
float getDiffuseSamplingRatio(const PBR &p)
{
    float d = std::max(1.0f - p.metallic, 0.1f);
    float g = std::max(1.0f - p.roughness, 0.1f);
    return d / (d + g);
}
V3 evalPBRStandard(const PBR &p, V3 wi, V3 wo, V3 H)
{
    float NdotL = wi.y, NdotV = wo.y;
    if (NdotL < 0.0f || NdotV < 0.0f)
        return v3s(0.0f);
    float NdotH = H.y, LdotH = dot(wi, H);
    V3 diffuse = evalDisneyDiffuse(NdotL, NdotV, LdotH, p);
    V3 glossy = evalDisneyMicrofacetIsotropic(NdotL, NdotV, NdotH, LdotH, p);
    return (diffuse * (1.0f - p.metallic) + glossy) * NdotL;
}
float pdfPBRStandard(V3 wi, V3 wo, const PBR &p)
{
    float c = wi.y;
    if (c < 0)
        return 0.0f;
    float pd = cosineSampleHemispherePdf(c);
    float pm = pdfDisneyMicrofacetIsotropic(wi, wo, p);
    float r = getDiffuseSamplingRatio(p);
    return pd * r + pm * (1.0f - r);
}
V3 samplePBRStandard(V3 &wi, V3 wo, float &pdf, const PBR &p, float u0, float u1, float rnd)
{
    pdf = 0.0f;
    wi = v3s(0.0f);
    float r = getDiffuseSamplingRatio(p);
    if (rnd <= r)
        wi = cosineSampleHemisphere(u0, u1, pdf);
    else
        sampleDisneyMicrofacetIsotropic(wi, wo, pdf, u0, u1, p);
    V3 F = evalPBRStandard(p, wi, wo, normalize(wi + wo));
    pdf = pdfPBRStandard(wi, wo, p);
    if (pdf < EPSILON)
        return v3s(0.0f);
    return F;
}
// pt/MIS.glsl:5-10
// With an overflowing square (a light sample grazing the emitter's own
// plane) the weight is the limit from the ratio of the pdfs instead of
// inf / inf, as the library computes it; finite squares are unchanged.
float PowerHeuristic(float fPdf, float gPdf)
{
    float f = fPdf, g = gPdf;
    const float ff = f * f, gg = g * g;
    if (std::isinf(ff) || std::isinf(gg)) {
        if (std::isinf(f) || std::isinf(g))
            return std::isinf(g) ? (std::isinf(f) ? 0.5f : 0.0f) : 1.0f;
        const float r = g / f;
        return 1.0f / (1.0f + r * r);
    }
    return ff / (ff + gg);
}
// phaseFunctions.glsl:1-31
float HenyeyGreenstein(float cosTheta, float g)
{
    float denom = 1.0f + g * g + 2.0f * g * cosTheta;
    return INV_4PI * (1.0f - g * g) / (denom * std::sqrt(denom));
}
float HG_Sample(V3 wo, V3 &wi, float r0, float r1, float g)
{
    float cosTheta;
    if (std::fabs(g) < 1e-3f)
        cosTheta = 1.0f - 2.0f * r0;
    else {
        float sqrTerm = (1.0f - g * g) / (1.0f + g - 2.0f * g * r0);
        cosTheta = -(1.0f + g * g - sqrTerm * sqrTerm) / (2.0f * g);
    }
    float sinTheta = std::sqrt(std::max(0.0f, 1.0f - cosTheta * cosTheta));
    float phi = 2.0f * PI * r1;
    V3 v1, v2;
    createCoordinateSystem(wo, v1, v2);
    wi = sinTheta * std::cos(phi) * v1 + sinTheta * std::sin(phi) * v2 + cosTheta * wo;
    return HenyeyGreenstein(cosTheta, g);
}

// ------------------------------------------------------------------ integrator
struct Params {
    float viewInv[16], projInv[16]; // column-major
    V3 background;
    float envType, lensRadius, focalDistance, envIntensity, zfar;
    int camVolume;
    uint32_t W, H, batchSize, batches, depth, totalSamples, totalLights;
    uint32_t envLight = 0; // the environment is one more light of the pick
    uint32_t sampler = 0;  // 0: RTGEMS, 1: PMJ (VVPT_RENDER_SAMPLER_PMJ)
    bool altOrder = false; // also render the emitter rays' other candidate order
};

// RayPayloadPrimary, shaders/pt/structs_pt.glsl:4-30
struct Payload {
    V3 radiance, beta;
    uint32_t recursionDepth, surfaceDepth;
    V3 albedo, normal;
    V3 origin, direction;
    bool stop, insideVolume;
    float vtmin;
    uint32_t volumeMaterialIndex;
    uint32_t rngState;      // RTGEMS state; the dimension under the PMJ sampler
    bool sampled = false;   // direction drawn by BSDF/phase sampling (env MIS)
    float samplePdf = 0.0f;
    // PMJ sampler (structs_pt.glsl:24-29)
    uint32_t pmj = 0;
    uint32_t pixelX = 0, pixelY = 0, sampleIndex = 0, samplesPerPixel = 0;
    V3 altDelta{0.0f, 0.0f, 0.0f}; // second image minus first, this sample
};

// ---- PMJ sampler, shaders/include/rng/rng_pmj.glsl:20-107, over the tables
// set by oracle_set_sampler_tables ([16][16384][2], [48][128][128])
const float *g_pmj = nullptr, *g_blue_noise = nullptr;
constexpr uint32_t kPmjSeed = 2873468793u; // rng_pmj_defines.glsl
constexpr float kOneMinusEps = 0.999999f;  // constants.glsl:2

uint64_t mixBits(uint64_t v) // rng_pmj.glsl:28-35
{
    v ^= (v >> 31);
    v *= 9202493588570546565ULL;
    v ^= (v >> 27);
    v *= 9357036318526133325ULL;
    v ^= (v >> 33);
    return v;
}

uint32_t permutationElement(uint32_t i, uint32_t l, uint32_t p) // rng_pmj.glsl:37-64
{
    uint32_t w = l - 1;
    w |= w >> 1;
    w |= w >> 2;
    w |= w >> 4;
    w |= w >> 8;
    w |= w >> 16;
    do {
        i ^= p;
        i *= 0xe170893du;
        i ^= p >> 16;
        i ^= (i & w) >> 4;
        i ^= p >> 8;
        i *= 0x0929eb3fu;
        i ^= p >> 23;
        i ^= (i & w) >> 1;
        i *= 1u | p >> 27;
        i *= 0x6935fa69u;
        i ^= (i & w) >> 11;
        i *= 0x74dcb303u;
        i ^= (i & w) >> 2;
        i *= 0x9e501cc3u;
        i ^= (i & w) >> 2;
        i *= 0xc860a3dfu;
        i &= w;
        i ^= i >> 5;
    } while (i >= l);
    return (i + p) % l;
}

uint32_t pmjHash(const Payload &pl)
{
    return (uint32_t)mixBits(((uint64_t)pl.pixelX << 48) ^ ((uint64_t)pl.pixelY << 32) ^
                             ((uint64_t)pl.rngState << 16) ^ (uint64_t)kPmjSeed);
}

inline float rand1D(Payload &p)
{
    if (!p.pmj)
        return uintToFloat(xorshift(p.rngState));
    // rng_pmj.glsl:66-78
    uint32_t index = permutationElement(p.sampleIndex, p.samplesPerPixel, pmjHash(p));
    float delta = g_blue_noise[((size_t)(p.rngState % 48u) * 128u + p.pixelX % 128u) * 128u + p.pixelY % 128u];
    p.rngState++;
    return std::min(((float)index + delta) / (float)p.samplesPerPixel, kOneMinusEps);
}

// rand2D: rng_def.glsl (two rand1D draws) or rng_pmj.glsl:80-107
inline void rand2D(Payload &p, float &u0, float &u1)
{
    if (!p.pmj) {
        u0 = rand1D(p);
        u1 = rand1D(p);
        return;
    }
    uint32_t index = p.sampleIndex;
    const uint32_t inst = p.rngState / 2;
    if (inst >= 16)
        index = permutationElement(p.sampleIndex, p.samplesPerPixel, pmjHash(p));
    const float *u = g_pmj + ((size_t)(inst % 16u) * 16384u + index % 16384u) * 2;
    p.rngState += 2;
    u0 = std::min(u[0], kOneMinusEps);
    u1 = std::min(u[1], kOneMinusEps);
}

struct HitInfo { // process_hit.glsl + construct_frame.glsl
    const vvpt_material *material;
    const Inst *inst;
    const vvpt_vertex *v0, *v1, *v2;
    float bx, by, bz;
    float uvx, uvy;
    V3 worldPosition;
    Frame frame;
    bool flipped;
};

HitInfo process_hit(const Scene &s, const Hit &h, V3 rayDir)
{
    HitInfo hi;
    const Inst &in = s.inst[h.inst];
    const Mesh &m = s.meshes[in.mesh];
    hi.inst = &in;
    hi.material = &s.mats[in.src->material_index];
    const uint32_t *ix = m.idx + 3 * h.prim;
    hi.v0 = &m.v[ix[0]];
    hi.v1 = &m.v[ix[1]];
    hi.v2 = &m.v[ix[2]];
    hi.bx = 1.0f - h.u - h.v;
    hi.by = h.u;
    hi.bz = h.v;
    hi.uvx = hi.v0->uv[0] * hi.bx + hi.v1->uv[0] * hi.by + hi.v2->uv[0] * hi.bz;
    hi.uvy = hi.v0->uv[1] * hi.bx + hi.v1->uv[1] * hi.by + hi.v2->uv[1] * hi.bz;
    auto interp = [&](const float *a, const float *b, const float *c) {
        return v3(a[0], a[1], a[2]) * hi.bx + v3(b[0], b[1], b[2]) * hi.by + v3(c[0], c[1], c[2]) * hi.bz;
    };
    V3 lp = interp(hi.v0->position, hi.v1->position, hi.v2->position);
    hi.worldPosition = xpoint(in.o2w, lp);
    V3 ln = interp(hi.v0->normal, hi.v1->normal, hi.v2->normal);
    V3 lt = interp(hi.v0->tangent, hi.v1->tangent, hi.v2->tangent);
    V3 lb = interp(hi.v0->bitangent, hi.v1->bitangent, hi.v2->bitangent);
    hi.frame.normal = normalize(xnormalT(in.w2o, ln));
    hi.frame.tangent = normalize(xnormalT(in.w2o, lt));
    hi.frame.bitangent = normalize(xnormalT(in.w2o, lb));
    hi.flipped = fixFrame(hi.frame.normal, hi.frame.tangent, hi.frame.bitangent, rayDir);
    return hi;
}

struct Ctx {
    const Scene &s;
    const Params &p;
};

// process_volume_transmittance.glsl:1-9
V3 volumeTransmittance(const Ctx &c, uint32_t vol, float vtstart, float vtend)
{
    const vvpt_material &m = c.s.mats[vol];
    V3 sa = v3(m.albedo[0], m.albedo[1], m.albedo[2]);
    V3 ss = v3(std::max(m.metallic_roughness_ao[0], EPSILON), std::max(m.metallic_roughness_ao[1], EPSILON),
               std::max(m.metallic_roughness_ao[2], EPSILON));
    V3 st = sa + ss;
    float d = std::max(vtend - vtstart, EPSILON);
    return vexp(-st * d);
}

struct LSR { // LightSamplingRecord
    V3 direction, radiance;
    float pdf;
    bool isDeltaLight;
};

inline V3 emissive_of(const Ctx &c, const vvpt_material &m, float u, float v)
{
    C4 t = texture(c.s, m.textures2[0], u * m.uv_tiling[0], v * m.uv_tiling[1]);
    return (m.emissive[3] * v3(m.emissive[0], m.emissive[1], m.emissive[2])) * rgb(t);
}
inline float alpha_of(const Ctx &c, const vvpt_material &m, float u, float v)
{
    return m.albedo[3] * texture(c.s, m.textures2[3], u * m.uv_tiling[0], v * m.uv_tiling[1]).r;
}

// Shadow-ray loop: lightSampling.glsl:108-144 with raySecondary.rahit/.rchit/.rmiss.
// Any-hit candidates are visited nearest first.
V3 shadow(const Ctx &c, const Payload &pl, V3 originPosition, V3 dir, float tmax)
{
    const float tmin = 0.0001f;
    V3 origin = originPosition;
    V3 throughput = v3s(1.0f);
    bool shadowed = false, stop = false;
    bool inside = pl.insideVolume;
    uint32_t vol = pl.volumeMaterialIndex;
    float distanceT = tmax - tmin;
    for (uint32_t d = 0; d < c.p.depth; d++) {
        float vtmin = tmin;
        Hit after;
        bool accepted = false;
        Hit acc;
        for (int guard = 0;; guard++) {
            Hit h = trace_after(c.s, origin, dir, tmin, distanceT, after);
            if (h.inst == NOHIT)
                break;
            const Inst &in = c.s.inst[h.inst];
            const vvpt_material &m = c.s.mats[in.src->material_index];
            bool isTransparent = m.metallic_roughness_ao[3] >= 0.99f;
            if (!isTransparent || guard > 1024) {
                stop = shadowed = true;
                accepted = true;
                acc = h;
                break;
            }
            HitInfo hi = process_hit(c.s, h, dir);
            float alpha = alpha_of(c, m, hi.uvx, hi.uvy);
            throughput = throughput * v3s(1.0f - alpha);
            if (in.src->id[1] != in.src->id[2]) {
                accepted = true;
                acc = h;
                break;
            }
            if (max3(throughput) > EPSILON) {
                shadowed = false;
                after = h;
                continue;
            }
            stop = shadowed = true;
            accepted = true;
            acc = h;
            break;
        }
        if (!accepted) {
            stop = true;
            shadowed = false;
            if (inside) {
                float vtend = std::min((float)(uint32_t)c.p.zfar, distanceT);
                throughput = throughput * volumeTransmittance(c, vol, vtmin, vtend);
                shadowed = !(max3(throughput) > EPSILON);
            }
        } else if (!stop) {
            HitInfo hi = process_hit(c.s, acc, dir);
            bool ret = false;
            if (inside) {
                throughput = throughput * volumeTransmittance(c, vol, vtmin, acc.t);
                if (max3(throughput) < EPSILON) {
                    stop = shadowed = true;
                    ret = true;
                }
            }
            if (!ret) {
                vtmin = acc.t;
                inside = false;
                const Inst &in = c.s.inst[acc.inst];
                float nv = hi.flipped ? in.src->id[1] : in.src->id[2];
                if (nv != -1.0f) {
                    inside = true;
                    vol = (uint32_t)nv;
                }
                origin = hi.worldPosition;
            }
        }
        distanceT -= vtmin;
        if (stop)
            break;
    }
    if (shadowed)
        throughput = v3s(0.0f);
    return throughput;
}

// sampleLight, lightSampling.glsl:1-147
// allowEnv: with the environment as a light (VVPT_RENDER_ENV_IS), whether
// picking it contributes (not at a path's last event).
LSR sampleLight(const Ctx &c, Payload &pl, V3 originPosition, bool allowEnv)
{
    LSR lsr;
    lsr.isDeltaLight = true;
    lsr.radiance = v3s(0.0f);
    lsr.pdf = 1.0f;
    lsr.direction = v3s(0.0f);
    uint32_t totalLights = c.p.totalLights + c.p.envLight;
    if (totalLights == 0)
        return lsr;
    float pdf = 1.0f / (float)totalLights;
    uint32_t randomLight = (uint32_t)(rand1D(pl) * (float)totalLights);
    if (randomLight >= totalLights)
        randomLight = totalLights - 1;
    float tmax = 10000.0f;
    if (randomLight == c.p.totalLights) {
        lsr.isDeltaLight = false;
        if (!allowEnv)
            return lsr;
        float uRow, uCol;
        rand2D(pl, uRow, uCol);
        float epdf;
        lsr.direction = envSampleDir(c.s, uRow, uCol, epdf);
        tmax = c.p.zfar;
        if (epdf > 0.0f) {
            lsr.radiance = env_sample(c.s, lsr.direction) * ((int)c.p.envType == 1 ? c.p.envIntensity : 1.0f);
            lsr.pdf = pdf * epdf;
            lsr.radiance = lsr.radiance * shadow(c, pl, originPosition, lsr.direction, tmax);
        }
        return lsr;
    }
    const vvpt_light_instance &L = c.s.lights[randomLight];
    V3 lpos = v3(L.position[0], L.position[1], L.position[2]);
    if (L.info[3] == 0) {
        const vvpt_light_data &ld = c.s.ldata[L.info[0]];
        V3 direction = lpos - originPosition;
        tmax = length(direction);
        lsr.direction = direction / tmax;
        float dd = length(originPosition - lpos);
        lsr.radiance = v3(ld.color[0], ld.color[1], ld.color[2]) * (1.0f / (dd * dd)) * ld.color[3];
        lsr.pdf = pdf * 1.0f;
        lsr.isDeltaLight = true;
    } else if (L.info[3] == 1) {
        const vvpt_light_data &ld = c.s.ldata[L.info[0]];
        lsr.direction = -lpos;
        tmax = c.p.zfar;
        lsr.radiance = v3(ld.color[0], ld.color[1], ld.color[2]) * ld.color[3];
        lsr.pdf = pdf * 1.0f;
        lsr.isDeltaLight = true;
    } else if (L.info[3] == 2) {
        const Inst &in = c.s.inst[L.info[1]];
        const Mesh &m = c.s.meshes[in.mesh];
        const vvpt_material &mat = c.s.mats[in.src->material_index];
        Rows T;
        for (int k = 0; k < 4; k++) {
            T.m[0][k] = L.position[k];
            T.m[1][k] = L.position1[k];
            T.m[2][k] = L.position2[k];
        }
        uint32_t ntri = in.src->num_triangles;
        uint32_t randomTriangle = (uint32_t)(rand1D(pl) * (float)ntri);
        if (randomTriangle >= ntri)
            randomTriangle = ntri - 1;
        const uint32_t *ix = m.idx + 3 * randomTriangle;
        float trianglePdf = 1.0f / (float)ntri;
        float r0, r1;
        rand2D(pl, r0, r1);
        float bx, by;
        uniformSampleTriangle(r0, r1, bx, by);
        float bz = 1.0f - bx - by;
        const vvpt_vertex &v0 = m.v[ix[0]], &v1 = m.v[ix[1]], &v2 = m.v[ix[2]];
        auto P = [](const float *a) { return v3(a[0], a[1], a[2]); };
        V3 p0 = xpoint(T, P(v0.position)), p1 = xpoint(T, P(v1.position)), p2 = xpoint(T, P(v2.position));
        float area = 0.5f * length(cross(p1 - p0, p2 - p0));
        float sampledPointPdf = 1.0f / area;
        V3 sp = bx * P(v0.position) + by * P(v1.position) + bz * P(v2.position);
        V3 sn = bx * P(v0.normal) + by * P(v1.normal) + bz * P(v2.normal);
        float su = bx * v0.uv[0] + by * v1.uv[0] + bz * v2.uv[0];
        float sv = bx * v0.uv[1] + by * v1.uv[1] + bz * v2.uv[1];
        sp = xpoint(T, sp);
        // transpose(inverse(transform)) * vec4(n, 0)
        float tm[16] = {L.position[0], L.position1[0], L.position2[0], 0, L.position[1], L.position1[1], L.position2[1], 0,
                        L.position[2], L.position1[2], L.position2[2], 0, L.position[3], L.position1[3], L.position2[3], 1};
        Rows inv;
        invert_rows(tm, inv);
        sn = v3(inv.m[0][0] * sn.x + inv.m[1][0] * sn.y + inv.m[2][0] * sn.z,
                inv.m[0][1] * sn.x + inv.m[1][1] * sn.y + inv.m[2][1] * sn.z,
                inv.m[0][2] * sn.x + inv.m[1][2] * sn.y + inv.m[2][2] * sn.z);
        V3 direction = sp - originPosition;
        tmax = length(direction);
        lsr.direction = direction / tmax;
        float dp = dot(-lsr.direction, sn);
        if (dp > 0) {
            lsr.radiance = emissive_of(c, mat, su, sv);
            float dd = length(originPosition - sp);
            lsr.pdf = pdf * trianglePdf * sampledPointPdf * (dd * dd) / dp;
        } else {
            lsr.radiance = v3s(0.0f);
            lsr.pdf = 0.0f;
        }
        lsr.isDeltaLight = false;
    }
    if (!isBlack(lsr.radiance))
        lsr.radiance = lsr.radiance * shadow(c, pl, originPosition, lsr.direction, tmax);
    return lsr;
}

// Entry distance of a ray into an instance's world box (the mesh box in
// object space, entered along the object-space ray; same parameter t).
float instance_entry(const Scene &s, uint32_t id, V3 o, V3 d, float tmin)
{
    const Inst &in = s.inst[id];
    const Mesh &m = s.meshes[in.mesh];
    V3 oo = xpoint(in.w2o, o), od = xvector(in.w2o, d);
    float t0 = tmin;
    for (int a = 0; a < 3; a++) {
        float oa = comp(oo, a), da = comp(od, a);
        float ta = (m.lo[a] - oa) / da, tb = (m.hi[a] - oa) / da;
        if (std::isnan(ta) || std::isnan(tb))
            continue;
        if (ta > tb)
            std::swap(ta, tb);
        t0 = std::max(t0, ta);
    }
    return t0;
}

// Every candidate of a ray on [tmin, tmax] in instance-box-entry order: the
// instances by the distance at which the ray enters their boxes (ties by
// slot), each instance's candidates nearest first. This is the order a
// stack traversal that visits the nearer child box first reports any-hit
// candidates in when the instance boxes are TLAS leaves: a ray that starts
// inside an instance's box sees all of that instance's candidates before
// those of an instance it enters later, whatever their distances.
std::vector<Hit> candidates_instance_order(const Scene &s, V3 o, V3 d, float tmin, float tmax)
{
    std::vector<Hit> all;
    Hit after;
    for (int k = 0; k < 4096; k++) {
        Hit h = trace_after(s, o, d, tmin, tmax, after);
        if (h.inst == NOHIT)
            break;
        all.push_back(h);
        after = h;
    }
    std::vector<float> te(all.size());
    for (size_t i = 0; i < all.size(); i++)
        te[i] = instance_entry(s, all[i].inst, o, d, tmin);
    std::vector<size_t> idx(all.size());
    for (size_t i = 0; i < idx.size(); i++)
        idx[i] = i;
    std::stable_sort(idx.begin(), idx.end(), [&](size_t a, size_t b) {
        if (te[a] != te[b])
            return te[a] < te[b];
        return all[a].inst < all[b].inst;
    });
    std::vector<Hit> r;
    r.reserve(all.size());
    for (size_t i : idx)
        r.push_back(all[i]);
    return r;
}

// next_event_estimation.glsl with rayNEE.rahit/.rchit/.rmiss. The any-hit
// shader sees candidates in the order the hardware reports them; the defined
// order here is nearest first (instanceOrder false). With instanceOrder the
// walk takes the candidates in instance-box-entry order instead
// (candidates_instance_order), the other end of what a traversal may report;
// it only feeds the oracle's diagnostic second image. Returns the radiance
// the emitter ray adds.
V3 emitterRay(const Ctx &c, const Payload &pl, float sampleDirectionPDF, bool instanceOrder)
{
    const float tmin = 0.0001f;
    const float tmax = c.p.zfar;
    V3 origin = pl.origin;
    V3 dir = pl.direction;
    V3 throughput = v3s(1.0f), emissive = v3s(0.0f);
    float pdf = 0.0f;
    bool stop = false;
    bool inside = pl.insideVolume;
    uint32_t vol = pl.volumeMaterialIndex;
    for (uint32_t d = 0; d < c.p.depth; d++) {
        float vtmin = tmin;
        Hit after;
        bool accepted = false;
        Hit acc;
        std::vector<Hit> ordered;
        if (instanceOrder)
            ordered = candidates_instance_order(c.s, origin, dir, tmin, tmax);
        for (int guard = 0;; guard++) {
            Hit h;
            if (instanceOrder) {
                if (guard >= (int)ordered.size())
                    break;
                h = ordered[guard];
            } else {
                h = trace_after(c.s, origin, dir, tmin, tmax, after);
            }
            if (h.inst == NOHIT)
                break;
            const Inst &in = c.s.inst[h.inst];
            const vvpt_material &m = c.s.mats[in.src->material_index];
            HitInfo hi = process_hit(c.s, h, dir);
            V3 em = emissive_of(c, m, hi.uvx, hi.uvy);
            bool isTransparent = m.metallic_roughness_ao[3] >= 0.99f;
            if (isBlackEps(em, 0.05f)) {
                if (!isTransparent || guard > 1024) {
                    stop = true;
                    throughput = v3s(0.0f);
                    emissive = v3s(0.0f);
                    accepted = true;
                    acc = h;
                    break;
                }
                float alpha = alpha_of(c, m, hi.uvx, hi.uvy);
                throughput = throughput * v3s(1.0f - alpha);
                if (in.src->id[1] != in.src->id[2]) {
                    accepted = true;
                    acc = h;
                    break;
                }
                after = h;
                continue;
            }
            stop = true;
            accepted = true;
            acc = h;
            if (inside) {
                throughput = throughput * volumeTransmittance(c, vol, vtmin, h.t);
                if (max3(throughput) < EPSILON) {
                    throughput = v3s(0.0f);
                    emissive = v3s(0.0f);
                    break;
                }
            }
            auto P = [](const float *a) { return v3(a[0], a[1], a[2]); };
            V3 ln = P(hi.v0->normal) * hi.bx + P(hi.v1->normal) * hi.by + P(hi.v2->normal) * hi.bz;
            V3 wn = normalize(xnormalT(in.w2o, ln));
            bool flipped = dot(wn, dir) > 0;
            if (flipped) {
                emissive = v3s(0.0f);
                throughput = v3s(0.0f);
                break;
            }
            emissive = em;
            V3 lp = P(hi.v0->position) * hi.bx + P(hi.v1->position) * hi.by + P(hi.v2->position) * hi.bz;
            V3 wp = xpoint(in.o2w, lp);
            V3 w0 = xpoint(in.o2w, P(hi.v0->position)), w1 = xpoint(in.o2w, P(hi.v1->position)),
               w2 = xpoint(in.o2w, P(hi.v2->position));
            float area = 0.5f * length(cross(w1 - w0, w2 - w0));
            float sampledPointPdf = (1.0f / (float)in.src->num_triangles) * (1.0f / area);
            float dp = dot(-dir, wn);
            if (dp > 0) {
                V3 objOrigin = xpoint(in.w2o, origin); // gl_ObjectRayOriginEXT, rayNEE.rahit.glsl:122
                float dd = length(objOrigin - wp);
                float lightDirectPdf = sampledPointPdf * (dd * dd) / dp;
                pdf = lightDirectPdf * (1.0f / (float)(c.p.totalLights + c.p.envLight));
            } else {
                pdf = 0.0f;
                emissive = v3s(0.0f);
            }
            break;
        }
        if (!accepted) {
            stop = true;
            emissive = v3s(0.0f);
            pdf = 0.0f;
        } else if (!stop) {
            HitInfo hi = process_hit(c.s, acc, dir);
            bool ret = false;
            if (inside) {
                throughput = throughput * volumeTransmittance(c, vol, vtmin, acc.t);
                if (max3(throughput) < EPSILON) {
                    stop = true;
                    throughput = v3s(0.0f);
                    emissive = v3s(0.0f);
                    ret = true;
                }
            }
            if (!ret) {
                vtmin = acc.t;
                inside = false;
                const Inst &in = c.s.inst[acc.inst];
                float nv = hi.flipped ? in.src->id[1] : in.src->id[2];
                if (nv != -1.0f) {
                    inside = true;
                    vol = (uint32_t)nv;
                }
                origin = hi.worldPosition;
            }
        }
        if (stop)
            break;
    }
    if (isBlack(emissive))
        return v3s(0.0f);
    float w = PowerHeuristic(sampleDirectionPDF, pdf);
    return w * throughput * emissive * pl.beta;
}

void nextEventEstimation(const Ctx &c, Payload &pl, float sampleDirectionPDF)
{
    V3 add = emitterRay(c, pl, sampleDirectionPDF, false);
    if (c.p.altOrder) {
        // the second image differs from the first only by what this emitter
        // ray adds under the other candidate order
        V3 alt = emitterRay(c, pl, sampleDirectionPDF, true);
        pl.altDelta = pl.altDelta + (alt - add);
    }
    if (!isBlack(add))
        pl.radiance = pl.radiance + add;
}

void russianRoulette(Payload &pl)
{
    float rrsample = rand1D(pl);
    if (pl.recursionDepth > RUSSIAN_ROULETTE_DEPTH) {
        float maxBeta = std::max(pl.beta.x, std::max(pl.beta.y, pl.beta.z));
        if (rrsample >= maxBeta) {
            pl.stop = true;
            return;
        }
        pl.beta = pl.beta * (1.0f / maxBeta);
    }
}

// process_volume_hit.glsl:1-80 (returns sampledMedium)
bool processVolumeHit(const Ctx &c, Payload &pl, uint32_t vol, float vtstart, float vtend, V3 worldRayDir)
{
    const vvpt_material &m = c.s.mats[vol];
    V3 sigma_a = v3(m.albedo[0], m.albedo[1], m.albedo[2]);
    V3 sigma_s = v3(std::max(m.metallic_roughness_ao[0], EPSILON), std::max(m.metallic_roughness_ao[1], EPSILON),
                    std::max(m.metallic_roughness_ao[2], EPSILON));
    V3 sigma_t = sigma_a + sigma_s;
    float g = std::max(std::min(m.emissive[0], 0.99f), -0.99f);
    V3 dirn = normalize(worldRayDir);
    V3 wo = -dirn;
    float dist = std::max(vtend - vtstart, EPSILON);
    uint32_t channel = std::min((uint32_t)(rand1D(pl) * 3.0f), 2u);
    float hit_distance = -std::log(1.0f - rand1D(pl)) / comp(sigma_t, channel);
    bool sampledMedium = hit_distance < dist;
    float td = std::min(hit_distance, dist);
    V3 transmittance = vexp(-sigma_t * td);
    V3 density = sampledMedium ? (sigma_t * transmittance) : transmittance;
    float pdf = 0;
    pdf += density.x;
    pdf += density.y;
    pdf += density.z;
    pdf *= 0.3333333f;
    if (pdf == 0)
        pdf = 1.0f;
    V3 F = sampledMedium ? (transmittance * sigma_s / pdf) : (transmittance / pdf);
    pl.beta = pl.beta * F;
    if (sampledMedium) {
        V3 scatteringPosition = pl.origin + (vtstart + hit_distance) * dirn;
        bool lastEvent = pl.recursionDepth + 1 >= c.p.depth;
        LSR lsr = sampleLight(c, pl, scatteringPosition,
                              !lastEvent && !((int)c.p.envType == 2 && pl.surfaceDepth == 0));
        if (!isBlack(lsr.radiance)) {
            float p = HenyeyGreenstein(dot(wo, lsr.direction), g);
            V3 Fp = v3s(p);
            if (!isBlack(Fp)) {
                if (lsr.isDeltaLight)
                    pl.radiance = pl.radiance + lsr.radiance * Fp * pl.beta / lsr.pdf;
                else {
                    float w = PowerHeuristic(lsr.pdf, p);
                    pl.radiance = pl.radiance + w * lsr.radiance * Fp * pl.beta / lsr.pdf;
                }
            }
        }
        V3 sdir;
        float r0, r1;
        rand2D(pl, r0, r1);
        float spdf = HG_Sample(wo, sdir, r0, r1, g);
        pl.origin = scatteringPosition;
        pl.direction = sdir;
        pl.sampled = true;
        pl.samplePdf = spdf;
        nextEventEstimation(c, pl, spdf);
    }
    return sampledMedium;
}

// rayPrimaryPBRStandard.rchit.glsl:45-175 and rayPrimaryLambert.rchit.glsl:45-163
void closestHit(const Ctx &c, Payload &pl, const Hit &h, V3 rayDir)
{
    HitInfo hi = process_hit(c.s, h, rayDir);
    const vvpt_material &mat = *hi.material;
    const bool lambert = (uint32_t)mat.uv_tiling[2] == VVPT_MATERIAL_LAMBERT;
    bool sampledMedium = false;
    if (pl.insideVolume)
        sampledMedium = processVolumeHit(c, pl, pl.volumeMaterialIndex, pl.vtmin, h.t, rayDir);
    if (!sampledMedium) {
        float tu = hi.uvx * mat.uv_tiling[0], tv = hi.uvy * mat.uv_tiling[1];
        float alpha = mat.albedo[3] * texture(c.s, mat.textures2[3], tu, tv).r;
        float transparent = mat.metallic_roughness_ao[3];
        if (transparent > 0) {
            float r = rand1D(pl);
            if (alpha < EPSILON || r > alpha) {
                const vvpt_instance &src = *hi.inst->src;
                if (src.id[1] != src.id[2]) {
                    pl.insideVolume = false;
                    float nv = hi.flipped ? src.id[1] : src.id[2];
                    if (nv != -1.0f) {
                        pl.insideVolume = true;
                        pl.volumeMaterialIndex = (uint32_t)nv;
                    }
                }
                pl.origin = hi.worldPosition;
                pl.direction = normalize(rayDir);
                return;
            }
        }
        C4 nm = texture(c.s, mat.textures2[1], tu, tv);
        applyNormalToFrame(hi.frame, processNormalFromNormalMap(rgb(nm)));
        V3 albedo = v3(mat.albedo[0], mat.albedo[1], mat.albedo[2]) * rgb(texture(c.s, mat.textures1[0], tu, tv));
        PBR pbr{};
        if (!lambert) {
            pbr.albedo = albedo;
            pbr.metallic = mat.metallic_roughness_ao[0] * texture(c.s, mat.textures1[1], tu, tv).r;
            pbr.roughness = mat.metallic_roughness_ao[1] * texture(c.s, mat.textures1[2], tu, tv).r;
            pbr.roughness = std::max(pbr.roughness, 0.035f);
        }
        V3 emissive = (mat.emissive[3] * v3(mat.emissive[0], mat.emissive[1], mat.emissive[2])) *
                      rgb(texture(c.s, mat.textures2[0], tu, tv));
        if (pl.surfaceDepth == 0) {
            pl.albedo = albedo;
            pl.normal = hi.frame.normal * 0.5f + v3s(0.5f);
        }
        if (pl.surfaceDepth == 0 && !isBlackEps(emissive, lambert ? 0.05f : 0.1f) && !hi.flipped) {
            pl.radiance = pl.radiance + emissive * pl.beta;
            pl.stop = true;
            return;
        }
        pl.surfaceDepth += 1;
        V3 wo = worldToLocal(hi.frame, -rayDir);
        LSR lsr = sampleLight(c, pl, hi.worldPosition, pl.recursionDepth + 1 < c.p.depth);
        if (!isBlack(lsr.radiance)) {
            V3 wi = worldToLocal(hi.frame, lsr.direction);
            V3 F;
            float bsdfPdf = 0.0f;
            if (lambert) {
                float cosTheta = std::min(std::max(wi.y, 0.0f), 1.0f);
                F = albedo * INV_PI * cosTheta;
                bsdfPdf = cosineSampleHemispherePdf(cosTheta);
            } else {
                F = evalPBRStandard(pbr, wi, wo, normalize(wo + wi));
            }
            if (!isBlack(F)) {
                if (lsr.isDeltaLight)
                    pl.radiance = pl.radiance + lsr.radiance * F * pl.beta / lsr.pdf;
                else {
                    if (!lambert)
                        bsdfPdf = pdfPBRStandard(wi, wo, pbr);
                    float w = PowerHeuristic(lsr.pdf, bsdfPdf);
                    pl.radiance = pl.radiance + w * lsr.radiance * F * pl.beta / lsr.pdf;
                }
            }
        }
        float sampleDirectionPDF;
        V3 sdl;
        if (lambert) {
            float r0, r1;
            rand2D(pl, r0, r1);
            sdl = cosineSampleHemisphere(r0, r1, sampleDirectionPDF);
            pl.origin = hi.worldPosition;
            pl.direction = localToWorld(hi.frame, sdl);
            pl.beta = pl.beta * albedo;
        } else {
            float r0, r1;
            rand2D(pl, r0, r1);
            float r2 = rand1D(pl);
            V3 F = samplePBRStandard(sdl, wo, sampleDirectionPDF, pbr, r0, r1, r2);
            pl.origin = hi.worldPosition;
            pl.direction = localToWorld(hi.frame, sdl);
            if (isBlack(F)) {
                pl.stop = true;
                return;
            }
            V3 q = F / sampleDirectionPDF;
            pl.beta = pl.beta * v3(std::min(std::max(q.x, 0.0f), 1.0f), std::min(std::max(q.y, 0.0f), 1.0f),
                                   std::min(std::max(q.z, 0.0f), 1.0f));
        }
        pl.sampled = true;
        pl.samplePdf = sampleDirectionPDF;
        nextEventEstimation(c, pl, sampleDirectionPDF);
    }
    russianRoulette(pl);
}

// rayPrimary.rmiss.glsl:40-106
void miss(const Ctx &c, Payload &pl, V3 rayDir)
{
    bool sampledMedium = false;
    if (pl.insideVolume) {
        float vtend = std::min((float)(uint32_t)c.p.zfar, 10000.0f);
        sampledMedium = processVolumeHit(c, pl, pl.volumeMaterialIndex, pl.vtmin, vtend, rayDir);
    }
    if (!sampledMedium) {
        pl.stop = true;
        int mode = (int)c.p.envType;
        // environment light-sampled: BSDF side of the MIS weight for an
        // escape along a sampled direction
        float wenv = 1.0f;
        if (c.p.envLight && pl.sampled)
            wenv = PowerHeuristic(pl.samplePdf, envPdf(c.s, rayDir) / (float)(c.p.totalLights + 1));
        if (mode == 0) {
            V3 bg = c.p.background;
            if (pl.surfaceDepth == 0) {
                pl.albedo = bg;
                pl.normal = v3s(0.0f);
            }
            pl.radiance = pl.radiance + bg * pl.beta;
        } else if (mode == 1) {
            V3 bg = c.p.envIntensity * env_sample(c.s, rayDir);
            if (pl.surfaceDepth == 0) {
                pl.albedo = bg;
                pl.normal = v3s(0.0f);
            }
            pl.radiance = pl.radiance + bg * pl.beta * wenv;
        } else if (mode == 2) {
            if (pl.surfaceDepth == 0) {
                pl.albedo = c.p.background;
                pl.normal = v3s(0.0f);
                pl.radiance = pl.radiance + c.p.background * pl.beta;
            } else {
                pl.radiance = pl.radiance + env_sample(c.s, rayDir) * pl.beta * wenv;
            }
        }
        return;
    }
    russianRoulette(pl);
}

inline void mat4mul(const float *m, float x, float y, float z, float w, float out[4])
{
    for (int r = 0; r < 4; r++)
        out[r] = m[0 + r] * x + m[4 + r] * y + m[8 + r] * z + m[12 + r] * w;
}

// raygen.rgen.glsl:24-145 for one pixel and one batch; returns the batch sums
template <class Acc>
// cum[0..2]: radiance, albedo, normal; cum[3]: the radiance of the second
// candidate order (Params::altOrder)
void raygen_batch(const Ctx &c, uint32_t px, uint32_t py, uint32_t batchIndex, Acc cum[4])
{
    const Params &p = c.p;
    Payload pl{};
    pl.rngState = initRNG(px, py, p.W, batchIndex);
    // PMJ sampler state, raygen.rgen.glsl:32-43
    pl.pmj = p.sampler;
    pl.samplesPerPixel = p.totalSamples;
    pl.pixelX = px;
    pl.pixelY = py;
    float lensRadius = p.lensRadius, focalDistance = p.focalDistance;
    bool insideVolume = p.camVolume != -1;
    for (int k = 0; k < 4; k++)
        cum[k] = Acc{0, 0, 0};
    for (uint32_t s = 0; s < p.batchSize; s++) {
        pl.altDelta = v3s(0.0f);
        if (pl.pmj) {
            // raygen.rgen.glsl:57-61 (dimension start y * width + y, as written there)
            pl.rngState = py * p.W + py;
            pl.sampleIndex = batchIndex * p.batchSize + s;
        }
        float ox, oy;
        rand2D(pl, ox, oy);
        float ux = ((float)px + ox) / (float)p.W, uy = ((float)py + oy) / (float)p.H;
        float dx = ux * 2.0f - 1.0f, dy = uy * 2.0f - 1.0f;
        float target[4];
        mat4mul(p.projInv, dx, dy, 1.0f, 1.0f, target);
        V3 dcam = normalize(v3(target[0], target[1], target[2]));
        V3 ocam = v3s(0.0f);
        if (lensRadius > 0) {
            float lx, ly;
            rand2D(pl, lx, ly);
            float cx, cy;
            concentricSampleDisk(lx, ly, cx, cy);
            float lox = lensRadius * cx, loy = lensRadius * cy;
            float ft = focalDistance / (-dcam.z);
            V3 focus = dcam * ft;
            ocam = v3(lox, loy, 0.0f);
            dcam = normalize(focus - ocam);
        }
        float o4[4], d4[4];
        mat4mul(p.viewInv, ocam.x, ocam.y, ocam.z, 1.0f, o4);
        mat4mul(p.viewInv, dcam.x, dcam.y, dcam.z, 0.0f, d4);
        V3 origin = v3(o4[0], o4[1], o4[2]), direction = v3(d4[0], d4[1], d4[2]);
        pl.origin = origin;
        pl.direction = direction;
        pl.surfaceDepth = 0;
        pl.sampled = false;
        pl.insideVolume = insideVolume;
        pl.volumeMaterialIndex = (uint32_t)p.camVolume;
        V3 beta = v3s(1.0f), radiance = v3s(0.0f), albedo = v3s(0.0f), normal = v3s(0.0f);
        for (uint32_t d = 0; d < p.depth; d++) {
            pl.stop = false;
            pl.radiance = radiance;
            pl.beta = beta;
            pl.recursionDepth = d;
            pl.vtmin = 0.001f;
            Hit h = trace_closest(c.s, origin, direction, 0.001f, 10000.0f);
            if (h.inst == NOHIT)
                miss(c, pl, direction);
            else
                closestHit(c, pl, h, direction);
            beta = pl.beta;
            radiance = pl.radiance;
            albedo = pl.albedo;
            normal = pl.normal;
            if (pl.stop)
                break;
            origin = pl.origin;
            direction = pl.direction;
        }
        float total = (float)p.totalSamples;
        V3 rr = radiance / total, aa = albedo / total, nn = normal / total;
        cum[0] = cum[0] + Acc{rr.x, rr.y, rr.z};
        cum[1] = cum[1] + Acc{aa.x, aa.y, aa.z};
        cum[2] = cum[2] + Acc{nn.x, nn.y, nn.z};
        if (p.altOrder) {
            V3 ra = (radiance + pl.altDelta) / total;
            cum[3] = cum[3] + Acc{ra.x, ra.y, ra.z};
        }
    }
}

struct F3 {
    float x, y, z;
    F3 operator+(const F3 &o) const { return {x + o.x, y + o.y, z + o.z}; }
};
struct D3 {
    double x, y, z;
    D3 operator+(const D3 &o) const { return {x + o.x, y + o.y, z + o.z}; }
};

bool build_scene(const vvpt_scene_desc *desc, Scene &s)
{
    s.meshes.resize(desc->num_meshes);
    for (uint32_t m = 0; m < desc->num_meshes; m++) {
        const vvpt_mesh_desc &md = desc->meshes[m];
        Mesh &mesh = s.meshes[m];
        mesh.v = md.vertices;
        mesh.idx = md.indices;
        mesh.ntri = md.num_triangles;
        std::vector<std::array<float, 6>> boxes(md.num_triangles);
        for (int a = 0; a < 3; a++) {
            mesh.lo[a] = FLT_MAX;
            mesh.hi[a] = -FLT_MAX;
        }
        for (uint32_t t = 0; t < md.num_triangles; t++) {
            auto &b = boxes[t];
            for (int a = 0; a < 3; a++) {
                b[a] = FLT_MAX;
                b[3 + a] = -FLT_MAX;
            }
            for (int k = 0; k < 3; k++) {
                const float *p = md.vertices[md.indices[3 * t + k]].position;
                for (int a = 0; a < 3; a++) {
                    b[a] = std::min(b[a], p[a]);
                    b[3 + a] = std::max(b[3 + a], p[a]);
                    mesh.lo[a] = std::min(mesh.lo[a], p[a]);
                    mesh.hi[a] = std::max(mesh.hi[a], p[a]);
                }
            }
        }
        if (md.num_triangles == 0)
            continue;
        build_bvh(boxes, mesh.bvh);
        mesh.tris.resize(md.num_triangles);
        for (uint32_t k = 0; k < md.num_triangles; k++) {
            uint32_t prim = mesh.bvh.order[k];
            const float *p0 = md.vertices[md.indices[3 * prim]].position;
            const float *p1 = md.vertices[md.indices[3 * prim + 1]].position;
            const float *p2 = md.vertices[md.indices[3 * prim + 2]].position;
            mesh.tris[k] = {v3(p0[0], p0[1], p0[2]), v3(p1[0], p1[1], p1[2]), v3(p2[0], p2[1], p2[2]), prim};
        }
    }
    s.inst.resize(desc->num_instances);
    std::vector<std::array<float, 6>> tboxes;
    // Small instances: at most kFlatMaxTriangles triangles, two or more of
    // them. They leave the TLAS; their triangles, baked into world space, form
    // one mesh under an identity instance, each triangle naming its instance
    // (the library's layout, which changes the rounding of their hits: the
    // test runs in world space on baked vertices).
    const uint32_t kFlatMaxTriangles = 64;
    std::vector<uint8_t> flat(desc->num_instances, 0);
    uint32_t nflat = 0;
    for (uint32_t i = 0; i < desc->num_instances; i++) {
        const vvpt_instance &src = desc->instances[i];
        Rows tmp;
        if ((src.flags & VVPT_INSTANCE_IN_TLAS) && src.mesh_index < desc->num_meshes &&
            s.meshes[src.mesh_index].ntri > 0 && s.meshes[src.mesh_index].ntri <= kFlatMaxTriangles &&
            invert_rows(src.model, tmp)) {
            flat[i] = 1;
            nflat++;
        }
    }
    if (nflat < 2)
        std::fill(flat.begin(), flat.end(), 0);
    for (uint32_t i = 0; i < desc->num_instances; i++) {
        const vvpt_instance &src = desc->instances[i];
        Inst &in = s.inst[i];
        in.src = &src;
        for (int r = 0; r < 3; r++)
            for (int c = 0; c < 4; c++)
                in.o2w.m[r][c] = src.model[c * 4 + r];
        if (!invert_rows(src.model, in.w2o) && (src.flags & VVPT_INSTANCE_IN_TLAS))
            return false;
        in.mesh = src.mesh_index < desc->num_meshes ? (int)src.mesh_index : -1;
        in.in_tlas = (src.flags & VVPT_INSTANCE_IN_TLAS) && in.mesh >= 0 && s.meshes[in.mesh].ntri > 0 && !flat[i];
        if (in.in_tlas) {
            const Mesh &m = s.meshes[in.mesh];
            std::array<float, 6> b;
            for (int a = 0; a < 3; a++) {
                b[a] = FLT_MAX;
                b[3 + a] = -FLT_MAX;
            }
            for (int k = 0; k < 8; k++) {
                V3 p = v3((k & 1) ? m.hi[0] : m.lo[0], (k & 2) ? m.hi[1] : m.lo[1], (k & 4) ? m.hi[2] : m.lo[2]);
                V3 q = xpoint(in.o2w, p);
                for (int a = 0; a < 3; a++) {
                    float pad = 1e-5f * (std::fabs(comp(q, a)) + 1.0f);
                    b[a] = std::min(b[a], comp(q, a) - pad);
                    b[3 + a] = std::max(b[3 + a], comp(q, a) + pad);
                }
            }
            // culling bound: |o_obj| <= |W|(|o| + |t|), |d_obj| >= |d| / |M|
            double nm = 0.0, nw = 0.0, tt = 0.0, pm = 0.0;
            for (int r = 0; r < 3; r++) {
                nm = std::max(nm, (double)std::fabs(in.o2w.m[r][0]) + std::fabs(in.o2w.m[r][1]) + std::fabs(in.o2w.m[r][2]));
                nw = std::max(nw, (double)std::fabs(in.w2o.m[r][0]) + std::fabs(in.w2o.m[r][1]) + std::fabs(in.w2o.m[r][2]));
                tt = std::max(tt, (double)std::fabs(in.o2w.m[r][3]));
                pm = std::max(pm, (double)std::max(std::fabs(m.lo[r]), std::fabs(m.hi[r])));
            }
            s.cull_o = std::max(s.cull_o, (float)(nm * nw));
            s.cull_r = std::max(s.cull_r, (float)(nm * (nw * tt + pm)));
            tboxes.push_back(b);
            s.tlas_ids.push_back(i);
        }
    }
    if (nflat >= 2) {
        // world = ((r0 * x + r1 * y) + r2 * z) + r3 per model row, in double,
        // rounded to float
        Mesh fm;
        std::vector<std::array<float, 6>> fboxes;
        std::vector<Tri> ftris;
        double mag = 0.0;
        for (uint32_t i = 0; i < desc->num_instances; i++) {
            if (!flat[i])
                continue;
            const Inst &in = s.inst[i];
            const Mesh &m = s.meshes[in.mesh];
            for (uint32_t t = 0; t < m.ntri; t++) {
                V3 q[3];
                std::array<float, 6> b;
                for (int a = 0; a < 3; a++) {
                    b[a] = FLT_MAX;
                    b[3 + a] = -FLT_MAX;
                }
                for (int k = 0; k < 3; k++) {
                    const float *p = m.v[m.idx[3 * t + k]].position;
                    float w[3];
                    for (int a = 0; a < 3; a++) {
                        double v = (double)in.o2w.m[a][0] * p[0];
                        v = v + (double)in.o2w.m[a][1] * p[1];
                        v = v + (double)in.o2w.m[a][2] * p[2];
                        v = v + (double)in.o2w.m[a][3];
                        w[a] = (float)v;
                        b[a] = std::min(b[a], w[a]);
                        b[3 + a] = std::max(b[3 + a], w[a]);
                        mag = std::max(mag, (double)std::fabs(w[a]));
                    }
                    q[k] = v3(w[0], w[1], w[2]);
                }
                Tri tr;
                tr.p0 = q[0];
                tr.p1 = q[1];
                tr.p2 = q[2];
                tr.prim = t;
                tr.inst = i;
                ftris.push_back(tr);
                fboxes.push_back(b);
            }
        }
        fm.ntri = (uint32_t)ftris.size();
        for (int a = 0; a < 3; a++) {
            fm.lo[a] = FLT_MAX;
            fm.hi[a] = -FLT_MAX;
        }
        for (const auto &b : fboxes)
            for (int a = 0; a < 3; a++) {
                fm.lo[a] = std::min(fm.lo[a], b[a]);
                fm.hi[a] = std::max(fm.hi[a], b[3 + a]);
            }
        build_bvh(fboxes, fm.bvh);
        fm.tris.resize(ftris.size());
        for (size_t k = 0; k < ftris.size(); k++)
            fm.tris[k] = ftris[fm.bvh.order[k]];
        const int fmi = (int)s.meshes.size();
        std::array<float, 6> wb;
        for (int a = 0; a < 3; a++) {
            const float pad = 1e-5f * (std::fabs(fm.lo[a]) + std::fabs(fm.hi[a]) + 1e-3f);
            wb[a] = fm.lo[a] - pad;
            wb[3 + a] = fm.hi[a] + pad;
        }
        s.meshes.push_back(std::move(fm));
        Inst syn;
        const float ident[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
        for (int r = 0; r < 3; r++)
            for (int c = 0; c < 4; c++)
                syn.o2w.m[r][c] = ident[c * 4 + r];
        invert_rows(ident, syn.w2o);
        for (uint32_t i = 0; i < desc->num_instances; i++)
            if (flat[i]) {
                syn.src = &desc->instances[i]; // never reported: hits name the baked triangle's instance
                break;
            }
        syn.mesh = fmi;
        syn.in_tlas = true;
        s.cull_o = std::max(s.cull_o, 1.0f);
        s.cull_r = std::max(s.cull_r, (float)mag);
        s.tlas_ids.push_back((uint32_t)s.inst.size());
        s.inst.push_back(syn);
        tboxes.push_back(wb);
    }
    if (!tboxes.empty())
        build_bvh(tboxes, s.tlas);
    s.mats = desc->materials;
    s.nmats = desc->num_materials;
    s.lights = desc->lights;
    s.nlights = desc->num_lights;
    s.ldata = desc->light_data;
    for (uint32_t t = 0; t < desc->num_textures; t++) {
        const vvpt_texture_desc &td = desc->textures[t];
        s.tex.push_back({td.width, td.height, td.format, (const uint8_t *)td.data});
    }
    if (desc->environment) {
        s.env = (int)s.tex.size();
        s.tex.push_back({desc->environment->width, desc->environment->height, desc->environment->format,
                         (const uint8_t *)desc->environment->data});
        if (desc->environment->format == VVPT_TEXTURE_RGBA32F)
            build_env_tables(s, (const float *)desc->environment->data, desc->environment->width,
                             desc->environment->height);
    }
    return true;
}

void make_params(const vvpt_scene_desc *desc, const vvpt_scene_data *sd, const vvpt_render_info *ri, Params &p)
{
    std::memcpy(p.viewInv, sd->view_inverse, sizeof(p.viewInv));
    std::memcpy(p.projInv, sd->projection_inverse, sizeof(p.projInv));
    p.background = v3(sd->background[0], sd->background[1], sd->background[2]);
    p.envType = sd->background[3];
    p.envIntensity = sd->exposure[1];
    p.lensRadius = sd->exposure[2];
    p.focalDistance = sd->exposure[3];
    p.zfar = sd->volumes[2];
    p.camVolume = (int)sd->volumes[0];
    p.W = ri->width;
    p.H = ri->height;
    p.batchSize = ri->batch_size;
    p.batches = ri->batch_size ? ri->samples / ri->batch_size : 0;
    p.depth = ri->depth;
    p.totalSamples = p.batchSize * p.batches;
    p.totalLights = desc->num_lights;
    p.sampler = (ri->flags & VVPT_RENDER_SAMPLER_PMJ) ? 1u : 0u;
}

void set_env_light(const Scene &s, const vvpt_render_info *ri, Params &p)
{
    int mode = (int)p.envType;
    p.envLight = ((ri->flags & VVPT_RENDER_ENV_IS) && s.envInt > 0.0f && (mode == 1 || mode == 2)) ? 1u : 0u;
}

}  // namespace

extern "C" {

// Tables of the PMJ sampler (VVPT_RENDER_SAMPLER_PMJ): [16][16384][2] and
// [48][128][128] floats, kept by the caller while it renders.
void oracle_set_sampler_tables(const float *pmj, const float *blue_noise)
{
    g_pmj = pmj;
    g_blue_noise = blue_noise;
}

// Renders the listed pixels (all pixels when pixels == NULL) over every batch.
// Outputs are W*H*4 floats (RGBA, A = 1); pixels not listed are left untouched.
// fp64 != 0 accumulates the per-batch sums and the image in double precision.
// options: bit 0 accumulates the radiance in double precision; bit 1 also
// renders radiance_alt, the image with every emitter ray's candidates taken in
// instance-box-entry order instead of nearest first (emitterRay).
int oracle_render(const vvpt_scene_desc *desc, const vvpt_scene_data *sd, const vvpt_render_info *ri,
                  const uint32_t *pixels, uint32_t num_pixels, int threads, int options, float *radiance,
                  float *albedo, float *normal, float *radiance_m2, float *radiance_alt)
{
    const bool fp64 = (options & 1) != 0;
    if (!desc || !sd || !ri || ri->width == 0 || ri->height == 0 || ri->batch_size == 0)
        return 1;
    Scene s;
    if (!build_scene(desc, s))
        return 2;
    Params p;
    make_params(desc, sd, ri, p);
    set_env_light(s, ri, p);
    if (p.sampler && (!g_pmj || !g_blue_noise))
        return 3;
    p.altOrder = (options & 2) != 0 && radiance_alt != nullptr;
    const Ctx c{s, p};
    const uint32_t npix = pixels ? num_pixels : p.W * p.H;
    if (threads <= 0)
        threads = (int)std::max(1u, std::thread::hardware_concurrency());
    if (fp64 && !p.altOrder && p.depth > 0 && p.batches >= 128 && npix < 4u * (uint32_t)threads) {
        // Few pixels and many batches (converged reference images): each
        // pixel's batches are split into chunks of 64 rendered in parallel,
        // and the chunks' double-precision sums are added in chunk order.
        const uint32_t chunk = 64, nchunks = (p.batches + chunk - 1) / chunk;
        const uint64_t units = (uint64_t)npix * nchunks;
        std::vector<double> part(units * 12, 0.0);
        std::atomic<uint64_t> nextu{0};
        auto workc = [&]() {
            for (;;) {
                const uint64_t u = nextu.fetch_add(1);
                if (u >= units)
                    break;
                const uint32_t k = (uint32_t)(u / nchunks), ch = (uint32_t)(u % nchunks);
                const uint32_t pix = pixels ? pixels[k] : k;
                if (pix >= p.W * p.H)
                    continue;
                double *acc = &part[u * 12];
                for (uint32_t b = ch * chunk; b < std::min(p.batches, (ch + 1) * chunk); b++) {
                    D3 cum[4];
                    raygen_batch(c, pix % p.W, pix / p.W, b, cum);
                    for (int q = 0; q < 3; q++) {
                        acc[3 * q + 0] += cum[q].x;
                        acc[3 * q + 1] += cum[q].y;
                        acc[3 * q + 2] += cum[q].z;
                    }
                    acc[9] += cum[0].x * cum[0].x;
                    acc[10] += cum[0].y * cum[0].y;
                    acc[11] += cum[0].z * cum[0].z;
                }
            }
        };
        std::vector<std::thread> cpool;
        for (int t = 0; t < threads; t++)
            cpool.emplace_back(workc);
        for (auto &t : cpool)
            t.join();
        float *outs[4] = {radiance, albedo, normal, radiance_m2};
        for (uint32_t k = 0; k < npix; k++) {
            const uint32_t pix = pixels ? pixels[k] : k;
            if (pix >= p.W * p.H)
                continue;
            double sum[12] = {0};
            for (uint32_t ch = 0; ch < nchunks; ch++)
                for (int i = 0; i < 12; i++)
                    sum[i] += part[((uint64_t)k * nchunks + ch) * 12 + i];
            for (int q = 0; q < 4; q++) {
                if (!outs[q])
                    continue;
                for (int chn = 0; chn < 3; chn++)
                    outs[q][4 * (size_t)pix + chn] = (float)sum[3 * q + chn];
                outs[q][4 * (size_t)pix + 3] = 1.0f;
            }
        }
        return 0;
    }
    std::atomic<uint32_t> next{0};
    auto work = [&]() {
        for (;;) {
            uint32_t k0 = next.fetch_add(16);
            if (k0 >= npix)
                break;
            for (uint32_t k = k0; k < std::min(npix, k0 + 16); k++) {
                uint32_t pix = pixels ? pixels[k] : k;
                if (pix >= p.W * p.H)
                    continue;
                uint32_t px = pix % p.W, py = pix / p.W;
                double img[4][3] = {{0}};
                float imgf[4][3] = {{0}};
                double m2[3] = {0, 0, 0};
                const int nq = p.altOrder ? 4 : 3;
                if (p.depth > 0) {
                    for (uint32_t b = 0; b < p.batches; b++) {
                        if (fp64) {
                            D3 cum[4];
                            raygen_batch(c, px, py, b, cum);
                            for (int q = 0; q < nq; q++) {
                                img[q][0] += cum[q].x;
                                img[q][1] += cum[q].y;
                                img[q][2] += cum[q].z;
                            }
                            m2[0] += cum[0].x * cum[0].x;
                            m2[1] += cum[0].y * cum[0].y;
                            m2[2] += cum[0].z * cum[0].z;
                        } else {
                            F3 cum[4];
                            raygen_batch(c, px, py, b, cum);
                            for (int q = 0; q < nq; q++) {
                                imgf[q][0] = imgf[q][0] + cum[q].x;
                                imgf[q][1] = imgf[q][1] + cum[q].y;
                                imgf[q][2] = imgf[q][2] + cum[q].z;
                            }
                            m2[0] += (double)cum[0].x * cum[0].x;
                            m2[1] += (double)cum[0].y * cum[0].y;
                            m2[2] += (double)cum[0].z * cum[0].z;
                        }
                    }
                }
                float *outs[4] = {radiance, albedo, normal, p.altOrder ? radiance_alt : nullptr};
                for (int q = 0; q < 4; q++) {
                    if (!outs[q])
                        continue;
                    for (int ch = 0; ch < 3; ch++)
                        outs[q][4 * (size_t)pix + ch] = fp64 ? (float)img[q][ch] : imgf[q][ch];
                    outs[q][4 * (size_t)pix + 3] = 1.0f;
                }
                if (radiance_m2) {
                    for (int ch = 0; ch < 3; ch++)
                        radiance_m2[4 * (size_t)pix + ch] = (float)m2[ch];
                    radiance_m2[4 * (size_t)pix + 3] = 1.0f;
                }
            }
        }
    };
    std::vector<std::thread> pool;
    for (int t = 0; t < threads; t++)
        pool.emplace_back(work);
    for (auto &t : pool)
        t.join();
    return 0;
}

// Closest hit for rays (origin, tmin, direction, tmax), 8 floats each.
int oracle_trace_closest(const vvpt_scene_desc *desc, const float *rays, uint32_t n, vvpt_hit *hits)
{
    Scene s;
    if (!build_scene(desc, s))
        return 2;
    for (uint32_t i = 0; i < n; i++) {
        const float *r = rays + 8 * (size_t)i;
        Hit h = trace_closest(s, v3(r[0], r[1], r[2]), v3(r[4], r[5], r[6]), r[3], r[7]);
        hits[i].t = h.t;
        hits[i].u = h.u;
        hits[i].v = h.v;
        hits[i].instance = h.inst;
        hits[i].primitive = h.prim;
    }
    return 0;
}

}  // extern "C"
