// Test harness: the device traversal of vviewer_gb300/csrc/traverse.cuh
// compiled for the host, over the scene arrays that vvpt_scene_upload would
// upload (pack_scene). The rounding intrinsics map to plain IEEE float /
// double operations, which round to nearest like the device's _rn forms
// (compile with -ffp-contract=off so no multiply-add is fused). Used only by
// the tests to check the traversal's bookkeeping (stack, instance entry and
// return, culling order) against the oracle without a GPU; it is not a
// rendering path.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <string>

static inline float __fadd_rn(float a, float b) { return a + b; }
static inline float __fsub_rn(float a, float b) { return a - b; }
static inline float __fmul_rn(float a, float b) { return a * b; }
static inline float __fdiv_rn(float a, float b) { return a / b; }
static inline double __dmul_rn(double a, double b) { return a * b; }
static inline double __dsub_rn(double a, double b) { return a - b; }
static inline int __float_as_int(float f) { int i; std::memcpy(&i, &f, 4); return i; }
static inline unsigned __float_as_uint(float f) { unsigned i; std::memcpy(&i, &f, 4); return i; }
static inline float __int_as_float(int i) { float f; std::memcpy(&f, &i, 4); return f; }
static inline float __uint_as_float(unsigned i) { float f; std::memcpy(&f, &i, 4); return f; }
static inline float __fmaf_rn(float a, float b, float c) { return std::fma(a, b, c); }
static inline int __ffs(int x) { return x ? __builtin_ctz((unsigned)x) + 1 : 0; }
static inline int __popc(unsigned x) { return __builtin_popcount(x); }
// byte i of the result = byte (s >> 4i) & 7 of the pair {y, x} (x bytes 0-3)
static inline unsigned __byte_perm(unsigned x, unsigned y, unsigned s)
{
    const unsigned long long pool = ((unsigned long long)y << 32) | x;
    unsigned r = 0;
    for (int i = 0; i < 4; i++)
        r |= (unsigned)((pool >> (8 * ((s >> (4 * i)) & 7u))) & 0xffu) << (8 * i);
    return r;
}
template <class T>
static inline T __ldg(const T *p) { return *p; }
// one lane per "warp": the speculative-traversal vote sees only this ray
static inline unsigned __activemask() { return 1u; }
static inline int __all_sync(unsigned, int pred) { return pred; }

#include "scene_pack.h"
#include "traverse.cuh"

using namespace vvpt;

// the shared-memory TLAS cache of the device kernels: never filled here
// (vvpt_tlas_cache_count stays 0)
namespace vvpt {
float4 vvpt_tlas_cache[4];
}

extern "C" int host_trace_closest(const vvpt_scene_desc *desc, const vvpt_ray *rays, uint32_t n, vvpt_hit *hits,
                                  uint32_t *err_bits, char *msg, int msg_len)
{
    PackedScene pk;
    std::string err;
    vvpt_status st = pack_scene(desc, pk, err, 1);
    if (st != VVPT_OK) {
        std::strncpy(msg, err.c_str(), msg_len - 1);
        msg[msg_len - 1] = 0;
        return (int)st;
    }
    SceneView v{};
    v.nodes = pk.nodes.data();
    v.wnodes = pk.wnodes.data();
    v.tris = pk.tris.data();
    v.verts = pk.verts.data();
    v.indices = pk.indices.data();
    v.instances = pk.instances.data();
    v.tlas_order = pk.tlas_order.data();
    v.tlas_root = pk.tlas_root;
    v.tlas_count = (uint32_t)(pk.nodes.size() - pk.tlas_root);
    v.num_instances = desc->num_instances;
    v.cull_o = pk.cull_o;
    v.cull_r = pk.cull_r;
    uint32_t e = 0;
    for (uint32_t i = 0; i < n; i++) {
        const vvpt_ray &r = rays[i];
        Hit h = trace_closest(v, f3(r.origin[0], r.origin[1], r.origin[2]),
                              f3(r.direction[0], r.direction[1], r.direction[2]), r.tmin, r.tmax, e);
        hits[i].t = h.t;
        hits[i].u = h.u;
        hits[i].v = h.v;
        hits[i].instance = h.inst;
        hits[i].primitive = h.prim;
    }
    *err_bits = e;
    return 0;
}

// may_reach_emitter for each ray over the packed scene's emissive boxes;
// also returns the number of boxes.
extern "C" int host_may_reach_emitter(const vvpt_scene_desc *desc, const vvpt_ray *rays, uint32_t n, uint8_t *out,
                                      uint32_t *num_boxes, char *msg, int msg_len)
{
    PackedScene pk;
    std::string err;
    vvpt_status st = pack_scene(desc, pk, err, 1);
    if (st != VVPT_OK) {
        std::strncpy(msg, err.c_str(), msg_len - 1);
        msg[msg_len - 1] = 0;
        return (int)st;
    }
    SceneView v{};
    v.emit_boxes = pk.emit_boxes.data();
    v.num_emit_boxes = (uint32_t)(pk.emit_boxes.size() / 2);
    *num_boxes = v.num_emit_boxes;
    for (uint32_t i = 0; i < n; i++) {
        const vvpt_ray &r = rays[i];
        out[i] = may_reach_emitter(v, f3(r.origin[0], r.origin[1], r.origin[2]),
                                   f3(r.direction[0], r.direction[1], r.direction[2]))
                     ? 1
                     : 0;
    }
    return 0;
}
