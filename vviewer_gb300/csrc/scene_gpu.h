// Device-resident scene layout. Shared by the host-side builder (bvh_build.cpp,
// api.cu) and the kernels. Plain structs, 16-byte aligned where the kernels do
// 128-bit loads.
#pragma once
#include <stdint.h>

#include <vector_types.h>

namespace vvpt {

// Entries of the single traversal stack (TLAS and BLAS levels together). The
// scene builder rejects BVHs whose worst-case depth would not fit.
constexpr int kTraversalStack = 128;

// Binary BVH node, 64 bytes: both children's boxes plus child links, so one
// node visit is four 128-bit loads. lxy = (l.lo.x, l.hi.x, l.lo.y, l.hi.y),
// rxy likewise, lrz = (l.lo.z, l.hi.z, r.lo.z, r.hi.z).
// c = (left, right, left_count, right_count): count > 0 -> leaf covering
// primitives [index, index + count) of the leaf-ordered primitive array;
// count == 0 -> internal node `index` (relative to the BVH's first node);
// index == -1 -> empty child.
struct alignas(16) BVHNode {
    float4 lxy;
    float4 rxy;
    float4 lrz;
    int4 c;
};
static_assert(sizeof(BVHNode) == 64, "BVHNode must be 64 bytes");

// Bottom-level acceleration structures use the binary nodes above
// (VVPT_BLAS_WIDE = 0, the default) or compressed 8-wide nodes
// (VVPT_BLAS_WIDE = 1, a build option). Both give the same closest hits. With
// the wide nodes the traversal kernels trace one ray per lane, or with
// VVPT_GROUP_TRAVERSAL = 1 one ray per group of eight lanes (a child slot or
// a triangle per lane). On GB300 the binary layout with one ray per lane is
// the fastest: the traversal kernels are issue-bound under divergence, the
// wide nodes cost more instructions per visit, and eight lanes per ray leave
// too few rays in flight to cover the memory latency of each node fetch.
// The TLAS uses binary nodes in every form.
#ifndef VVPT_BLAS_WIDE
#define VVPT_BLAS_WIDE 0
#endif
#ifndef VVPT_GROUP_TRAVERSAL
#define VVPT_GROUP_TRAVERSAL 0
#endif

// Compressed 8-wide node (80 bytes, five 128-bit loads). Child box planes are
// p + q * 2^(e - 127) per axis with 8-bit q (qlo, qhi); p is a multiple of the
// scale and every plane is exactly representable. imask bit i: slot i holds an
// internal child; internal children are consecutive wide nodes from
// child_base in slot order (index = child_base + number of internal slots
// below i). meta[i] of a leaf slot: (triangle count 1..4) << 5 | offset
// (0..31) of its first triangle from tri_base; 0 for empty and internal
// slots. child_base and tri_base are relative to the BLAS's first wide node
// and first triangle.
struct alignas(16) WideNode {
    float px, py, pz;
    uint8_t ex, ey, ez, imask;
    uint32_t child_base;
    uint32_t tri_base;
    uint8_t meta[8];
    uint8_t qlox[8], qloy[8], qloz[8];
    uint8_t qhix[8], qhiy[8], qhiz[8];
};
static_assert(sizeof(WideNode) == 80, "WideNode must be 80 bytes");

// Triangle in leaf order for intersection: v0.w carries the original
// primitive index (gl_PrimitiveID) as raw bits; v1.w is 0, or for the
// baked world-space triangles of small instances (kFlattenMaxTriangles) the
// instance slot + 1 as raw bits, the instance a hit on it reports.
struct alignas(16) TriVerts {
    float4 v0, v1, v2;
};
constexpr uint32_t kFlattenMaxTriangles = 64;

// Shading vertex: position + u, normal + v, tangent (+pad). Bitangents are not
// kept: fixFrame (shaders/include/frame.glsl:7-36) overwrites the bitangent in
// both of its branches, so the input value never reaches the result.
struct alignas(16) ShadeVertex {
    float4 pos_u;
    float4 nrm_v;
    float4 tan_;
};

struct MeshInfo {
    uint32_t node_offset;   // first node of the BLAS (WideNode or BVHNode)
    uint32_t tri_offset;    // first TriVerts (leaf order)
    uint32_t vertex_offset; // first ShadeVertex
    uint32_t index_offset;  // first index triple (in uint32 units / 3)
    uint32_t num_triangles;
    uint32_t num_nodes;
    uint32_t pad0, pad1;
};

// Per-instance data the kernels read (128 bytes).
struct alignas(16) DevInstance {
    float4 w2o[3];  // world-to-object rows
    float4 o2w[3];  // object-to-world rows
    uint32_t node_offset;
    uint32_t tri_offset;
    uint32_t vertex_offset;
    uint32_t index_offset;
    uint32_t material;
    uint32_t num_triangles;
    int32_t front_volume; // id.g (-1 none)
    int32_t back_volume;  // id.b (-1 none)
};
static_assert(sizeof(DevInstance) == 128, "DevInstance must be 128 bytes");

struct DevMaterial {
    float4 albedo;
    float4 mrao;
    float4 emissive;
    uint32_t tex1[4];
    uint32_t tex2[4];
    float4 uv_tiling;
    uint32_t padding[8];
};
static_assert(sizeof(DevMaterial) == 128, "DevMaterial must be 128 bytes");

struct DevLightInstance {
    uint32_t info[4];
    float4 position;
    float4 position1;
    float4 position2;
    // host-precomputed transpose(inverse(M)) rows for mesh lights (the
    // reference computes it per sample in lightSampling.glsl:80)
    float4 nrm0, nrm1, nrm2;
    float4 color; // LightData colour of point/directional lights
};

struct DevTexture {
    uint32_t width, height, format, pad;
    uint64_t offset; // byte offset into the texel pool
};

// Everything a kernel needs about the scene.
struct SceneView {
    const BVHNode *nodes;      // all BLAS nodes (binary layout), then TLAS nodes
    const WideNode *wnodes;    // all BLAS nodes (wide layout)
    const TriVerts *tris;
    const ShadeVertex *verts;
    const uint32_t *indices;   // 3 per triangle, original order
    const DevInstance *instances;
    const uint32_t *tlas_order; // TLAS leaf order -> instance slot
    uint32_t tlas_root;        // node index of the TLAS root
    uint32_t tlas_count;       // TLAS nodes (from tlas_root to the end of `nodes`)
    uint32_t num_instances;
    const DevMaterial *materials;
    uint32_t num_materials;
    const DevLightInstance *lights;
    uint32_t num_lights;
    const DevTexture *textures;
    uint32_t num_textures;
    const uint8_t *texels;
    int32_t env_texture;       // texture index of the equirect environment, -1 none
    uint32_t has_transparent;  // any material with the transparent flag set
    // culling-margin bound: over the TLAS instances, the object-space
    // coordinate magnitude a triangle test sees per unit of world-space ray
    // direction is at most cull_o * |origin| + cull_r (max-norms)
    float cull_o, cull_r;
    // importance sampling of the environment (piecewise constant over the
    // equirect texels, function = dilated luminance x cos(latitude));
    // env_func_int == 0: not samplable
    const float *env_func;     // env_h x env_w
    const float *env_cond_cdf; // env_h x (env_w + 1), per-row CDFs
    const float *env_marg_cdf; // env_h + 1
    uint32_t env_w, env_h;
    float env_func_int;        // integral of env_func over [0,1]^2
    // World boxes (lo, hi pairs, padded) that hold every TLAS instance whose
    // material can emit (emission above the emitter rays' 0.05 threshold):
    // a BSDF-direction emitter ray whose line misses all of them adds nothing.
    // At most kMaxEmitBoxes; more emissive instances are merged into that many.
    const float4 *emit_boxes;
    uint32_t num_emit_boxes;
};

constexpr uint32_t kMaxEmitBoxes = 32;

}  // namespace vvpt
