// Host-side scene preparation: validates a vvpt_scene_desc and packs it into
// the device layout of scene_gpu.h (BLAS per mesh, TLAS over the instances,
// leaf-ordered triangles, shading vertices, materials, lights, texel pool).
// The arrays are uploaded as they are by vvpt_scene_upload; nothing here
// touches the GPU, so the packed scene can also be inspected on the host.
#pragma once
#include <stdint.h>

#include <functional>
#include <string>
#include <vector>

#include "../../include/vvpt.h"
#include "scene_gpu.h"

namespace vvpt {

struct PackedScene {
    std::vector<BVHNode> nodes;       // every binary BLAS, then the TLAS
    std::vector<WideNode> wnodes;     // every wide BLAS (VVPT_BLAS_WIDE)
    std::vector<TriVerts> tris;       // leaf order per BLAS
    std::vector<ShadeVertex> verts;
    std::vector<uint32_t> indices;    // original triangle order
    std::vector<DevInstance> instances;
    std::vector<uint32_t> tlas_order; // TLAS leaf order -> instance slot
    uint32_t tlas_root = 0;
    std::vector<DevMaterial> materials;
    std::vector<DevLightInstance> lights;
    std::vector<DevTexture> textures;
    std::vector<uint8_t> texels;
    int32_t env_texture = -1;
    bool has_transparent = false;
    float cull_o = 0.0f, cull_r = 0.0f; // SceneView culling-margin bound
    // environment sampling tables, one array: function (h x w), per-row CDFs
    // (h x (w + 1)), marginal CDF (h + 1); empty without an environment
    std::vector<float> env_dist;
    uint32_t env_w = 0, env_h = 0;
    float env_func_int = 0.0f;
    int tlas_depth = 0;
    int max_blas_depth = 0;
    std::vector<float4> emit_boxes;   // SceneView::emit_boxes (lo, hi pairs)
};

// Builder for large BLAS (e.g. the GPU builder): fills `out` and returns true,
// or returns false to leave the mesh to the host builder (err set on failure).
struct Box3;
struct BVHBuildOptions;
struct BVHBuildResult;
using BlasBuilder = std::function<bool(const std::vector<Box3> &, const BVHBuildOptions &, BVHBuildResult &,
                                       std::string &)>;

// Returns VVPT_OK or an error status with `err` set. `threads` = 0 uses every
// hardware thread for the BLAS builds. Meshes of at least `large_min`
// triangles go to `large_builder` when one is given (one at a time); with
// `builder_for_all` the baked small instances' BLAS and the TLAS go to it too.
vvpt_status pack_scene(const vvpt_scene_desc *desc, PackedScene &out, std::string &err, unsigned threads = 0,
                       const BlasBuilder &large_builder = BlasBuilder(), uint32_t large_min = 65536,
                       bool builder_for_all = false);

// Piecewise-constant sampling tables of an RGBA32F equirect environment
// (PackedScene::env_dist layout): function = luminance dilated over the 3x3
// texel neighbourhood (so every texel the bilinear lookup can reach has
// probability) times cos(latitude of the row centre), CDFs accumulated in
// double. Returns the function's integral over [0,1]^2 (0: nothing to sample).
float build_env_distribution(const float *rgba, uint32_t w, uint32_t h, std::vector<float> &out);

// Row form of the 3x4 affine part of a column-major 4x4 matrix, and of its
// inverse (computed in double, rounded to float). False when singular.
void affine_rows(const float m[16], float4 rows[3]);
bool affine_inverse_rows(const float m[16], float4 rows[3]);

}  // namespace vvpt
