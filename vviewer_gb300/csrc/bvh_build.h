// Host-side binned-SAH BVH builder (binary nodes). Used for every BLAS (over
// triangles) and for the TLAS (over instance world boxes).
//
// Replaces the driver-built acceleration structures of the reference
// (src/lib/vengine/vulkan/resources/VulkanAccelerationStructure.cpp:14-279,
// built with VK_BUILD_ACCELERATION_STRUCTURE_PREFER_FAST_TRACE_BIT_KHR).
#pragma once
#include <stdint.h>

#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "scene_gpu.h"

namespace vvpt {

struct Box3 {
    float lo[3];
    float hi[3];
};

// BLAS build parameters (build-time overridable for tuning experiments)
#ifndef VVPT_BVH_BINS
#define VVPT_BVH_BINS 32
#endif
#ifndef VVPT_BVH_MAX_LEAF
#define VVPT_BVH_MAX_LEAF 4
#endif
#ifndef VVPT_BVH_COST_TRAVERSAL
#define VVPT_BVH_COST_TRAVERSAL 1.0
#endif

struct BVHBuildOptions {
    int bins = VVPT_BVH_BINS;         // SAH bins per axis
    int max_leaf = VVPT_BVH_MAX_LEAF; // preferred leaf size
    int max_depth = 56;     // force leaves below this depth (traversal stack bound)
    double cost_traversal = VVPT_BVH_COST_TRAVERSAL;
    double cost_intersect = 1.0;
    int threads = 0;        // 0 = hardware concurrency (large builds only)
};

struct BVHBuildResult {
    std::vector<BVHNode> nodes; // node 0 is the root
    std::vector<uint32_t> order; // leaf order -> primitive index
    int depth = 0;
};

// Builds a BVH over `boxes`. Always emits at least a root node (an empty
// input gives a root with two empty children).
BVHBuildResult build_bvh2(const std::vector<Box3> &boxes, const BVHBuildOptions &opt = BVHBuildOptions());

// Compressed 8-wide BVH collapsed from a binary one (bvh_wide.cpp): node 0 is
// the root; `order` lists the primitives in the wide leaf order (each wide
// node's leaf triangles contiguous from its tri_base).
struct WideBuildResult {
    std::vector<WideNode> nodes;
    std::vector<uint32_t> order;
    int depth = 0;
};
WideBuildResult collapse_to_wide(const BVHBuildResult &bin, const std::vector<Box3> &boxes);

// The same BVH built on the GPU (bvh_gpu.cu), one tree level per round of
// kernels on `stream`; node and order arrays come back to the host. Returns
// false (err set, or err empty for trees the host builds trivially: at most
// max_leaf primitives) when it did not build.
bool build_bvh2_gpu(const std::vector<Box3> &boxes, const BVHBuildOptions &opt, cudaStream_t stream,
                    BVHBuildResult &out, std::string &err);

}  // namespace vvpt
