// Library-internal state behind the C ABI: device buffers, the context and
// scene handles, error helpers, and the pieces of a render shared by the
// one-shot render (api.cu) and the job engine (engine.cu).
#pragma once
#include <atomic>
#include <chrono>
#include <memory>
#include <mutex>
#include <string>

#include <cuda_runtime.h>

#include "../../include/vvpt.h"
#include "scene_gpu.h"
#include "wavefront.cuh"

namespace vvpt {

struct DevBuf {
    void *ptr = nullptr;
    size_t bytes = 0;
    DevBuf() = default;
    DevBuf(const DevBuf &) = delete;
    DevBuf &operator=(const DevBuf &) = delete;
    ~DevBuf() { release(); }
    void release()
    {
        if (ptr)
            cudaFree(ptr);
        ptr = nullptr;
        bytes = 0;
    }
    cudaError_t alloc(size_t n)
    {
        release();
        if (n == 0)
            n = 16;
        cudaError_t e = cudaMalloc(&ptr, n);
        if (e == cudaSuccess)
            bytes = n;
        else
            ptr = nullptr;
        return e;
    }
    // grow-only reuse
    cudaError_t reserve(size_t n)
    {
        if (ptr && bytes >= n)
            return cudaSuccess;
        return alloc(n);
    }
    template <class T>
    T *as() const
    {
        return reinterpret_cast<T *>(ptr);
    }
};

struct Engine; // engine.cu

}  // namespace vvpt

struct vvpt_scene {
    vvpt::DevBuf nodes, wnodes, tris, verts, indices, instances, tlas_order, materials, lights, textures, texels, env_dist,
        emit_boxes;
    vvpt::SceneView view{};
    uint64_t bytes = 0;
    uint32_t num_materials = 0;
    std::atomic<uint32_t> jobs_in_flight{0}; // engine jobs that still read this scene
};

struct vvpt_ctx {
    int device = 0;
    int num_sms = 0;
    cudaStream_t stream = nullptr;
    std::mutex mu;
    std::string last_error;
    std::atomic<float> progress{0.0f};
    vvpt_render_stats stats{};
    vvpt_tuning tuning{};
    // render buffers (grow-only, reused across renders)
    vvpt::DevBuf state, queues, results, params, outputs;
    uint32_t *counters_pinned = nullptr;
    vvpt::DevBuf rays, hits_tuv, hits_ids, err_word;
    cudaStream_t user_stream = nullptr;
    vvpt_kernel_profile profile{};
    // job engine (vvpt_submit ...), created on first use
    std::mutex engine_mu;
    vvpt::Engine *engine = nullptr;
    uint64_t budget_bytes = 0; // 0: no limit beyond the device's memory
    int bvh_builder = 0;       // VVPT_BVH_BUILDER_*
    // low-discrepancy sampler tables (VVPT_RENDER_SAMPLER_PMJ), uploaded on first use
    std::mutex sampler_mu;
    vvpt::DevBuf pmj_table, blue_noise_table;
    std::chrono::steady_clock::time_point created = std::chrono::steady_clock::now();
};

namespace vvpt {

inline cudaStream_t vv_stream(const vvpt_ctx *ctx) { return ctx->user_stream ? ctx->user_stream : ctx->stream; }

inline vvpt_status fail(vvpt_ctx *ctx, vvpt_status code, const std::string &msg)
{
    if (ctx)
        ctx->last_error = msg;
    return code;
}

inline vvpt_status cuda_fail(vvpt_ctx *ctx, cudaError_t e, const char *what)
{
    cudaGetLastError();
    std::string m = std::string(what) + ": " + cudaGetErrorString(e);
    return fail(ctx, e == cudaErrorMemoryAllocation ? VVPT_ERR_OOM : VVPT_ERR_DEVICE, m);
}

#define VV_CUDA(call, what)                  \
    do {                                     \
        cudaError_t _e = (call);             \
        if (_e != cudaSuccess)               \
            return cuda_fail(ctx, _e, what); \
    } while (0)

constexpr size_t aligned256(size_t b) { return (b + 255) & ~size_t(255); }

// RenderParams of one render request (SceneData and RenderInfo of the
// reference: VulkanRendererPathTracing.cpp:143-199, raygen.rgen.glsl:24-40).
// Checks the request; on error sets ctx's message and returns its status.
vvpt_status make_render_params(vvpt_ctx *ctx, const vvpt_scene *scene, const vvpt_scene_data *sd,
                               const vvpt_render_info *info, RenderParams &hp);

// Path state and queues for `slots` paths carved from one allocation each.
size_t path_state_bytes(size_t slots);
size_t queue_bytes(size_t slots);
PathState carve_path_state(char *base, size_t slots);
Queues carve_queues(char *base, size_t slots);

// Engine teardown (vvpt_destroy): stops the worker, fails unfinished jobs.
void engine_shutdown(vvpt_ctx *ctx);

}  // namespace vvpt
