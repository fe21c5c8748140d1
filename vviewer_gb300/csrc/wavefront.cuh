// Wavefront path-tracer state and launch interface.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "scene_gpu.h"

namespace vvpt {

// Per-render constants (SceneData + PathTracingData of the reference,
// src/lib/vengine/core/Scene.hpp:27-35 and
// src/lib/vengine/vulkan/renderers/VulkanRendererPathTracing.hpp:57-61).
struct RenderParams {
    float4 view_inv[4]; // columns
    float4 proj_inv[4]; // columns
    float3 background;
    float env_type;     // background.a: 0 solid, 1 HDRI, 2 solid + HDRI lighting
    float lens_radius;
    float focal_distance;
    float env_intensity;
    float zfar;          // sceneData.volumes.b
    float zfar_trunc;    // float(uint(zfar)), rayPrimary.rmiss.glsl:49
    int32_t cam_volume;  // sceneData.volumes.r (-1: camera not in a medium)
    uint32_t width, height;
    uint32_t batch_size, batches, depth, total_samples;
    uint32_t num_lights;  // pathTracingData.lights.r
    uint32_t total_items; // width * height * batches
    uint32_t want_m2;
    uint32_t reduce_fp64; // 1: batch sums added in double (VVPT_RENDER_REDUCE_FP64)
    uint32_t env_light;   // 1: the environment is sampled as one more light (VVPT_RENDER_ENV_IS)
    uint32_t sampler;     // 0: RTGEMS stream, 1: PMJ (VVPT_RENDER_SAMPLER_PMJ)
    const float *pmj;        // [16][16384][2] (sampler 1)
    const float *blue_noise; // [48][128][128] (sampler 1)
};

// Structure-of-arrays path state, one entry per slot. A slot runs one
// (pixel, batch) work item: its batch_size samples in order, because the
// RTGEMS state carries from one sample to the next (raygen.rgen.glsl:36-55).
struct PathState {
    float4 *o;       // ray origin (xyz)
    float4 *d;       // ray direction (xyz)
    float4 *beta;    // throughput (xyz)
    float4 *rad;     // sample radiance (xyz)
    float4 *alb;     // first-hit albedo carried across samples (payload semantics)
    float4 *nrm;     // first-hit normal carried across samples
    float4 *cum_rad; // per-batch sums (cumRadiance/cumAlbedo/cumNormal)
    float4 *cum_alb;
    float4 *cum_nrm;
    float4 *hit;     // t, u, v, prim bits
    uint32_t *hit_inst;
    float4 *sh_dir;  // shadow direction (xyz), tmax (w)
    float4 *sh_c;    // unoccluded light contribution (xyz)
    float4 *nee_b;   // beta for the emitter-ray contribution (xyz), BSDF pdf (w)
    float4 *nee_c;   // emitter-ray contribution of a path flagged F_NEE (xyz), added by regen or shade
    uint32_t *rng;
    uint32_t *flags;
    uint32_t *vol;
    uint32_t *item;   // work item within its job: batch * width * height + pixel
    uint32_t *sample;
    uint32_t *job;    // index into the job table
};

enum CounterIndex {
    C_EXT0 = 0,
    C_EXT1 = 1,
    C_SHADE_L = 2,
    C_SHADE_P = 3,
    C_SHADE_M = 4,
    C_CONN = 5,
    C_REGEN0 = 6,
    C_REGEN1 = 7,
    C_NEXT_ITEM = 8,
    C_ACTIVE = 9,
    C_ERR = 10,
    C_SEGMENTS = 11,
    C_SHADOW = 12,
    C_NEE = 13,
    C_PATHS = 14,
    C_WALK = 15,
    C_NEEQ = 16,
    C_FETCH_EXT = 17,    // extension rays handed out so far in this iteration (lane refill)
    C_FETCH_SHADOW = 18, // shadow and emitter rays handed out so far in this iteration
    C_COUNT = 19
};

struct Queues {
    uint32_t *ext[2];
    uint32_t *ext_key;  // per extension-queue entry: shade bin (0 Lambert, 1 PBR, 2 miss) | 4 = emitter walk
    uint32_t *shade_l, *shade_p, *shade_m;
    uint32_t *walk;     // paths whose pending emitter ray needs the full candidate walk
    uint32_t *conn;     // paths with a shadow ray
    uint32_t *nee;      // paths that end with an emitter ray (k_shadow, after the shadow rays)
    uint32_t *regen[2];
    uint32_t *counters; // CounterIndex
};

// Per-(pixel, batch) sums written when a work item finishes, reduced in batch
// order at the end so the image equals the reference's per-batch
// read-modify-write sequence (raygen.rgen.glsl:134-144).
struct BatchResults {
    float4 *rad;
    float4 *alb;
    float4 *nrm;
};

// One render job: its scene, its parameters and its per-batch sums. The
// table holds one per job slot; a slot is reused once its job has finished.
struct JobView {
    SceneView scene;
    RenderParams params;
    BatchResults results;
};

// Work items of all admitted jobs form one global sequence, handed out in
// admission order: global item range_begin[r] + i is work item i of job slot
// range_job[r] (ranges ascending). Fused per stage, every queue holds paths of
// all live jobs; a path finds its job through ps.job.
struct JobTable {
    const JobView *jobs;                   // per job slot
    const unsigned long long *range_begin; // per hand-out range, ascending
    const uint32_t *range_job;
    uint32_t *item_done;                   // per job slot: work items finished
    unsigned long long *next_item;         // next global work item to hand out
    unsigned long long *total_items;       // end of the last range
    uint32_t *num_ranges;
    uint32_t *idle;                        // slots that found no work
    uint32_t *idle_count;
};

struct LaunchShape {
    int grid;
    int block;
};

// Kernel launchers (wavefront.cu). Each reads its work count from `counters`,
// so a sequence of them can be captured in a CUDA graph.
void launch_iteration(const JobTable &jt, const PathState &ps, const Queues &q, int pingpong, const LaunchShape &shape,
                      cudaStream_t stream);
void launch_reduce(const RenderParams &hparams, const BatchResults &br, float4 *radiance, float4 *albedo,
                   float4 *normal, float4 *radiance_m2, cudaStream_t stream);
// Resets counters, the job table counters and puts every slot on the first
// regeneration queue (its flags cleared).
void launch_init_slots(const Queues &q, const PathState &ps, const JobTable &jt, uint32_t slots, cudaStream_t stream);
// Admits work: raises the global item count to `total_items` over
// `num_ranges` hand-out ranges (after work items ran out, the hand-out counter
// is brought back to the old total) and returns idle slots to the first
// regeneration queue. Launched between graph replays, stream-ordered, after
// the range arrays were written.
void launch_admit(const Queues &q, const JobTable &jt, unsigned long long total_items, uint32_t num_ranges,
                  cudaStream_t stream);
void launch_trace_closest(const SceneView &s, const float4 *rays, uint32_t n, float4 *hits_tuv, uint32_t *hits_ids,
                          uint32_t *err, cudaStream_t stream);
// One wavefront kernel, launched on its own (profiling mode); an iteration
// launches all of them in this order.
enum KernelId {
    K_BEGIN = 0,
    K_REGEN = 1,
    K_EXTEND = 2,
    K_PARTITION = 3,
    K_WALK = 4,
    K_SHADE = 5,
    K_SHADOW = 6, // shadow rays, then the emitter rays of paths that end
    K_NUM = 7
};
// K_SHADE launches one kernel over the three material-sorted queues, or with
// VVPT_SHADE_SPLIT = 1 (a build option) one kernel per queue, each compiled
// for its own surface model. Measured on the 1080p medium scene: the same
// shading time either way (the split kernels need the same 128 registers,
// set by the medium, light-sampling and emitter-ray code they share; capped
// at 3 blocks per SM they spill and run slower), so one launch.
#ifndef VVPT_SHADE_SPLIT
#define VVPT_SHADE_SPLIT 0
#endif
// Lane refill in the extension kernel (binary BLAS). With
// VVPT_EXTEND_PARTITION = 1 (a build option, measured, not kept) the refill
// kernel also appends its hits to the material-sorted shade queues and the
// emitter-walk queue itself and k_partition is not launched: the extension
// kernel grew by what the partition launch took (1920 x 1080 x 64 medium
// scene: 174.3 against 174.5 M paths/s).
#ifndef VVPT_EXTEND_REFILL
#define VVPT_EXTEND_REFILL (!VVPT_BLAS_WIDE)
#endif
#ifndef VVPT_EXTEND_PARTITION
#define VVPT_EXTEND_PARTITION 0
#endif
constexpr int kShadeLaunches = VVPT_SHADE_SPLIT ? 3 : 1;
constexpr int kPartitionLaunches = (VVPT_EXTEND_REFILL && VVPT_EXTEND_PARTITION) ? 0 : 1;
constexpr int launches_of(int k)
{
    return k == K_SHADE ? kShadeLaunches : (k == K_PARTITION ? kPartitionLaunches : 1);
}
constexpr int kKernelsPerIteration = K_NUM + kShadeLaunches - 1 + kPartitionLaunches - 1;
void launch_kernel(KernelId k, const JobTable &jt, const PathState &ps, const Queues &q, int pingpong,
                   const LaunchShape &shape, cudaStream_t stream);

// Algorithmic bytes per work unit of each kernel: the path-state, queue and
// hit-record loads and stores the kernel's code performs for one queue entry
// (nominal branch), plus the three shading vertices and their indices read by
// shade. BVH nodes, triangles and textures are excluded.
constexpr double kBytesRegen = 4 + 3 * 4 + 3 * sizeof(float4) + 3 * sizeof(float4) + 4 + 9 * sizeof(float4) + 5 * 4 + 4;
constexpr double kBytesExtend = 4 + 4 /* flags */ + 2 * sizeof(float4) + sizeof(float4) + 4 + 4 /* key */;
constexpr double kBytesPartition = 4 + 4 + 4;
constexpr double kBytesWalk = 4 + 4 + 4 + 4 * sizeof(float4) /* o d nee_b rad */ + sizeof(float4) + 4;
constexpr double kBytesShade = 4 + (4 + 4 + 4 + 4) + 5 * sizeof(float4) /* beta rad o d hit */ + 3 * 4 +
                               3 * sizeof(ShadeVertex) /* vertices */ + (4 + 4 + 4) + 4 * sizeof(float4) /* writes */ +
                               5 * sizeof(float4) /* alb nrm sh_dir sh_c nee_b */ + sizeof(float4) /* nee_b read */ +
                               2 * 4;
constexpr double kBytesShadow = 4 + 4 + 4 + 4 * sizeof(float4) /* o sh_dir rad sh_c */ + sizeof(float4) + 4;

}  // namespace vvpt
