/*
 * vvpt.h — C ABI of the GB300-native offline path tracer.
 *
 * This is the drop-in boundary for vengine's path-traced offline renderer
 * (kwstanths/vviewer). Everything below is plain C: pointers, sizes and POD
 * structs, no C++ or torch types. Every entry point returns a vvpt_status and
 * never throws; device-side failures surface through status words that the
 * library reads back on the host.
 *
 * Reference interfaces replaced (paths relative to the vviewer project):
 *   - RendererPathTracing (src/lib/vengine/core/Renderer.hpp:11-39):
 *       renderInfo()/render()/renderProgress()/isRayTracingEnabled()
 *       -> vvpt_render / vvpt_progress / vvpt_create
 *   - VulkanRendererPathTracing::render() and its batch loop
 *       (src/lib/vengine/vulkan/renderers/VulkanRendererPathTracing.cpp:121-226, 791-901)
 *       -> vvpt_render
 *   - The GPU-side scene buffers the shaders read (InstanceData, MaterialData,
 *       LightData, LightInstance, SceneData, PathTracingData;
 *       src/lib/vengine/shaders/include/structs.glsl:4-69,
 *       src/lib/vengine/core/Scene.hpp:27-35,
 *       src/lib/vengine/vulkan/renderers/VulkanRendererPathTracing.hpp:57-61)
 *       -> vvpt_scene_desc / vvpt_scene_data, uploaded by vvpt_scene_upload
 *   - TLAS/BLAS creation (src/lib/vengine/vulkan/resources/VulkanAccelerationStructure.cpp:14-279,
 *       src/lib/vengine/vulkan/VulkanScene.cpp:306-381) -> vvpt_scene_upload
 *   - traceRayEXT closest hit (shaders/pt/raygen.rgen.glsl:110 with the empty
 *       any-hit of shaders/pt/rayPrimary.rahit.glsl:32-71) -> vvpt_trace_closest
 */
#ifndef VVPT_H
#define VVPT_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(_WIN32)
#define VVPT_API __declspec(dllexport)
#else
#define VVPT_API __attribute__((visibility("default")))
#endif

/* Error model: the reference logs and breaks out of its batch loop on a
 * fence timeout or device loss (VulkanRendererPathTracing.cpp:869-882) and
 * returns early on an empty scene (:132-136). Here every call reports. */
typedef enum vvpt_status {
    VVPT_OK = 0,
    VVPT_ERR_INVALID_ARG = 1,     /* null pointer, bad size, index out of range */
    VVPT_ERR_OOM = 2,             /* device or host allocation failed */
    VVPT_ERR_BUDGET_EXCEEDED = 3, /* a job does not fit the device-memory budget */
    VVPT_ERR_TIMEOUT = 4,         /* deadline passed before the work finished */
    VVPT_ERR_DEVICE = 5,          /* CUDA error or a device status word was set */
    VVPT_ERR_NOT_READY = 6,       /* job still running (vvpt_poll) */
    VVPT_ERR_EMPTY_SCENE = 7,     /* nothing to render (reference: warning + return) */
    VVPT_ERR_UNSUPPORTED = 8
} vvpt_status;

typedef struct vvpt_ctx vvpt_ctx;
typedef struct vvpt_scene vvpt_scene;

/* ---- Scene buffers (mirrors of the reference GPU structs) ---------------- */

/* Vertex, shaders/include/structs.glsl:4-12 (scalar layout, 68 bytes). */
typedef struct vvpt_vertex {
    float position[3];
    float uv[2];
    float normal[3];
    float color[3];
    float tangent[3];
    float bitangent[3];
} vvpt_vertex;

/* One mesh = one BLAS (VulkanMesh.cpp:15-26). indices: 3 per triangle. */
typedef struct vvpt_mesh_desc {
    const vvpt_vertex *vertices;
    uint32_t num_vertices;
    const uint32_t *indices;
    uint32_t num_triangles;
} vvpt_mesh_desc;

/* MaterialData, shaders/include/structs.glsl:41-52 (128 bytes).
 * albedo: RGB albedo, A alpha. metallic_roughness_ao: R metallic, G roughness,
 * B AO, A transparent flag. emissive: RGB colour, A intensity.
 * textures1: albedo, metallic, roughness, AO texture indices.
 * textures2: emissive, normal, BRDF-LUT, alpha texture indices.
 * uv_tiling: R u tiling, G v tiling, B material type (0 PBR, 2 Lambert, 3 volume).
 * Volumes pack sigma_a in albedo, sigma_s in metallic_roughness_ao and g in
 * emissive[0] (src/lib/vengine/vulkan/resources/VulkanMaterial.cpp:438-483). */
typedef struct vvpt_material {
    float albedo[4];
    float metallic_roughness_ao[4];
    float emissive[4];
    uint32_t textures1[4];
    uint32_t textures2[4];
    float uv_tiling[4];
    uint32_t padding[8];
} vvpt_material;

enum {
    VVPT_MATERIAL_PBR_STANDARD = 0,
    VVPT_MATERIAL_LAMBERT = 2,
    VVPT_MATERIAL_VOLUME = 3
};

/* InstanceData, src/lib/vengine/core/Instances.hpp:17-35, with the buffer
 * device addresses replaced by a mesh index. model: column-major 4x4
 * object-to-world. id: R object id, G front-facing volume material index,
 * B back-facing volume material index (-1 = none). flags bit 0: the instance
 * is in the TLAS (opaque groups and transparent objects are, light-only
 * objects are not; VulkanScene.cpp:306-357). */
typedef struct vvpt_instance {
    float model[16];
    float id[4];
    uint32_t material_index;
    uint32_t mesh_index;
    uint32_t num_triangles;
    uint32_t flags;
} vvpt_instance;

enum { VVPT_INSTANCE_IN_TLAS = 1u };

/* LightData, shaders/include/structs.glsl:55-61: RGB colour, A intensity;
 * type[0] = LightType (0 point, 1 directional). */
typedef struct vvpt_light_data {
    float color[4];
    uint32_t type[4];
    uint32_t padding[8];
} vvpt_light_data;

/* LightInstance, src/lib/vengine/core/Instances.hpp:39-44, filled as in
 * src/lib/vengine/vulkan/VulkanInstances.cpp:66-109. info: R LightData index,
 * G InstanceData index, A light type (0 point, 1 directional, 2 mesh).
 * position: world position (point) or -direction source (directional: the
 * model matrix applied to +Z) or row 0 of the model matrix (mesh);
 * position1/position2: rows 1/2 of the model matrix (mesh). */
typedef struct vvpt_light_instance {
    uint32_t info[4];
    float position[4];
    float position1[4];
    float position2[4];
} vvpt_light_instance;

enum {
    VVPT_TEXTURE_RGBA8_LINEAR = 0,
    VVPT_TEXTURE_RGBA8_SRGB = 1,
    VVPT_TEXTURE_RGBA32F = 2
};

/* A 2D texture sampled bilinearly at LOD 0 with repeat addressing
 * (VulkanTexture.cpp:219-230). The environment map is an equirectangular
 * RGBA32F image looked up with the mapping of
 * shaders/include/environmentMap.glsl:3-10. */
typedef struct vvpt_texture_desc {
    uint32_t width;
    uint32_t height;
    uint32_t format;
    uint32_t reserved;
    const void *data;
} vvpt_texture_desc;

typedef struct vvpt_scene_desc {
    const vvpt_mesh_desc *meshes;
    uint32_t num_meshes;
    const vvpt_instance *instances;
    uint32_t num_instances;
    const vvpt_material *materials;
    uint32_t num_materials;
    const vvpt_light_data *light_data;
    uint32_t num_light_data;
    const vvpt_light_instance *lights; /* point/directional first, then mesh lights */
    uint32_t num_lights;
    const vvpt_texture_desc *textures;
    uint32_t num_textures;
    const vvpt_texture_desc *environment; /* may be NULL */
} vvpt_scene_desc;

/* SceneData, src/lib/vengine/core/Scene.hpp:27-35, column-major matrices,
 * projection already flipped ([1][1] *= -1) for the render resolution
 * (VulkanRendererPathTracing.cpp:143-170). exposure: R exposure, G environment
 * intensity, B lens radius, A focal distance. background: RGB colour, A
 * environment type (0 solid, 1 HDRI, 2 solid + HDRI lighting). volumes: R
 * camera volume material index (-1 none), G znear, B zfar. */
typedef struct vvpt_scene_data {
    float view[16];
    float view_inverse[16];
    float projection[16];
    float projection_inverse[16];
    float exposure[4];
    float background[4];
    float volumes[4];
} vvpt_scene_data;

/* RendererPathTracing::RenderInfo (src/lib/vengine/core/Renderer.hpp:14-28),
 * compute fields only; file naming and writing stay in the host adapter. */
typedef struct vvpt_render_info {
    uint32_t samples;    /* total samples per pixel; batches = samples / batch_size */
    uint32_t depth;      /* max traced segments per sample */
    uint32_t batch_size; /* samples per batch (one RNG seed per batch) */
    uint32_t width;
    uint32_t height;
    uint32_t flags;      /* VVPT_RENDER_* */
} vvpt_render_info;

enum {
    /* also return per-pixel sum over batches of the squared batch sums
     * (radiance only), for Monte Carlo error estimates */
    VVPT_RENDER_WANT_BATCH_M2 = 1u,
    /* launch the wavefront kernels one by one with CUDA events around each
     * (no graphs) and record per-kernel times: see vvpt_last_kernel_profile */
    VVPT_RENDER_PROFILE_KERNELS = 2u,
    /* Estimator addition with no counterpart in the reference (which never
     * light-samples the environment, lightSampling.glsl:101-106): with an
     * environment image and background mode 1 or 2, the environment joins
     * the uniform light pick as one more light, importance sampled by
     * texel luminance, and escapes of sampled directions take the BSDF side
     * of the power-heuristic MIS weight. The environment sample of a path's
     * last event contributes nothing (the reference never adds environment
     * light from the last event either), so the expected image is the
     * reference estimator's; the variance under bright skies is far lower. */
    VVPT_RENDER_ENV_IS = 4u,
    /* The reference's low-discrepancy sampler (shaders/include/rng/
     * rng_pmj.glsl, selected there by SAMPLING_PMJ in pt/defines_pt.glsl:3)
     * instead of the RTGEMS xorshift stream: 2D draws (pixel jitter, lens,
     * BSDF/phase directions, triangle points) from 16 progressive
     * multi-jittered (0,2) sequences, 1D draws from a hashed permutation of
     * the sample index plus a blue-noise offset; per-sample dimension start
     * pixel.y * width + pixel.y and sample index batch * batch_size + s as
     * in raygen.rgen.glsl:57-61. Tables: vvpt_sampler_tables. */
    VVPT_RENDER_SAMPLER_PMJ = 8u,
    /* No counterpart in the reference (whose images accumulate in float,
     * raygen.rgen.glsl:134-144): the per-batch sums are added in double
     * precision, in batch order, and rounded to float once. For reference
     * images of many batches (an FP64-accumulated high-spp render); the
     * default float sum in batch order is the reference's sequence. */
    VVPT_RENDER_REDUCE_FP64 = 16u
};

/* Sizes of the low-discrepancy sampler's tables
 * (shaders/include/rng/rng_pmj_defines.glsl, bluenoise_defines.glsl). */
enum {
    VVPT_PMJ_SEQUENCES = 16,
    VVPT_PMJ_SAMPLES = 16384,
    VVPT_BLUE_NOISE_TEXTURES = 48,
    VVPT_BLUE_NOISE_RES = 128
};

/* Copies the sampler's tables (generated once per process, deterministic):
 * pmj [VVPT_PMJ_SEQUENCES][VVPT_PMJ_SAMPLES][2] and blue_noise
 * [VVPT_BLUE_NOISE_TEXTURES][x][y], floats in [0, 1). Either pointer may be
 * NULL. The reference ships these as data (math/PMJSequences.hpp,
 * math/BlueNoise.hpp, uploaded by vulkan/resources/VulkanRandom.cpp); here
 * they are regenerated: (0,2) sequences as Owen-scrambled Sobol points,
 * blue noise by void-and-cluster. */
VVPT_API vvpt_status vvpt_sampler_tables(float *pmj, float *blue_noise);

/* Output images, RGBA32F row-major W*H*4 floats each, A = 1 (the three
 * storage images of raygen.rgen.glsl:131-144). Any pointer may be NULL.
 * on_device != 0: pointers are device pointers (stay valid, written in
 * place); else host pointers (copied back before the call returns). */
typedef struct vvpt_outputs {
    float *radiance;
    float *albedo;
    float *normal;
    float *radiance_m2;
    int32_t on_device;
} vvpt_outputs;

/* Closest-hit ray record for vvpt_trace_closest: origin, tmin, direction, tmax. */
typedef struct vvpt_ray {
    float origin[3];
    float tmin;
    float direction[3];
    float tmax;
} vvpt_ray;

/* Hit record: instance = InstanceData slot (gl_InstanceCustomIndexEXT),
 * primitive = triangle index in the mesh (gl_PrimitiveID), u/v = barycentric
 * weights of vertices 1 and 2 (hitAttributeEXT attribs). instance = 0xFFFFFFFF
 * on a miss. */
typedef struct vvpt_hit {
    float t;
    float u;
    float v;
    uint32_t instance;
    uint32_t primitive;
} vvpt_hit;

/* ---- Context ------------------------------------------------------------- */

/* Creates a context on CUDA device `device` (one stream set per context).
 * Fails with VVPT_ERR_DEVICE when no usable GPU is present (the reference
 * throws at init without ray-tracing support, VulkanRendererPathTracing.cpp:48-51). */
VVPT_API vvpt_status vvpt_create(int device, vvpt_ctx **out_ctx);
VVPT_API vvpt_status vvpt_destroy(vvpt_ctx *ctx);
/* Last error message of this context (thread-local copy owned by ctx). */
VVPT_API const char *vvpt_last_error(vvpt_ctx *ctx);
/* Library version string, no context needed. */
VVPT_API const char *vvpt_version(void);

/* ---- Scene --------------------------------------------------------------- */

/* Uploads meshes, instances, materials, lights and textures, and builds the
 * BLAS per mesh and the instance TLAS on the device. The scene stays resident
 * until vvpt_scene_release. */
VVPT_API vvpt_status vvpt_scene_upload(vvpt_ctx *ctx, const vvpt_scene_desc *desc, vvpt_scene **out_scene);
VVPT_API vvpt_status vvpt_scene_release(vvpt_ctx *ctx, vvpt_scene *scene);
/* Bytes of device memory held by the scene (geometry, BVH, textures). */
VVPT_API vvpt_status vvpt_scene_device_bytes(vvpt_ctx *ctx, const vvpt_scene *scene, uint64_t *out_bytes);

/* ---- Render -------------------------------------------------------------- */

/* One synchronous render (RendererPathTracing::render). */
VVPT_API vvpt_status vvpt_render(vvpt_ctx *ctx,
                                 vvpt_scene *scene,
                                 const vvpt_scene_data *scene_data,
                                 const vvpt_render_info *info,
                                 vvpt_outputs *outputs);
/* Render that makes no device allocations (no counterpart in the reference).
 *
 * For callers that cannot let a library call cudaMalloc: engines that manage
 * a fixed device-memory pool and forbid allocations they did not make,
 * processes under a hard memory cap, or frame loops that must not take the
 * implicit device synchronisation of the allocator. Same result as
 * vvpt_render (bit for bit), from the same render parameters (sizes checked
 * the same way, VVPT_RENDER_ENV_IS honoured); the PMJ sampler, whose tables
 * would need an allocation, is refused with VVPT_ERR_UNSUPPORTED. All scratch
 * (parameters, counters, ray queues,
 * path state for up to 65,536 paths in flight, per-batch sums) comes from one
 * 64 MiB array the library defines at file scope, which every GPU that loads
 * the library holds until the process exits. Limit: the request must fit it:
 * width * height * (samples / batch_size) <= 993,936 work items (48 bytes
 * each, beside 18.5 MiB of path state), e.g. 256 x 256 at 15 batches;
 * larger requests fail with
 * VVPT_ERR_INVALID_ARG before any GPU work. Outputs must be device buffers
 * (outputs->on_device = 1). The scene must already be resident
 * (vvpt_scene_upload allocates; this call does not).
 * The first call on a device looks up the array's device address and keeps
 * it for the life of the process; make that first call before any stream
 * capture, and do not call this entry point again after cudaDeviceReset (or
 * any other teardown of the device's primary context) in the same process:
 * the kept address would be stale. All calls in the process share the
 * array: calls that overlap on the GPU (two contexts on one device, or two
 * threads) race and corrupt each other's results, so serialise them. */
VVPT_API vvpt_status vvpt_render_noalloc(vvpt_ctx *ctx,
                                         vvpt_scene *scene,
                                         const vvpt_scene_data *scene_data,
                                         const vvpt_render_info *info,
                                         vvpt_outputs *outputs);

/* Fraction of the current/last render done, readable from any thread
 * (RendererPathTracing::renderProgress). */
VVPT_API vvpt_status vvpt_progress(vvpt_ctx *ctx, float *out_progress);

/* Closest hit for a batch of rays against the scene (no shading). rays/hits
 * are host pointers unless on_device != 0. */
VVPT_API vvpt_status vvpt_trace_closest(vvpt_ctx *ctx,
                                        vvpt_scene *scene,
                                        const vvpt_ray *rays,
                                        uint32_t num_rays,
                                        vvpt_hit *hits,
                                        int32_t on_device);

/* Launch statistics of the last vvpt_render: kernels launched, wavefront
 * iterations, segments traced, shadow and emitter rays traced. */
typedef struct vvpt_render_stats {
    uint64_t kernel_launches;
    uint64_t iterations;
    uint64_t segments;
    uint64_t shadow_rays;
    uint64_t emitter_rays;
    uint64_t paths;
    double device_ms;
} vvpt_render_stats;
VVPT_API vvpt_status vvpt_last_render_stats(vvpt_ctx *ctx, vvpt_render_stats *out_stats);

/* Per-kernel profile of the last render made with
 * VVPT_RENDER_PROFILE_KERNELS: for each wavefront kernel, launches, work
 * units (queue entries) processed, summed CUDA-event time, and the kernel's
 * algorithmic bytes per unit (compulsory path-state and queue traffic plus
 * shading-vertex fetches; BVH nodes and textures excluded). */
typedef struct vvpt_kernel_profile_entry {
    char name[24];
    uint64_t launches;
    uint64_t units;
    double total_ms;
    double bytes_per_unit;
} vvpt_kernel_profile_entry;
typedef struct vvpt_kernel_profile {
    uint32_t count;
    vvpt_kernel_profile_entry kernels[8];
} vvpt_kernel_profile;
VVPT_API vvpt_status vvpt_last_kernel_profile(vvpt_ctx *ctx, vvpt_kernel_profile *out_profile);

/* Runs the context's work on a caller-owned CUDA stream (a cudaStream_t
 * passed as void*); NULL restores the context's own stream. Calls stay
 * synchronous with respect to the host. */
VVPT_API vvpt_status vvpt_set_stream(vvpt_ctx *ctx, void *cuda_stream);

/* Tuning knobs (path-slot pool size and blocks per SM for the wavefront
 * kernels); 0 = automatic. */
typedef struct vvpt_tuning {
    uint32_t slots;
    uint32_t blocks_per_sm;
    uint32_t threads_per_block;
    uint32_t iterations_per_graph;
} vvpt_tuning;
VVPT_API vvpt_status vvpt_set_tuning(vvpt_ctx *ctx, const vvpt_tuning *tuning);
VVPT_API vvpt_status vvpt_get_tuning(vvpt_ctx *ctx, vvpt_tuning *out_tuning);

/* Autotuner (no counterpart in the reference): times short renders of the
 * request (its image size and depth, a few batches sized to about
 * budget_ms / 12 each) and picks blocks per SM, path slots and iterations
 * per CUDA graph by coordinate descent on measured paths/s. The result is
 * stored as the context's tuning (used by vvpt_render and by a job engine
 * started afterwards) and returned in out_tuning (may be NULL). Images do
 * not depend on the tuning. */
VVPT_API vvpt_status vvpt_autotune(vvpt_ctx *ctx,
                                   vvpt_scene *scene,
                                   const vvpt_scene_data *scene_data,
                                   const vvpt_render_info *info,
                                   double budget_ms,
                                   vvpt_tuning *out_tuning);

/* BVH builder of vvpt_scene_upload: AUTO builds meshes of at least 65,536
 * triangles on the GPU (binned SAH, one tree level per round of kernels) and
 * the rest, the baked small instances and the TLAS on the host; HOST builds
 * every tree on the host (binned SAH with FP64 costs); GPU builds every BLAS,
 * the baked small instances' BLAS and the TLAS on the GPU (trees of at most
 * one leaf stay on the host). All give the same closest hits. */
enum { VVPT_BVH_BUILDER_AUTO = 0, VVPT_BVH_BUILDER_HOST = 1, VVPT_BVH_BUILDER_GPU = 2 };
VVPT_API vvpt_status vvpt_set_bvh_builder(vvpt_ctx *ctx, int builder);

/* ---- Jobs: batched and served renders ------------------------------------
 *
 * No counterpart in the reference, whose render() is synchronous and
 * non-reentrant (VulkanRendererPathTracing.cpp:121-226). A submitted job is
 * the same request as vvpt_render; the context's engine thread runs all
 * admitted jobs together, with the work items of every job in one hand-out
 * sequence and one queue per wavefront stage, so small jobs fill the GPU
 * beside large ones. A job's images are bit-identical to vvpt_render of the
 * same request (its RNG streams depend only on pixel and batch). Admission is
 * first come first served, bounded by the device budget.
 *
 * Thread-safe: submit, poll, wait and release may be called from any thread.
 * The scene must stay resident until its jobs have finished
 * (vvpt_scene_release returns VVPT_ERR_NOT_READY while they run). Output
 * buffers must stay valid until the job is done; host outputs are written
 * by the engine's completion thread. */
typedef uint64_t vvpt_job;

typedef enum vvpt_job_state {
    VVPT_JOB_QUEUED = 0,  /* submitted, waiting for admission */
    VVPT_JOB_RUNNING = 1, /* admitted: its work items are being traced */
    VVPT_JOB_DONE = 2,    /* outputs written */
    VVPT_JOB_FAILED = 3   /* see status */
} vvpt_job_state;

typedef struct vvpt_job_info {
    uint32_t state;       /* vvpt_job_state */
    int32_t status;       /* vvpt_status of a failed job, else VVPT_OK */
    double submit_ms;     /* host steady clock, ms since the context was created */
    double start_ms;      /* admission */
    double end_ms;        /* outputs written */
    uint64_t paths;       /* width * height * (samples / batch_size) * batch_size */
    uint64_t device_bytes; /* engine memory the job holds while admitted */
} vvpt_job_info;

/* Queues one render. `outputs` is copied; its buffers (host or device) are
 * written when the job completes. Fails with VVPT_ERR_BUDGET_EXCEEDED if the
 * job alone could never fit the budget. */
VVPT_API vvpt_status vvpt_submit(vvpt_ctx *ctx,
                                 vvpt_scene *scene,
                                 const vvpt_scene_data *scene_data,
                                 const vvpt_render_info *info,
                                 const vvpt_outputs *outputs,
                                 vvpt_job *out_job);
/* Non-blocking state of a job. */
VVPT_API vvpt_status vvpt_poll(vvpt_ctx *ctx, vvpt_job job, vvpt_job_info *out_info);
/* Blocks until the job is done (VVPT_OK), failed (its status) or
 * `timeout_ms` passed (VVPT_ERR_TIMEOUT; the job keeps running). A negative
 * timeout waits without limit. */
VVPT_API vvpt_status vvpt_wait(vvpt_ctx *ctx, vvpt_job job, double timeout_ms);
/* Forgets a finished job's record (VVPT_ERR_NOT_READY while it runs). */
VVPT_API vvpt_status vvpt_job_release(vvpt_ctx *ctx, vvpt_job job);
/* Device-memory budget of the engine in bytes (path state, queues, per-job
 * batch sums and output staging); 0 = no limit but the device's memory.
 * Applies to admissions after the call. */
VVPT_API vvpt_status vvpt_set_budget(vvpt_ctx *ctx, uint64_t bytes);
/* Engine occupancy: its fixed pool (path slots, queues, job table), the
 * memory admitted jobs hold, and job counts by state (records not yet
 * released). Starts the engine if it is not running. */
typedef struct vvpt_engine_stats {
    uint64_t fixed_bytes;
    uint64_t job_bytes;
    uint32_t queued;
    uint32_t running;
    uint32_t finished;
    uint32_t slots;
} vvpt_engine_stats;
VVPT_API vvpt_status vvpt_engine_stats_get(vvpt_ctx *ctx, vvpt_engine_stats *out_stats);
/* Renders n requests together through the engine and waits for all of them;
 * returns the first failure. Each output equals vvpt_render's. */
VVPT_API vvpt_status vvpt_render_batch(vvpt_ctx *ctx,
                                       uint32_t n,
                                       vvpt_scene *const *scenes,
                                       const vvpt_scene_data *scene_data,
                                       const vvpt_render_info *infos,
                                       const vvpt_outputs *outputs);

/* ---- Learned denoiser ------------------------------------------------------
 *
 * Stands in for the reference's OpenImageDenoise call in storeToDisk
 * (VulkanRendererPathTracing.cpp:985-1018): a 5-level U-Net (3x3 convs of
 * 32/48/64/96/128 channels) over noisy radiance, albedo and normal, trained on
 * the GPU on pairs the tracer renders (few-spp inputs, many-spp targets).
 * Every convolution (forward, input gradient, weight gradient) runs on the
 * BF16 tensor cores with FP32 accumulation in the library's own kernels;
 * parameters are FP32 with an Adam optimiser. Images are device RGBA32F
 * buffers (A ignored on input, 1 on output); width and height must be
 * multiples of 16. Parameter layout: per layer, weights [cout][3][3][cin]
 * then biases [cout]; layers: encoder (2 per level), decoder (2 per level,
 * coarsest first), output. */
typedef struct vvpt_denoiser vvpt_denoiser;

typedef struct vvpt_denoise_batch {
    const float *radiance; /* count x height x width RGBA32F, device */
    const float *albedo;
    const float *normal;
    const float *target;   /* high-spp radiance, same layout */
    uint32_t count;
    uint32_t width;
    uint32_t height;
} vvpt_denoise_batch;

/* New network with seeded initial weights (He-normal; the output layer
 * small). */
VVPT_API vvpt_status vvpt_denoiser_create(vvpt_ctx *ctx, uint64_t seed, vvpt_denoiser **out_denoiser);
VVPT_API vvpt_status vvpt_denoiser_destroy(vvpt_denoiser *denoiser);
VVPT_API vvpt_status vvpt_denoiser_num_params(vvpt_denoiser *denoiser, uint64_t *out_count);
VVPT_API vvpt_status vvpt_denoiser_get_params(vvpt_denoiser *denoiser, float *host_params, uint64_t count);
VVPT_API vvpt_status vvpt_denoiser_set_params(vvpt_denoiser *denoiser, const float *host_params, uint64_t count);
/* Loss (mean absolute error of log(1 + radiance)) and its gradient with
 * respect to every parameter, copied to the host; parameters unchanged. */
VVPT_API vvpt_status vvpt_denoiser_gradients(vvpt_denoiser *denoiser,
                                             const vvpt_denoise_batch *batch,
                                             float *host_grads,
                                             uint64_t count,
                                             float *out_loss);
/* One Adam step (beta 0.9 / 0.999) on the batch; returns the loss before it. */
VVPT_API vvpt_status vvpt_denoiser_train_step(vvpt_denoiser *denoiser,
                                              const vvpt_denoise_batch *batch,
                                              float learning_rate,
                                              float *out_loss);
/* Convolution kernels. TCGEN05 (default): tcgen05 tensor cores with TMEM
 * accumulators; layers whose weights fit in shared memory run the strip
 * kernel (TMA-fed ring of input rows, weights resident, one wave of
 * persistent CTAs), the others a per-tile kernel. MMA_SYNC: the warp-level
 * BF16 m16n8k16 path. TCGEN05_TILES: the per-tile tcgen05 kernels only.
 * TCGEN05_PERSISTENT: the strip kernel on a small grid, so that every CTA
 * walks several row segments. TCGEN05_UNFUSED: as TCGEN05, but inference
 * writes the upsample + concat tensor instead of reading both halves in the
 * convolution. TCGEN05_WGRAD: as TCGEN05, and the weight gradients on the
 * tcgen05 tensor cores as well (by default they run on the mma.sync kernel,
 * which is faster for these channel counts). All accumulate in FP32; the
 * variants serve as cross-checks of the first. */
enum {
    VVPT_DENOISER_TCGEN05 = 0,
    VVPT_DENOISER_MMA_SYNC = 1,
    VVPT_DENOISER_TCGEN05_TILES = 2,
    VVPT_DENOISER_TCGEN05_PERSISTENT = 3,
    VVPT_DENOISER_TCGEN05_UNFUSED = 4,
    VVPT_DENOISER_TCGEN05_WGRAD = 5
};
VVPT_API vvpt_status vvpt_denoiser_set_kernels(vvpt_denoiser *denoiser, int kind);
/* Diagnostics for failure handling: the next tcgen05 strip convolution of
 * the process (of any denoiser) withholds its accumulator-ready signal, its
 * drain warps' bounded waits (2 s) run out, and the call that launched it
 * returns VVPT_ERR_DEVICE; the kernel frees its tensor memory and the
 * denoiser stays usable. */
VVPT_API vvpt_status vvpt_denoiser_inject_wait_timeout(vvpt_denoiser *denoiser);
/* Denoises one image: out = exp(network(log1p radiance, albedo, normal)) - 1. */
VVPT_API vvpt_status vvpt_denoiser_apply(vvpt_denoiser *denoiser,
                                         const float *radiance,
                                         const float *albedo,
                                         const float *normal,
                                         float *out,
                                         uint32_t width,
                                         uint32_t height);

/* ---- Model textures -------------------------------------------------------
 *
 * Replaces stb_image's JPEG path in assimpLoadTextureData
 * (src/lib/vengine/core/io/AssimpLoadModel.cpp): sequential Huffman JPEG
 * (ITU-T T.81 baseline and extended, 8-bit, grey or YCbCr with sampling
 * factors 1 and 2, restart intervals) decoded on the host to RGBA8 (grey
 * replicated to RGB; alpha 255). With rgba = NULL only width, height and
 * channels (1 or 3) are returned; otherwise rgba must hold width * height * 4
 * bytes. Progressive, lossless, arithmetic-coded and 12-bit files return
 * VVPT_ERR_UNSUPPORTED; malformed files VVPT_ERR_INVALID_ARG. No context or
 * GPU is needed. */
VVPT_API vvpt_status vvpt_jpeg_decode(const uint8_t *data,
                                      uint64_t size,
                                      uint32_t *width,
                                      uint32_t *height,
                                      uint32_t *channels,
                                      uint8_t *rgba,
                                      uint64_t rgba_bytes);

#ifdef __cplusplus
}
#endif

#endif /* VVPT_H */
