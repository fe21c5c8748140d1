// C ABI of the path tracer (include/vvpt.h): context, scene upload with BVH
// builds, and the render loop that drives the wavefront kernels through CUDA
// graphs.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/vvpt.h"
#include "internal.h"
#include "bvh_build.h"
#include "sampler_tables.h"
#include "scene_pack.h"
#include "scene_gpu.h"
#include "traverse.cuh"
#include "wavefront.cuh"

using namespace vvpt;

namespace vvpt {

vvpt_status make_render_params(vvpt_ctx *ctx, const vvpt_scene *scene, const vvpt_scene_data *sd,
                               const vvpt_render_info *info, RenderParams &hp)
{
    if (info->width == 0 || info->height == 0 || info->batch_size == 0)
        return fail(ctx, VVPT_ERR_INVALID_ARG, "width, height and batch_size must be positive");
    if ((uint64_t)info->width * info->height > (1ull << 28))
        return fail(ctx, VVPT_ERR_INVALID_ARG, "resolution too large");
    const uint32_t batches = info->samples / info->batch_size; // integer truncation, as the reference
    hp = RenderParams{};
    for (int c = 0; c < 4; c++) {
        hp.view_inv[c] = make_float4(sd->view_inverse[c * 4 + 0], sd->view_inverse[c * 4 + 1],
                                     sd->view_inverse[c * 4 + 2], sd->view_inverse[c * 4 + 3]);
        hp.proj_inv[c] = make_float4(sd->projection_inverse[c * 4 + 0], sd->projection_inverse[c * 4 + 1],
                                     sd->projection_inverse[c * 4 + 2], sd->projection_inverse[c * 4 + 3]);
    }
    hp.background = make_float3(sd->background[0], sd->background[1], sd->background[2]);
    hp.env_type = sd->background[3];
    hp.lens_radius = sd->exposure[2];
    hp.focal_distance = sd->exposure[3];
    hp.env_intensity = sd->exposure[1];
    hp.zfar = sd->volumes[2];
    hp.zfar_trunc = (float)(uint32_t)std::max(0.0f, sd->volumes[2]);
    hp.cam_volume = (int32_t)sd->volumes[0];
    if (hp.cam_volume != -1 && (hp.cam_volume < 0 || (uint32_t)hp.cam_volume >= scene->num_materials))
        return fail(ctx, VVPT_ERR_INVALID_ARG, "camera volume material index out of range");
    hp.width = info->width;
    hp.height = info->height;
    hp.batch_size = info->batch_size;
    hp.batches = batches;
    hp.depth = std::min(info->depth, 255u);
    hp.total_samples = info->batch_size * batches;
    hp.num_lights = scene->view.num_lights;
    const uint64_t total_items64 = (uint64_t)info->width * info->height * batches;
    if (total_items64 >= 0xFFFFFFF0ull)
        return fail(ctx, VVPT_ERR_INVALID_ARG, "width * height * batches exceeds 2^32");
    hp.total_items = (uint32_t)total_items64;
    hp.want_m2 = (info->flags & VVPT_RENDER_WANT_BATCH_M2) ? 1u : 0u;
    hp.reduce_fp64 = (info->flags & VVPT_RENDER_REDUCE_FP64) ? 1u : 0u;
    const int mode = (int)hp.env_type;
    hp.env_light = ((info->flags & VVPT_RENDER_ENV_IS) && scene->view.env_func_int > 0.0f && (mode == 1 || mode == 2))
                       ? 1u
                       : 0u;
    if (info->flags & VVPT_RENDER_SAMPLER_PMJ) {
        std::lock_guard<std::mutex> lk(ctx->sampler_mu);
        if (!ctx->pmj_table.ptr) {
            const SamplerTables &t = sampler_tables();
            cudaSetDevice(ctx->device);
            VV_CUDA(ctx->pmj_table.alloc(t.pmj.size() * sizeof(float)), "cudaMalloc sampler tables");
            VV_CUDA(ctx->blue_noise_table.alloc(t.blue_noise.size() * sizeof(float)), "cudaMalloc sampler tables");
            VV_CUDA(cudaMemcpy(ctx->pmj_table.ptr, t.pmj.data(), t.pmj.size() * sizeof(float), cudaMemcpyHostToDevice),
                    "upload sampler tables");
            VV_CUDA(cudaMemcpy(ctx->blue_noise_table.ptr, t.blue_noise.data(), t.blue_noise.size() * sizeof(float),
                               cudaMemcpyHostToDevice),
                    "upload sampler tables");
        }
        hp.sampler = 1u;
        hp.pmj = ctx->pmj_table.as<float>();
        hp.blue_noise = ctx->blue_noise_table.as<float>();
    }
    return VVPT_OK;
}

// 14 float4 arrays (one spare) and 7 uint32 arrays per slot
size_t path_state_bytes(size_t slots)
{
    return 14 * aligned256(slots * sizeof(float4)) + 7 * aligned256(slots * sizeof(uint32_t));
}

size_t queue_bytes(size_t slots)
{
    return 11 * aligned256(slots * sizeof(uint32_t)) + aligned256(C_COUNT * sizeof(uint32_t));
}

PathState carve_path_state(char *base, size_t n)
{
    const size_t f4 = aligned256(n * sizeof(float4)), u4 = aligned256(n * sizeof(uint32_t));
    auto take = [&](size_t b) {
        char *p = base;
        base += b;
        return p;
    };
    PathState ps;
    ps.o = (float4 *)take(f4);
    ps.d = (float4 *)take(f4);
    ps.beta = (float4 *)take(f4);
    ps.rad = (float4 *)take(f4);
    ps.alb = (float4 *)take(f4);
    ps.nrm = (float4 *)take(f4);
    ps.cum_rad = (float4 *)take(f4);
    ps.cum_alb = (float4 *)take(f4);
    ps.cum_nrm = (float4 *)take(f4);
    ps.hit = (float4 *)take(f4);
    ps.sh_dir = (float4 *)take(f4);
    ps.sh_c = (float4 *)take(f4);
    ps.nee_b = (float4 *)take(f4);
    ps.nee_c = (float4 *)take(f4);
    ps.hit_inst = (uint32_t *)take(u4);
    ps.rng = (uint32_t *)take(u4);
    ps.flags = (uint32_t *)take(u4);
    ps.vol = (uint32_t *)take(u4);
    ps.item = (uint32_t *)take(u4);
    ps.sample = (uint32_t *)take(u4);
    ps.job = (uint32_t *)take(u4);
    return ps;
}

Queues carve_queues(char *base, size_t n)
{
    const size_t u4 = aligned256(n * sizeof(uint32_t));
    auto take = [&](size_t b) {
        char *p = base;
        base += b;
        return p;
    };
    Queues q;
    q.ext[0] = (uint32_t *)take(u4);
    q.ext[1] = (uint32_t *)take(u4);
    q.shade_l = (uint32_t *)take(u4);
    q.shade_p = (uint32_t *)take(u4);
    q.shade_m = (uint32_t *)take(u4);
    q.conn = (uint32_t *)take(u4);
    q.nee = (uint32_t *)take(u4);
    q.ext_key = (uint32_t *)take(u4);
    q.walk = (uint32_t *)take(u4);
    q.regen[0] = (uint32_t *)take(u4);
    q.regen[1] = (uint32_t *)take(u4);
    q.counters = (uint32_t *)take(aligned256(C_COUNT * sizeof(uint32_t)));
    return q;
}

}  // namespace vvpt

namespace {

template <class T>
vvpt_status upload(vvpt_ctx *ctx, DevBuf &buf, const std::vector<T> &v, uint64_t &bytes)
{
    size_t n = v.size() * sizeof(T);
    VV_CUDA(buf.alloc(n), "cudaMalloc scene buffer");
    if (n)
        VV_CUDA(cudaMemcpyAsync(buf.ptr, v.data(), n, cudaMemcpyHostToDevice, vv_stream(ctx)), "upload scene buffer");
    bytes += buf.bytes;
    return VVPT_OK;
}

// Device block of a one-job table (single renders): the job, its one
// hand-out range and the table's counters in one struct, filled on the host
// and copied with one memcpy.
struct SingleJobBlock {
    JobView job;
    unsigned long long range_begin;
    unsigned long long next_item;
    unsigned long long total_items;
    uint32_t range_job;
    uint32_t num_ranges;
    uint32_t idle_count;
    uint32_t item_done;
};

JobTable single_job_table(SingleJobBlock *d, uint32_t *idle)
{
    JobTable jt;
    jt.jobs = &d->job;
    jt.range_begin = &d->range_begin;
    jt.range_job = &d->range_job;
    jt.item_done = &d->item_done;
    jt.next_item = &d->next_item;
    jt.total_items = &d->total_items;
    jt.num_ranges = &d->num_ranges;
    jt.idle = idle;
    jt.idle_count = &d->idle_count;
    return jt;
}

SingleJobBlock single_job_host(const SceneView &view, const RenderParams &hp, const BatchResults &br)
{
    SingleJobBlock h{};
    h.job.scene = view;
    h.job.params = hp;
    h.job.results = br;
    h.range_begin = 0;
    h.range_job = 0;
    h.total_items = hp.total_items;
    h.num_ranges = 1;
    return h;
}

}  // namespace

extern "C" {

VVPT_API const char *vvpt_version(void) { return "vvpt-gb300 0.1 (sm_103a)"; }

VVPT_API vvpt_status vvpt_create(int device, vvpt_ctx **out_ctx)
{
    if (!out_ctx)
        return VVPT_ERR_INVALID_ARG;
    *out_ctx = nullptr;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count <= device || device < 0) {
        cudaGetLastError();
        return VVPT_ERR_DEVICE;
    }
    vvpt_ctx *ctx = new vvpt_ctx();
    ctx->device = device;
    if (cudaSetDevice(device) != cudaSuccess) {
        delete ctx;
        return VVPT_ERR_DEVICE;
    }
    cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device);
    if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete ctx;
        return VVPT_ERR_DEVICE;
    }
    // counters plus room for per-job done counts read alongside them
    if (cudaMallocHost(&ctx->counters_pinned, (C_COUNT + 4096) * sizeof(uint32_t)) != cudaSuccess) {
        cudaStreamDestroy(ctx->stream);
        delete ctx;
        return VVPT_ERR_OOM;
    }
    *out_ctx = ctx;
    return VVPT_OK;
}

VVPT_API vvpt_status vvpt_destroy(vvpt_ctx *ctx)
{
    if (!ctx)
        return VVPT_ERR_INVALID_ARG;
    engine_shutdown(ctx);
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(vv_stream(ctx));
    if (ctx->counters_pinned)
        cudaFreeHost(ctx->counters_pinned);
    cudaStreamDestroy(ctx->stream);
    delete ctx;
    return VVPT_OK;
}

VVPT_API const char *vvpt_last_error(vvpt_ctx *ctx)
{
    if (!ctx)
        return "null context";
    return ctx->last_error.c_str();
}

VVPT_API vvpt_status vvpt_set_tuning(vvpt_ctx *ctx, const vvpt_tuning *t)
{
    if (!ctx || !t)
        return VVPT_ERR_INVALID_ARG;
    if (t->threads_per_block && (t->threads_per_block % 32 != 0 || t->threads_per_block > 256))
        return fail(ctx, VVPT_ERR_INVALID_ARG, "threads_per_block must be a multiple of 32, at most 256");
    if (t->blocks_per_sm > 64 || t->iterations_per_graph > 256)
        return fail(ctx, VVPT_ERR_INVALID_ARG, "blocks_per_sm at most 64, iterations_per_graph at most 256");
    std::lock_guard<std::mutex> lk(ctx->mu);
    ctx->tuning = *t;
    return VVPT_OK;
}

VVPT_API vvpt_status vvpt_set_bvh_builder(vvpt_ctx *ctx, int builder)
{
    if (!ctx || (builder != VVPT_BVH_BUILDER_AUTO && builder != VVPT_BVH_BUILDER_HOST &&
                 builder != VVPT_BVH_BUILDER_GPU))
        return VVPT_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> lk(ctx->mu);
    ctx->bvh_builder = builder;
    return VVPT_OK;
}

VVPT_API vvpt_status vvpt_get_tuning(vvpt_ctx *ctx, vvpt_tuning *t)
{
    if (!ctx || !t)
        return VVPT_ERR_INVALID_ARG;
    *t = ctx->tuning;
    return VVPT_OK;
}

VVPT_API vvpt_status vvpt_scene_upload(vvpt_ctx *ctx, const vvpt_scene_desc *desc, vvpt_scene **out_scene)
{
    if (!ctx || !desc || !out_scene)
        return fail(ctx, VVPT_ERR_INVALID_ARG, "null argument");
    *out_scene = nullptr;
    std::lock_guard<std::mutex> lk(ctx->mu);
    cudaSetDevice(ctx->device);

    PackedScene pk;
    std::string err;
    BlasBuilder gpu_builder;
    if (ctx->bvh_builder != VVPT_BVH_BUILDER_HOST) {
        cudaStream_t bs = vv_stream(ctx);
        gpu_builder = [bs](const std::vector<Box3> &boxes, const BVHBuildOptions &opt, BVHBuildResult &res,
                           std::string &e) { return build_bvh2_gpu(boxes, opt, bs, res, e); };
    }
    const bool all_gpu = ctx->bvh_builder == VVPT_BVH_BUILDER_GPU;
    vvpt_status st = pack_scene(desc, pk, err, 0, gpu_builder, all_gpu ? 1u : 65536u, all_gpu);
    if (st != VVPT_OK)
        return fail(ctx, st, err);
    auto scene = new vvpt_scene();
    std::unique_ptr<vvpt_scene> guard(scene);

    // ---- upload
    uint64_t bytes = 0;
    if ((st = upload(ctx, scene->nodes, pk.nodes, bytes)) != VVPT_OK)
        return st;
    if ((st = upload(ctx, scene->wnodes, pk.wnodes, bytes)) != VVPT_OK)
        return st;
    if ((st = upload(ctx, scene->tris, pk.tris, bytes)) != VVPT_OK)
        return st;
    if ((st = upload(ctx, scene->verts, pk.verts, bytes)) != VVPT_OK)
        return st;
    if ((st = upload(ctx, scene->indices, pk.indices, bytes)) != VVPT_OK)
        return st;
    if ((st = upload(ctx, scene->instances, pk.instances, bytes)) != VVPT_OK)
        return st;
    if ((st = upload(ctx, scene->tlas_order, pk.tlas_order, bytes)) != VVPT_OK)
        return st;
    if ((st = upload(ctx, scene->materials, pk.materials, bytes)) != VVPT_OK)
        return st;
    if ((st = upload(ctx, scene->lights, pk.lights, bytes)) != VVPT_OK)
        return st;
    if ((st = upload(ctx, scene->textures, pk.textures, bytes)) != VVPT_OK)
        return st;
    if ((st = upload(ctx, scene->texels, pk.texels, bytes)) != VVPT_OK)
        return st;
    if ((st = upload(ctx, scene->env_dist, pk.env_dist, bytes)) != VVPT_OK)
        return st;
    if ((st = upload(ctx, scene->emit_boxes, pk.emit_boxes, bytes)) != VVPT_OK)
        return st;
    VV_CUDA(cudaStreamSynchronize(vv_stream(ctx)), "scene upload");

    SceneView &v = scene->view;
    v.nodes = scene->nodes.as<BVHNode>();
    v.wnodes = scene->wnodes.as<WideNode>();
    v.tris = scene->tris.as<TriVerts>();
    v.verts = scene->verts.as<ShadeVertex>();
    v.indices = scene->indices.as<uint32_t>();
    v.instances = scene->instances.as<DevInstance>();
    v.tlas_order = scene->tlas_order.as<uint32_t>();
    v.tlas_root = pk.tlas_root;
    v.tlas_count = (uint32_t)(pk.nodes.size() - pk.tlas_root);
    v.num_instances = desc->num_instances;
    v.materials = scene->materials.as<DevMaterial>();
    v.num_materials = desc->num_materials;
    v.lights = scene->lights.as<DevLightInstance>();
    v.num_lights = desc->num_lights;
    v.textures = scene->textures.as<DevTexture>();
    v.num_textures = (uint32_t)pk.textures.size();
    v.texels = scene->texels.as<uint8_t>();
    v.env_texture = pk.env_texture;
    v.has_transparent = pk.has_transparent ? 1u : 0u;
    v.cull_o = pk.cull_o;
    v.cull_r = pk.cull_r;
    v.env_w = pk.env_w;
    v.env_h = pk.env_h;
    v.env_func_int = pk.env_func_int;
    v.env_func = scene->env_dist.as<float>();
    v.env_cond_cdf = v.env_func + (size_t)pk.env_w * pk.env_h;
    v.env_marg_cdf = v.env_cond_cdf + (size_t)(pk.env_w + 1) * pk.env_h;
    v.emit_boxes = scene->emit_boxes.as<float4>();
    v.num_emit_boxes = (uint32_t)(pk.emit_boxes.size() / 2);
    scene->bytes = bytes;
    scene->num_materials = desc->num_materials;
    *out_scene = guard.release();
    return VVPT_OK;
}

VVPT_API vvpt_status vvpt_scene_release(vvpt_ctx *ctx, vvpt_scene *scene)
{
    if (!ctx || !scene)
        return VVPT_ERR_INVALID_ARG;
    if (scene->jobs_in_flight.load() != 0)
        return fail(ctx, VVPT_ERR_NOT_READY, "scene still used by submitted jobs");
    std::lock_guard<std::mutex> lk(ctx->mu);
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(vv_stream(ctx));
    delete scene;
    return VVPT_OK;
}

VVPT_API vvpt_status vvpt_scene_device_bytes(vvpt_ctx *ctx, const vvpt_scene *scene, uint64_t *out_bytes)
{
    if (!ctx || !scene || !out_bytes)
        return VVPT_ERR_INVALID_ARG;
    *out_bytes = scene->bytes;
    return VVPT_OK;
}

VVPT_API vvpt_status vvpt_progress(vvpt_ctx *ctx, float *out)
{
    if (!ctx || !out)
        return VVPT_ERR_INVALID_ARG;
    *out = ctx->progress.load();
    return VVPT_OK;
}

VVPT_API vvpt_status vvpt_last_render_stats(vvpt_ctx *ctx, vvpt_render_stats *out)
{
    if (!ctx || !out)
        return VVPT_ERR_INVALID_ARG;
    *out = ctx->stats;
    return VVPT_OK;
}

VVPT_API vvpt_status vvpt_last_kernel_profile(vvpt_ctx *ctx, vvpt_kernel_profile *out)
{
    if (!ctx || !out)
        return VVPT_ERR_INVALID_ARG;
    *out = ctx->profile;
    return VVPT_OK;
}

VVPT_API vvpt_status vvpt_set_stream(vvpt_ctx *ctx, void *cuda_stream)
{
    if (!ctx)
        return VVPT_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> lk(ctx->mu);
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(vv_stream(ctx));
    ctx->user_stream = reinterpret_cast<cudaStream_t>(cuda_stream);
    return VVPT_OK;
}

VVPT_API vvpt_status vvpt_render(vvpt_ctx *ctx, vvpt_scene *scene, const vvpt_scene_data *sd,
                                 const vvpt_render_info *info, vvpt_outputs *out)
{
    if (!ctx || !scene || !sd || !info || !out)
        return fail(ctx, VVPT_ERR_INVALID_ARG, "null argument");
    RenderParams hp;
    vvpt_status pst0 = make_render_params(ctx, scene, sd, info, hp);
    if (pst0 != VVPT_OK)
        return pst0;
    std::lock_guard<std::mutex> lk(ctx->mu);
    cudaSetDevice(ctx->device);
    ctx->progress.store(0.0f);
    const uint32_t npix = hp.width * hp.height;
    const uint32_t batches = hp.batches;

    vvpt_render_stats stats{};
    // ---- output buffers
    const size_t img_bytes = (size_t)npix * sizeof(float4);
    float4 *d_out[4] = {nullptr, nullptr, nullptr, nullptr};
    float *host_out[4] = {out->radiance, out->albedo, out->normal, out->radiance_m2};
    if (out->on_device) {
        for (int k = 0; k < 4; k++)
            d_out[k] = reinterpret_cast<float4 *>(host_out[k]);
    } else {
        VV_CUDA(ctx->outputs.reserve(4 * img_bytes), "cudaMalloc outputs");
        for (int k = 0; k < 4; k++)
            d_out[k] = host_out[k] ? ctx->outputs.as<float4>() + (size_t)k * npix : nullptr;
    }

    if (batches == 0 || hp.depth == 0 || hp.total_items == 0) {
        // nothing traced: the reference's images stay zero (alpha untouched)
        for (int k = 0; k < 4; k++)
            if (d_out[k])
                VV_CUDA(cudaMemsetAsync(d_out[k], 0, img_bytes, vv_stream(ctx)), "clear outputs");
    } else {
        // ---- path state and queues
        uint32_t slots = ctx->tuning.slots ? ctx->tuning.slots : (1u << 20);
        slots = std::max<uint32_t>(32u, std::min<uint32_t>(slots, hp.total_items));
        const size_t n = slots;
        const size_t u4 = n * sizeof(uint32_t);
        auto aligned = [](size_t b) { return aligned256(b); };
        char *base = nullptr;
        auto take = [&](size_t b) {
            char *p = base;
            base += aligned(b);
            return p;
        };
        VV_CUDA(ctx->state.reserve(path_state_bytes(n)), "cudaMalloc path state");
        const PathState ps = carve_path_state(ctx->state.as<char>(), n);
        VV_CUDA(ctx->queues.reserve(queue_bytes(n)), "cudaMalloc queues");
        const Queues q = carve_queues(ctx->queues.as<char>(), n);

        const size_t rb = (size_t)hp.total_items * sizeof(float4);
        size_t rneed = 3 * aligned(rb);
        VV_CUDA(ctx->results.reserve(rneed), "cudaMalloc batch results");
        base = ctx->results.as<char>();
        BatchResults br;
        br.rad = (float4 *)take(rb);
        br.alb = (float4 *)take(rb);
        br.nrm = (float4 *)take(rb);

        VV_CUDA(ctx->params.reserve(aligned(sizeof(SingleJobBlock)) + u4), "cudaMalloc job table");
        base = ctx->params.as<char>();
        SingleJobBlock *djob = (SingleJobBlock *)take(sizeof(SingleJobBlock));
        const JobTable jt = single_job_table(djob, (uint32_t *)take(u4));
        const SingleJobBlock hjob = single_job_host(scene->view, hp, br);
        VV_CUDA(cudaMemcpyAsync(djob, &hjob, sizeof(hjob), cudaMemcpyHostToDevice, vv_stream(ctx)), "upload job");
        uint32_t *d_item_done = &djob->item_done;

        LaunchShape shape;
        shape.block = ctx->tuning.threads_per_block ? (int)ctx->tuning.threads_per_block : 256;
        int bps = ctx->tuning.blocks_per_sm ? (int)ctx->tuning.blocks_per_sm : 4;
        shape.grid = std::max(1, ctx->num_sms * bps);
        const int K = ctx->tuning.iterations_per_graph ? (int)ctx->tuning.iterations_per_graph : 8;

        cudaEvent_t tev[2];
        cudaEventCreate(&tev[0]);
        cudaEventCreate(&tev[1]);
        struct EventGuard {
            cudaEvent_t *e;
            ~EventGuard()
            {
                cudaEventDestroy(e[0]);
                cudaEventDestroy(e[1]);
            }
        } tev_guard{tev};
        VV_CUDA(cudaEventRecord(tev[0], vv_stream(ctx)), "event");
        launch_init_slots(q, ps, jt, slots, vv_stream(ctx));
        stats.kernel_launches += 1;
        VV_CUDA(cudaGetLastError(), "launch init");
        const uint64_t max_iters =
            (uint64_t)hp.batch_size * (hp.depth + 1) * ((hp.total_items + slots - 1) / slots + 1) + 64;

        if (info->flags & VVPT_RENDER_PROFILE_KERNELS) {
            // one kernel at a time with events around each launch
            static const char *names[K_NUM] = {"k_begin", "k_regen",  "k_extend", "k_partition",
                                               "k_walk",  "k_shade", "k_shadow"};
            static const double bpu[K_NUM] = {0.0,        kBytesRegen, kBytesExtend, kBytesPartition,
                                              kBytesWalk, kBytesShade, kBytesShadow};
            vvpt_kernel_profile prof{};
            prof.count = K_NUM;
            for (int k = 0; k < K_NUM; k++) {
                std::snprintf(prof.kernels[k].name, sizeof(prof.kernels[k].name), "%s", names[k]);
                prof.kernels[k].bytes_per_unit = bpu[k];
            }
            cudaEvent_t ka, kb;
            cudaEventCreate(&ka);
            cudaEventCreate(&kb);
            uint64_t it = 0;
            vvpt_status pst = VVPT_OK;
            for (;; it++) {
                const int pp = (int)(it & 1);
                for (int k = 0; k < K_NUM; k++) {
                    VV_CUDA(cudaMemcpyAsync(ctx->counters_pinned, q.counters, C_COUNT * sizeof(uint32_t),
                                            cudaMemcpyDeviceToHost, vv_stream(ctx)),
                            "read counters");
                    VV_CUDA(cudaStreamSynchronize(vv_stream(ctx)), "profile sync");
                    const uint32_t *c = ctx->counters_pinned;
                    uint64_t units = k == K_REGEN    ? c[C_REGEN0 + pp]
                                     : (k == K_EXTEND || k == K_PARTITION) ? c[C_EXT0 + pp]
                                     : k == K_WALK   ? c[C_WALK]
                                     : k == K_SHADE  ? (uint64_t)c[C_SHADE_L] + c[C_SHADE_P] + c[C_SHADE_M]
                                     : k == K_SHADOW ? (uint64_t)c[C_CONN] + c[C_NEEQ]
                                                      : 1;
                    cudaEventRecord(ka, vv_stream(ctx));
                    launch_kernel((KernelId)k, jt, ps, q, pp, shape, vv_stream(ctx));
                    cudaEventRecord(kb, vv_stream(ctx));
                    VV_CUDA(cudaEventSynchronize(kb), "profile kernel");
                    float ms = 0.0f;
                    cudaEventElapsedTime(&ms, ka, kb);
                    prof.kernels[k].launches += (uint64_t)launches_of(k);
                    prof.kernels[k].units += launches_of(k) ? units : 0;
                    prof.kernels[k].total_ms += ms;
                    stats.kernel_launches += launches_of(k);
                }
                VV_CUDA(cudaMemcpy(ctx->counters_pinned, q.counters, C_COUNT * sizeof(uint32_t), cudaMemcpyDeviceToHost),
                        "read counters");
                VV_CUDA(cudaMemcpy(ctx->counters_pinned + C_COUNT, d_item_done, sizeof(uint32_t),
                                   cudaMemcpyDeviceToHost),
                        "read done count");
                const uint32_t *c = ctx->counters_pinned;
                if (c[C_ERR]) {
                    pst = fail(ctx, VVPT_ERR_DEVICE, "device status word set: " + std::to_string(c[C_ERR]));
                    break;
                }
                if (c[C_COUNT] >= hp.total_items)
                    break;
                if (it > max_iters) {
                    pst = fail(ctx, VVPT_ERR_TIMEOUT, "wavefront did not drain within the iteration bound");
                    break;
                }
            }
            cudaEventDestroy(ka);
            cudaEventDestroy(kb);
            if (pst != VVPT_OK)
                return pst;
            ctx->profile = prof;
            stats.iterations = it + 1;
        } else {
        // capture K iterations (K even keeps the ping-pong phase aligned)
        const int Ke = (K + 1) & ~1;
        cudaGraph_t graph;
        cudaGraphExec_t exec;
        VV_CUDA(cudaStreamBeginCapture(vv_stream(ctx), cudaStreamCaptureModeThreadLocal), "begin capture");
        for (int it = 0; it < Ke; it++)
            launch_iteration(jt, ps, q, it & 1, shape, vv_stream(ctx));
        cudaError_t ce = cudaStreamEndCapture(vv_stream(ctx), &graph);
        if (ce != cudaSuccess)
            return cuda_fail(ctx, ce, "end capture");
        ce = cudaGraphInstantiate(&exec, graph, 0);
        cudaGraphDestroy(graph);
        if (ce != cudaSuccess)
            return cuda_fail(ctx, ce, "graph instantiate");

        cudaEvent_t ev[2];
        cudaEventCreateWithFlags(&ev[0], cudaEventDisableTiming);
        cudaEventCreateWithFlags(&ev[1], cudaEventDisableTiming);
        // Bound on iterations (max_iters): every slot-iteration advances a
        // path by one segment, so the total is at most samples * depth
        // segments per work item times the work items per slot.
        uint64_t iters = 0;
        int launched = 0;
        bool done = false;
        vvpt_status loop_status = VVPT_OK;
        // keep one graph in flight ahead of the counter check
        VV_CUDA(cudaGraphLaunch(exec, vv_stream(ctx)), "graph launch");
        VV_CUDA(cudaEventRecord(ev[0], vv_stream(ctx)), "event");
        launched = 1;
        iters += Ke;
        while (!done) {
            VV_CUDA(cudaMemcpyAsync(ctx->counters_pinned, q.counters, C_COUNT * sizeof(uint32_t),
                                    cudaMemcpyDeviceToHost, vv_stream(ctx)),
                    "read counters");
            VV_CUDA(cudaMemcpyAsync(ctx->counters_pinned + C_COUNT, d_item_done, sizeof(uint32_t),
                                    cudaMemcpyDeviceToHost, vv_stream(ctx)),
                    "read done count");
            VV_CUDA(cudaEventRecord(ev[launched & 1], vv_stream(ctx)), "event");
            int check = launched & 1;
            VV_CUDA(cudaGraphLaunch(exec, vv_stream(ctx)), "graph launch");
            launched++;
            iters += Ke;
            VV_CUDA(cudaEventSynchronize(ev[check]), "wait counters");
            const uint32_t *c = ctx->counters_pinned;
            ctx->progress.store((float)std::min<uint32_t>(c[C_COUNT], hp.total_items) / (float)hp.total_items);
            if (c[C_ERR]) {
                loop_status = fail(ctx, VVPT_ERR_DEVICE,
                                   "device status word set (traversal stack overflow or loop cap): " +
                                       std::to_string(c[C_ERR]));
                break;
            }
            if (c[C_COUNT] >= hp.total_items)
                done = true;
            else if (iters > max_iters + 4 * (uint64_t)Ke) {
                loop_status = fail(ctx, VVPT_ERR_TIMEOUT, "wavefront did not drain within the iteration bound");
                break;
            }
        }
        VV_CUDA(cudaStreamSynchronize(vv_stream(ctx)), "render");
        cudaGraphExecDestroy(exec);
        cudaEventDestroy(ev[0]);
        cudaEventDestroy(ev[1]);
        if (loop_status != VVPT_OK)
            return loop_status;
        stats.iterations = iters;
        stats.kernel_launches += (uint64_t)iters * kKernelsPerIteration;
        }
        VV_CUDA(cudaMemcpy(ctx->counters_pinned, q.counters, C_COUNT * sizeof(uint32_t), cudaMemcpyDeviceToHost),
                "final counters");
        stats.segments = ctx->counters_pinned[C_SEGMENTS];
        stats.shadow_rays = ctx->counters_pinned[C_SHADOW];
        stats.emitter_rays = ctx->counters_pinned[C_NEE];
        stats.paths = ctx->counters_pinned[C_PATHS];
        if (ctx->counters_pinned[C_ERR])
            return fail(ctx, VVPT_ERR_DEVICE, "device status word set: " + std::to_string(ctx->counters_pinned[C_ERR]));

        launch_reduce(hp, br, d_out[0], d_out[1], d_out[2], d_out[3], vv_stream(ctx));
        stats.kernel_launches += 1;
        VV_CUDA(cudaGetLastError(), "launch reduce");
        VV_CUDA(cudaEventRecord(tev[1], vv_stream(ctx)), "event");
        VV_CUDA(cudaEventSynchronize(tev[1]), "render");
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, tev[0], tev[1]);
        stats.device_ms = ms;
    }

    if (!out->on_device) {
        for (int k = 0; k < 4; k++)
            if (host_out[k])
                VV_CUDA(cudaMemcpyAsync(host_out[k], d_out[k], img_bytes, cudaMemcpyDeviceToHost, vv_stream(ctx)),
                        "download outputs");
    }
    VV_CUDA(cudaStreamSynchronize(vv_stream(ctx)), "render finish");
    ctx->stats = stats;
    ctx->progress.store(1.0f);
    return VVPT_OK;
}

VVPT_API vvpt_status vvpt_autotune(vvpt_ctx *ctx, vvpt_scene *scene, const vvpt_scene_data *sd,
                                   const vvpt_render_info *info, double budget_ms, vvpt_tuning *out)
{
    if (!ctx || !scene || !sd || !info)
        return fail(ctx, VVPT_ERR_INVALID_ARG, "null argument");
    RenderParams hp;
    vvpt_status st = make_render_params(ctx, scene, sd, info, hp);
    if (st != VVPT_OK)
        return st;
    if (hp.total_items == 0 || hp.depth == 0)
        return fail(ctx, VVPT_ERR_INVALID_ARG, "autotune needs a request that traces paths");
    const size_t img = (size_t)hp.width * hp.height * sizeof(float4);
    DevBuf outb;
    {
        std::lock_guard<std::mutex> lk(ctx->mu);
        cudaSetDevice(ctx->device);
        VV_CUDA(outb.alloc(3 * img), "cudaMalloc autotune outputs");
    }
    vvpt_outputs o{};
    o.radiance = outb.as<float>();
    o.albedo = o.radiance + img / sizeof(float);
    o.normal = o.albedo + img / sizeof(float);
    o.on_device = 1;
    // probe: the request's image size and depth, few batches
    vvpt_render_info probe = *info;
    probe.flags &= ~(uint32_t)VVPT_RENDER_PROFILE_KERNELS;
    probe.samples = info->batch_size;
    const vvpt_tuning start = ctx->tuning;
    auto trial = [&](const vvpt_tuning &t, double &paths_per_ms) -> vvpt_status {
        {
            std::lock_guard<std::mutex> lk(ctx->mu);
            ctx->tuning = t;
        }
        vvpt_status r = vvpt_render(ctx, scene, sd, &probe, &o);
        if (r != VVPT_OK)
            return r;
        paths_per_ms = (double)ctx->stats.paths / std::max(ctx->stats.device_ms, 1e-3);
        return VVPT_OK;
    };
    // size the probe so that one trial takes about budget / 12
    double ppm = 0.0;
    vvpt_tuning best = start;
    if ((st = trial(best, ppm)) != VVPT_OK)
        return st;
    const double per_trial_ms = std::max(budget_ms, 100.0) / 12.0;
    const double want_paths = ppm * per_trial_ms;
    const double batch_paths = (double)hp.width * hp.height * info->batch_size;
    const uint32_t batches = (uint32_t)std::min<double>(std::max(1.0, want_paths / batch_paths), hp.batches);
    probe.samples = info->batch_size * batches;
    if ((st = trial(best, ppm)) != VVPT_OK) // warm-up at the probe size
        return st;
    double best_ppm = 0.0;
    if ((st = trial(best, best_ppm)) != VVPT_OK)
        return st;
    // coordinate descent: blocks per SM, slots, iterations per graph
    auto sweep = [&](auto apply, std::initializer_list<uint32_t> values) -> vvpt_status {
        vvpt_tuning base = best;
        for (uint32_t v : values) {
            vvpt_tuning t = base;
            apply(t, v);
            double p = 0.0;
            vvpt_status r = trial(t, p);
            if (r == VVPT_ERR_OOM)
                continue; // candidate too large for this device: skip it
            if (r != VVPT_OK)
                return r;
            if (p > best_ppm * 1.01) {
                best_ppm = p;
                best = t;
            }
        }
        return VVPT_OK;
    };
    if ((st = sweep([](vvpt_tuning &t, uint32_t v) { t.blocks_per_sm = v; }, {2u, 3u, 4u, 6u, 8u})) != VVPT_OK)
        return st;
    if ((st = sweep([](vvpt_tuning &t, uint32_t v) { t.slots = v; }, {1u << 19, 1u << 20, 3u << 19, 1u << 21})) !=
        VVPT_OK)
        return st;
    if ((st = sweep([](vvpt_tuning &t, uint32_t v) { t.iterations_per_graph = v; }, {4u, 8u, 16u})) != VVPT_OK)
        return st;
    {
        std::lock_guard<std::mutex> lk(ctx->mu);
        ctx->tuning = best;
        outb.release();
    }
    if (out)
        *out = best;
    return VVPT_OK;
}

VVPT_API vvpt_status vvpt_trace_closest(vvpt_ctx *ctx, vvpt_scene *scene, const vvpt_ray *rays, uint32_t n,
                                        vvpt_hit *hits, int32_t on_device)
{
    if (!ctx || !scene || (n && (!rays || !hits)))
        return fail(ctx, VVPT_ERR_INVALID_ARG, "null argument");
    if (n == 0)
        return VVPT_OK;
    std::lock_guard<std::mutex> lk(ctx->mu);
    cudaSetDevice(ctx->device);
    static_assert(sizeof(vvpt_ray) == 32, "ray layout");
    const float4 *d_rays;
    if (on_device) {
        d_rays = reinterpret_cast<const float4 *>(rays);
    } else {
        VV_CUDA(ctx->rays.reserve((size_t)n * 32), "cudaMalloc rays");
        VV_CUDA(cudaMemcpyAsync(ctx->rays.ptr, rays, (size_t)n * 32, cudaMemcpyHostToDevice, vv_stream(ctx)), "upload rays");
        d_rays = ctx->rays.as<float4>();
    }
    VV_CUDA(ctx->hits_tuv.reserve((size_t)n * 16), "cudaMalloc hits");
    VV_CUDA(ctx->hits_ids.reserve((size_t)n * 8), "cudaMalloc hits");
    VV_CUDA(ctx->err_word.reserve(16), "cudaMalloc err");
    VV_CUDA(cudaMemsetAsync(ctx->err_word.ptr, 0, 4, vv_stream(ctx)), "clear err");
    launch_trace_closest(scene->view, d_rays, n, ctx->hits_tuv.as<float4>(), ctx->hits_ids.as<uint32_t>(),
                         ctx->err_word.as<uint32_t>(), vv_stream(ctx));
    VV_CUDA(cudaGetLastError(), "launch trace");
    std::vector<float4> tuv(n);
    std::vector<uint32_t> ids(2 * (size_t)n);
    uint32_t err = 0;
    VV_CUDA(cudaMemcpyAsync(tuv.data(), ctx->hits_tuv.ptr, (size_t)n * 16, cudaMemcpyDeviceToHost, vv_stream(ctx)), "d2h");
    VV_CUDA(cudaMemcpyAsync(ids.data(), ctx->hits_ids.ptr, (size_t)n * 8, cudaMemcpyDeviceToHost, vv_stream(ctx)), "d2h");
    VV_CUDA(cudaMemcpyAsync(&err, ctx->err_word.ptr, 4, cudaMemcpyDeviceToHost, vv_stream(ctx)), "d2h");
    VV_CUDA(cudaStreamSynchronize(vv_stream(ctx)), "trace");
    std::vector<vvpt_hit> hv(n);
    for (uint32_t i = 0; i < n; i++) {
        hv[i].t = tuv[i].x;
        hv[i].u = tuv[i].y;
        hv[i].v = tuv[i].z;
        hv[i].instance = ids[2 * i];
        hv[i].primitive = ids[2 * i + 1];
    }
    if (on_device)
        VV_CUDA(cudaMemcpy(hits, hv.data(), (size_t)n * sizeof(vvpt_hit), cudaMemcpyHostToDevice), "store hits");
    else
        std::memcpy(hits, hv.data(), (size_t)n * sizeof(vvpt_hit));
    if (err)
        return fail(ctx, VVPT_ERR_DEVICE, "traversal status word set: " + std::to_string(err));
    return VVPT_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Render without device allocations.
//
// Some callers cannot let a library call cudaMalloc: an engine that owns a
// fixed device-memory pool and forbids allocations behind its back, a process
// under a hard memory cap, or code that must not hit the allocator's implicit
// device synchronisation in the middle of a frame. vvpt_render_noalloc renders
// with every piece of its scratch (render parameters, counters, ray queues,
// path state and per-batch sums) carved out of one fixed device array that the
// library defines at file scope. The array is part of the module, so every GPU
// that loads this library holds it until the process exits.

namespace {

constexpr size_t kNoAllocScratchBytes = 64ull << 20; // 64 MiB
constexpr uint32_t kNoAllocMaxSlots = 65536;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

// The array's address on each device, looked up once per device with that
// device current. On the host, `g_noalloc_scratch` is only a stand-in symbol,
// never a device address: kernels receive the looked-up pointer.
std::mutex g_noalloc_mu;
unsigned char *g_noalloc_ptr[64] = {};

vvpt_status noalloc_scratch(vvpt_ctx *ctx, unsigned char **out)
{
    if (ctx->device < 0 || ctx->device >= 64)
        return fail(ctx, VVPT_ERR_UNSUPPORTED, "device index beyond 63");
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_ptr[ctx->device]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p)
            return cuda_fail(ctx, e == cudaSuccess ? cudaErrorInvalidSymbol : e, "cudaGetSymbolAddress(scratch)");
        g_noalloc_ptr[ctx->device] = static_cast<unsigned char *>(p);
    }
    *out = g_noalloc_ptr[ctx->device];
    return VVPT_OK;
}

}  // namespace

extern "C" {

VVPT_API vvpt_status vvpt_render_noalloc(vvpt_ctx *ctx, vvpt_scene *scene, const vvpt_scene_data *sd,
                                         const vvpt_render_info *info, vvpt_outputs *out)
{
    if (!ctx || !scene || !sd || !info || !out)
        return fail(ctx, VVPT_ERR_INVALID_ARG, "null argument");
    if (!out->on_device)
        return fail(ctx, VVPT_ERR_INVALID_ARG, "vvpt_render_noalloc writes device buffers only (outputs.on_device = 1)");
    if (info->flags & VVPT_RENDER_SAMPLER_PMJ)
        return fail(ctx, VVPT_ERR_UNSUPPORTED, "vvpt_render_noalloc renders with the RTGEMS sampler only");
    // The same parameters as vvpt_render, from the same function: it checks
    // the sizes (width * height <= 2^28, width * height * batches < 2^32) and
    // the camera volume, and sets every field, environment importance
    // sampling included. With the RTGEMS sampler it allocates nothing.
    RenderParams hp;
    vvpt_status pst = make_render_params(ctx, scene, sd, info, hp);
    if (pst != VVPT_OK)
        return pst;
    hp.want_m2 = out->radiance_m2 ? 1u : 0u;
    // every product below is of checked sizes: items < 2^32, so the largest
    // term, 3 * 16 * items, stays below 2^38
    const uint64_t npix64 = (uint64_t)hp.width * hp.height;
    const uint32_t batches = hp.batches;
    const uint64_t items64 = hp.total_items;
    const uint64_t slots64 = std::max<uint64_t>(32, std::min<uint64_t>(items64, kNoAllocMaxSlots));
    auto aligned = [](uint64_t b) { return (b + 255) & ~uint64_t(255); };
    const uint64_t f4 = slots64 * sizeof(float4), u4 = slots64 * sizeof(uint32_t);
    const uint64_t need = aligned(sizeof(SingleJobBlock)) + aligned(C_COUNT * sizeof(uint32_t)) + 14 * aligned(f4) +
                          7 * aligned(u4) + aligned(u4) /* idle slots */ + 11 * aligned(u4) +
                          3 * aligned(items64 * sizeof(float4));
    if (need > kNoAllocScratchBytes)
        return fail(ctx, VVPT_ERR_INVALID_ARG,
                    "render needs " + std::to_string(need) + " bytes of scratch; vvpt_render_noalloc has " +
                        std::to_string(kNoAllocScratchBytes) + " (width * height * samples / batch_size too large)");

    std::lock_guard<std::mutex> lk(ctx->mu);
    cudaSetDevice(ctx->device);
    ctx->progress.store(0.0f);
    unsigned char *scratch = nullptr;
    vvpt_status st = noalloc_scratch(ctx, &scratch);
    if (st != VVPT_OK)
        return st;
    cudaStream_t stream = vv_stream(ctx);

    float4 *d_out[4] = {reinterpret_cast<float4 *>(out->radiance), reinterpret_cast<float4 *>(out->albedo),
                        reinterpret_cast<float4 *>(out->normal), reinterpret_cast<float4 *>(out->radiance_m2)};
    if (batches == 0 || hp.depth == 0) {
        for (int k = 0; k < 4; k++)
            if (d_out[k])
                VV_CUDA(cudaMemsetAsync(d_out[k], 0, npix64 * sizeof(float4), stream), "clear outputs");
        VV_CUDA(cudaStreamSynchronize(stream), "render");
        ctx->progress.store(1.0f);
        return VVPT_OK;
    }

    // carve the scratch array; everything below is rewritten by this call
    // before it is read (the counters and slot queue by k_init_slots, path
    // state by k_regen, every per-batch sum once per work item)
    unsigned char *base = scratch;
    auto take = [&](uint64_t b) {
        unsigned char *p = base;
        base += aligned(b);
        return p;
    };
    SingleJobBlock *djob = reinterpret_cast<SingleJobBlock *>(take(sizeof(SingleJobBlock)));
    Queues q;
    q.counters = reinterpret_cast<uint32_t *>(take(C_COUNT * sizeof(uint32_t)));
    PathState ps;
    float4 **f4s[14] = {&ps.o, &ps.d, &ps.beta, &ps.rad, &ps.alb, &ps.nrm, &ps.cum_rad,
                        &ps.cum_alb, &ps.cum_nrm, &ps.hit, &ps.sh_dir, &ps.sh_c, &ps.nee_b, &ps.nee_c};
    for (float4 **p : f4s) {
        float4 *m = reinterpret_cast<float4 *>(take(f4));
        if (p)
            *p = m;
    }
    uint32_t **u4s[7] = {&ps.hit_inst, &ps.rng, &ps.flags, &ps.vol, &ps.item, &ps.sample, &ps.job};
    for (uint32_t **p : u4s)
        *p = reinterpret_cast<uint32_t *>(take(u4));
    const JobTable jt = single_job_table(djob, reinterpret_cast<uint32_t *>(take(u4)));
    uint32_t **qs[11] = {&q.ext[0], &q.ext[1],  &q.shade_l, &q.shade_p,  &q.shade_m, &q.conn,
                         &q.nee,    &q.ext_key, &q.walk,    &q.regen[0], &q.regen[1]};
    for (uint32_t **p : qs)
        *p = reinterpret_cast<uint32_t *>(take(u4));
    BatchResults br;
    br.rad = reinterpret_cast<float4 *>(take(items64 * sizeof(float4)));
    br.alb = reinterpret_cast<float4 *>(take(items64 * sizeof(float4)));
    br.nrm = reinterpret_cast<float4 *>(take(items64 * sizeof(float4)));

    const SingleJobBlock hjob = single_job_host(scene->view, hp, br);
    VV_CUDA(cudaMemcpyAsync(djob, &hjob, sizeof(hjob), cudaMemcpyHostToDevice, stream), "upload job");
    LaunchShape shape;
    shape.block = 256;
    shape.grid = std::max(1, ctx->num_sms * 4);
    const uint32_t slots = (uint32_t)slots64;
    launch_init_slots(q, ps, jt, slots, stream);
    VV_CUDA(cudaGetLastError(), "launch init");
    const uint64_t max_iters =
        (uint64_t)hp.batch_size * (hp.depth + 1) * ((hp.total_items + slots - 1) / slots + 1) + 64;
    // kernels are launched one by one (no graph objects); the pinned counter
    // buffer was allocated when the context was created
    vvpt_render_stats stats{};
    stats.kernel_launches = 1;
    uint64_t it = 0;
    for (;;) {
        for (int k = 0; k < 8; k++) {
            for (int kk = 0; kk < K_NUM; kk++)
                launch_kernel((KernelId)kk, jt, ps, q, (int)(it & 1), shape, stream);
            it++;
        }
        stats.kernel_launches += 8 * kKernelsPerIteration;
        VV_CUDA(cudaGetLastError(), "launch iteration");
        VV_CUDA(cudaMemcpyAsync(ctx->counters_pinned, q.counters, C_COUNT * sizeof(uint32_t), cudaMemcpyDeviceToHost,
                                stream),
                "read counters");
        VV_CUDA(cudaMemcpyAsync(ctx->counters_pinned + C_COUNT, &djob->item_done, sizeof(uint32_t),
                                cudaMemcpyDeviceToHost, stream),
                "read done count");
        VV_CUDA(cudaStreamSynchronize(stream), "render");
        const uint32_t *c = ctx->counters_pinned;
        if (c[C_ERR])
            return fail(ctx, VVPT_ERR_DEVICE, "device status word set: " + std::to_string(c[C_ERR]));
        ctx->progress.store((float)std::min<uint32_t>(c[C_COUNT], hp.total_items) / (float)hp.total_items);
        if (c[C_COUNT] >= hp.total_items)
            break;
        if (it > max_iters + 16)
            return fail(ctx, VVPT_ERR_TIMEOUT, "wavefront did not drain within the iteration bound");
    }
    stats.iterations = it;
    stats.segments = ctx->counters_pinned[C_SEGMENTS];
    stats.shadow_rays = ctx->counters_pinned[C_SHADOW];
    stats.emitter_rays = ctx->counters_pinned[C_NEE];
    stats.paths = ctx->counters_pinned[C_PATHS];
    launch_reduce(hp, br, d_out[0], d_out[1], d_out[2], d_out[3], stream);
    stats.kernel_launches += 1;
    VV_CUDA(cudaGetLastError(), "launch reduce");
    VV_CUDA(cudaStreamSynchronize(stream), "render finish");
    ctx->stats = stats;
    ctx->progress.store(1.0f);
    return VVPT_OK;
}

}  // extern "C"

VVPT_API vvpt_status vvpt_sampler_tables(float *pmj, float *blue_noise)
{
    const SamplerTables &t = sampler_tables();
    if (pmj)
        std::memcpy(pmj, t.pmj.data(), t.pmj.size() * sizeof(float));
    if (blue_noise)
        std::memcpy(blue_noise, t.blue_noise.data(), t.blue_noise.size() * sizeof(float));
    return VVPT_OK;
}
