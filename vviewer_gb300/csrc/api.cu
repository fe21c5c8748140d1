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
#include "bvh_build.h"
#include "scene_gpu.h"
#include "wavefront.cuh"

using namespace vvpt;

namespace {

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

struct StatusError {
    vvpt_status code;
    std::string msg;
};

}  // namespace

struct vvpt_scene {
    DevBuf nodes, tris, verts, indices, instances, tlas_order, materials, lights, textures, texels;
    SceneView view{};
    uint64_t bytes = 0;
    uint32_t num_materials = 0;
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
    DevBuf state, queues, results, params, outputs;
    uint32_t *counters_pinned = nullptr;
    DevBuf rays, hits_tuv, hits_ids, err_word;
    cudaStream_t user_stream = nullptr;
    vvpt_kernel_profile profile{};
};

namespace {

inline cudaStream_t vv_stream(const vvpt_ctx *ctx) { return ctx->user_stream ? ctx->user_stream : ctx->stream; }

vvpt_status fail(vvpt_ctx *ctx, vvpt_status code, const std::string &msg)
{
    if (ctx)
        ctx->last_error = msg;
    return code;
}

vvpt_status cuda_fail(vvpt_ctx *ctx, cudaError_t e, const char *what)
{
    cudaGetLastError();
    std::string m = std::string(what) + ": " + cudaGetErrorString(e);
    return fail(ctx, e == cudaErrorMemoryAllocation ? VVPT_ERR_OOM : VVPT_ERR_DEVICE, m);
}

#define VV_CUDA(call, what)                       \
    do {                                          \
        cudaError_t _e = (call);                  \
        if (_e != cudaSuccess)                    \
            return cuda_fail(ctx, _e, what);      \
    } while (0)

// column-major 4x4 -> rows of the 3x4 affine part
void affine_rows(const float m[16], float4 rows[3])
{
    for (int r = 0; r < 3; r++)
        rows[r] = make_float4(m[0 * 4 + r], m[1 * 4 + r], m[2 * 4 + r], m[3 * 4 + r]);
}

// inverse of the 3x4 affine part in double, rounded to float rows
bool affine_inverse_rows(const float m[16], float4 rows[3])
{
    double a[3][3], t[3];
    for (int r = 0; r < 3; r++) {
        for (int c = 0; c < 3; c++)
            a[r][c] = m[c * 4 + r];
        t[r] = m[3 * 4 + r];
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
        double tt = -(inv[r][0] * t[0] + inv[r][1] * t[1] + inv[r][2] * t[2]);
        rows[r] = make_float4((float)inv[r][0], (float)inv[r][1], (float)inv[r][2], (float)tt);
    }
    return true;
}

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

struct MeshBuild {
    BVHBuildResult bvh;
    Box3 root{};
};

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
    if (cudaMallocHost(&ctx->counters_pinned, C_COUNT * sizeof(uint32_t)) != cudaSuccess) {
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
    if (t->threads_per_block && (t->threads_per_block % 32 != 0 || t->threads_per_block > 1024))
        return fail(ctx, VVPT_ERR_INVALID_ARG, "threads_per_block must be a multiple of 32, at most 1024");
    std::lock_guard<std::mutex> lk(ctx->mu);
    ctx->tuning = *t;
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

    // ---- validation (indices the shaders would dereference)
    if ((desc->num_meshes && !desc->meshes) || (desc->num_instances && !desc->instances) ||
        (desc->num_materials && !desc->materials) || (desc->num_lights && !desc->lights) ||
        (desc->num_light_data && !desc->light_data) || (desc->num_textures && !desc->textures))
        return fail(ctx, VVPT_ERR_INVALID_ARG, "array pointer is null while its count is not zero");
    for (uint32_t m = 0; m < desc->num_meshes; m++) {
        const vvpt_mesh_desc &md = desc->meshes[m];
        if ((md.num_vertices && !md.vertices) || (md.num_triangles && !md.indices))
            return fail(ctx, VVPT_ERR_INVALID_ARG, "mesh " + std::to_string(m) + ": null vertex or index array");
        for (uint64_t i = 0; i < 3ull * md.num_triangles; i++)
            if (md.indices[i] >= md.num_vertices)
                return fail(ctx, VVPT_ERR_INVALID_ARG, "mesh " + std::to_string(m) + ": index out of range");
    }
    auto check_tex = [&](uint32_t t) { return t < desc->num_textures; };
    bool has_transparent = false;
    for (uint32_t i = 0; i < desc->num_materials; i++) {
        const vvpt_material &mt = desc->materials[i];
        for (int k = 0; k < 4; k++) {
            if (k != 2 && !check_tex(mt.textures2[k]) && (uint32_t)mt.uv_tiling[2] != VVPT_MATERIAL_VOLUME)
                return fail(ctx, VVPT_ERR_INVALID_ARG, "material " + std::to_string(i) + ": texture index out of range");
            if (!check_tex(mt.textures1[k]) && (uint32_t)mt.uv_tiling[2] != VVPT_MATERIAL_VOLUME &&
                !((uint32_t)mt.uv_tiling[2] == VVPT_MATERIAL_LAMBERT && (k == 1 || k == 2)))
                return fail(ctx, VVPT_ERR_INVALID_ARG, "material " + std::to_string(i) + ": texture index out of range");
        }
        if (mt.metallic_roughness_ao[3] > 0.0f && (uint32_t)mt.uv_tiling[2] != VVPT_MATERIAL_VOLUME)
            has_transparent = true;
    }
    for (uint32_t i = 0; i < desc->num_instances; i++) {
        const vvpt_instance &in = desc->instances[i];
        if (!(in.flags & VVPT_INSTANCE_IN_TLAS))
            continue;
        if (in.mesh_index >= desc->num_meshes)
            return fail(ctx, VVPT_ERR_INVALID_ARG, "instance " + std::to_string(i) + ": mesh index out of range");
        if (in.material_index >= desc->num_materials)
            return fail(ctx, VVPT_ERR_INVALID_ARG, "instance " + std::to_string(i) + ": material index out of range");
        uint32_t mtype = (uint32_t)desc->materials[in.material_index].uv_tiling[2];
        if (mtype != VVPT_MATERIAL_PBR_STANDARD && mtype != VVPT_MATERIAL_LAMBERT)
            return fail(ctx, VVPT_ERR_INVALID_ARG,
                        "instance " + std::to_string(i) + ": surface material must be PBR standard or Lambert");
        for (int k = 1; k <= 2; k++) {
            float v = in.id[k];
            if (v != -1.0f && !(v >= 0.0f && (uint32_t)v < desc->num_materials))
                return fail(ctx, VVPT_ERR_INVALID_ARG, "instance " + std::to_string(i) + ": volume index out of range");
        }
    }
    for (uint32_t i = 0; i < desc->num_lights; i++) {
        const vvpt_light_instance &L = desc->lights[i];
        if (L.info[3] <= 1 && L.info[0] >= desc->num_light_data)
            return fail(ctx, VVPT_ERR_INVALID_ARG, "light " + std::to_string(i) + ": light data index out of range");
        if (L.info[3] == 2) {
            if (L.info[1] >= desc->num_instances)
                return fail(ctx, VVPT_ERR_INVALID_ARG, "mesh light " + std::to_string(i) + ": instance out of range");
            const vvpt_instance &in = desc->instances[L.info[1]];
            if (in.mesh_index >= desc->num_meshes || in.material_index >= desc->num_materials ||
                desc->meshes[in.mesh_index].num_triangles == 0)
                return fail(ctx, VVPT_ERR_INVALID_ARG, "mesh light " + std::to_string(i) + ": instance has no mesh");
        }
        if (L.info[3] > 2)
            return fail(ctx, VVPT_ERR_UNSUPPORTED, "light " + std::to_string(i) + ": unsupported light type");
    }
    for (uint32_t t = 0; t < desc->num_textures; t++) {
        const vvpt_texture_desc &td = desc->textures[t];
        if (!td.data || td.width == 0 || td.height == 0 || td.format > VVPT_TEXTURE_RGBA32F)
            return fail(ctx, VVPT_ERR_INVALID_ARG, "texture " + std::to_string(t) + ": bad description");
    }

    auto scene = new vvpt_scene();
    std::unique_ptr<vvpt_scene> guard(scene);

    // ---- BLAS per mesh (largest first, meshes built in parallel)
    const uint32_t nm = desc->num_meshes;
    std::vector<MeshBuild> builds(nm);
    std::vector<uint32_t> order(nm);
    for (uint32_t i = 0; i < nm; i++)
        order[i] = i;
    std::sort(order.begin(), order.end(),
              [&](uint32_t a, uint32_t b) { return desc->meshes[a].num_triangles > desc->meshes[b].num_triangles; });
    std::atomic<uint32_t> next{0};
    unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    auto worker = [&]() {
        for (;;) {
            uint32_t k = next.fetch_add(1);
            if (k >= nm)
                break;
            uint32_t m = order[k];
            const vvpt_mesh_desc &md = desc->meshes[m];
            std::vector<Box3> boxes(md.num_triangles);
            for (uint32_t t = 0; t < md.num_triangles; t++) {
                Box3 &b = boxes[t];
                for (int a = 0; a < 3; a++) {
                    b.lo[a] = INFINITY;
                    b.hi[a] = -INFINITY;
                }
                for (int c = 0; c < 3; c++) {
                    const float *p = md.vertices[md.indices[3 * t + c]].position;
                    for (int a = 0; a < 3; a++) {
                        b.lo[a] = std::min(b.lo[a], p[a]);
                        b.hi[a] = std::max(b.hi[a], p[a]);
                    }
                }
            }
            BVHBuildOptions opt;
            opt.threads = (k == 0 && md.num_triangles > 100000) ? (int)hw : 1;
            builds[m].bvh = build_bvh2(boxes, opt);
            Box3 r;
            for (int a = 0; a < 3; a++) {
                r.lo[a] = INFINITY;
                r.hi[a] = -INFINITY;
            }
            for (const Box3 &b : boxes)
                for (int a = 0; a < 3; a++) {
                    r.lo[a] = std::min(r.lo[a], b.lo[a]);
                    r.hi[a] = std::max(r.hi[a], b.hi[a]);
                }
            builds[m].root = r;
        }
    };
    {
        std::vector<std::thread> th;
        unsigned nth = std::min<unsigned>(hw, std::max<uint32_t>(nm, 1));
        for (unsigned i = 0; i < nth; i++)
            th.emplace_back(worker);
        for (auto &t : th)
            t.join();
    }

    std::vector<MeshInfo> minfo(nm);
    std::vector<BVHNode> nodes;
    std::vector<TriVerts> tris;
    std::vector<ShadeVertex> verts;
    std::vector<uint32_t> indices;
    size_t total_nodes = 0, total_tris = 0, total_verts = 0;
    for (uint32_t m = 0; m < nm; m++) {
        total_nodes += builds[m].bvh.nodes.size();
        total_tris += desc->meshes[m].num_triangles;
        total_verts += desc->meshes[m].num_vertices;
    }
    nodes.reserve(total_nodes + 2 * desc->num_instances + 2);
    tris.reserve(total_tris);
    verts.reserve(total_verts);
    indices.reserve(3 * total_tris);
    for (uint32_t m = 0; m < nm; m++) {
        const vvpt_mesh_desc &md = desc->meshes[m];
        MeshInfo &mi = minfo[m];
        mi.node_offset = (uint32_t)nodes.size();
        mi.tri_offset = (uint32_t)tris.size();
        mi.vertex_offset = (uint32_t)verts.size();
        mi.index_offset = (uint32_t)indices.size();
        mi.num_triangles = md.num_triangles;
        mi.num_nodes = (uint32_t)builds[m].bvh.nodes.size();
        nodes.insert(nodes.end(), builds[m].bvh.nodes.begin(), builds[m].bvh.nodes.end());
        for (uint32_t k = 0; k < md.num_triangles; k++) {
            uint32_t prim = builds[m].bvh.order[k];
            TriVerts tv;
            const float *p0 = md.vertices[md.indices[3 * prim + 0]].position;
            const float *p1 = md.vertices[md.indices[3 * prim + 1]].position;
            const float *p2 = md.vertices[md.indices[3 * prim + 2]].position;
            float pid;
            std::memcpy(&pid, &prim, 4);
            tv.v0 = make_float4(p0[0], p0[1], p0[2], pid);
            tv.v1 = make_float4(p1[0], p1[1], p1[2], 0.0f);
            tv.v2 = make_float4(p2[0], p2[1], p2[2], 0.0f);
            tris.push_back(tv);
        }
        for (uint32_t v = 0; v < md.num_vertices; v++) {
            const vvpt_vertex &x = md.vertices[v];
            ShadeVertex sv;
            sv.pos_u = make_float4(x.position[0], x.position[1], x.position[2], x.uv[0]);
            sv.nrm_v = make_float4(x.normal[0], x.normal[1], x.normal[2], x.uv[1]);
            sv.tan_ = make_float4(x.tangent[0], x.tangent[1], x.tangent[2], 0.0f);
            verts.push_back(sv);
        }
        indices.insert(indices.end(), md.indices, md.indices + 3ull * md.num_triangles);
    }

    // ---- instances + TLAS
    const uint32_t ni = desc->num_instances;
    std::vector<DevInstance> dinst(ni);
    std::vector<Box3> tlas_boxes;
    std::vector<uint32_t> tlas_ids;
    for (uint32_t i = 0; i < ni; i++) {
        const vvpt_instance &in = desc->instances[i];
        DevInstance &d = dinst[i];
        std::memset(&d, 0, sizeof(d));
        affine_rows(in.model, d.o2w);
        if (!affine_inverse_rows(in.model, d.w2o)) {
            if (in.flags & VVPT_INSTANCE_IN_TLAS)
                return fail(ctx, VVPT_ERR_INVALID_ARG, "instance " + std::to_string(i) + ": singular model matrix");
        }
        d.material = in.material_index < desc->num_materials ? in.material_index : 0;
        d.front_volume = (int32_t)in.id[1];
        d.back_volume = (int32_t)in.id[2];
        if (in.mesh_index < nm) {
            const MeshInfo &mi = minfo[in.mesh_index];
            d.node_offset = mi.node_offset;
            d.tri_offset = mi.tri_offset;
            d.vertex_offset = mi.vertex_offset;
            d.index_offset = mi.index_offset;
            d.num_triangles = mi.num_triangles;
        }
        if ((in.flags & VVPT_INSTANCE_IN_TLAS) && in.mesh_index < nm && minfo[in.mesh_index].num_triangles > 0) {
            const Box3 &r = builds[in.mesh_index].root;
            Box3 w;
            for (int a = 0; a < 3; a++) {
                w.lo[a] = INFINITY;
                w.hi[a] = -INFINITY;
            }
            for (int c = 0; c < 8; c++) {
                double p[3] = {(c & 1) ? r.hi[0] : r.lo[0], (c & 2) ? r.hi[1] : r.lo[1], (c & 4) ? r.hi[2] : r.lo[2]};
                const float4 *rows = d.o2w;
                double q[3] = {rows[0].x * p[0] + rows[0].y * p[1] + rows[0].z * p[2] + rows[0].w,
                               rows[1].x * p[0] + rows[1].y * p[1] + rows[1].z * p[2] + rows[1].w,
                               rows[2].x * p[0] + rows[2].y * p[1] + rows[2].z * p[2] + rows[2].w};
                for (int a = 0; a < 3; a++) {
                    // widen by a few ulps: the box must contain every
                    // object-space hit mapped back to world space
                    double pad = 1e-5 * (std::fabs(q[a]) + 1.0);
                    w.lo[a] = std::min(w.lo[a], (float)(q[a] - pad));
                    w.hi[a] = std::max(w.hi[a], (float)(q[a] + pad));
                }
            }
            tlas_boxes.push_back(w);
            tlas_ids.push_back(i);
        }
    }
    BVHBuildResult tlas = build_bvh2(tlas_boxes);
    const uint32_t tlas_root = (uint32_t)nodes.size();
    nodes.insert(nodes.end(), tlas.nodes.begin(), tlas.nodes.end());
    std::vector<uint32_t> tlas_order(tlas.order.size());
    for (size_t k = 0; k < tlas.order.size(); k++)
        tlas_order[k] = tlas_ids[tlas.order[k]];
    if (tlas.depth > 30 || [&] {
            int md = 0;
            for (auto &b : builds)
                md = std::max(md, b.bvh.depth);
            return md > 62;
        }())
        return fail(ctx, VVPT_ERR_UNSUPPORTED, "BVH deeper than the traversal stack");

    // ---- materials, lights, textures
    std::vector<DevMaterial> mats(desc->num_materials);
    static_assert(sizeof(DevMaterial) == sizeof(vvpt_material), "material layout");
    if (desc->num_materials)
        std::memcpy(mats.data(), desc->materials, sizeof(vvpt_material) * desc->num_materials);
    std::vector<DevLightInstance> lights(desc->num_lights);
    for (uint32_t i = 0; i < desc->num_lights; i++) {
        const vvpt_light_instance &L = desc->lights[i];
        DevLightInstance &d = lights[i];
        std::memset(&d, 0, sizeof(d));
        std::memcpy(d.info, L.info, sizeof(d.info));
        d.position = make_float4(L.position[0], L.position[1], L.position[2], L.position[3]);
        d.position1 = make_float4(L.position1[0], L.position1[1], L.position1[2], L.position1[3]);
        d.position2 = make_float4(L.position2[0], L.position2[1], L.position2[2], L.position2[3]);
        if (L.info[3] <= 1) {
            const vvpt_light_data &ld = desc->light_data[L.info[0]];
            d.color = make_float4(ld.color[0], ld.color[1], ld.color[2], ld.color[3]);
        } else {
            // transpose(inverse(M)) for the sampled normal (lightSampling.glsl:80)
            float m[16] = {L.position[0], L.position1[0], L.position2[0], 0.0f, L.position[1], L.position1[1],
                           L.position2[1], 0.0f, L.position[2], L.position1[2], L.position2[2], 0.0f,
                           L.position[3], L.position1[3], L.position2[3], 1.0f};
            float4 inv[3];
            if (!affine_inverse_rows(m, inv))
                return fail(ctx, VVPT_ERR_INVALID_ARG, "mesh light " + std::to_string(i) + ": singular transform");
            d.nrm0 = make_float4(inv[0].x, inv[1].x, inv[2].x, 0.0f);
            d.nrm1 = make_float4(inv[0].y, inv[1].y, inv[2].y, 0.0f);
            d.nrm2 = make_float4(inv[0].z, inv[1].z, inv[2].z, 0.0f);
        }
    }
    std::vector<DevTexture> texs;
    std::vector<uint8_t> texels;
    auto add_texture = [&](const vvpt_texture_desc &td) {
        DevTexture t{};
        t.width = td.width;
        t.height = td.height;
        t.format = td.format;
        size_t texel_bytes = td.format == VVPT_TEXTURE_RGBA32F ? 16 : 4;
        size_t off = (texels.size() + 15) & ~size_t(15);
        texels.resize(off + texel_bytes * td.width * td.height);
        std::memcpy(texels.data() + off, td.data, texel_bytes * td.width * td.height);
        t.offset = off;
        texs.push_back(t);
    };
    for (uint32_t t = 0; t < desc->num_textures; t++)
        add_texture(desc->textures[t]);
    int env_index = -1;
    if (desc->environment) {
        if (!desc->environment->data || desc->environment->format != VVPT_TEXTURE_RGBA32F)
            return fail(ctx, VVPT_ERR_INVALID_ARG, "environment must be an RGBA32F equirectangular image");
        env_index = (int)texs.size();
        add_texture(*desc->environment);
    }

    // ---- upload
    vvpt_status st;
    uint64_t bytes = 0;
    if ((st = upload(ctx, scene->nodes, nodes, bytes)) != VVPT_OK)
        return st;
    if ((st = upload(ctx, scene->tris, tris, bytes)) != VVPT_OK)
        return st;
    if ((st = upload(ctx, scene->verts, verts, bytes)) != VVPT_OK)
        return st;
    if ((st = upload(ctx, scene->indices, indices, bytes)) != VVPT_OK)
        return st;
    if ((st = upload(ctx, scene->instances, dinst, bytes)) != VVPT_OK)
        return st;
    if ((st = upload(ctx, scene->tlas_order, tlas_order, bytes)) != VVPT_OK)
        return st;
    if ((st = upload(ctx, scene->materials, mats, bytes)) != VVPT_OK)
        return st;
    if ((st = upload(ctx, scene->lights, lights, bytes)) != VVPT_OK)
        return st;
    if ((st = upload(ctx, scene->textures, texs, bytes)) != VVPT_OK)
        return st;
    if ((st = upload(ctx, scene->texels, texels, bytes)) != VVPT_OK)
        return st;
    VV_CUDA(cudaStreamSynchronize(vv_stream(ctx)), "scene upload");

    SceneView &v = scene->view;
    v.nodes = scene->nodes.as<BVHNode>();
    v.tris = scene->tris.as<TriVerts>();
    v.verts = scene->verts.as<ShadeVertex>();
    v.indices = scene->indices.as<uint32_t>();
    v.instances = scene->instances.as<DevInstance>();
    v.tlas_order = scene->tlas_order.as<uint32_t>();
    v.tlas_root = tlas_root;
    v.num_instances = ni;
    v.materials = scene->materials.as<DevMaterial>();
    v.num_materials = desc->num_materials;
    v.lights = scene->lights.as<DevLightInstance>();
    v.num_lights = desc->num_lights;
    v.textures = scene->textures.as<DevTexture>();
    v.num_textures = (uint32_t)texs.size();
    v.texels = scene->texels.as<uint8_t>();
    v.env_texture = env_index;
    v.has_transparent = has_transparent ? 1u : 0u;
    scene->bytes = bytes;
    scene->num_materials = desc->num_materials;
    *out_scene = guard.release();
    return VVPT_OK;
}

VVPT_API vvpt_status vvpt_scene_release(vvpt_ctx *ctx, vvpt_scene *scene)
{
    if (!ctx || !scene)
        return VVPT_ERR_INVALID_ARG;
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
    if (info->width == 0 || info->height == 0 || info->batch_size == 0)
        return fail(ctx, VVPT_ERR_INVALID_ARG, "width, height and batch_size must be positive");
    if ((uint64_t)info->width * info->height > (1ull << 28))
        return fail(ctx, VVPT_ERR_INVALID_ARG, "resolution too large");
    std::lock_guard<std::mutex> lk(ctx->mu);
    cudaSetDevice(ctx->device);
    ctx->progress.store(0.0f);
    auto t_start = std::chrono::steady_clock::now();

    const uint32_t W = info->width, H = info->height;
    const uint32_t npix = W * H;
    const uint32_t batches = info->samples / info->batch_size; // integer truncation, as the reference
    RenderParams hp{};
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
    hp.width = W;
    hp.height = H;
    hp.batch_size = info->batch_size;
    hp.batches = batches;
    hp.depth = std::min(info->depth, 255u);
    hp.total_samples = info->batch_size * batches;
    hp.num_lights = scene->view.num_lights;
    uint64_t total_items64 = (uint64_t)npix * batches;
    if (total_items64 >= 0xFFFFFFF0ull)
        return fail(ctx, VVPT_ERR_INVALID_ARG, "width * height * batches exceeds 2^32");
    hp.total_items = (uint32_t)total_items64;
    hp.want_m2 = (info->flags & VVPT_RENDER_WANT_BATCH_M2) ? 1u : 0u;

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
        const size_t f4 = n * sizeof(float4), u4 = n * sizeof(uint32_t);
        auto aligned = [](size_t b) { return (b + 255) & ~size_t(255); };
        char *base = nullptr;
        auto take = [&](size_t b) {
            char *p = base;
            base += aligned(b);
            return p;
        };
        VV_CUDA(ctx->state.reserve(14 * aligned(f4) + 7 * aligned(u4)), "cudaMalloc path state");
        base = ctx->state.as<char>();
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
        take(f4); // spare
        ps.hit_inst = (uint32_t *)take(u4);
        ps.rng = (uint32_t *)take(u4);
        ps.flags = (uint32_t *)take(u4);
        ps.vol = (uint32_t *)take(u4);
        ps.item = (uint32_t *)take(u4);
        ps.sample = (uint32_t *)take(u4);
        take(u4);

        size_t qneed = 10 * aligned(u4) + aligned(C_COUNT * sizeof(uint32_t));
        VV_CUDA(ctx->queues.reserve(qneed), "cudaMalloc queues");
        base = ctx->queues.as<char>();
        Queues q;
        q.ext[0] = (uint32_t *)take(u4);
        q.ext[1] = (uint32_t *)take(u4);
        q.shade_l = (uint32_t *)take(u4);
        q.shade_p = (uint32_t *)take(u4);
        q.shade_m = (uint32_t *)take(u4);
        q.conn = (uint32_t *)take(u4);
        q.ext_key = (uint32_t *)take(u4);
        q.walk = (uint32_t *)take(u4);
        q.regen[0] = (uint32_t *)take(u4);
        q.regen[1] = (uint32_t *)take(u4);
        q.counters = (uint32_t *)take(C_COUNT * sizeof(uint32_t));

        const size_t rb = (size_t)hp.total_items * sizeof(float4);
        size_t rneed = 3 * aligned(rb);
        VV_CUDA(ctx->results.reserve(rneed), "cudaMalloc batch results");
        base = ctx->results.as<char>();
        BatchResults br;
        br.rad = (float4 *)take(rb);
        br.alb = (float4 *)take(rb);
        br.nrm = (float4 *)take(rb);

        VV_CUDA(ctx->params.reserve(sizeof(RenderParams)), "cudaMalloc params");
        RenderParams *dparams = ctx->params.as<RenderParams>();
        VV_CUDA(cudaMemcpyAsync(dparams, &hp, sizeof(hp), cudaMemcpyHostToDevice, vv_stream(ctx)), "upload params");

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
        launch_init_slots(q, ps, slots, vv_stream(ctx));
        stats.kernel_launches += 1;
        VV_CUDA(cudaGetLastError(), "launch init");
        const uint64_t max_iters =
            (uint64_t)hp.batch_size * (hp.depth + 1) * ((hp.total_items + slots - 1) / slots + 1) + 64;

        if (info->flags & VVPT_RENDER_PROFILE_KERNELS) {
            // one kernel at a time with events around each launch
            static const char *names[K_NUM] = {"k_begin", "k_regen",  "k_extend", "k_partition",
                                               "k_walk",  "k_shade", "k_shadow", "k_emitter"};
            static const double bpu[K_NUM] = {0.0,        kBytesRegen, kBytesExtend, kBytesPartition,
                                              kBytesWalk, kBytesShade, kBytesShadow, kBytesEmitter};
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
                                     : (k == K_SHADOW || k == K_EMITTER) ? c[C_CONN]
                                                      : 1;
                    cudaEventRecord(ka, vv_stream(ctx));
                    launch_kernel((KernelId)k, scene->view, dparams, ps, q, br, pp, shape, vv_stream(ctx));
                    cudaEventRecord(kb, vv_stream(ctx));
                    VV_CUDA(cudaEventSynchronize(kb), "profile kernel");
                    float ms = 0.0f;
                    cudaEventElapsedTime(&ms, ka, kb);
                    prof.kernels[k].launches += 1;
                    prof.kernels[k].units += units;
                    prof.kernels[k].total_ms += ms;
                    stats.kernel_launches += 1;
                }
                VV_CUDA(cudaMemcpy(ctx->counters_pinned, q.counters, C_COUNT * sizeof(uint32_t), cudaMemcpyDeviceToHost),
                        "read counters");
                const uint32_t *c = ctx->counters_pinned;
                if (c[C_ERR]) {
                    pst = fail(ctx, VVPT_ERR_DEVICE, "device status word set: " + std::to_string(c[C_ERR]));
                    break;
                }
                if (c[C_NEXT_ITEM] >= hp.total_items && c[C_ACTIVE] == 0)
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
            launch_iteration(scene->view, dparams, ps, q, br, it & 1, shape, vv_stream(ctx));
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
            VV_CUDA(cudaEventRecord(ev[launched & 1], vv_stream(ctx)), "event");
            int check = launched & 1;
            VV_CUDA(cudaGraphLaunch(exec, vv_stream(ctx)), "graph launch");
            launched++;
            iters += Ke;
            VV_CUDA(cudaEventSynchronize(ev[check]), "wait counters");
            const uint32_t *c = ctx->counters_pinned;
            float prog = hp.total_items ? (float)std::min<uint32_t>(c[C_NEXT_ITEM] - std::min(c[C_NEXT_ITEM], c[C_ACTIVE]),
                                                                   hp.total_items) /
                                              (float)hp.total_items
                                        : 1.0f;
            ctx->progress.store(prog);
            if (c[C_ERR]) {
                loop_status = fail(ctx, VVPT_ERR_DEVICE,
                                   "device status word set (traversal stack overflow or loop cap): " +
                                       std::to_string(c[C_ERR]));
                break;
            }
            if (c[C_NEXT_ITEM] >= hp.total_items && c[C_ACTIVE] == 0)
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
    (void)t_start;
    ctx->stats = stats;
    ctx->progress.store(1.0f);
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
    if (info->width == 0 || info->height == 0 || info->batch_size == 0)
        return fail(ctx, VVPT_ERR_INVALID_ARG, "width, height and batch_size must be positive");
    const uint64_t npix64 = (uint64_t)info->width * info->height;
    const uint32_t batches = info->samples / info->batch_size;
    const uint64_t items64 = npix64 * batches;
    const uint64_t slots64 = std::max<uint64_t>(32, std::min<uint64_t>(items64, kNoAllocMaxSlots));
    auto aligned = [](uint64_t b) { return (b + 255) & ~uint64_t(255); };
    const uint64_t f4 = slots64 * sizeof(float4), u4 = slots64 * sizeof(uint32_t);
    const uint64_t need = aligned(sizeof(RenderParams)) + aligned(C_COUNT * sizeof(uint32_t)) + 14 * aligned(f4) +
                          7 * aligned(u4) + 10 * aligned(u4) + 3 * aligned(items64 * sizeof(float4));
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

    RenderParams hp{};
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
    hp.total_items = (uint32_t)items64;
    hp.want_m2 = out->radiance_m2 ? 1u : 0u;

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
    RenderParams *dparams = reinterpret_cast<RenderParams *>(take(sizeof(RenderParams)));
    Queues q;
    q.counters = reinterpret_cast<uint32_t *>(take(C_COUNT * sizeof(uint32_t)));
    PathState ps;
    float4 **f4s[14] = {&ps.o, &ps.d, &ps.beta, &ps.rad, &ps.alb, &ps.nrm, &ps.cum_rad,
                        &ps.cum_alb, &ps.cum_nrm, &ps.hit, &ps.sh_dir, &ps.sh_c, &ps.nee_b, nullptr};
    for (float4 **p : f4s) {
        float4 *m = reinterpret_cast<float4 *>(take(f4));
        if (p)
            *p = m;
    }
    uint32_t **u4s[7] = {&ps.hit_inst, &ps.rng, &ps.flags, &ps.vol, &ps.item, &ps.sample, nullptr};
    for (uint32_t **p : u4s) {
        uint32_t *m = reinterpret_cast<uint32_t *>(take(u4));
        if (p)
            *p = m;
    }
    uint32_t **qs[10] = {&q.ext[0], &q.ext[1], &q.shade_l, &q.shade_p, &q.shade_m,
                         &q.conn,   &q.ext_key, &q.walk,  &q.regen[0], &q.regen[1]};
    for (uint32_t **p : qs)
        *p = reinterpret_cast<uint32_t *>(take(u4));
    BatchResults br;
    br.rad = reinterpret_cast<float4 *>(take(items64 * sizeof(float4)));
    br.alb = reinterpret_cast<float4 *>(take(items64 * sizeof(float4)));
    br.nrm = reinterpret_cast<float4 *>(take(items64 * sizeof(float4)));

    VV_CUDA(cudaMemcpyAsync(dparams, &hp, sizeof(hp), cudaMemcpyHostToDevice, stream), "upload params");
    LaunchShape shape;
    shape.block = 256;
    shape.grid = std::max(1, ctx->num_sms * 4);
    const uint32_t slots = (uint32_t)slots64;
    launch_init_slots(q, ps, slots, stream);
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
                launch_kernel((KernelId)kk, scene->view, dparams, ps, q, br, (int)(it & 1), shape, stream);
            it++;
        }
        stats.kernel_launches += 8 * K_NUM;
        VV_CUDA(cudaGetLastError(), "launch iteration");
        VV_CUDA(cudaMemcpyAsync(ctx->counters_pinned, q.counters, C_COUNT * sizeof(uint32_t), cudaMemcpyDeviceToHost,
                                stream),
                "read counters");
        VV_CUDA(cudaStreamSynchronize(stream), "render");
        const uint32_t *c = ctx->counters_pinned;
        if (c[C_ERR])
            return fail(ctx, VVPT_ERR_DEVICE, "device status word set: " + std::to_string(c[C_ERR]));
        ctx->progress.store((float)std::min<uint32_t>(c[C_NEXT_ITEM] - std::min(c[C_NEXT_ITEM], c[C_ACTIVE]),
                                                     hp.total_items) /
                            (float)hp.total_items);
        if (c[C_NEXT_ITEM] >= hp.total_items && c[C_ACTIVE] == 0)
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
