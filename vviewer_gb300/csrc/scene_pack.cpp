// Host-side scene preparation (scene_pack.h). Validation follows the indices
// the reference's shaders dereference: MaterialData texture slots
// (shaders/include/structs.glsl:41-52), InstanceData material / volume ids
// (src/lib/vengine/core/Instances.hpp:17-35), LightInstance data and
// instance links (src/lib/vengine/vulkan/VulkanInstances.cpp:66-109).
#include "scene_pack.h"

#include <vector_functions.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <mutex>
#include <thread>

#include "bvh_build.h"

namespace vvpt {

namespace {

vvpt_status fail(std::string &err, vvpt_status code, const std::string &msg)
{
    err = msg;
    return code;
}

struct MeshBuild {
    BVHBuildResult bvh;
    WideBuildResult wide; // collapsed from bvh (VVPT_BLAS_WIDE)
    Box3 root{};
};

}  // namespace

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

float build_env_distribution(const float *rgba, uint32_t w, uint32_t h, std::vector<float> &out)
{
    const size_t W = w, H = h;
    std::vector<double> lum(W * H), f(W * H);
    for (size_t i = 0; i < W * H; i++) {
        const double v = 0.2126 * rgba[4 * i] + 0.7152 * rgba[4 * i + 1] + 0.0722 * rgba[4 * i + 2];
        lum[i] = v > 0.0 && std::isfinite(v) ? v : 0.0;
    }
    for (size_t r = 0; r < H; r++) {
        // latitude of the row centre: w = asin(y) * 0.3183 + 0.5
        const double lat = (((double)r + 0.5) / (double)H - 0.5) / (double)0.3183f;
        const double cosl = std::max(0.0, std::cos(std::min(std::max(lat, -0.5 * M_PI), 0.5 * M_PI)));
        for (size_t c = 0; c < W; c++) {
            double m = 0.0;
            for (int dr = -1; dr <= 1; dr++) {
                const size_t rr = (size_t)std::min<long>(std::max<long>((long)r + dr, 0), (long)H - 1);
                for (int dc = -1; dc <= 1; dc++) {
                    const size_t cc = (c + W + dc) % W;
                    m = std::max(m, lum[rr * W + cc]);
                }
            }
            f[r * W + c] = m * cosl;
        }
    }
    out.assign(W * H + H * (W + 1) + (H + 1), 0.0f);
    float *func = out.data(), *cond = func + W * H, *marg = cond + H * (W + 1);
    std::vector<double> row_int(H, 0.0);
    for (size_t r = 0; r < H; r++) {
        double acc = 0.0;
        for (size_t c = 0; c < W; c++)
            acc += f[r * W + c];
        row_int[r] = acc / (double)W;
        double run = 0.0;
        float *cr = cond + r * (W + 1);
        cr[0] = 0.0f;
        for (size_t c = 0; c < W; c++) {
            run += f[r * W + c];
            cr[c + 1] = acc > 0.0 ? (float)(run / acc) : (float)((double)(c + 1) / (double)W);
        }
        cr[W] = 1.0f;
        for (size_t c = 0; c < W; c++)
            func[r * W + c] = (float)f[r * W + c];
    }
    double total = 0.0;
    for (size_t r = 0; r < H; r++)
        total += row_int[r];
    double run = 0.0;
    marg[0] = 0.0f;
    for (size_t r = 0; r < H; r++) {
        run += row_int[r];
        marg[r + 1] = total > 0.0 ? (float)(run / total) : (float)((double)(r + 1) / (double)H);
    }
    marg[H] = 1.0f;
    return (float)(total / (double)H);
}

vvpt_status pack_scene(const vvpt_scene_desc *desc, PackedScene &out, std::string &err, unsigned threads,
                       const BlasBuilder &large_builder, uint32_t large_min, bool builder_for_all)
{
    // a tree for the TLAS or the baked small instances: on the given builder
    // when it takes every tree, else (or when it declines) on the host
    auto build_other = [&](const std::vector<Box3> &boxes, const BVHBuildOptions &opt,
                           BVHBuildResult &res) -> bool {
        if (builder_for_all && large_builder) {
            std::string e;
            if (large_builder(boxes, opt, res, e))
                return true;
            if (!e.empty()) {
                err = e;
                return false;
            }
        }
        res = build_bvh2(boxes, opt);
        return true;
    };
    out = PackedScene();
    // ---- validation (indices the shaders would dereference)
    if ((desc->num_meshes && !desc->meshes) || (desc->num_instances && !desc->instances) ||
        (desc->num_materials && !desc->materials) || (desc->num_lights && !desc->lights) ||
        (desc->num_light_data && !desc->light_data) || (desc->num_textures && !desc->textures))
        return fail(err, VVPT_ERR_INVALID_ARG, "array pointer is null while its count is not zero");
    for (uint32_t m = 0; m < desc->num_meshes; m++) {
        const vvpt_mesh_desc &md = desc->meshes[m];
        if ((md.num_vertices && !md.vertices) || (md.num_triangles && !md.indices))
            return fail(err, VVPT_ERR_INVALID_ARG, "mesh " + std::to_string(m) + ": null vertex or index array");
        for (uint64_t i = 0; i < 3ull * md.num_triangles; i++)
            if (md.indices[i] >= md.num_vertices)
                return fail(err, VVPT_ERR_INVALID_ARG, "mesh " + std::to_string(m) + ": index out of range");
    }
    auto check_tex = [&](uint32_t t) { return t < desc->num_textures; };
    bool &has_transparent = out.has_transparent;
    has_transparent = false;
    for (uint32_t i = 0; i < desc->num_materials; i++) {
        const vvpt_material &mt = desc->materials[i];
        for (int k = 0; k < 4; k++) {
            if (k != 2 && !check_tex(mt.textures2[k]) && (uint32_t)mt.uv_tiling[2] != VVPT_MATERIAL_VOLUME)
                return fail(err, VVPT_ERR_INVALID_ARG, "material " + std::to_string(i) + ": texture index out of range");
            if (!check_tex(mt.textures1[k]) && (uint32_t)mt.uv_tiling[2] != VVPT_MATERIAL_VOLUME &&
                !((uint32_t)mt.uv_tiling[2] == VVPT_MATERIAL_LAMBERT && (k == 1 || k == 2)))
                return fail(err, VVPT_ERR_INVALID_ARG, "material " + std::to_string(i) + ": texture index out of range");
        }
        if (mt.metallic_roughness_ao[3] > 0.0f && (uint32_t)mt.uv_tiling[2] != VVPT_MATERIAL_VOLUME)
            has_transparent = true;
    }
    for (uint32_t i = 0; i < desc->num_instances; i++) {
        const vvpt_instance &in = desc->instances[i];
        if (!(in.flags & VVPT_INSTANCE_IN_TLAS))
            continue;
        if (in.mesh_index >= desc->num_meshes)
            return fail(err, VVPT_ERR_INVALID_ARG, "instance " + std::to_string(i) + ": mesh index out of range");
        if (in.material_index >= desc->num_materials)
            return fail(err, VVPT_ERR_INVALID_ARG, "instance " + std::to_string(i) + ": material index out of range");
        uint32_t mtype = (uint32_t)desc->materials[in.material_index].uv_tiling[2];
        if (mtype != VVPT_MATERIAL_PBR_STANDARD && mtype != VVPT_MATERIAL_LAMBERT)
            return fail(err, VVPT_ERR_INVALID_ARG,
                        "instance " + std::to_string(i) + ": surface material must be PBR standard or Lambert");
        for (int k = 1; k <= 2; k++) {
            float v = in.id[k];
            if (v != -1.0f && !(v >= 0.0f && (uint32_t)v < desc->num_materials))
                return fail(err, VVPT_ERR_INVALID_ARG, "instance " + std::to_string(i) + ": volume index out of range");
        }
    }
    for (uint32_t i = 0; i < desc->num_lights; i++) {
        const vvpt_light_instance &L = desc->lights[i];
        if (L.info[3] <= 1 && L.info[0] >= desc->num_light_data)
            return fail(err, VVPT_ERR_INVALID_ARG, "light " + std::to_string(i) + ": light data index out of range");
        if (L.info[3] == 2) {
            if (L.info[1] >= desc->num_instances)
                return fail(err, VVPT_ERR_INVALID_ARG, "mesh light " + std::to_string(i) + ": instance out of range");
            const vvpt_instance &in = desc->instances[L.info[1]];
            if (in.mesh_index >= desc->num_meshes || in.material_index >= desc->num_materials ||
                desc->meshes[in.mesh_index].num_triangles == 0)
                return fail(err, VVPT_ERR_INVALID_ARG, "mesh light " + std::to_string(i) + ": instance has no mesh");
        }
        if (L.info[3] > 2)
            return fail(err, VVPT_ERR_UNSUPPORTED, "light " + std::to_string(i) + ": unsupported light type");
    }
    for (uint32_t t = 0; t < desc->num_textures; t++) {
        const vvpt_texture_desc &td = desc->textures[t];
        if (!td.data || td.width == 0 || td.height == 0 || td.format > VVPT_TEXTURE_RGBA32F)
            return fail(err, VVPT_ERR_INVALID_ARG, "texture " + std::to_string(t) + ": bad description");
    }

    // ---- BLAS per mesh (largest first, meshes built in parallel)
    const uint32_t nm = desc->num_meshes;
    std::vector<MeshBuild> builds(nm);
    std::vector<uint32_t> order(nm);
    for (uint32_t i = 0; i < nm; i++)
        order[i] = i;
    std::sort(order.begin(), order.end(),
              [&](uint32_t a, uint32_t b) { return desc->meshes[a].num_triangles > desc->meshes[b].num_triangles; });
    std::atomic<uint32_t> next{0};
    std::mutex large_mu;
    std::string large_err; // a failed large build falls back to the host builder
    const unsigned hw = threads ? threads : std::max(1u, std::thread::hardware_concurrency());
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
            bool built = false;
            if (large_builder && md.num_triangles >= large_min) {
                std::lock_guard<std::mutex> lk(large_mu);
                std::string e;
                built = large_builder(boxes, opt, builds[m].bvh, e);
                if (!built && !e.empty() && large_err.empty())
                    large_err = e;
            }
            if (!built)
                builds[m].bvh = build_bvh2(boxes, opt);
#if VVPT_BLAS_WIDE
            builds[m].wide = collapse_to_wide(builds[m].bvh, boxes);
            builds[m].bvh.nodes = std::vector<BVHNode>();
#endif
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

    if (!large_err.empty())
        return fail(err, VVPT_ERR_DEVICE, large_err);

    std::vector<MeshInfo> minfo(nm);
    std::vector<BVHNode> &nodes = out.nodes;
    std::vector<WideNode> &wnodes = out.wnodes;
    std::vector<TriVerts> &tris = out.tris;
    std::vector<ShadeVertex> &verts = out.verts;
    std::vector<uint32_t> &indices = out.indices;
    size_t total_nodes = 0, total_tris = 0, total_verts = 0;
    for (uint32_t m = 0; m < nm; m++) {
        total_nodes += builds[m].bvh.nodes.size() + builds[m].wide.nodes.size();
        total_tris += desc->meshes[m].num_triangles;
        total_verts += desc->meshes[m].num_vertices;
    }
#if VVPT_BLAS_WIDE
    wnodes.reserve(total_nodes);
    nodes.reserve(2 * desc->num_instances + 2);
#else
    nodes.reserve(total_nodes + 2 * desc->num_instances + 2);
#endif
    tris.reserve(total_tris);
    verts.reserve(total_verts);
    indices.reserve(3 * total_tris);
    for (uint32_t m = 0; m < nm; m++) {
        const vvpt_mesh_desc &md = desc->meshes[m];
        MeshInfo &mi = minfo[m];
        mi.tri_offset = (uint32_t)tris.size();
        mi.vertex_offset = (uint32_t)verts.size();
        mi.index_offset = (uint32_t)indices.size();
        mi.num_triangles = md.num_triangles;
#if VVPT_BLAS_WIDE
        mi.node_offset = (uint32_t)wnodes.size();
        mi.num_nodes = (uint32_t)builds[m].wide.nodes.size();
        wnodes.insert(wnodes.end(), builds[m].wide.nodes.begin(), builds[m].wide.nodes.end());
        const std::vector<uint32_t> &leaf_order = builds[m].wide.order;
#else
        mi.node_offset = (uint32_t)nodes.size();
        mi.num_nodes = (uint32_t)builds[m].bvh.nodes.size();
        nodes.insert(nodes.end(), builds[m].bvh.nodes.begin(), builds[m].bvh.nodes.end());
        const std::vector<uint32_t> &leaf_order = builds[m].bvh.order;
#endif
        for (uint32_t k = 0; k < md.num_triangles; k++) {
            uint32_t prim = leaf_order[k];
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

    // ---- which materials can emit: the emitter rays add radiance where
    // emissive.w * emissive.rgb * texel exceeds 0.05 in some channel; bound it
    // by the largest texel of the emissive texture (1 for 8-bit formats). The
    // 0.04 cut leaves a margin for rounding; NaN counts as emitting.
    std::vector<char> may_emit(desc->num_materials, 0);
    {
        std::vector<double> tex_max(desc->num_textures, -1.0);
        auto texel_bound = [&](uint32_t t) -> double {
            if (t >= desc->num_textures)
                return INFINITY;
            const vvpt_texture_desc &td = desc->textures[t];
            if (td.format != VVPT_TEXTURE_RGBA32F)
                return 1.0;
            if (tex_max[t] < 0.0) {
                const float *px = static_cast<const float *>(td.data);
                double mx = 0.0;
                for (uint64_t k = 0; k < (uint64_t)td.width * td.height && !std::isinf(mx); k++)
                    for (int c = 0; c < 3; c++) {
                        const double v = std::fabs((double)px[4 * k + c]);
                        mx = std::isnan(v) ? INFINITY : std::max(mx, v);
                    }
                tex_max[t] = mx;
            }
            return tex_max[t];
        };
        for (uint32_t i = 0; i < desc->num_materials; i++) {
            const vvpt_material &mt = desc->materials[i];
            if ((uint32_t)mt.uv_tiling[2] == VVPT_MATERIAL_VOLUME)
                continue;
            double b = 0.0;
            for (int c = 0; c < 3; c++) {
                const double v = std::fabs((double)mt.emissive[3] * (double)mt.emissive[c]);
                b = std::isnan(v) ? INFINITY : std::max(b, v);
            }
            may_emit[i] = !(b == 0.0 || b * texel_bound(mt.textures2[0]) <= 0.04);
        }
    }
    std::vector<Box3> emit;

    // ---- instances + TLAS
    const uint32_t ni = desc->num_instances;
    std::vector<DevInstance> &dinst = out.instances;
    dinst.assign(ni, DevInstance{});
    std::vector<Box3> tlas_boxes;
    std::vector<uint32_t> tlas_ids;
    // Small instances (at most kFlattenMaxTriangles triangles each, two or
    // more of them) leave the TLAS: their triangles, baked into world space,
    // form one extra BLAS under an identity instance, and each baked
    // triangle carries its instance slot, which the traversal reports as the
    // hit's instance. Rays then enter one BLAS instead of several small ones
    // whose boxes span the scene (a room's walls, a medium's boundary).
    std::vector<uint8_t> flat(ni, 0);
    uint32_t nflat = 0;
    for (uint32_t i = 0; i < ni; i++) {
        const vvpt_instance &in = desc->instances[i];
        if ((in.flags & VVPT_INSTANCE_IN_TLAS) && in.mesh_index < nm && minfo[in.mesh_index].num_triangles > 0 &&
            minfo[in.mesh_index].num_triangles <= kFlattenMaxTriangles) {
            float4 inv[3];
            if (affine_inverse_rows(in.model, inv)) {
                flat[i] = 1;
                nflat++;
            }
        }
    }
    if (nflat < 2)
        std::fill(flat.begin(), flat.end(), 0);
    for (uint32_t i = 0; i < ni; i++) {
        const vvpt_instance &in = desc->instances[i];
        DevInstance &d = dinst[i];
        std::memset(&d, 0, sizeof(d));
        affine_rows(in.model, d.o2w);
        if (!affine_inverse_rows(in.model, d.w2o)) {
            if (in.flags & VVPT_INSTANCE_IN_TLAS)
                return fail(err, VVPT_ERR_INVALID_ARG, "instance " + std::to_string(i) + ": singular model matrix");
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
            const bool in_flat = flat[i] != 0;
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
            // culling-margin bound (traverse.cuh cull_slack), max-norms:
            // |o_obj| <= |A^-1| (|o| + |b|), |d_obj| >= |d| / |A|
            auto row_norm = [](const float4 *m) {
                double n = 0.0;
                for (int k = 0; k < 3; k++)
                    n = std::max(n, (double)std::fabs(m[k].x) + std::fabs(m[k].y) + std::fabs(m[k].z));
                return n;
            };
            const double na = row_norm(d.o2w), ninv = row_norm(d.w2o);
            const double bt = std::max({std::fabs((double)d.o2w[0].w), std::fabs((double)d.o2w[1].w),
                                        std::fabs((double)d.o2w[2].w)});
            double pm = 0.0;
            for (int a = 0; a < 3; a++)
                pm = std::max({pm, (double)std::fabs(r.lo[a]), (double)std::fabs(r.hi[a])});
            if (!in_flat) {
                out.cull_o = std::max(out.cull_o, (float)(na * ninv));
                out.cull_r = std::max(out.cull_r, (float)(na * (ninv * bt + pm)));
                tlas_boxes.push_back(w);
                tlas_ids.push_back(i);
            }
            if (may_emit[d.material])
                emit.push_back(w);
        }
    }
    if (nflat >= 2) {
        // baked triangles: world = ((r.x * x + r.y * y) + r.z * z) + r.w per
        // row of the instance's model matrix, in double, rounded to float
        std::vector<TriVerts> ft;
        std::vector<Box3> fb;
        double fm = 0.0;
        for (uint32_t i = 0; i < ni; i++) {
            if (!flat[i])
                continue;
            const vvpt_instance &in = desc->instances[i];
            const vvpt_mesh_desc &md = desc->meshes[in.mesh_index];
            const float4 *R = dinst[i].o2w;
            const float rr[3][4] = {{R[0].x, R[0].y, R[0].z, R[0].w},
                                    {R[1].x, R[1].y, R[1].z, R[1].w},
                                    {R[2].x, R[2].y, R[2].z, R[2].w}};
            for (uint32_t t = 0; t < md.num_triangles; t++) {
                float q[3][3];
                Box3 b;
                for (int a = 0; a < 3; a++) {
                    b.lo[a] = INFINITY;
                    b.hi[a] = -INFINITY;
                }
                for (int c = 0; c < 3; c++) {
                    const float *p = md.vertices[md.indices[3 * t + c]].position;
                    for (int a = 0; a < 3; a++) {
                        double v = (double)rr[a][0] * p[0];
                        v = v + (double)rr[a][1] * p[1];
                        v = v + (double)rr[a][2] * p[2];
                        v = v + (double)rr[a][3];
                        q[c][a] = (float)v;
                        b.lo[a] = std::min(b.lo[a], q[c][a]);
                        b.hi[a] = std::max(b.hi[a], q[c][a]);
                        fm = std::max(fm, (double)std::fabs(q[c][a]));
                    }
                }
                TriVerts tv;
                float pid, iid;
                const uint32_t slot = i + 1;
                std::memcpy(&pid, &t, 4);
                std::memcpy(&iid, &slot, 4);
                tv.v0 = make_float4(q[0][0], q[0][1], q[0][2], pid);
                tv.v1 = make_float4(q[1][0], q[1][1], q[1][2], iid);
                tv.v2 = make_float4(q[2][0], q[2][1], q[2][2], 0.0f);
                ft.push_back(tv);
                fb.push_back(b);
            }
        }
        BVHBuildResult fbvh;
        if (!build_other(fb, BVHBuildOptions(), fbvh))
            return VVPT_ERR_DEVICE;
        DevInstance syn;
        std::memset(&syn, 0, sizeof(syn));
        const float ident[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
        affine_rows(ident, syn.o2w);
        affine_rows(ident, syn.w2o);
        syn.tri_offset = (uint32_t)tris.size();
        syn.num_triangles = (uint32_t)ft.size();
        syn.front_volume = syn.back_volume = -1;
#if VVPT_BLAS_WIDE
        WideBuildResult fw = collapse_to_wide(fbvh, fb);
        syn.node_offset = (uint32_t)wnodes.size();
        wnodes.insert(wnodes.end(), fw.nodes.begin(), fw.nodes.end());
        const std::vector<uint32_t> &forder = fw.order;
#else
        syn.node_offset = (uint32_t)nodes.size();
        nodes.insert(nodes.end(), fbvh.nodes.begin(), fbvh.nodes.end());
        const std::vector<uint32_t> &forder = fbvh.order;
#endif
        for (uint32_t k = 0; k < (uint32_t)ft.size(); k++)
            tris.push_back(ft[forder[k]]);
        Box3 w;
        for (int a = 0; a < 3; a++) {
            w.lo[a] = INFINITY;
            w.hi[a] = -INFINITY;
        }
        for (const Box3 &b : fb)
            for (int a = 0; a < 3; a++) {
                w.lo[a] = std::min(w.lo[a], b.lo[a]);
                w.hi[a] = std::max(w.hi[a], b.hi[a]);
            }
        for (int a = 0; a < 3; a++) {
            const float pad = 1e-5f * (std::fabs(w.lo[a]) + std::fabs(w.hi[a]) + 1e-3f);
            w.lo[a] -= pad;
            w.hi[a] += pad;
        }
        out.cull_o = std::max(out.cull_o, 1.0f);
        out.cull_r = std::max(out.cull_r, (float)fm);
        out.max_blas_depth = std::max(out.max_blas_depth, fbvh.depth);
        dinst.push_back(syn);
        tlas_boxes.push_back(w);
        tlas_ids.push_back(ni);
    }
    if (emit.size() > kMaxEmitBoxes) {
        // merge into kMaxEmitBoxes boxes: runs of neighbours along the axis
        // of widest centroid spread (unions stay conservative)
        double clo[3] = {INFINITY, INFINITY, INFINITY}, chi[3] = {-INFINITY, -INFINITY, -INFINITY};
        for (const Box3 &b : emit)
            for (int a = 0; a < 3; a++) {
                const double c = 0.5 * ((double)b.lo[a] + (double)b.hi[a]);
                clo[a] = std::min(clo[a], c);
                chi[a] = std::max(chi[a], c);
            }
        int ax = 0;
        for (int a = 1; a < 3; a++)
            if (chi[a] - clo[a] > chi[ax] - clo[ax])
                ax = a;
        std::stable_sort(emit.begin(), emit.end(), [ax](const Box3 &x, const Box3 &y) {
            return (double)x.lo[ax] + x.hi[ax] < (double)y.lo[ax] + y.hi[ax];
        });
        std::vector<Box3> merged;
        const size_t n = emit.size();
        for (size_t g = 0; g < kMaxEmitBoxes; g++) {
            const size_t k = g * n / kMaxEmitBoxes, end = (g + 1) * n / kMaxEmitBoxes;
            Box3 u = emit[k];
            for (size_t j = k + 1; j < end; j++)
                for (int a = 0; a < 3; a++) {
                    u.lo[a] = std::min(u.lo[a], emit[j].lo[a]);
                    u.hi[a] = std::max(u.hi[a], emit[j].hi[a]);
                }
            merged.push_back(u);
        }
        emit.swap(merged);
    }
    for (const Box3 &b : emit) {
        out.emit_boxes.push_back(make_float4(b.lo[0], b.lo[1], b.lo[2], 0.0f));
        out.emit_boxes.push_back(make_float4(b.hi[0], b.hi[1], b.hi[2], 0.0f));
    }
    // one instance per TLAS leaf: entering an instance costs a BLAS traversal
#ifndef VVPT_TLAS_MAX_LEAF
#define VVPT_TLAS_MAX_LEAF 1
#endif
    BVHBuildOptions tlas_opt;
    tlas_opt.max_leaf = VVPT_TLAS_MAX_LEAF;
    BVHBuildResult tlas;
    if (!build_other(tlas_boxes, tlas_opt, tlas))
        return VVPT_ERR_DEVICE;
    out.tlas_root = (uint32_t)nodes.size();
    nodes.insert(nodes.end(), tlas.nodes.begin(), tlas.nodes.end());
    std::vector<uint32_t> &tlas_order = out.tlas_order;
    tlas_order.resize(tlas.order.size());
    for (size_t k = 0; k < tlas.order.size(); k++)
        tlas_order[k] = tlas_ids[tlas.order[k]];
    {
        // the traversal stack holds at most two entries per TLAS level, the
        // instance return marker and one entry per BLAS level
        int md = out.max_blas_depth;
        for (auto &b : builds)
            md = std::max(md, b.bvh.depth);
        out.tlas_depth = tlas.depth;
        out.max_blas_depth = md;
        if (2 * tlas.depth + md + 2 > kTraversalStack)
            return fail(err, VVPT_ERR_UNSUPPORTED, "BVH deeper than the traversal stack");
    }

    // ---- materials, lights, textures
    std::vector<DevMaterial> &mats = out.materials;
    mats.resize(desc->num_materials);
    static_assert(sizeof(DevMaterial) == sizeof(vvpt_material), "material layout");
    if (desc->num_materials)
        std::memcpy(mats.data(), desc->materials, sizeof(vvpt_material) * desc->num_materials);
    std::vector<DevLightInstance> &lights = out.lights;
    lights.resize(desc->num_lights);
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
                return fail(err, VVPT_ERR_INVALID_ARG, "mesh light " + std::to_string(i) + ": singular transform");
            d.nrm0 = make_float4(inv[0].x, inv[1].x, inv[2].x, 0.0f);
            d.nrm1 = make_float4(inv[0].y, inv[1].y, inv[2].y, 0.0f);
            d.nrm2 = make_float4(inv[0].z, inv[1].z, inv[2].z, 0.0f);
        }
    }
    std::vector<DevTexture> &texs = out.textures;
    std::vector<uint8_t> &texels = out.texels;
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
    int &env_index = out.env_texture;
    env_index = -1;
    if (desc->environment) {
        if (!desc->environment->data || desc->environment->format != VVPT_TEXTURE_RGBA32F)
            return fail(err, VVPT_ERR_INVALID_ARG, "environment must be an RGBA32F equirectangular image");
        env_index = (int)texs.size();
        add_texture(*desc->environment);
        out.env_w = desc->environment->width;
        out.env_h = desc->environment->height;
        out.env_func_int = build_env_distribution(static_cast<const float *>(desc->environment->data), out.env_w,
                                                  out.env_h, out.env_dist);
    }

    return VVPT_OK;
}

}  // namespace vvpt
