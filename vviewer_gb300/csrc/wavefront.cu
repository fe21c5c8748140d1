// Wavefront integrator kernels: regen (camera rays), extend (closest hit),
// shade (surface / medium / miss events, light and BSDF sampling, Russian
// roulette) and connect (shadow rays and BSDF-direction emitter rays).
//
// One iteration of the five kernels advances every live path by one traced
// segment, i.e. one pass of the `for d < depth` loop of
// src/lib/vengine/shaders/pt/raygen.rgen.glsl:100-124 with the closest-hit /
// miss shader that follows it. The shadow and emitter rays the reference
// traces inside its hit shaders (lightSampling.glsl:108-144,
// next_event_estimation.glsl:1-33) are deferred to `connect`; they consume no
// random numbers, so the RNG stream per path is the reference's.
#include "shade.cuh"
#include "traverse.cuh"
#include "wavefront.cuh"

namespace vvpt {

// path flag bits
constexpr uint32_t F_SAMPLED = 128u;     // ray direction sampled (BSDF or phase), pdf in nee_b.w
constexpr uint32_t F_INSIDE = 1u;       // rayPayloadPrimary.insideVolume
constexpr uint32_t F_DONE = 2u;         // sample finished, finalize in regen
constexpr uint32_t F_ITEM = 4u;         // slot holds a work item
constexpr uint32_t F_SHADOW = 8u;       // pending shadow connection
constexpr uint32_t F_NEE = 16u;         // pending emitter connection (path ends at this event)
constexpr uint32_t F_NEE_FUSED = 32u;   // emitter ray rides on the next extension ray
constexpr uint32_t F_NEE_FULL = 64u;    // ... but needs the full candidate walk (set by extend)
constexpr int kDepthShift = 8;          // recursionDepth d
constexpr int kSurfShift = 16;          // surfaceDepth
constexpr uint32_t kByteMask = 0xFFu;

constexpr float kExtTmin = 0.001f;      // raygen.rgen.glsl:110
constexpr float kExtTmax = 10000.0f;
constexpr float kConnTmin = 0.0001f;    // lightSampling.glsl:112, next_event_estimation.glsl:3
constexpr int kCandidateCap = 1024;     // per-segment candidate bound for any-hit loops

// Who traces a ray in the candidate walks below: one lane on its own
// (trace_after), or a group of eight lanes that all run the walk with the
// same data (trace_after_group, the traversal kernels' form).
struct LaneTracer {
    __device__ __forceinline__ Hit operator()(const SceneView &s, const float3 &o, const float3 &d, float tmin,
                                              float tmax, const Hit &after, uint32_t &err) const
    {
        return trace_after(s, o, d, tmin, tmax, after, err);
    }
};
#if VVPT_BLAS_WIDE && VVPT_GROUP_TRAVERSAL
struct GroupTracer {
    LaneGroup g;
    __device__ __forceinline__ Hit operator()(const SceneView &s, const float3 &o, const float3 &d, float tmin,
                                              float tmax, const Hit &after, uint32_t &err) const
    {
        return trace_after_group(s, o, d, tmin, tmax, after, err, g);
    }
};
#endif

// One atomic per warp for a per-lane count. All 32 lanes call it.
__device__ __forceinline__ void warp_add(uint32_t *counter, uint32_t v)
{
    const uint32_t sum = __reduce_add_sync(0xFFFFFFFFu, v);
    if ((threadIdx.x & 31u) == 0 && sum)
        atomicAdd(counter, sum);
}

// Warp-aggregated queue append. Must be called by all 32 lanes of the warp
// at a convergence point (the kernels below keep their loop bounds
// warp-uniform); lanes with want == false get no slot.
__device__ __forceinline__ uint32_t warp_append_all(bool want, uint32_t *counter)
{
    const uint32_t mask = __ballot_sync(0xFFFFFFFFu, want);
    const int lane = threadIdx.x & 31;
    const int leader = mask ? __ffs(mask) - 1 : 0;
    uint32_t base = 0;
    if (want && lane == leader)
        base = atomicAdd(counter, (uint32_t)__popc(mask));
    base = __shfl_sync(0xFFFFFFFFu, base, leader);
    return base + (uint32_t)__popc(mask & ((1u << lane) - 1u));
}

__device__ __forceinline__ float4 mat4_mul(const float4 *cols, float x, float y, float z, float w)
{
    return make_float4(cols[0].x * x + cols[1].x * y + cols[2].x * z + cols[3].x * w,
                       cols[0].y * x + cols[1].y * y + cols[2].y * z + cols[3].y * w,
                       cols[0].z * x + cols[1].z * y + cols[2].z * z + cols[3].z * w,
                       cols[0].w * x + cols[1].w * y + cols[2].w * z + cols[3].w * w);
}

// ---------------------------------------------------------------------------
// Hit reconstruction (shaders/pt/process_hit.glsl:1-17, construct_frame.glsl:1-15)

struct SurfaceHit {
    float3 wpos;
    float2 uv;
    Frame frame;
    bool flipped;
    uint32_t material;
    int32_t front_volume, back_volume;
};

__device__ __forceinline__ void fetch_triangle(const SceneView &s, const DevInstance &inst, uint32_t prim,
                                               ShadeVertex &a, ShadeVertex &b, ShadeVertex &c)
{
    const uint32_t *ix = s.indices + inst.index_offset + 3u * prim;
    uint32_t i0 = __ldg(ix), i1 = __ldg(ix + 1), i2 = __ldg(ix + 2);
    const ShadeVertex *v = s.verts + inst.vertex_offset;
    const float4 *p0 = reinterpret_cast<const float4 *>(v + i0);
    const float4 *p1 = reinterpret_cast<const float4 *>(v + i1);
    const float4 *p2 = reinterpret_cast<const float4 *>(v + i2);
    a.pos_u = __ldg(p0); a.nrm_v = __ldg(p0 + 1); a.tan_ = __ldg(p0 + 2);
    b.pos_u = __ldg(p1); b.nrm_v = __ldg(p1 + 1); b.tan_ = __ldg(p1 + 2);
    c.pos_u = __ldg(p2); c.nrm_v = __ldg(p2 + 1); c.tan_ = __ldg(p2 + 2);
}

__device__ __forceinline__ Affine34 rows_of(const float4 *r) { return Affine34{r[0], r[1], r[2]}; }

// Full hit record with the shading frame; `ray_dir` is gl_WorldRayDirectionEXT.
__device__ __forceinline__ SurfaceHit make_surface_hit(const SceneView &s, uint32_t inst_id, uint32_t prim, float hu,
                                                       float hv, const float3 &ray_dir)
{
    const DevInstance &inst = s.instances[inst_id];
    ShadeVertex a, b, c;
    fetch_triangle(s, inst, prim, a, b, c);
    const float bx = 1.0f - hu - hv, by = hu, bz = hv;
    SurfaceHit h;
    h.uv = make_float2(a.pos_u.w * bx + b.pos_u.w * by + c.pos_u.w * bz, a.nrm_v.w * bx + b.nrm_v.w * by + c.nrm_v.w * bz);
    float3 lp = f3(a.pos_u) * bx + f3(b.pos_u) * by + f3(c.pos_u) * bz;
    Affine34 o2w = rows_of(inst.o2w), w2o = rows_of(inst.w2o);
    h.wpos = xform_point(o2w, lp);
    float3 ln = f3(a.nrm_v) * bx + f3(b.nrm_v) * by + f3(c.nrm_v) * bz;
    float3 lt = f3(a.tan_) * bx + f3(b.tan_) * by + f3(c.tan_) * bz;
    h.frame.n = normalize3(xform_normal_transposed(w2o, ln));
    h.frame.t = normalize3(xform_normal_transposed(w2o, lt));
    h.frame.b = f3(0.0f, 0.0f, 1.0f); // overwritten by fix_frame in both branches
    h.flipped = fix_frame(h.frame, ray_dir);
    h.material = inst.material;
    h.front_volume = inst.front_volume;
    h.back_volume = inst.back_volume;
    return h;
}

__device__ __forceinline__ float3 material_emissive(const SceneView &s, const DevMaterial &m, float2 tuv)
{
    float4 te = tex2d(s, m.tex2[0], tuv.x, tuv.y);
    return (m.emissive.w * f3(m.emissive)) * f3(te);
}
__device__ __forceinline__ float material_alpha(const SceneView &s, const DevMaterial &m, float2 tuv)
{
    return m.albedo.w * tex2d(s, m.tex2[3], tuv.x, tuv.y).x;
}


// ---------------------------------------------------------------------------
// Light sampling (shaders/pt/lightSampling.glsl:1-106), without the shadow
// trace, which `connect` performs.

// ---- Sampler. RTGEMS (default): the xorshift stream of
// shaders/include/rng/rng_def.glsl:4-36, rand2D = two rand1D draws.
// PMJ (VVPT_RENDER_SAMPLER_PMJ): shaders/include/rng/rng_pmj.glsl:20-107,
// whose state is the pixel, the sample index and a dimension counter.
struct PathRng {
    uint32_t s;     // RTGEMS xorshift state, or the PMJ dimension
    uint32_t pix;   // PMJ: pixel x | y << 16
    uint32_t index; // PMJ: sample index within the pixel
};

// 64-bit finaliser, rng_pmj.glsl:28-35
__device__ __forceinline__ uint64_t pmj_mix_bits(uint64_t v)
{
    v ^= v >> 31;
    v *= 9202493588570546565ull;
    v ^= v >> 27;
    v *= 9357036318526133325ull;
    v ^= v >> 33;
    return v;
}

// Element i of a pseudo-random permutation of [0, l) keyed by p (cycle
// walking over the next power of two), rng_pmj.glsl:37-64. The walk ends
// within a few steps; the cap only guards the loop.
__device__ __forceinline__ uint32_t pmj_permutation_element(uint32_t i, uint32_t l, uint32_t p)
{
    uint32_t w = l - 1;
    w |= w >> 1;
    w |= w >> 2;
    w |= w >> 4;
    w |= w >> 8;
    w |= w >> 16;
    for (int it = 0; it < 1024; it++) {
        i ^= p;
        i *= 0xe170893du;
        i ^= p >> 16;
        i ^= (i & w) >> 4;
        i ^= p >> 8;
        i *= 0x0929eb3fu;
        i ^= p >> 23;
        i ^= (i & w) >> 1;
        i *= 1u | p >> 27;
        i *= 0x6935fa69u;
        i ^= (i & w) >> 11;
        i *= 0x74dcb303u;
        i ^= (i & w) >> 2;
        i *= 0x9e501cc3u;
        i ^= (i & w) >> 2;
        i *= 0xc860a3dfu;
        i &= w;
        i ^= i >> 5;
        if (i < l)
            break;
    }
    return (i + p) % l;
}

constexpr uint32_t kPmjSeed = 2873468793u;
constexpr float kOneMinusEpsilon = 0.999999f; // ONEMINUSEPSILON, shaders/include/constants.glsl:2

__device__ __forceinline__ uint32_t pmj_hash(const PathRng &r)
{
    const uint64_t px = r.pix & 0xFFFFu, py = r.pix >> 16;
    return (uint32_t)pmj_mix_bits((px << 48) ^ (py << 32) ^ ((uint64_t)r.s << 16) ^ (uint64_t)kPmjSeed);
}

__device__ __forceinline__ float rnd1(const RenderParams &p, PathRng &r)
{
    if (!p.sampler)
        return rand1(r.s);
    const uint32_t index = pmj_permutation_element(r.index, p.total_samples, pmj_hash(r));
    const uint32_t px = (r.pix & 0xFFFFu) % 128u, py = (r.pix >> 16) % 128u;
    const float delta = __ldg(p.blue_noise + ((size_t)(r.s % 48u) * 128u + px) * 128u + py);
    r.s++;
    return fminf(__fdiv_rn(__fadd_rn((float)index, delta), (float)p.total_samples), kOneMinusEpsilon);
}

__device__ __forceinline__ float2 rnd2(const RenderParams &p, PathRng &r)
{
    if (!p.sampler) {
        const float a = rand1(r.s);
        const float b = rand1(r.s);
        return make_float2(a, b);
    }
    uint32_t index = r.index;
    const uint32_t inst = r.s / 2u;
    if (inst >= 16u)
        index = pmj_permutation_element(r.index, p.total_samples, pmj_hash(r));
    const float2 u = __ldg(reinterpret_cast<const float2 *>(p.pmj) + (size_t)(inst % 16u) * 16384u + index % 16384u);
    r.s += 2u;
    return make_float2(fminf(u.x, kOneMinusEpsilon), fminf(u.y, kOneMinusEpsilon));
}

// The path's sampler state as the shade kernels use it.
__device__ __forceinline__ PathRng load_rng(const RenderParams &p, const PathState &ps, uint32_t slot)
{
    PathRng r;
    r.s = ps.rng[slot];
    r.pix = 0;
    r.index = 0;
    if (p.sampler) {
        const uint32_t npix = p.width * p.height, item = ps.item[slot];
        const uint32_t batch = item / npix, pix = item - batch * npix;
        r.pix = (pix % p.width) | ((pix / p.width) << 16);
        r.index = batch * p.batch_size + ps.sample[slot];
    }
    return r;
}

struct LightSample {
    float3 dir;
    float3 radiance;
    float pdf;
    float tmax;
    bool delta;
};

// With env_light set, the environment is light number num_lights of the
// uniform pick (importance sampled by sample_env); `allow_env` = false makes
// that pick contribute nothing (the last event of a path, whose environment
// contribution the reference's estimator never adds either).
// Out of line with VVPT_SHADE_OUTLINE = 1 (a build option, measured, not
// kept): the shading kernel samples a light at a medium scatter point and at
// a surface, and one copy instead of two shortens its instruction stream,
// but the call's register saves cost more (1920 x 1080 x 64 medium scene:
// 158.0 against 160.0 M paths/s).
#ifndef VVPT_SHADE_OUTLINE
#define VVPT_SHADE_OUTLINE 0
#endif
#if VVPT_SHADE_OUTLINE
#define VVPT_SHADE_FN __noinline__
#else
#define VVPT_SHADE_FN __forceinline__
#endif
__device__ VVPT_SHADE_FN LightSample sample_light(const SceneView &s, const RenderParams &p, const float3 origin,
                                                  PathRng &rng, bool allow_env)
{
    LightSample ls;
    ls.delta = true;
    ls.radiance = f3(0.0f);
    ls.pdf = 1.0f;
    ls.dir = f3(0.0f);
    ls.tmax = 10000.0f;
    const uint32_t total = p.num_lights + p.env_light;
    if (total == 0)
        return ls;
    float pdf = 1.0f / (float)total;
    uint32_t li = (uint32_t)(rnd1(p, rng) * (float)total);
    if (li >= total)
        li = total - 1;
    if (li == p.num_lights) {
        ls.delta = false;
        if (!allow_env)
            return ls;
        const float2 uv = rnd2(p, rng);
        const float u_row = uv.x, u_col = uv.y;
        float epdf;
        ls.dir = sample_env(s, u_row, u_col, epdf);
        ls.tmax = p.zfar;
        if (epdf > 0.0f) {
            ls.radiance = env_lookup(s, ls.dir) * ((int)p.env_type == 1 ? p.env_intensity : 1.0f);
            ls.pdf = pdf * epdf;
        }
        return ls;
    }
    const DevLightInstance &L = s.lights[li];
    const uint32_t type = L.info[3];
    if (type == 0) {
        float3 lp = f3(L.position);
        float3 dir = lp - origin;
        float tmax = length3(dir);
        ls.tmax = tmax;
        ls.dir = dir / tmax;
        float dist = length3(origin - lp);
        ls.radiance = f3(L.color) * (1.0f / (dist * dist)) * L.color.w;
        ls.pdf = pdf * 1.0f;
        ls.delta = true;
    } else if (type == 1) {
        ls.dir = -f3(L.position);
        ls.tmax = p.zfar;
        ls.radiance = f3(L.color) * L.color.w;
        ls.pdf = pdf * 1.0f;
        ls.delta = true;
    } else if (type == 2) {
        const uint32_t mesh_inst = L.info[1];
        const DevInstance &inst = s.instances[mesh_inst];
        const DevMaterial &m = s.materials[inst.material];
        uint32_t tri = (uint32_t)(rnd1(p, rng) * (float)inst.num_triangles);
        if (tri >= inst.num_triangles)
            tri = inst.num_triangles - 1;
        float tri_pdf = 1.0f / (float)inst.num_triangles;
        const float2 uu = rnd2(p, rng);
        float2 bc = uniform_sample_triangle(uu.x, uu.y);
        float b0 = bc.x, b1 = bc.y, b2 = 1.0f - bc.x - bc.y;
        ShadeVertex a, b, c;
        fetch_triangle(s, inst, tri, a, b, c);
        Affine34 M{L.position, L.position1, L.position2};
        float3 p0 = xform_point(M, f3(a.pos_u)), p1 = xform_point(M, f3(b.pos_u)), p2 = xform_point(M, f3(c.pos_u));
        float area = 0.5f * length3(cross3(p1 - p0, p2 - p0));
        float point_pdf = 1.0f / area;
        float3 sp = f3(a.pos_u) * b0 + f3(b.pos_u) * b1 + f3(c.pos_u) * b2;
        float3 sn = f3(a.nrm_v) * b0 + f3(b.nrm_v) * b1 + f3(c.nrm_v) * b2;
        float2 suv = make_float2(a.pos_u.w * b0 + b.pos_u.w * b1 + c.pos_u.w * b2,
                                 a.nrm_v.w * b0 + b.nrm_v.w * b1 + c.nrm_v.w * b2);
        sp = xform_point(M, sp);
        Affine34 N{L.nrm0, L.nrm1, L.nrm2};
        sn = xform_vector(N, sn);
        float3 dir = sp - origin;
        float tmax = length3(dir);
        ls.tmax = tmax;
        ls.dir = dir / tmax;
        float dp = dot3(-ls.dir, sn);
        if (dp > 0.0f) {
            float2 tuv = make_float2(suv.x * m.uv_tiling.x, suv.y * m.uv_tiling.y);
            ls.radiance = material_emissive(s, m, tuv);
            float dist = length3(origin - sp);
            ls.pdf = pdf * tri_pdf * point_pdf * (dist * dist) / dp;
        } else {
            ls.radiance = f3(0.0f);
            ls.pdf = 0.0f;
        }
        ls.delta = false;
    }
    return ls;
}

// ---------------------------------------------------------------------------
// Homogeneous medium free flight (shaders/pt/process_volume_hit.glsl:1-40)

struct Medium {
    float3 sigma_s, sigma_t;
    float g;
};
__device__ __forceinline__ Medium load_medium(const SceneView &s, uint32_t vol)
{
    const DevMaterial &m = s.materials[vol];
    Medium md;
    float3 sa = f3(m.albedo);
    md.sigma_s = fmax3(f3(m.mrao), kEps);
    md.sigma_t = sa + md.sigma_s;
    md.g = fmaxf(fminf(m.emissive.x, 0.99f), -0.99f);
    return md;
}
// process_volume_transmittance.glsl:1-9
__device__ __forceinline__ float3 medium_transmittance(const SceneView &s, uint32_t vol, float vtstart, float vtend)
{
    const DevMaterial &m = s.materials[vol];
    float3 ss = fmax3(f3(m.mrao), kEps);
    float3 st = f3(m.albedo) + ss;
    float dist = fmaxf(vtend - vtstart, kEps);
    return f3(expf(-st.x * dist), expf(-st.y * dist), expf(-st.z * dist));
}

// ---------------------------------------------------------------------------
// Kernels

__global__ void k_init_slots(Queues q, PathState ps, JobTable jt, uint32_t slots)
{
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < slots; i += gridDim.x * blockDim.x) {
        q.regen[0][i] = i;
        ps.flags[i] = 0u;
        ps.item[i] = 0xFFFFFFFFu;
        ps.job[i] = 0u;
    }
    if (blockIdx.x == 0)
        vvpt_srgb_lut[threadIdx.x & 255u] = srgb_to_linear((float)(threadIdx.x & 255u) / 255.0f);
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        for (int c = 0; c < C_COUNT; c++)
            q.counters[c] = 0u;
        q.counters[C_REGEN0] = slots;
        *jt.next_item = 0ull;
        *jt.idle_count = 0u;
    }
}

// New work for idle slots (see launch_admit). One block: the counters it
// resets are read by all of its threads first.
__global__ void k_admit(Queues q, JobTable jt, unsigned long long total_items, uint32_t num_ranges)
{
    const uint32_t n = *jt.idle_count;
    const uint32_t base = q.counters[C_REGEN0];
    for (uint32_t i = threadIdx.x; i < n; i += blockDim.x)
        q.regen[0][base + i] = jt.idle[i];
    __syncthreads();
    if (threadIdx.x == 0) {
        // hand-out attempts past the old end claimed nothing
        const unsigned long long old_total = *jt.total_items;
        if (*jt.next_item > old_total)
            *jt.next_item = old_total;
        *jt.total_items = total_items;
        *jt.num_ranges = num_ranges;
        q.counters[C_REGEN0] = base + n;
        *jt.idle_count = 0u;
    }
}

// Hand-out range holding global work item g (the last range beginning at or
// before g).
__device__ __forceinline__ uint32_t find_range(const JobTable &jt, uint32_t num_ranges, unsigned long long g)
{
    uint32_t lo = 0, hi = num_ranges;
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (jt.range_begin[mid] <= g)
            lo = mid;
        else
            hi = mid;
    }
    return lo;
}

__global__ void k_begin(Queues q, int pp)
{
    if (threadIdx.x == 0) {
        q.counters[C_SHADE_L] = 0u;
        q.counters[C_SHADE_P] = 0u;
        q.counters[C_SHADE_M] = 0u;
        q.counters[C_WALK] = 0u;
        q.counters[C_CONN] = 0u;
        q.counters[C_NEEQ] = 0u;
        q.counters[C_FETCH_EXT] = 0u;
        q.counters[C_FETCH_SHADOW] = 0u;
        q.counters[C_EXT0 + (1 - pp)] = 0u;
        q.counters[C_REGEN0 + (1 - pp)] = 0u;
    }
}

// Finalizes finished samples, hands out work items, and generates camera
// rays (raygen.rgen.glsl:24-99, 126-129).
#ifndef VVPT_REGEN_MIN_BLOCKS
#define VVPT_REGEN_MIN_BLOCKS 1
#endif
__global__ void __launch_bounds__(256, VVPT_REGEN_MIN_BLOCKS) k_regen(JobTable jt, PathState ps, Queues q, int pp)
{
    const uint32_t n = q.counters[C_REGEN0 + pp];
    const uint32_t *queue = q.regen[pp];
    const unsigned long long total_items = *jt.total_items;
    const uint32_t num_ranges = *jt.num_ranges;
    // camera ray of a slot that holds a work item (fresh: a new item, its
    // sums and RNG state start from zero)
    auto body = [&](const uint32_t slot, uint32_t sample, uint32_t item, uint32_t job, bool fresh, float3 cr,
                    float3 ca, float3 cn) -> bool {
        const RenderParams &p = jt.jobs[job].params;
        const uint32_t npix = p.width * p.height;
        const uint32_t batch = item / npix;
        const uint32_t pix = item - batch * npix;
        const uint32_t px = pix % p.width, py = pix / p.width;
        PathRng rng;
        float3 alb, nrm;
        if (fresh) {
            rng.s = init_rng(px, py, p.width, batch);
            alb = nrm = f3(0.0f);
        } else {
            rng.s = ps.rng[slot];
            alb = f3(ps.alb[slot]);
            nrm = f3(ps.nrm[slot]);
        }
        rng.pix = px | (py << 16);
        rng.index = batch * p.batch_size + sample;
        if (p.sampler)
            rng.s = py * p.width + py; // dimension start of every sample, raygen.rgen.glsl:57-60
        // camera ray, raygen.rgen.glsl:63-91
        const float2 oxy = rnd2(p, rng);
        const float ox = oxy.x, oy = oxy.y;
        float uvx = ((float)px + ox) / (float)p.width;
        float uvy = ((float)py + oy) / (float)p.height;
        float dx = uvx * 2.0f - 1.0f, dy = uvy * 2.0f - 1.0f;
        float4 target = mat4_mul(p.proj_inv, dx, dy, 1.0f, 1.0f);
        float3 dcam = normalize3(f3(target.x, target.y, target.z));
        float3 ocam = f3(0.0f);
        if (p.lens_radius > 0.0f) {
            const float2 lxy = rnd2(p, rng);
            const float lx = lxy.x, ly = lxy.y;
            float2 disk = concentric_sample_disk(lx, ly);
            float2 lens = make_float2(p.lens_radius * disk.x, p.lens_radius * disk.y);
            float ft = p.focal_distance / (-dcam.z);
            float3 focus = dcam * ft;
            ocam = f3(lens.x, lens.y, 0.0f);
            dcam = normalize3(focus - ocam);
        }
        float4 wo = mat4_mul(p.view_inv, ocam.x, ocam.y, ocam.z, 1.0f);
        float4 wd = mat4_mul(p.view_inv, dcam.x, dcam.y, dcam.z, 0.0f);
        ps.o[slot] = make_float4(wo.x, wo.y, wo.z, 0.0f);
        ps.d[slot] = make_float4(wd.x, wd.y, wd.z, 0.0f);
        ps.beta[slot] = make_float4(1.0f, 1.0f, 1.0f, 0.0f);
        ps.rad[slot] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        ps.alb[slot] = f4(alb, 0.0f);
        ps.nrm[slot] = f4(nrm, 0.0f);
        ps.cum_rad[slot] = f4(cr, 0.0f);
        ps.cum_alb[slot] = f4(ca, 0.0f);
        ps.cum_nrm[slot] = f4(cn, 0.0f);
        ps.rng[slot] = rng.s;
        uint32_t nf = F_ITEM;
        if (p.cam_volume != -1)
            nf |= F_INSIDE;
        ps.flags[slot] = nf;
        ps.vol[slot] = (uint32_t)p.cam_volume;
        ps.item[slot] = item;
        ps.sample[slot] = sample;
        ps.job[slot] = job;
        return true;
    };
    // The loop bound is warp-uniform: the counters below take one atomic per
    // warp (one per job for finished items) instead of one per slot, as the
    // slots of a launch all update the same few addresses.
    const uint32_t lane = threadIdx.x & 31u;
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
        const uint32_t i = base + threadIdx.x;
        const bool valid = i < n;
        uint32_t slot = 0, flags = 0, sample = 0, item = 0, job = 0;
        float3 cr = f3(0.0f), ca = f3(0.0f), cn = f3(0.0f);
        bool path_done = false, item_done = false;
        if (valid) {
            slot = queue[i];
            flags = ps.flags[slot];
            sample = ps.sample[slot];
            item = ps.item[slot];
            job = ps.job[slot];
            if (flags & F_ITEM) {
                cr = f3(ps.cum_rad[slot]);
                ca = f3(ps.cum_alb[slot]);
                cn = f3(ps.cum_nrm[slot]);
            }
            if (flags & F_DONE) {
                const float total = (float)jt.jobs[job].params.total_samples;
                float3 r = f3(ps.rad[slot]);
                if (flags & F_NEE) // the emitter ray's contribution, after the shadow ray's
                    r = r + f3(ps.nee_c[slot]);
                cr += r / total;
                ca += f3(ps.alb[slot]) / total;
                cn += f3(ps.nrm[slot]) / total;
                sample++;
                path_done = true;
            }
            if ((flags & F_ITEM) && sample >= jt.jobs[job].params.batch_size) {
                // the item's batch sums; the host and k_reduce read them after
                // this launch, in stream order
                const BatchResults br = jt.jobs[job].results;
                br.rad[item] = f4(cr, 1.0f);
                br.alb[item] = f4(ca, 1.0f);
                br.nrm[item] = f4(cn, 1.0f);
                flags &= ~F_ITEM;
                item_done = true;
            }
        }
        const uint32_t paths = (uint32_t)__popc(__ballot_sync(0xFFFFFFFFu, path_done));
        const uint32_t fin = __ballot_sync(0xFFFFFFFFu, item_done);
        if (item_done) {
            const uint32_t same = __match_any_sync(fin, job);
            if (lane == (uint32_t)(__ffs(same) - 1))
                atomicAdd(&jt.item_done[job], (uint32_t)__popc(same));
        }
        // next work items, in lane order, for the slots without one
        const bool need = valid && !(flags & F_ITEM);
        const uint32_t need_mask = __ballot_sync(0xFFFFFFFFu, need);
        unsigned long long g0 = 0;
        if (lane == 0 && need_mask)
            g0 = atomicAdd(jt.next_item, (unsigned long long)__popc(need_mask));
        g0 = __shfl_sync(0xFFFFFFFFu, g0, 0);
        const unsigned long long g = g0 + (unsigned long long)__popc(need_mask & ((1u << lane) - 1u));
        const bool got = need && g < total_items;
        const bool idle = need && !got;
        const uint32_t started = (uint32_t)__popc(__ballot_sync(0xFFFFFFFFu, got));
        if (lane == 0) {
            if (paths)
                atomicAdd(&q.counters[C_PATHS], paths);
            if (started != (uint32_t)__popc(fin))
                atomicAdd(&q.counters[C_ACTIVE], started - (uint32_t)__popc(fin)); // mod 2^32
        }
        const uint32_t ipos = warp_append_all(idle, jt.idle_count);
        bool emit = false;
        if (idle) {
            ps.flags[slot] = 0u;
            ps.item[slot] = 0xFFFFFFFFu;
            jt.idle[ipos] = slot;
        } else if (got) {
            const uint32_t r = find_range(jt, num_ranges, g);
            emit = body(slot, 0u, (uint32_t)(g - jt.range_begin[r]), jt.range_job[r], true, f3(0.0f), f3(0.0f),
                        f3(0.0f));
        } else if (valid) {
            emit = body(slot, sample, item, job, false, cr, ca, cn);
        }
        const uint32_t pos = warp_append_all(emit, &q.counters[C_EXT0 + pp]);
        if (emit)
            q.ext[pp][pos] = slot;
    }
}

// Closest hit for every queued extension ray; hits are binned by material
// model into the shade queues (material-sorted shading).
// Minimum resident blocks of 256 threads per SM requested for the traversal
// kernels, which caps their registers (4: 64 registers, 50% occupancy); the
// traversal is latency bound and gains more from resident warps than it
// loses to the few spilled registers.
#ifndef VVPT_EXTEND_MIN_BLOCKS
#define VVPT_EXTEND_MIN_BLOCKS 4
#endif
#ifndef VVPT_TRACE_MIN_BLOCKS
#define VVPT_TRACE_MIN_BLOCKS 4
#endif
#ifndef VVPT_SHADE_MIN_BLOCKS
#define VVPT_SHADE_MIN_BLOCKS 2
#endif
// the Lambert and miss shading kernels
#ifndef VVPT_SHADE_LM_MIN_BLOCKS
#define VVPT_SHADE_LM_MIN_BLOCKS 2
#endif
// Rays per traversal-kernel lane: one (the one-ray-per-lane loop) or, with
// the wide BLAS, one per group of eight lanes (trace_after_group). first_ray
// is the queue index of a block's first ray, ray_stride the grid stride.
#if VVPT_BLAS_WIDE && VVPT_GROUP_TRAVERSAL
constexpr uint32_t kLanesPerRay = 8;
#else
constexpr uint32_t kLanesPerRay = 1;
#endif
__device__ __forceinline__ uint32_t first_ray() { return blockIdx.x * (blockDim.x / kLanesPerRay); }
__device__ __forceinline__ uint32_t my_ray() { return (blockIdx.x * blockDim.x + threadIdx.x) / kLanesPerRay; }
__device__ __forceinline__ uint32_t ray_stride() { return gridDim.x * blockDim.x / kLanesPerRay; }
// Before a group's lane 0 writes what every lane of the group has read.
__device__ __forceinline__ void group_sync()
{
#if VVPT_BLAS_WIDE && VVPT_GROUP_TRAVERSAL
    __syncwarp(0xFFu << (threadIdx.x & 24u));
#endif
}

// Shade bin of a closest hit (0 Lambert, 1 PBR, 2 miss; | 4: the fused
// emitter ray takes the full candidate walk).
__device__ __forceinline__ uint32_t extend_key(const SceneView &s, const Hit &h, bool fused, uint32_t key)
{
    if (h.inst == kNoHit)
        return key | 2u;
    const DevMaterial &m = s.materials[s.instances[h.inst].material];
    key |= (uint32_t)m.uv_tiling.z == 2u ? 0u : 1u;
    // a transparent first candidate also needs the walk
    if (fused && h.t <= kExtTmax && m.mrao.w >= 0.99f)
        key |= 4u;
    return key;
}

// Lane refill: a warp traces its rays step by step (trace_step). A lane is
// free, tracing, or done (its traversal ended, its result not yet used).
// When no more than VVPT_REFILL_BELOW of the warp's lanes are tracing, the
// done lanes finish their rays together and the free lanes take the next
// rays of the queue (one atomic per warp). Rays of very different lengths
// then share a warp's steps instead of the warp running until its longest
// ray ends, and the code between traversals runs for many lanes at once.
// Per-lane values that only that code reads stay in shared memory (one entry
// per thread), so the traversal state keeps the registers. Binary BLAS only.
#ifndef VVPT_REFILL_BELOW
#define VVPT_REFILL_BELOW 16
#endif
constexpr uint32_t kLaneFree = 0, kLaneTracing = 1, kLaneDone = 2;
// Step turns (k_extend): triangle tests and the other kinds of step in
// separate warp steps, triangle tests when at least VVPT_TRI_TURN_PCT % of
// the tracing lanes have one pending.
#ifndef VVPT_STEP_TURNS
#define VVPT_STEP_TURNS 1
#endif
#ifndef VVPT_TRI_TURN_PCT
#define VVPT_TRI_TURN_PCT 33
#endif

// Hands the next queue entries to the free lanes of the warp: returns the
// entry index of this lane (meaningful when `mine`), and clears `open` when
// the queue has no entries left after these. Warp-uniform call.
__device__ __forceinline__ uint32_t refill_take(bool free, uint32_t *counter, uint32_t n, bool &open, bool &mine)
{
    const uint32_t want = __ballot_sync(0xFFFFFFFFu, free);
    const uint32_t cnt = (uint32_t)__popc(want);
    const uint32_t lane = threadIdx.x & 31u;
    uint32_t base = 0;
    if (lane == 0 && cnt)
        base = atomicAdd(counter, cnt);
    base = __shfl_sync(0xFFFFFFFFu, base, 0);
    if (cnt)
        open = base + cnt < n;
    const uint32_t idx = base + (uint32_t)__popc(want & ((1u << lane) - 1u));
    mine = free && idx < n;
    return idx;
}

__global__ void __launch_bounds__(256, VVPT_EXTEND_MIN_BLOCKS) k_extend(JobTable jt, PathState ps, Queues q, int pp)
{
    const uint32_t n = q.counters[C_EXT0 + pp];
    const uint32_t *queue = q.ext[pp];
    uint32_t err = 0;
#if VVPT_EXTEND_REFILL
    if (n > 0)
        tlas_cache_fill(jt.jobs[ps.job[queue[min(first_ray(), n - 1u)]]].scene);
    else
        tlas_cache_none();
    // per lane: queue index, slot, fused (bit 0) | shade-bin bits (<< 1)
    __shared__ uint4 cold[256];
    TraceState st;
    TraceStack stack;
    uint32_t state = kLaneFree, job = 0;
    bool open = true; // warp-uniform: the queue may still hold rays
    for (;;) {
        uint32_t tr = __ballot_sync(0xFFFFFFFFu, state == kLaneTracing);
        if (__popc(tr) <= VVPT_REFILL_BELOW) {
            // finished rays go straight to the shade queues (material
            // bins) and the emitter-walk queue: warp-uniform appends
            uint32_t fin_slot = 0, fin_key = 0xFFu, fin_i = 0;
            if (state == kLaneDone) {
                const uint4 c = cold[threadIdx.x];
                const SceneView &s = jt.jobs[job].scene;
                const Hit &h = st.best;
                const bool fused = (c.z & 1u) != 0;
                const uint32_t key = c.z >> 1;
                if (fused && key == 0 && h.inst != kNoHit && h.t < kExtTmin) {
                    // the emitter ray's first candidate lies below the
                    // extension ray's tmin: the emitter ray takes the full
                    // candidate walk, and this lane goes on with the
                    // extension ray from its tmin
                    cold[threadIdx.x].z = 1u | (4u << 1);
                    trace_begin(st, s, st.o, st.d, kExtTmin, kExtTmax, no_hit());
                    state = kLaneTracing;
                } else {
                    ps.hit[c.y] = make_float4(h.t, h.u, h.v, __uint_as_float(h.prim));
                    ps.hit_inst[c.y] = h.inst;
                    fin_slot = c.y;
                    fin_i = c.x;
                    fin_key = extend_key(s, h, fused, key);
                    state = kLaneFree;
                }
            }
#if VVPT_EXTEND_PARTITION
            const uint32_t bin = fin_key & 3u;
            uint32_t pos = warp_append_all(bin == 0, &q.counters[C_SHADE_L]);
            if (bin == 0)
                q.shade_l[pos] = fin_slot;
            pos = warp_append_all(bin == 1, &q.counters[C_SHADE_P]);
            if (bin == 1)
                q.shade_p[pos] = fin_slot;
            pos = warp_append_all(bin == 2, &q.counters[C_SHADE_M]);
            if (bin == 2)
                q.shade_m[pos] = fin_slot;
            const bool walk = fin_key != 0xFFu && (fin_key & 4u);
            pos = warp_append_all(walk, &q.counters[C_WALK]);
            if (walk)
                q.walk[pos] = fin_slot;
#else
            if (fin_key != 0xFFu)
                q.ext_key[fin_i] = fin_key;
#endif
            if (open) {
                bool mine;
                const uint32_t i = refill_take(state == kLaneFree, &q.counters[C_FETCH_EXT], n, open, mine);
                if (mine) {
                    const uint32_t slot = queue[i];
                    job = ps.job[slot];
                    // with an emitter ray riding on this ray, start at its tmin
                    const bool fused = (ps.flags[slot] & F_NEE_FUSED) != 0;
                    cold[threadIdx.x] = make_uint4(i, slot, fused ? 1u : 0u, 0u);
                    trace_begin(st, jt.jobs[job].scene, f3(ps.o[slot]), f3(ps.d[slot]), fused ? kConnTmin : kExtTmin,
                                kExtTmax, no_hit());
                    state = kLaneTracing;
                }
            }
            tr = __ballot_sync(0xFFFFFFFFu, state == kLaneTracing);
            if (tr == 0) {
                if (!open)
                    break;
                continue;
            }
        }
#if VVPT_STEP_TURNS
        // triangle tests and node visits in separate warp steps: triangle
        // tests run when enough of the tracing lanes have one pending, the
        // other kinds of step otherwise (a lane whose kind is not this
        // step's waits; every lane's kind gets its turn, since the lanes
        // that step move on to a leaf, finish, or leave the tracing set)
        const bool tri = state == kLaneTracing && st.leaf_count > 0;
        const bool tri_turn =
            100 * __popc(__ballot_sync(0xFFFFFFFFu, tri)) >= VVPT_TRI_TURN_PCT * __popc(tr);
        if (state == kLaneTracing && tri == tri_turn && !trace_step(st, stack, jt.jobs[job].scene, no_hit(), err))
            state = kLaneDone;
#else
        if (state == kLaneTracing && !trace_step(st, stack, jt.jobs[job].scene, no_hit(), err))
            state = kLaneDone;
#endif
    }
#else
    if (first_ray() < n)
        tlas_cache_fill(jt.jobs[ps.job[queue[first_ray()]]].scene);
    else
        tlas_cache_none();
#if VVPT_BLAS_WIDE && VVPT_GROUP_TRAVERSAL
    // One ray per group of eight lanes; the group's lanes share the
    // traversal (trace_after_group) and lane 0 writes the result.
    const LaneGroup g = lane_group();
#endif
    // A lane (group) takes its next ray as soon as its current one is done,
    // so a warp is never held by its slowest ray. The shade bin is written
    // per queue entry and compacted by k_partition.
    for (uint32_t i = my_ray(); i < n; i += ray_stride()) {
        const uint32_t slot = queue[i];
        const SceneView &s = jt.jobs[ps.job[slot]].scene;
        const float3 o = f3(ps.o[slot]);
        const float3 d = f3(ps.d[slot]);
        const uint32_t flags = ps.flags[slot];
        // with an emitter ray riding on this ray, start at its tmin
        const bool fused = (flags & F_NEE_FUSED) != 0;
#if VVPT_BLAS_WIDE && VVPT_GROUP_TRAVERSAL
        Hit h = trace_after_group(s, o, d, fused ? kConnTmin : kExtTmin, kExtTmax, no_hit(), err, g);
#else
        Hit h = trace_closest(s, o, d, fused ? kConnTmin : kExtTmin, kExtTmax, err);
#endif
        uint32_t key = 0;
        if (fused && h.inst != kNoHit && h.t < kExtTmin) {
            // the emitter ray's first candidate lies below the extension
            // ray's tmin: the emitter ray takes the full candidate walk
            key = 4;
#if VVPT_BLAS_WIDE && VVPT_GROUP_TRAVERSAL
            h = trace_after_group(s, o, d, kExtTmin, kExtTmax, no_hit(), err, g);
#else
            h = trace_closest(s, o, d, kExtTmin, kExtTmax, err);
#endif
        }
        key = extend_key(s, h, fused, key);
#if VVPT_BLAS_WIDE && VVPT_GROUP_TRAVERSAL
        if (g.gl == 0)
#endif
        {
            ps.hit[slot] = make_float4(h.t, h.u, h.v, __uint_as_float(h.prim));
            ps.hit_inst[slot] = h.inst;
            q.ext_key[i] = key;
        }
    }
#endif
    if (blockIdx.x == 0 && threadIdx.x == 0)
        atomicAdd(&q.counters[C_SEGMENTS], n);
    if (err)
        atomicOr(&q.counters[C_ERR], err);
}

// Compacts the extension queue into the material-sorted shade queues and the
// emitter-walk queue (warp-uniform loop; uniform, cheap work per entry).
__global__ void __launch_bounds__(256) k_partition(PathState ps, Queues q, int pp)
{
    const uint32_t n = q.counters[C_EXT0 + pp];
    const uint32_t *queue = q.ext[pp];
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
        const uint32_t i = base + threadIdx.x;
        uint32_t slot = 0, key = 0xFFu;
        if (i < n) {
            slot = queue[i];
            key = q.ext_key[i];
        }
        const uint32_t bin = key & 3u;
        uint32_t pos = warp_append_all(bin == 0, &q.counters[C_SHADE_L]);
        if (bin == 0)
            q.shade_l[pos] = slot;
        pos = warp_append_all(bin == 1, &q.counters[C_SHADE_P]);
        if (bin == 1)
            q.shade_p[pos] = slot;
        pos = warp_append_all(bin == 2, &q.counters[C_SHADE_M]);
        if (bin == 2)
            q.shade_m[pos] = slot;
        const bool walk = key != 0xFFu && (key & 4u);
        pos = warp_append_all(walk, &q.counters[C_WALK]);
        if (walk)
            q.walk[pos] = slot;
    }
}

template <class Tracer>
__device__ __noinline__ void emitter_ray(const Tracer &trace, const SceneView &s, const RenderParams &p, float3 o,
                                         const float3 &dir, bool inside, uint32_t vol, float3 &out_em_T,
                                         float3 &out_T, float3 &out_em, float &out_pdf, uint32_t &err);

// The pending emitter rays whose first candidate is transparent (or below the
// extension ray's tmin): the full candidate walk, before shade adds this
// iteration's contributions.
__global__ void __launch_bounds__(256, VVPT_TRACE_MIN_BLOCKS) k_walk(JobTable jt, PathState ps, Queues q)
{
    const uint32_t n = q.counters[C_WALK];
    uint32_t err = 0;
    if (first_ray() < n)
        tlas_cache_fill(jt.jobs[ps.job[q.walk[first_ray()]]].scene);
    else
        tlas_cache_none();
#if VVPT_BLAS_WIDE && VVPT_GROUP_TRAVERSAL
    const GroupTracer trace{lane_group()};
    const bool writer = trace.g.gl == 0;
#else
    const LaneTracer trace{};
    const bool writer = true;
#endif
    for (uint32_t i = my_ray(); i < n; i += ray_stride()) {
        const uint32_t slot = q.walk[i];
        const JobView &J = jt.jobs[ps.job[slot]];
        const SceneView &s = J.scene;
        const RenderParams &p = J.params;
        const uint32_t flags = ps.flags[slot];
        const float4 nb = ps.nee_b[slot];
        float3 emT, T, em;
        float lpdf;
        emitter_ray(trace, s, p, f3(ps.o[slot]), f3(ps.d[slot]), (flags & F_INSIDE) != 0, ps.vol[slot], emT, T, em,
                    lpdf, err);
        group_sync();
        if (writer) {
            if (!is_black(em))
                ps.rad[slot] = f4(f3(ps.rad[slot]) + power_heuristic(nb.w, lpdf) * T * em * f3(nb), 0.0f);
            ps.flags[slot] = flags & ~(F_NEE_FUSED | F_NEE_FULL);
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0 && n)
        atomicAdd(&q.counters[C_NEE], n);
    if (err)
        atomicOr(&q.counters[C_ERR], err);
}

// Volume free flight on the current segment; returns true when the path
// scattered in the medium (sampledMedium) and writes the scatter point.
__device__ __forceinline__ bool medium_event(const SceneView &s, const RenderParams &p, uint32_t vol, float vtstart,
                                             float vtend, const float3 &origin, const float3 &raydir, float3 &beta,
                                             PathRng &rng, float3 &scatter_pos, float &g)
{
    Medium md = load_medium(s, vol);
    g = md.g;
    float3 dirn = normalize3(raydir);
    float dist_in = fmaxf(vtend - vtstart, kEps);
    uint32_t channel = min((uint32_t)(rnd1(p, rng) * 3.0f), 2u);
    float u = rnd1(p, rng);
    float hit_dist = -logf(1.0f - u) / comp(md.sigma_t, channel);
    bool sampled = hit_dist < dist_in;
    float td = fminf(hit_dist, dist_in);
    float3 tr = f3(expf(-md.sigma_t.x * td), expf(-md.sigma_t.y * td), expf(-md.sigma_t.z * td));
    float3 density = sampled ? md.sigma_t * tr : tr;
    float pdf = 0.0f;
    pdf += density.x;
    pdf += density.y;
    pdf += density.z;
    pdf *= 0.3333333f;
    if (pdf == 0.0f)
        pdf = 1.0f;
    float3 F = sampled ? (tr * md.sigma_s / pdf) : (tr / pdf);
    beta *= F;
    if (sampled)
        scatter_pos = origin + (vtstart + hit_dist) * dirn;
    return sampled;
}

__device__ __noinline__ float3 fused_nee(const SceneView &s, const RenderParams &p, bool full, bool is_hit,
                                         uint32_t inst_id, float4 hv, float3 o, float3 dir, bool inside, uint32_t vol,
                                         float4 nb, uint32_t &err, uint32_t &walks);

// One shading event per queued path: the body of rayPrimary*.rchit.glsl:45-175
// (hits) or rayPrimary.rmiss.glsl:40-106 (misses), followed by Russian
// roulette (russian_roulette.glsl:1-11).
// One kernel per material-sorted queue (k_partition): KIND 0 shades the
// Lambert hits, 1 the metallic/roughness hits, 2 the misses. Each is compiled
// for its own case only (the other surface models are dead code there), so
// the Lambert and miss kernels fit more resident blocks than the
// metallic/roughness one.
// VVPT_SHADE_SHARED_BSDF: one call site for the cosine-weighted warp and one
// copy of the metallic/roughness evaluation in the surface event.
#ifndef VVPT_SHADE_SHARED_BSDF
#define VVPT_SHADE_SHARED_BSDF 1
#endif
template <int KIND>
__global__ void __launch_bounds__(256, KIND == 0 || KIND == 2 ? VVPT_SHADE_LM_MIN_BLOCKS : VVPT_SHADE_MIN_BLOCKS)
    k_shade(JobTable jt, PathState ps, Queues q, int pp)
{
    // KIND 3: all three queues in one launch (VVPT_SHADE_SPLIT = 0)
    const uint32_t nl = q.counters[C_SHADE_L], np = q.counters[C_SHADE_P];
    const uint32_t n = KIND == 3 ? nl + np + q.counters[C_SHADE_M]
                                 : q.counters[KIND == 0 ? C_SHADE_L : (KIND == 1 ? C_SHADE_P : C_SHADE_M)];
    const uint32_t *queue = KIND == 0 ? q.shade_l : (KIND == 1 ? q.shade_p : q.shade_m);
    auto entry = [&](uint32_t i) {
        if (KIND != 3)
            return queue[i];
        return i < nl ? q.shade_l[i] : (i < nl + np ? q.shade_p[i - nl] : q.shade_m[i - nl - np]);
    };
    uint32_t err = 0, walks = 0;
    {
        const uint32_t f = blockIdx.x * blockDim.x;
        if (f < n)
            tlas_cache_fill(jt.jobs[ps.job[entry(f)]].scene);
        else
            tlas_cache_none();
    }
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
        const uint32_t i = base + threadIdx.x;
        uint32_t slot = 0;
        bool want_conn = false, want_nee = false, want_done = false, want_ext = false;
        if (i < n) {
        slot = entry(i);
        const JobView &J = jt.jobs[ps.job[slot]];
        const SceneView &s = J.scene;
        const RenderParams &p = J.params;

        uint32_t flags = ps.flags[slot];
        PathRng rng = load_rng(p, ps, slot);
        float3 beta = f3(ps.beta[slot]);
        float3 rad = f3(ps.rad[slot]);
        if (flags & F_NEE) // the previous event's emitter ray (a path that continued with zfar > kExtTmax)
            rad = rad + f3(ps.nee_c[slot]);
        float3 origin = f3(ps.o[slot]);
        float3 dir = f3(ps.d[slot]);
        uint32_t vol = ps.vol[slot];
        const uint32_t d = (flags >> kDepthShift) & kByteMask;
        uint32_t sdepth = (flags >> kSurfShift) & kByteMask;
        bool inside = (flags & F_INSIDE) != 0;
        const float4 hv = ps.hit[slot];
        const uint32_t inst_id = ps.hit_inst[slot];
        const bool is_hit = KIND == 3 ? inst_id != kNoHit : KIND != 2; // hits (0, 1) or misses (2)

        // the previous event's emitter ray, added before this event's own
        // contributions (next_event_estimation.glsl:28-32 runs inside the
        // previous hit shader)
        if (flags & F_NEE_FUSED)
            rad += fused_nee(s, p, (flags & F_NEE_FULL) != 0, is_hit, inst_id, hv, origin, dir, inside, vol,
                             ps.nee_b[slot], err, walks);

        bool stop = false;
        bool terminal_no_rr = false; // returns before the RR block
        bool has_shadow = false, has_nee = false;
        bool sampled = false;        // a new direction was sampled here (pdf in nee_pdf)
        bool keep_sampled = false;   // pass-through: the direction keeps its sampling pdf
        const bool last = (d + 1u >= p.depth);
        float3 sh_dir = f3(0.0f), sh_c = f3(0.0f);
        float sh_tmax = 0.0f;
        float3 nee_beta = f3(0.0f);
        float nee_pdf = 0.0f;
        bool write_alb = false;
        float3 new_alb = f3(0.0f), new_nrm = f3(0.0f);

        // ---- medium along the segment
        bool sampled_medium = false;
        float3 scatter_pos = f3(0.0f);
        float g = 0.0f;
        if (inside && vol < s.num_materials) {
            float vtend = is_hit ? hv.x : fminf(p.zfar_trunc, kExtTmax);
            sampled_medium = medium_event(s, p, vol, kExtTmin, vtend, origin, dir, beta, rng, scatter_pos, g);
        }
        // The event's own part first; an event that samples a light (a
        // scatter point in a medium, or a surface the path continues from)
        // then samples it at one call site, so that the light-sampling code
        // (mesh lights, environment) is inlined once; the evaluation after it
        // follows per event. The random numbers are drawn in the same order.
        SurfaceHit h;
        bool lambert = false, surface_light = false;
        float3 albedo = f3(0.0f);
        PBR pbr;
        if (sampled_medium) {
            // light sample at the scatter point with the HG phase function
            // (process_volume_hit.glsl:42-79), below
        } else if (!is_hit) {
            // miss: background (rayPrimary.rmiss.glsl:53-103)
            stop = true;
            terminal_no_rr = true;
            const int mode = (int)p.env_type;
            // with the environment light-sampled, a sampled direction's escape
            // takes the BSDF side of the MIS weight
            float wenv = 1.0f;
            if (p.env_light && (flags & F_SAMPLED))
                wenv = power_heuristic(ps.nee_b[slot].w, env_pdf(s, dir) / (float)(p.num_lights + 1u));
            // one environment lookup for modes 1 and 2 (one inlined copy)
            const bool env_seen = mode == 1 || (mode == 2 && sdepth != 0);
            const float3 envc = env_seen ? env_lookup(s, dir) : f3(0.0f);
            if (mode == 0) {
                if (sdepth == 0) {
                    write_alb = true;
                    new_alb = p.background;
                    new_nrm = f3(0.0f);
                }
                rad += p.background * beta;
            } else if (mode == 1) {
                float3 bg = p.env_intensity * envc;
                if (sdepth == 0) {
                    write_alb = true;
                    new_alb = bg;
                    new_nrm = f3(0.0f);
                }
                rad += bg * beta * wenv;
            } else if (mode == 2) {
                if (sdepth == 0) {
                    write_alb = true;
                    new_alb = p.background;
                    new_nrm = f3(0.0f);
                    rad += p.background * beta;
                } else {
                    rad += envc * beta * wenv;
                }
            }
        } else {
            // surface event
            const uint32_t prim = __float_as_uint(hv.w);
            h = make_surface_hit(s, inst_id, prim, hv.y, hv.z, dir);
            const DevMaterial &m = s.materials[h.material];
            const float2 tuv = make_float2(h.uv.x * m.uv_tiling.x, h.uv.y * m.uv_tiling.y);
            lambert = KIND == 3 ? (uint32_t)m.uv_tiling.z == 2u : KIND == 0;
            bool passthrough = false;
            if (m.mrao.w > 0.0f) {
                float alpha = material_alpha(s, m, tuv);
                float r = rnd1(p, rng);
                if (alpha < kEps || r > alpha) {
                    if (h.front_volume != h.back_volume) {
                        inside = false;
                        int nv = h.flipped ? h.front_volume : h.back_volume;
                        if (nv != -1) {
                            inside = true;
                            vol = (uint32_t)nv;
                        }
                    }
                    origin = h.wpos;
                    dir = normalize3(dir);
                    passthrough = true;
                    keep_sampled = (flags & F_SAMPLED) != 0;
                }
            }
            if (passthrough) {
                terminal_no_rr = true; // returns without RR and without stop
            } else {
                float4 nm = tex2d(s, m.tex2[1], tuv.x, tuv.y);
                apply_normal_to_frame(h.frame, normal_from_normal_map(f3(nm)));
                albedo = f3(m.albedo) * f3(tex2d(s, m.tex1[0], tuv.x, tuv.y));
                float3 emissive = material_emissive(s, m, tuv);
                if (!lambert) {
                    pbr.albedo = albedo;
                    pbr.metallic = m.mrao.x * tex2d(s, m.tex1[1], tuv.x, tuv.y).x;
                    pbr.roughness = m.mrao.y * tex2d(s, m.tex1[2], tuv.x, tuv.y).x;
                    pbr.roughness = fmaxf(pbr.roughness, 0.035f);
                }
                if (sdepth == 0) {
                    write_alb = true;
                    new_alb = albedo;
                    new_nrm = h.frame.n * 0.5f + f3(0.5f);
                }
                const float em_eps = lambert ? 0.05f : 0.1f;
                if (sdepth == 0 && !is_black_eps(emissive, em_eps) && !h.flipped) {
                    rad += emissive * beta;
                    stop = true;
                    terminal_no_rr = true;
                } else {
                    sdepth = min(sdepth + 1u, 255u);
                    surface_light = true;
                }
            }
        }
        if (sampled_medium || surface_light) {
            // in background mode 2 an escape before any surface event sees
            // the solid colour, so the environment is not a light there
            const LightSample ls =
                sample_light(s, p, sampled_medium ? scatter_pos : h.wpos, rng,
                             sampled_medium ? !last && !((int)p.env_type == 2 && sdepth == 0) : !last);
            if (sampled_medium) {
                float3 wo = -normalize3(dir);
                if (!is_black(ls.radiance)) {
                    float ph = henyey_greenstein(dot3(wo, ls.dir), g);
                    float3 F = f3(ph);
                    if (!is_black(F)) {
                        float w = ls.delta ? 1.0f : power_heuristic(ls.pdf, ph);
                        has_shadow = true;
                        sh_dir = ls.dir;
                        sh_tmax = ls.tmax;
                        sh_c = (ls.delta ? ls.radiance : w * ls.radiance) * F * beta / ls.pdf;
                    }
                }
                float3 wi;
                const float2 uu = rnd2(p, rng);
                const float u0 = uu.x, u1 = uu.y;
                float spdf = hg_sample(wo, wi, u0, u1, g);
                origin = scatter_pos;
                dir = wi;
                has_nee = true;
                sampled = true;
                nee_beta = beta;
                nee_pdf = spdf;
            } else {
                const float3 wo = world_to_local(h.frame, -dir);
#if VVPT_SHADE_SHARED_BSDF
                // The BSDF sample's numbers follow the light sample's, as
                // always; the cosine-weighted warp serves Lambert surfaces
                // and the metallic/roughness diffuse lobe from one call site,
                // and one copy of the metallic/roughness evaluation (a loop
                // that is not unrolled) takes the light's direction and the
                // sampled one. Same arithmetic as sample_pbr.
                const float2 uu = rnd2(p, rng);
                const float rl = lambert ? 0.0f : rnd1(p, rng);
                float spdf = 0.0f;
                float3 sdir_local;
                if (lambert || rl <= diffuse_sampling_ratio(pbr))
                    sdir_local = cosine_sample_hemisphere(uu.x, uu.y, spdf);
                else
                    sdir_local = ggx_sample_reflect(wo, pbr, uu.x, uu.y);
                const float3 wil = world_to_local(h.frame, ls.dir);
                float3 Fl = f3(0.0f), Fsm = f3(0.0f);
                float pl = 0.0f, psm = 0.0f;
                if (lambert) {
                    const float ct = fminf(fmaxf(wil.y, 0.0f), 1.0f);
                    Fl = albedo * kInvPi * ct;
                    pl = cosine_hemisphere_pdf(ct);
                } else {
#pragma unroll 1
                    for (int k = 0; k < 2; k++) {
                        const float3 wi = k == 0 ? wil : sdir_local;
                        const float3 F = eval_pbr(pbr, wi, wo, normalize3(wo + wi));
                        const float pd = pdf_pbr(wi, wo, pbr);
                        if (k == 0) {
                            Fl = F;
                            pl = ls.delta ? 0.0f : pd;
                        } else {
                            Fsm = F;
                            psm = pd;
                        }
                    }
                }
                if (!is_black(ls.radiance) && !is_black(Fl)) {
                    float w = ls.delta ? 1.0f : power_heuristic(ls.pdf, pl);
                    has_shadow = true;
                    sh_dir = ls.dir;
                    sh_tmax = ls.tmax;
                    sh_c = (ls.delta ? ls.radiance : w * ls.radiance) * Fl * beta / ls.pdf;
                }
                bool black_f = false;
                float3 Fs = f3(0.0f);
                if (!lambert) {
                    spdf = psm;
                    Fs = psm < kEps ? f3(0.0f) : Fsm;
                    black_f = is_black(Fs);
                }
#else
                if (!is_black(ls.radiance)) {
                    float3 wi = world_to_local(h.frame, ls.dir);
                    float3 F;
                    float bpdf;
                    if (lambert) {
                        float ct = fminf(fmaxf(wi.y, 0.0f), 1.0f);
                        F = albedo * kInvPi * ct;
                        bpdf = cosine_hemisphere_pdf(ct);
                    } else {
                        F = eval_pbr(pbr, wi, wo, normalize3(wo + wi));
                        bpdf = ls.delta ? 0.0f : pdf_pbr(wi, wo, pbr);
                    }
                    if (!is_black(F)) {
                        float w = ls.delta ? 1.0f : power_heuristic(ls.pdf, bpdf);
                        has_shadow = true;
                        sh_dir = ls.dir;
                        sh_tmax = ls.tmax;
                        sh_c = (ls.delta ? ls.radiance : w * ls.radiance) * F * beta / ls.pdf;
                    }
                }
                // BSDF sampling
                float spdf;
                float3 sdir_local;
                bool black_f = false;
                float3 Fs;
                if (lambert) {
                    const float2 uu = rnd2(p, rng);
                    const float u0 = uu.x, u1 = uu.y;
                    sdir_local = cosine_sample_hemisphere(u0, u1, spdf);
                } else {
                    const float2 uu = rnd2(p, rng);
                    const float u0 = uu.x, u1 = uu.y;
                    float r = rnd1(p, rng);
                    Fs = sample_pbr(sdir_local, wo, spdf, pbr, u0, u1, r);
                    black_f = is_black(Fs);
                }
#endif
                float3 sdir = local_to_world(h.frame, sdir_local);
                origin = h.wpos;
                dir = sdir;
                if (lambert) {
                    beta *= albedo;
                    has_nee = true;
                } else if (black_f) {
                    stop = true;
                    terminal_no_rr = true;
                } else {
                    beta *= clamp3(Fs / spdf, 0.0f, 1.0f);
                    has_nee = true;
                }
                sampled = has_nee;
                nee_beta = beta;
                nee_pdf = spdf;
            }
        }
        // Russian roulette (russian_roulette.glsl:1-11) for events that reach it
        if (!terminal_no_rr) {
            float rr = rnd1(p, rng);
            if (d > kRussianRouletteDepth) {
                float mb = fmaxf(beta.x, fmaxf(beta.y, beta.z));
                if (rr >= mb)
                    stop = true;
                else
                    beta = beta * (1.0f / mb);
            }
        }
        if (has_nee && p.num_lights == 0u) {
            // With no lights the reference's emitter pdf is
            // lightDirectPdf * (1 / 0) = inf (rayNEE.rahit.glsl:124), so the
            // MIS weight and the contribution are zero: skip the ray.
            has_nee = false;
        }
        if (has_nee && !may_reach_emitter(s, origin, dir))
            has_nee = false; // no emissive surface on its line: it adds zero

        const bool done = stop || last;
        uint32_t nf = F_ITEM | (inside ? F_INSIDE : 0u) | ((min(d + 1u, 255u)) << kDepthShift) | (sdepth << kSurfShift);
        if (done)
            nf |= F_DONE;
        if (has_shadow)
            nf |= F_SHADOW;
        if (sampled || keep_sampled)
            nf |= F_SAMPLED;
        // a continuing path's emitter ray shares origin and direction with its
        // next extension ray and is resolved from that traversal
        const bool fuse = has_nee && !done && p.zfar <= kExtTmax;
        if (has_nee)
            nf |= fuse ? F_NEE_FUSED : F_NEE;
        ps.flags[slot] = nf;
        ps.rng[slot] = rng.s;
        ps.beta[slot] = f4(beta, 0.0f);
        ps.rad[slot] = f4(rad, 0.0f);
        ps.o[slot] = f4(origin, 0.0f);
        ps.d[slot] = f4(dir, 0.0f);
        ps.vol[slot] = vol;
        if (write_alb) {
            ps.alb[slot] = f4(new_alb, 0.0f);
            ps.nrm[slot] = f4(new_nrm, 0.0f);
        }
        if (has_shadow) {
            ps.sh_dir[slot] = f4(sh_dir, sh_tmax);
            ps.sh_c[slot] = f4(sh_c, 0.0f);
        }
        if (sampled)
            ps.nee_b[slot] = f4(nee_beta, nee_pdf);
        want_conn = has_shadow;
        want_nee = has_nee && !fuse;
        want_done = done;
        want_ext = !done;
        }
        uint32_t pos = warp_append_all(want_conn, &q.counters[C_CONN]);
        if (want_conn)
            q.conn[pos] = slot;
        pos = warp_append_all(want_nee, &q.counters[C_NEEQ]);
        if (want_nee)
            q.nee[pos] = slot;
        pos = warp_append_all(want_done, &q.counters[C_REGEN0 + (1 - pp)]);
        if (want_done)
            q.regen[1 - pp][pos] = slot;
        pos = warp_append_all(want_ext, &q.counters[C_EXT0 + (1 - pp)]);
        if (want_ext)
            q.ext[1 - pp][pos] = slot;
    }
    warp_add(&q.counters[C_NEE], walks);
    if (err)
        atomicOr(&q.counters[C_ERR], err);
}

// Shadow ray with transparent surfaces and media (lightSampling.glsl:108-144,
// raySecondary.rahit.glsl:31-72, raySecondary.rchit.glsl:32-78,
// raySecondary.rmiss.glsl:17-44). Candidates are processed nearest first.
template <class Tracer>
__device__ float3 shadow_transmittance(const Tracer &trace, const SceneView &s, const RenderParams &p, float3 o,
                                       const float3 &dir, float tmax_light, bool inside, uint32_t vol, uint32_t &err)
{
    const float tmin = kConnTmin;
    float3 T = f3(1.0f);
    bool shadowed = false;
    bool stop = false;
    float distT = tmax_light - tmin;
    for (uint32_t seg = 0; seg < p.depth; seg++) {
        float vtmin = tmin;
        Hit after = no_hit();
        bool accepted = false;
        Hit acc;
        int guard = 0;
        for (;;) {
            Hit h = trace(s, o, dir, tmin, distT, after, err);
            if (h.inst == kNoHit)
                break;
            if (++guard > kCandidateCap) {
                err |= kErrLoopCap;
                stop = shadowed = true;
                accepted = true;
                acc = h;
                break;
            }
            const DevInstance &inst = s.instances[h.inst];
            const DevMaterial &m = s.materials[inst.material];
            if (!(m.mrao.w >= 0.99f)) {
                stop = shadowed = true;
                accepted = true;
                acc = h;
                break;
            }
            // alpha needs the hit's uv
            ShadeVertex a, b, c;
            fetch_triangle(s, inst, h.prim, a, b, c);
            float bx = 1.0f - h.u - h.v;
            float2 uv = make_float2(a.pos_u.w * bx + b.pos_u.w * h.u + c.pos_u.w * h.v,
                                    a.nrm_v.w * bx + b.nrm_v.w * h.u + c.nrm_v.w * h.v);
            float alpha = material_alpha(s, m, make_float2(uv.x * m.uv_tiling.x, uv.y * m.uv_tiling.y));
            T *= f3(1.0f - alpha);
            if (inst.front_volume != inst.back_volume) {
                accepted = true;
                acc = h;
                break;
            }
            if (max3f(T) > kEps) {
                shadowed = false;
                after = h;
                continue;
            }
            stop = shadowed = true;
            accepted = true;
            acc = h;
            break;
        }
        if (!accepted) {
            // miss shader
            stop = true;
            shadowed = false;
            if (inside && vol < s.num_materials) {
                float vtend = fminf(p.zfar_trunc, distT);
                T *= medium_transmittance(s, vol, vtmin, vtend);
                shadowed = !(max3f(T) > kEps);
            }
        } else if (!stop) {
            // closest hit on a volume boundary
            SurfaceHit sh = make_surface_hit(s, acc.inst, acc.prim, acc.u, acc.v, dir);
            bool ended = false;
            if (inside && vol < s.num_materials) {
                T *= medium_transmittance(s, vol, vtmin, acc.t);
                if (max3f(T) < kEps) {
                    stop = shadowed = true;
                    ended = true;
                }
            }
            if (!ended) {
                vtmin = acc.t;
                inside = false;
                int nv = sh.flipped ? sh.front_volume : sh.back_volume;
                if (nv != -1) {
                    inside = true;
                    vol = (uint32_t)nv;
                }
                o = sh.wpos;
            }
        }
        distT -= vtmin;
        if (stop)
            break;
    }
    if (shadowed)
        T = f3(0.0f);
    return T;
}

// An emitter reached by the BSDF-direction ray (rayNEE.rahit.glsl:73-131):
// medium transmittance up to the hit, back-face rejection, and the light pdf
// of having sampled that point, with the squared distance measured from the
// object-space ray origin as the reference does (rayNEE.rahit.glsl:122).
__device__ __forceinline__ void emitter_eval(const SceneView &s, const RenderParams &p, const DevInstance &inst,
                                             const ShadeVertex &a, const ShadeVertex &b, const ShadeVertex &c,
                                             const Hit &h, const float3 &e, const float3 &o, const float3 &dir,
                                             bool inside, uint32_t vol, float vtmin, float3 &T, float3 &em, float &pdf)
{
    if (inside && vol < s.num_materials) {
        T *= medium_transmittance(s, vol, vtmin, h.t);
        if (max3f(T) < kEps) {
            T = f3(0.0f);
            em = f3(0.0f);
            return;
        }
    }
    const float bx = 1.0f - h.u - h.v;
    Affine34 w2o = rows_of(inst.w2o), o2w = rows_of(inst.o2w);
    float3 ln = f3(a.nrm_v) * bx + f3(b.nrm_v) * h.u + f3(c.nrm_v) * h.v;
    float3 wn = normalize3(xform_normal_transposed(w2o, ln));
    if (dot3(wn, dir) > 0.0f) { // back face
        em = f3(0.0f);
        T = f3(0.0f);
        return;
    }
    em = e;
    float3 lp = f3(a.pos_u) * bx + f3(b.pos_u) * h.u + f3(c.pos_u) * h.v;
    float3 wp = xform_point(o2w, lp);
    float3 p0 = xform_point(o2w, f3(a.pos_u)), p1 = xform_point(o2w, f3(b.pos_u)), p2 = xform_point(o2w, f3(c.pos_u));
    float area = 0.5f * length3(cross3(p1 - p0, p2 - p0));
    float point_pdf = (1.0f / (float)inst.num_triangles) * (1.0f / area);
    float dp = dot3(-dir, wn);
    if (dp > 0.0f) {
        float3 obj_o = xform_point(w2o, o);
        float dist = length3(obj_o - wp);
        float light_pdf = point_pdf * (dist * dist) / dp;
        pdf = light_pdf * (1.0f / (float)(p.num_lights + p.env_light));
    } else {
        pdf = 0.0f;
        em = f3(0.0f);
    }
}

// BSDF-direction emitter ray (next_event_estimation.glsl:1-33,
// rayNEE.rahit.glsl:32-132, rayNEE.rchit.glsl:33-82, rayNEE.rmiss.glsl:12-19).
// Returns the emitter radiance times throughput and its light pdf.
template <class Tracer>
__device__ __noinline__ void emitter_ray(const Tracer &trace, const SceneView &s, const RenderParams &p, float3 o,
                                         const float3 &dir, bool inside, uint32_t vol, float3 &out_em_T,
                                         float3 &out_T, float3 &out_em, float &out_pdf, uint32_t &err)
{
    const float tmin = kConnTmin;
    const float tmax = p.zfar;
    float3 T = f3(1.0f);
    float3 em = f3(0.0f);
    float pdf = 0.0f;
    bool stop = false;
    for (uint32_t seg = 0; seg < p.depth; seg++) {
        float vtmin = tmin;
        Hit after = no_hit();
        bool accepted = false;
        Hit acc;
        int guard = 0;
        for (;;) {
            Hit h = trace(s, o, dir, tmin, tmax, after, err);
            if (h.inst == kNoHit)
                break;
            if (++guard > kCandidateCap) {
                err |= kErrLoopCap;
                stop = true;
                T = f3(0.0f);
                em = f3(0.0f);
                accepted = true;
                acc = h;
                break;
            }
            const DevInstance &inst = s.instances[h.inst];
            const DevMaterial &m = s.materials[inst.material];
            ShadeVertex a, b, c;
            fetch_triangle(s, inst, h.prim, a, b, c);
            float bx = 1.0f - h.u - h.v;
            float2 uv = make_float2(a.pos_u.w * bx + b.pos_u.w * h.u + c.pos_u.w * h.v,
                                    a.nrm_v.w * bx + b.nrm_v.w * h.u + c.nrm_v.w * h.v);
            float2 tuv = make_float2(uv.x * m.uv_tiling.x, uv.y * m.uv_tiling.y);
            float3 e = material_emissive(s, m, tuv);
            const bool transparent = m.mrao.w >= 0.99f;
            if (is_black_eps(e, 0.05f)) {
                if (!transparent) {
                    stop = true;
                    T = f3(0.0f);
                    em = f3(0.0f);
                    accepted = true;
                    acc = h;
                    break;
                }
                float alpha = material_alpha(s, m, tuv);
                T *= f3(1.0f - alpha);
                if (inst.front_volume != inst.back_volume) {
                    accepted = true;
                    acc = h;
                    break;
                }
                after = h;
                continue;
            }
            // emissive surface
            stop = true;
            accepted = true;
            acc = h;
            emitter_eval(s, p, inst, a, b, c, h, e, o, dir, inside, vol, vtmin, T, em, pdf);
            break;
        }
        if (!accepted) {
            stop = true;
            em = f3(0.0f);
            pdf = 0.0f;
        } else if (!stop) {
            SurfaceHit sh = make_surface_hit(s, acc.inst, acc.prim, acc.u, acc.v, dir);
            bool ended = false;
            if (inside && vol < s.num_materials) {
                T *= medium_transmittance(s, vol, vtmin, acc.t);
                if (max3f(T) < kEps) {
                    stop = true;
                    T = f3(0.0f);
                    em = f3(0.0f);
                    ended = true;
                }
            }
            if (!ended) {
                vtmin = acc.t;
                inside = false;
                int nv = sh.flipped ? sh.front_volume : sh.back_volume;
                if (nv != -1) {
                    inside = true;
                    vol = (uint32_t)nv;
                }
                o = sh.wpos;
            }
        }
        if (stop)
            break;
    }
    out_T = T;
    out_em = em;
    out_pdf = pdf;
    out_em_T = T * em;
}

// The previous event's BSDF-direction emitter ray, resolved from this
// iteration's extension hit: the two rays share origin and direction, and the
// extension traversal starts at the emitter ray's tmin (1e-4) when one is
// pending, so the extension hit is the emitter ray's first candidate unless
// extend flagged a candidate below 1e-3 (`full`). Candidates beyond zfar are a
// miss for the emitter ray; a transparent first candidate needs the complete
// candidate walk of emitter_ray.
__device__ __noinline__ float3 fused_nee(const SceneView &s, const RenderParams &p, bool full, bool is_hit,
                                         uint32_t inst_id, float4 hv, float3 o, float3 dir, bool inside, uint32_t vol,
                                         float4 nb, uint32_t &err, uint32_t &walks)
{
    float3 T = f3(1.0f), em = f3(0.0f);
    float pdf = 0.0f;
    if (!full && is_hit && hv.x <= p.zfar) {
        Hit h;
        h.t = hv.x;
        h.u = hv.y;
        h.v = hv.z;
        h.inst = inst_id;
        h.prim = __float_as_uint(hv.w);
        const DevInstance &inst = s.instances[inst_id];
        const DevMaterial &m = s.materials[inst.material];
        ShadeVertex a, b, c;
        fetch_triangle(s, inst, h.prim, a, b, c);
        const float bx = 1.0f - h.u - h.v;
        float2 uv = make_float2(a.pos_u.w * bx + b.pos_u.w * h.u + c.pos_u.w * h.v,
                                a.nrm_v.w * bx + b.nrm_v.w * h.u + c.nrm_v.w * h.v);
        float2 tuv = make_float2(uv.x * m.uv_tiling.x, uv.y * m.uv_tiling.y);
        float3 e = material_emissive(s, m, tuv);
        if (is_black_eps(e, 0.05f)) {
            if (m.mrao.w >= 0.99f)
                full = true; // transparent: walk the candidates
        } else {
            emitter_eval(s, p, inst, a, b, c, h, e, o, dir, inside, vol, kConnTmin, T, em, pdf);
        }
    }
    if (full) {
        float3 emT;
        emitter_ray(LaneTracer{}, s, p, o, dir, inside, vol, emT, T, em, pdf, err);
        walks++;
    }
    if (is_black(em))
        return f3(0.0f);
    return power_heuristic(nb.w, pdf) * T * em * f3(nb);
}

// Shadow rays of the events shaded this iteration, then the BSDF-direction
// emitter rays of the paths that end at this event (their own queue, after
// the shadow entries, in the same launch: the few long emitter walks overlap
// the shadow rays instead of forming a launch of their own). An emitter ray's
// contribution goes to nee_c, so the two parts never write the same word;
// regen (or shade, for a path that continues) adds it after the shadow ray's,
// in the order of the reference's additions.
// One shadow ray of shadow_transmittance as a resumable walk for the lane
// refill loop of k_shadow: the candidate logic between two traversals, with
// the same decisions in the same order. The walk's ray and traversal live in
// the TraceState (st.o is the current segment's origin); the candidate loop
// of a segment always starts at kConnTmin.
struct ShadowWalk {
    float3 T;
    float distT;
    uint32_t vol, seg, guard;
    bool inside;
};

// The transparent-candidate part of the walk (alpha, volume boundaries), out
// of line: it is rare on most scenes, and inline its registers would crowd
// the traversal state of the refill loop. Returns 0 when T is final, 1 to go
// on past the candidate, 2 to start the next segment at `next_o`.
__device__ __noinline__ int shadow_walk_transparent(ShadowWalk &w, const SceneView &s, const RenderParams &p,
                                                    const Hit h, const float3 dir, float3 &next_o)
{
    const float tmin = kConnTmin;
    const DevInstance &inst = s.instances[h.inst];
    const DevMaterial &m = s.materials[inst.material];
    // alpha needs the hit's uv
    ShadeVertex a, b, c;
    fetch_triangle(s, inst, h.prim, a, b, c);
    const float bx = 1.0f - h.u - h.v;
    const float2 uv = make_float2(a.pos_u.w * bx + b.pos_u.w * h.u + c.pos_u.w * h.v,
                                  a.nrm_v.w * bx + b.nrm_v.w * h.u + c.nrm_v.w * h.v);
    const float alpha = material_alpha(s, m, make_float2(uv.x * m.uv_tiling.x, uv.y * m.uv_tiling.y));
    w.T *= f3(1.0f - alpha);
    if (inst.front_volume != inst.back_volume) {
        // closest hit on a volume boundary: the segment ends here
        const SurfaceHit sh = make_surface_hit(s, h.inst, h.prim, h.u, h.v, dir);
        if (w.inside && w.vol < s.num_materials) {
            w.T *= medium_transmittance(s, w.vol, tmin, h.t);
            if (max3f(w.T) < kEps) {
                w.T = f3(0.0f);
                return 0;
            }
        }
        w.inside = false;
        const int nv = sh.flipped ? sh.front_volume : sh.back_volume;
        if (nv != -1) {
            w.inside = true;
            w.vol = (uint32_t)nv;
        }
        w.distT -= h.t;
        if (++w.seg >= p.depth)
            return 0;
        w.guard = 0;
        next_o = sh.wpos;
        return 2;
    }
    if (max3f(w.T) > kEps)
        return 1;
    w.T = f3(0.0f);
    return 0;
}

// Result of one finished traversal of the walk: true while the walk goes on
// (a new traversal has been begun, after the candidate `after`), false when
// T is final (zero if shadowed).
__device__ __forceinline__ bool shadow_walk_next(ShadowWalk &w, Hit &after, TraceState &st, const SceneView &s,
                                                 const RenderParams &p, uint32_t &err)
{
    const float tmin = kConnTmin;
    const Hit h = st.best;
    if (h.inst == kNoHit) {
        // miss shader
        if (w.inside && w.vol < s.num_materials) {
            w.T *= medium_transmittance(s, w.vol, tmin, fminf(p.zfar_trunc, w.distT));
            if (!(max3f(w.T) > kEps))
                w.T = f3(0.0f);
        }
        return false;
    }
    if (++w.guard > (uint32_t)kCandidateCap) {
        err |= kErrLoopCap;
        w.T = f3(0.0f);
        return false;
    }
    if (!(s.materials[s.instances[h.inst].material].mrao.w >= 0.99f)) {
        w.T = f3(0.0f);
        return false;
    }
    float3 next_o;
    const int r = shadow_walk_transparent(w, s, p, h, st.d, next_o);
    if (r == 0)
        return false;
    if (r == 2) {
        after = no_hit();
        trace_begin(st, s, next_o, st.d, tmin, w.distT, after);
    } else {
        after = h;
        trace_begin(st, s, st.o, st.d, tmin, w.distT, after);
    }
    return true;
}

// Lane refill for the shadow kernel (as in k_extend; binary BLAS only), a
// build option, off: shadow rays aim at the same few lights, and the rays of
// one warp taken together share their node fetches in L1; a warp of rays at
// different stages does not. Measured on the 1080p medium scene at 64 spp:
// shadow launch 37 % of the step with refill against 27 % without (L1 hit
// rate 50 against 62 %, long-scoreboard stalls 18 against 4 cycles per
// issued instruction), 137.6 against 160.4 M paths/s.
#ifndef VVPT_SHADOW_REFILL
#define VVPT_SHADOW_REFILL 0
#endif
#ifndef VVPT_SHADOW_REFILL_BELOW
#define VVPT_SHADOW_REFILL_BELOW VVPT_REFILL_BELOW
#endif

__global__ void __launch_bounds__(256, VVPT_TRACE_MIN_BLOCKS) k_shadow(JobTable jt, PathState ps, Queues q)
{
    const uint32_t nc = q.counters[C_CONN];
    const uint32_t n = nc + q.counters[C_NEEQ];
    uint32_t err = 0;
    uint32_t nsh = 0, nnee = 0;
#if VVPT_SHADOW_REFILL
    // Shadow rays step by step with refill; an emitter ray (the entries past
    // the connection queue, a few per cent) runs its whole walk when its lane
    // takes it.
    if (n > 0) {
        const uint32_t b0 = min(first_ray(), n - 1u);
        tlas_cache_fill(jt.jobs[ps.job[b0 < nc ? q.conn[b0] : q.nee[b0 - nc]]].scene);
    } else {
        tlas_cache_none();
    }
    // per lane: the walk's transmittance and remaining distance; slot,
    // volume, segment, candidate count | inside << 31
    __shared__ float4 cold_t[256];
    __shared__ uint4 cold_w[256];
    TraceState st;
    TraceStack stack;
    Hit after = no_hit();
    uint32_t state = kLaneFree, job = 0;
    bool open = true; // warp-uniform: the queues may still hold rays
    for (;;) {
        uint32_t tr = __ballot_sync(0xFFFFFFFFu, state == kLaneTracing);
        if (__popc(tr) <= VVPT_SHADOW_REFILL_BELOW) {
            if (state == kLaneDone) {
                const JobView &J = jt.jobs[job];
                const float4 ct = cold_t[threadIdx.x];
                const uint4 cw = cold_w[threadIdx.x];
                ShadowWalk w;
                w.T = f3(ct);
                w.distT = ct.w;
                w.vol = cw.y;
                w.seg = cw.z;
                w.guard = cw.w & 0x7FFFFFFFu;
                w.inside = (cw.w >> 31) != 0;
                if (shadow_walk_next(w, after, st, J.scene, J.params, err)) {
                    cold_t[threadIdx.x] = f4(w.T, w.distT);
                    cold_w[threadIdx.x] = make_uint4(cw.x, w.vol, w.seg, w.guard | (w.inside ? 0x80000000u : 0u));
                    state = kLaneTracing;
                } else {
                    const uint32_t slot = cw.x;
                    if (!is_black(w.T))
                        ps.rad[slot] = f4(f3(ps.rad[slot]) + f3(ps.sh_c[slot]) * w.T, 0.0f);
                    ps.flags[slot] = ps.flags[slot] & ~F_SHADOW;
                    nsh++;
                    state = kLaneFree;
                }
            }
            if (open) {
                bool mine;
                const uint32_t i = refill_take(state == kLaneFree, &q.counters[C_FETCH_SHADOW], n, open, mine);
                if (mine && i < nc) {
                    const uint32_t slot = q.conn[i];
                    const uint32_t flags = ps.flags[slot];
                    if (flags & F_SHADOW) {
                        job = ps.job[slot];
                        const JobView &J = jt.jobs[job];
                        const float4 sd = ps.sh_dir[slot];
                        const float distT = sd.w - kConnTmin;
                        if (J.params.depth > 0) {
                            cold_t[threadIdx.x] = make_float4(1.0f, 1.0f, 1.0f, distT);
                            cold_w[threadIdx.x] =
                                make_uint4(slot, ps.vol[slot], 0u, (flags & F_INSIDE) ? 0x80000000u : 0u);
                            after = no_hit();
                            trace_begin(st, J.scene, f3(ps.o[slot]), f3(sd), kConnTmin, distT, after);
                            state = kLaneTracing;
                        } else {
                            // no segment to walk: the light is visible
                            ps.rad[slot] = f4(f3(ps.rad[slot]) + f3(ps.sh_c[slot]), 0.0f);
                            ps.flags[slot] = flags & ~F_SHADOW;
                            nsh++;
                        }
                    }
                } else if (mine) {
                    const uint32_t eslot = q.nee[i - nc];
                    const uint32_t flags = ps.flags[eslot]; // F_INSIDE; the shadow rays may clear F_SHADOW meanwhile
                    const JobView &J = jt.jobs[ps.job[eslot]];
                    const float4 nb = ps.nee_b[eslot];
                    float3 emT, T, em;
                    float lpdf;
                    emitter_ray(LaneTracer{}, J.scene, J.params, f3(ps.o[eslot]), f3(ps.d[eslot]),
                                (flags & F_INSIDE) != 0, ps.vol[eslot], emT, T, em, lpdf, err);
                    float3 c = f3(0.0f);
                    if (!is_black(em))
                        c = power_heuristic(nb.w, lpdf) * T * em * f3(nb);
                    ps.nee_c[eslot] = f4(c, 0.0f);
                    nnee++;
                }
            }
            tr = __ballot_sync(0xFFFFFFFFu, state == kLaneTracing);
            if (tr == 0) {
                if (!open)
                    break;
                continue;
            }
        }
        if (state == kLaneTracing && !trace_step(st, stack, jt.jobs[job].scene, after, err))
            state = kLaneDone;
    }
#else
    const uint32_t b0 = first_ray();
    if (b0 < n)
        tlas_cache_fill(jt.jobs[ps.job[b0 < nc ? q.conn[b0] : q.nee[b0 - nc]]].scene);
    else
        tlas_cache_none();
#if VVPT_BLAS_WIDE && VVPT_GROUP_TRAVERSAL
    const GroupTracer trace{lane_group()};
    const bool writer = trace.g.gl == 0;
#else
    const LaneTracer trace{};
    const bool writer = true;
#endif
    for (uint32_t i = my_ray(); i < n; i += ray_stride()) {
        if (i < nc) {
            const uint32_t slot = q.conn[i];
            const uint32_t flags = ps.flags[slot];
            if (!(flags & F_SHADOW))
                continue;
            const JobView &J = jt.jobs[ps.job[slot]];
            const SceneView &s = J.scene;
            const RenderParams &p = J.params;
            const float4 sd = ps.sh_dir[slot];
            const float3 T = shadow_transmittance(trace, s, p, f3(ps.o[slot]), f3(sd), sd.w, (flags & F_INSIDE) != 0,
                                                  ps.vol[slot], err);
            group_sync();
            if (writer) {
                if (!is_black(T))
                    ps.rad[slot] = f4(f3(ps.rad[slot]) + f3(ps.sh_c[slot]) * T, 0.0f);
                ps.flags[slot] = flags & ~F_SHADOW;
                nsh++;
            }
        } else {
            const uint32_t slot = q.nee[i - nc];
            const uint32_t flags = ps.flags[slot]; // F_INSIDE; the shadow part may clear F_SHADOW meanwhile
            const JobView &J = jt.jobs[ps.job[slot]];
            const SceneView &s = J.scene;
            const RenderParams &p = J.params;
            const float4 nb = ps.nee_b[slot];
            float3 emT, T, em;
            float lpdf;
            emitter_ray(trace, s, p, f3(ps.o[slot]), f3(ps.d[slot]), (flags & F_INSIDE) != 0, ps.vol[slot], emT, T,
                        em, lpdf, err);
            float3 c = f3(0.0f);
            if (!is_black(em))
                c = power_heuristic(nb.w, lpdf) * T * em * f3(nb);
            if (writer) {
                ps.nee_c[slot] = f4(c, 0.0f);
                nnee++;
            }
        }
    }
#endif
    warp_add(&q.counters[C_SHADOW], nsh);
    warp_add(&q.counters[C_NEE], nnee);
    if (err)
        atomicOr(&q.counters[C_ERR], err);
}

// Final image: per pixel, add the per-batch sums in batch order starting from
// zero, exactly the sequence of read-modify-writes of raygen.rgen.glsl:134-144.
__global__ void k_reduce(RenderParams p, BatchResults br, float4 *rad, float4 *alb, float4 *nrm, float4 *m2)
{
    const uint32_t npix = p.width * p.height;
    for (uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x; pix < npix; pix += gridDim.x * blockDim.x) {
        float3 r = f3(0.0f), a = f3(0.0f), nn = f3(0.0f), q2 = f3(0.0f);
        if (p.reduce_fp64) {
            double s[12] = {0.0};
            for (uint32_t b = 0; b < p.batches; b++) {
                const size_t it = (size_t)b * npix + pix;
                const float4 rb = br.rad[it], ab = br.alb[it], nb = br.nrm[it];
                s[0] += rb.x, s[1] += rb.y, s[2] += rb.z;
                s[3] += ab.x, s[4] += ab.y, s[5] += ab.z;
                s[6] += nb.x, s[7] += nb.y, s[8] += nb.z;
                s[9] += (double)rb.x * rb.x, s[10] += (double)rb.y * rb.y, s[11] += (double)rb.z * rb.z;
            }
            r = f3((float)s[0], (float)s[1], (float)s[2]);
            a = f3((float)s[3], (float)s[4], (float)s[5]);
            nn = f3((float)s[6], (float)s[7], (float)s[8]);
            q2 = f3((float)s[9], (float)s[10], (float)s[11]);
        } else {
            for (uint32_t b = 0; b < p.batches; b++) {
                const size_t it = (size_t)b * npix + pix;
                float3 rb = f3(br.rad[it]);
                r = r + rb;
                a = a + f3(br.alb[it]);
                nn = nn + f3(br.nrm[it]);
                q2 = q2 + rb * rb;
            }
        }
        if (rad)
            rad[pix] = f4(r, 1.0f);
        if (alb)
            alb[pix] = f4(a, 1.0f);
        if (nrm)
            nrm[pix] = f4(nn, 1.0f);
        if (m2)
            m2[pix] = f4(q2, 1.0f);
    }
}

__global__ void k_trace_closest(SceneView s, const float4 *rays, uint32_t n, float4 *tuv, uint32_t *ids, uint32_t *err_out)
{
    uint32_t err = 0;
    tlas_cache_fill(s);
#if VVPT_BLAS_WIDE && VVPT_GROUP_TRAVERSAL
    const LaneGroup g = lane_group();
#endif
    for (uint32_t i = my_ray(); i < n; i += ray_stride()) {
        float4 a = rays[2 * i], b = rays[2 * i + 1];
#if VVPT_BLAS_WIDE && VVPT_GROUP_TRAVERSAL
        Hit h = trace_after_group(s, f3(a), f3(b), a.w, b.w, no_hit(), err, g);
        if (g.gl != 0)
            continue;
#else
        Hit h = trace_closest(s, f3(a), f3(b), a.w, b.w, err);
#endif
        tuv[i] = make_float4(h.t, h.u, h.v, 0.0f);
        ids[2 * i] = h.inst;
        ids[2 * i + 1] = h.prim;
    }
    if (err)
        atomicOr(err_out, err);
}

// ---------------------------------------------------------------------------
// Host launchers

void launch_init_slots(const Queues &q, const PathState &ps, const JobTable &jt, uint32_t slots, cudaStream_t stream)
{
    int grid = (int)std::min<uint32_t>((slots + 255) / 256, 65535u);
    k_init_slots<<<grid, 256, 0, stream>>>(q, ps, jt, slots);
}

void launch_admit(const Queues &q, const JobTable &jt, unsigned long long total_items, uint32_t num_ranges,
                  cudaStream_t stream)
{
    k_admit<<<1, 1024, 0, stream>>>(q, jt, total_items, num_ranges);
}

void launch_iteration(const JobTable &jt, const PathState &ps, const Queues &q, int pp, const LaunchShape &shape,
                      cudaStream_t stream)
{
    for (int k = 0; k < K_NUM; k++)
        launch_kernel((KernelId)k, jt, ps, q, pp, shape, stream);
}

void launch_kernel(KernelId k, const JobTable &jt, const PathState &ps, const Queues &q, int pp,
                   const LaunchShape &shape, cudaStream_t stream)
{
    switch (k) {
    case K_BEGIN:
        k_begin<<<1, 32, 0, stream>>>(q, pp);
        break;
    case K_REGEN:
        k_regen<<<shape.grid, shape.block, 0, stream>>>(jt, ps, q, pp);
        break;
    case K_EXTEND:
        k_extend<<<shape.grid, shape.block, kTlasCacheBytes, stream>>>(jt, ps, q, pp);
        break;
    case K_PARTITION:
        if (kPartitionLaunches)
            k_partition<<<shape.grid, shape.block, 0, stream>>>(ps, q, pp);
        break;
    case K_WALK:
        k_walk<<<shape.grid, shape.block, kTlasCacheBytes, stream>>>(jt, ps, q);
        break;
    case K_SHADE:
#if VVPT_SHADE_SPLIT
        k_shade<0><<<shape.grid, shape.block, kTlasCacheBytes, stream>>>(jt, ps, q, pp);
        k_shade<1><<<shape.grid, shape.block, kTlasCacheBytes, stream>>>(jt, ps, q, pp);
        k_shade<2><<<shape.grid, shape.block, kTlasCacheBytes, stream>>>(jt, ps, q, pp);
#else
        k_shade<3><<<shape.grid, shape.block, kTlasCacheBytes, stream>>>(jt, ps, q, pp);
#endif
        break;
    case K_SHADOW:
        k_shadow<<<shape.grid, shape.block, kTlasCacheBytes, stream>>>(jt, ps, q);
        break;
    default:
        break;
    }
}

void launch_reduce(const RenderParams &hp, const BatchResults &br, float4 *radiance, float4 *albedo, float4 *normal,
                   float4 *radiance_m2, cudaStream_t stream)
{
    uint32_t npix = hp.width * hp.height;
    int grid = (int)std::min<uint32_t>((npix + 255) / 256, 65535u);
    k_reduce<<<grid, 256, 0, stream>>>(hp, br, radiance, albedo, normal, radiance_m2);
}

void launch_trace_closest(const SceneView &s, const float4 *rays, uint32_t n, float4 *tuv, uint32_t *ids, uint32_t *err,
                          cudaStream_t stream)
{
    int grid = (int)std::min<uint64_t>(((uint64_t)n * kLanesPerRay + 255) / 256, 65535u);
    if (grid < 1)
        grid = 1;
    k_trace_closest<<<grid, 256, kTlasCacheBytes, stream>>>(s, rays, n, tuv, ids, err);
}

}  // namespace vvpt
