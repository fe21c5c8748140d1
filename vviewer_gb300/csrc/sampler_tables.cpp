// Tables of the low-discrepancy sampler (VVPT_RENDER_SAMPLER_PMJ): 16
// progressive multi-jittered (0,2) sequences of 16384 2D points and 48
// blue-noise textures of 128 x 128, the data the reference uploads for its
// PMJ02BN sampler (src/lib/vengine/vulkan/resources/VulkanRandom.cpp,
// math/PMJSequences.hpp:10-14, math/BlueNoise.hpp:27-32; shaders
// include/rng/rng_pmj_defines.glsl). The reference's own tables are data
// blobs not present in its tree, so they are regenerated here from the
// published methods, deterministically:
//
// - (0,2) sequences: the first two Sobol dimensions (van der Corput and the
//   x + 1 polynomial dimension) under Owen's nested uniform scrambling. Every
//   power-of-two prefix is stratified in all elementary intervals, the
//   defining property of pmj02 (Christensen, Kensler, Kilpatrick,
//   "Progressive Multi-Jittered Sample Sequences", EGSR 2018; Helmer,
//   Christensen, Kensler, "Stochastic Generation of (t, s) Sample
//   Sequences", EGSR 2021, show the equivalence). The best-candidate
//   refinement of PMJ02BN is not reproduced.
// - Blue noise: Ulichney's void-and-cluster method ("The void-and-cluster
//   method for dither array generation", SPIE 1913, 1993) on a torus with a
//   Gaussian filter of sigma 1.5, values rank / 16384.
#include "sampler_tables.h"

#include <algorithm>
#include <cmath>
#include <mutex>
#include <thread>

namespace vvpt {
namespace {

uint32_t hash32(uint32_t x)
{
    // lowbias32 (Wellons): an invertible 32-bit mix
    x ^= x >> 16;
    x *= 0x7feb352du;
    x ^= x >> 15;
    x *= 0x846ca68bu;
    x ^= x >> 16;
    return x;
}

uint32_t reverse_bits(uint32_t v)
{
    uint32_t r = 0;
    for (int b = 0; b < 32; b++)
        r |= ((v >> b) & 1u) << (31 - b);
    return r;
}

// Sobol dimension 1 (primitive polynomial x + 1): direction numbers
// v1 = 2^31, v_k = v_{k-1} ^ (v_{k-1} >> 1)
uint32_t sobol1(uint32_t i)
{
    uint32_t r = 0, v = 1u << 31;
    for (; i; i >>= 1, v ^= v >> 1)
        if (i & 1u)
            r ^= v;
    return r;
}

// Owen's nested uniform scrambling: bit b flips by a hash of the bits above
// it, so every elementary interval keeps its point count
uint32_t owen_scramble(uint32_t v, uint32_t seed)
{
    uint32_t out = 0;
    for (int b = 31; b >= 0; b--) {
        const uint32_t prefix = b == 31 ? 0u : (v >> (b + 1)) | (1u << (31 - b)); // level-tagged prefix
        const uint32_t flip = hash32(prefix ^ hash32(seed + 0x9e3779b9u * (uint32_t)b)) & 1u;
        out |= (((v >> b) & 1u) ^ flip) << b;
    }
    return out;
}

float unit_float(uint32_t v) { return (float)(v >> 8) * (1.0f / 16777216.0f); }

// Largest key per row, refreshed for the rows a change touches, so a
// step costs O(res * filter height) instead of a scan of every cell.
// key(i) = sign * energy for the cells of the class searched, else -inf.
struct RowMax {
    int res;
    std::vector<float> best;
    std::vector<int> arg;
    template <class Key>
    void row(int y, const Key &key)
    {
        float bv = -INFINITY;
        int ba = -1;
        for (int x = 0; x < res; x++) {
            const float k = key(y * res + x);
            if (k > bv) {
                bv = k;
                ba = y * res + x;
            }
        }
        best[y] = bv;
        arg[y] = ba;
    }
    template <class Key>
    void all(const Key &key)
    {
        for (int y = 0; y < res; y++)
            row(y, key);
    }
    template <class Key>
    void around(int p, int rad, const Key &key)
    {
        const int py = p / res;
        for (int dy = -rad; dy <= rad; dy++)
            row((py + dy + res) % res, key);
    }
    int top() const
    {
        int y = (int)(std::max_element(best.begin(), best.end()) - best.begin());
        return arg[y];
    }
};

// void-and-cluster on a res x res torus
void void_and_cluster(int res, uint32_t seed, float *out /* [x][y] */)
{
    const int n = res * res;
    const double sigma = 1.5;
    const int rad = 7;
    std::vector<float> kern((2 * rad + 1) * (2 * rad + 1));
    for (int dy = -rad; dy <= rad; dy++)
        for (int dx = -rad; dx <= rad; dx++)
            kern[(dy + rad) * (2 * rad + 1) + dx + rad] = (float)std::exp(-(dx * dx + dy * dy) / (2.0 * sigma * sigma));
    auto splat = [&](std::vector<float> &e, int p, float sgn) {
        const int px = p % res, py = p / res;
        for (int dy = -rad; dy <= rad; dy++) {
            const int y = (py + dy + res) % res;
            for (int dx = -rad; dx <= rad; dx++) {
                const int x = (px + dx + res) % res;
                e[y * res + x] += sgn * kern[(dy + rad) * (2 * rad + 1) + dx + rad];
            }
        }
    };
    // initial pattern: 10 % of the cells, chosen by a seeded hash
    std::vector<uint8_t> pat(n, 0);
    std::vector<float> en(n, 0.0f);
    int ones = 0;
    for (uint32_t k = 0; ones < n / 10; k++) {
        const int p = (int)(hash32(seed ^ hash32(k)) % (uint32_t)n);
        if (!pat[p]) {
            pat[p] = 1;
            splat(en, p, 1.0f);
            ones++;
        }
    }
    // relax: move the tightest cluster to the largest void until stable
    {
        auto kc = [&](int i) { return pat[i] ? en[i] : -INFINITY; };
        auto kv = [&](int i) { return pat[i] ? -INFINITY : -en[i]; };
        RowMax rc{res, std::vector<float>(res), std::vector<int>(res)};
        RowMax rv{res, std::vector<float>(res), std::vector<int>(res)};
        rc.all(kc);
        rv.all(kv);
        for (int it = 0; it < 4 * n; it++) {
            const int c = rc.top();
            pat[c] = 0;
            splat(en, c, -1.0f);
            rc.around(c, rad, kc);
            rv.around(c, rad, kv);
            const int v = rv.top();
            pat[v] = 1;
            splat(en, v, 1.0f);
            rc.around(v, rad, kc);
            rv.around(v, rad, kv);
            if (v == c)
                break;
        }
    }
    std::vector<int> rank(n, -1);
    // phase 1: rank the initial points, tightest cluster last
    {
        std::vector<uint8_t> p1 = pat;
        std::vector<float> e1 = en;
        auto key = [&](int i) { return p1[i] ? e1[i] : -INFINITY; };
        RowMax rm{res, std::vector<float>(res), std::vector<int>(res)};
        rm.all(key);
        for (int r = ones - 1; r >= 0; r--) {
            const int c = rm.top();
            p1[c] = 0;
            splat(e1, c, -1.0f);
            rm.around(c, rad, key);
            rank[c] = r;
        }
    }
    // phase 2: fill the largest voids up to half the cells
    int r = ones;
    {
        auto key = [&](int i) { return pat[i] ? -INFINITY : -en[i]; };
        RowMax rm{res, std::vector<float>(res), std::vector<int>(res)};
        rm.all(key);
        for (; r < n / 2; r++) {
            const int v = rm.top();
            pat[v] = 1;
            splat(en, v, 1.0f);
            rm.around(v, rad, key);
            rank[v] = r;
        }
    }
    // phase 3: the zeros are now the minority; energy of the zeros, fill
    // their tightest cluster
    {
        std::vector<float> ez(n, 0.0f);
        for (int i = 0; i < n; i++)
            if (!pat[i])
                splat(ez, i, 1.0f);
        auto key = [&](int i) { return pat[i] ? -INFINITY : ez[i]; };
        RowMax rm{res, std::vector<float>(res), std::vector<int>(res)};
        rm.all(key);
        for (; r < n; r++) {
            const int c = rm.top();
            pat[c] = 1;
            splat(ez, c, -1.0f);
            rm.around(c, rad, key);
            rank[c] = r;
        }
    }
    for (int y = 0; y < res; y++)
        for (int x = 0; x < res; x++)
            out[x * res + y] = (float)rank[y * res + x] / (float)n;
}

}  // namespace

void make_pmj02_table(float *out)
{
    for (int s = 0; s < kPmjSequences; s++) {
        const uint32_t sx = hash32(kPmjSeed ^ (2u * (uint32_t)s + 1u)), sy = hash32(kPmjSeed ^ (2u * (uint32_t)s + 2u));
        for (int i = 0; i < kPmjSamples; i++) {
            out[((size_t)s * kPmjSamples + i) * 2 + 0] = unit_float(owen_scramble(reverse_bits((uint32_t)i), sx));
            out[((size_t)s * kPmjSamples + i) * 2 + 1] = unit_float(owen_scramble(sobol1((uint32_t)i), sy));
        }
    }
}

void make_blue_noise_table(float *out)
{
    const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    const int nth = (int)std::min<unsigned>(hw, (unsigned)kBlueNoiseTextures);
    std::vector<std::thread> th;
    for (int t = 0; t < nth; t++)
        th.emplace_back([=]() {
            for (int k = t; k < kBlueNoiseTextures; k += nth)
                void_and_cluster(kBlueNoiseRes, kPmjSeed + 7919u * (uint32_t)k,
                                 out + (size_t)k * kBlueNoiseRes * kBlueNoiseRes);
        });
    for (auto &x : th)
        x.join();
}

const SamplerTables &sampler_tables()
{
    static SamplerTables t;
    static std::once_flag once;
    std::call_once(once, [] {
        t.pmj.resize((size_t)kPmjSequences * kPmjSamples * 2);
        t.blue_noise.resize((size_t)kBlueNoiseTextures * kBlueNoiseRes * kBlueNoiseRes);
        make_pmj02_table(t.pmj.data());
        make_blue_noise_table(t.blue_noise.data());
    });
    return t;
}

}  // namespace vvpt
