// Tables of the low-discrepancy sampler (sampler_tables.cpp): sizes follow
// the reference's shaders/include/rng/rng_pmj_defines.glsl and
// bluenoise_defines.glsl.
#pragma once
#include <stdint.h>

#include <vector>

namespace vvpt {

constexpr int kPmjSequences = 16;
constexpr int kPmjSamples = 16384;
constexpr uint32_t kPmjSeed = 2873468793u;
constexpr int kBlueNoiseTextures = 48;
constexpr int kBlueNoiseRes = 128;

// [sequence][sample][2] in [0, 1)
void make_pmj02_table(float *out);
// [texture][x][y] in [0, 1): rank / (128 * 128)
void make_blue_noise_table(float *out);

struct SamplerTables {
    std::vector<float> pmj;        // kPmjSequences * kPmjSamples * 2
    std::vector<float> blue_noise; // kBlueNoiseTextures * kBlueNoiseRes^2
};
// Generated once per process (about a second on 8 cores).
const SamplerTables &sampler_tables();

}  // namespace vvpt
