// Kernels of the learned denoiser: BF16 tensor-core 3x3 convolutions as
// implicit GEMMs (forward, input gradient, weight gradient) with FP32
// accumulation, and the elementwise kernels around them (feature packing,
// 2x2 average pool, nearest upsample + concat, L1 loss in the log domain,
// Adam). Activations are NHWC bf16, weights [Cout][3][3][Cin] bf16 with FP32
// master copies. Channel counts (inputs and outputs) are multiples of 16.
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace vvdn {

typedef __nv_bfloat16 bf16;

struct ConvArgs {
    const bf16 *in;    // [P][cin]
    int cin;
    const bf16 *wgt;   // [cout][9][cin]
    const float *bias; // [cout] or null
    void *out;         // [P][cout] bf16, or f32 when out_f32
    int cout;
    int out_f32;
    int relu;
    const bf16 *mask;  // [P][cout] or null: output *= (mask > 0)
    int n, h, wd;      // P = n * h * wd
    // Fused nearest-upsample + concat input (conv3x3_concat): channels
    // [0, cc) come from `coarse` ([n][h/2][wd/2][cc]) upsampled by 2, channels
    // [cc, cin) from `in` ([P][cin - cc]). cc = 0: `in` holds all cin.
    const bf16 *coarse;
    int cc;
    // Output layer at inference (tcgen05 kernels): the frame written as RGBA
    // f32, expm1(max(y, 0)) of channels 0-2 and alpha 1, instead of `out`.
    float4 *rgba;
};

enum ConvKernels {
    kConvAuto = 0,       // tcgen05: strip kernel where the weights fit, else per-tile
    kConvTiles = 1,      // tcgen05 per-tile kernels only
    kConvPersistent = 2, // strip kernel on a grid of 16 CTAs (several segments each)
    kConvNoFusion = 3,   // as kConvAuto, but no fused upsample + concat inputs
    kConvWgradTc = 4,    // as kConvAuto, and the weight gradient on tcgen05 too
};

// out = act(conv3x3(in, w) + bias) (zero padding); with transformed weights
// (w_t[ci][8 - tap][co]) and a mask the same kernel is the input gradient.
// With `err` set (and cout <= 256) it runs on the tcgen05 tensor cores and
// `err` receives a status bit if one of its waits timed out; with err null
// it runs the warp-level mma.sync kernel.
void conv3x3(const ConvArgs &a, cudaStream_t s, uint32_t *err, ConvKernels kind = kConvAuto);

// The same convolution over concat(upsample2(coarse), in) without writing the
// concatenated tensor (a.coarse, a.cc set): runs only on the strip kernel and
// returns false, launching nothing, when that kernel does not take the layer.
bool conv3x3_concat(const ConvArgs &a, cudaStream_t s, uint32_t *err, ConvKernels kind = kConvAuto);

// Diagnostics: the next strip-kernel launch withholds its accumulator-ready
// signal, so its drain warps' bounded waits run out and the launch records
// an error status instead of hanging (no GPU fault is involved).
void inject_wait_timeout();

// dw[co][tap][ci] += sum_p dout[p][co] * in[p shifted by tap][ci];
// dbias[co] += sum_p dout[p][co] (dbias may be null).
// With `err` set it runs on the tcgen05 tensor cores (err receives a status
// bit if a wait timed out), with err null on the warp-level mma.sync kernel
// (the faster of the two for this network: training step 3.2 vs 4.1 ms).
void conv3x3_wgrad(const bf16 *dout, int cout, const bf16 *in, int cin, int n, int h, int w, float *dw,
                   float *dbias, cudaStream_t s, uint32_t *err = nullptr);
// the mma.sync weight gradient (dw only)
void wgrad_mma_sync(const bf16 *dout, int cout, const bf16 *in, int cin, int n, int h, int w, float *dw,
                    cudaStream_t s);

// w_t[ci][8 - tap][co] = w[co][tap][ci]
void transform_weights(const bf16 *w, bf16 *wt, int cout, int cin, cudaStream_t s);

// f32 master weights -> bf16 copy
void to_bf16(const float *src, bf16 *dst, size_t n, cudaStream_t s);

// Input features from RGBA32F buffers: log(1 + max(radiance, 0)), albedo,
// normal, zeros to 16 channels. `target` (optional) -> log(1 + max(t, 0)),
// 3 floats per pixel.
void pack_features(const float *radiance, const float *albedo, const float *normal, bf16 *x, int npix,
                   cudaStream_t s);
void pack_target(const float *target, float *t3, int npix, cudaStream_t s);

void avgpool2(const bf16 *in, bf16 *out, int n, int h, int w, int c, cudaStream_t s);
// out[.., 0:cc] = nearest-upsampled coarse (h/2 x w/2), out[.., cc:cc+cs] = skip
void upcat(const bf16 *coarse, int cc, const bf16 *skip, int cs, bf16 *out, int n, int h, int w, cudaStream_t s);
// split the gradient of an upcat: dcoarse = sum over the 2x2 block of the
// first cc channels; dskip = the rest
void upcat_backward(const bf16 *dcat, int cc, int cs, bf16 *dcoarse, bf16 *dskip, int n, int h, int w,
                    cudaStream_t s);
// de = (dskip + dpooled[p / 2] / 4) * (e > 0); dskip may be null
void pool_backward_combine(const bf16 *dskip, const bf16 *dpooled, const bf16 *e, bf16 *de, int n, int h, int w,
                           int c, cudaStream_t s);
// L1 loss between out[.., 0:3] (f32, stride cout) and t3; dout (bf16, stride
// cout, zero beyond channel 3) = sign(out - t) / (3 * npix); loss_sum += |diff|
void l1_loss(const float *out, int cout, const float *t3, bf16 *dout, float *loss_sum, int npix, cudaStream_t s);
// Adam (Kingma and Ba 2015) with bias correction; t = step number from 1
void adam(float *p, const float *g, float *m, float *v, size_t n, float lr, float b1, float b2, float eps, int t,
          cudaStream_t s);
// out RGBA32F = exp(max(y, 0)) - 1 for the first 3 channels, A = 1
void unpack_output(const float *y, int cout, float *out_rgba, int npix, cudaStream_t s);

}  // namespace vvdn
