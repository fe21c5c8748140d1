// Learned denoiser behind vvpt_denoiser_* (include/vvpt.h): a 5-level U-Net
// over noisy radiance + albedo + normal, standing in for the reference's
// OpenImageDenoise step (VulkanRendererPathTracing.cpp:985-1018). Trained on
// the GPU with the project's own kernels (denoise_kernels.cu): BF16
// tensor-core convolutions with FP32 accumulation for the forward pass, the
// input gradients and the weight gradients, FP32 master weights and Adam.
//
// Network (channels C = 32, 48, 64, 96, 128; every conv 3x3, zero padded):
//   x0 = features (log1p radiance, albedo, normal; 16 channels)
//   encoder l = 0..4: x_l = avgpool2(e_{l-1}) (l > 0); a_l = relu(conv(x_l));
//                     e_l = relu(conv(a_l))
//   decoder l = 3..0: u_l = [upsample2(l == 3 ? e_4 : d_{l+1}), e_l];
//                     b_l = relu(conv(u_l)); d_l = relu(conv(b_l))
//   y = conv(d_0) (16 channels, the first 3 used): log1p of the radiance
//   loss = mean |y - log1p(target)| over pixels and the 3 channels.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "denoise_kernels.cuh"
#include "internal.h"

using namespace vvpt;
using vvdn::bf16;

namespace {

constexpr int kLevels = 5;
constexpr int kCh[kLevels] = {32, 48, 64, 96, 128};
constexpr int kInCh = 16;
constexpr int kOutCh = 16;
constexpr int kLayers = 19;

struct Layer {
    int cin, cout;
    bool relu;
    size_t w_off, b_off; // into the f32 parameter vector (floats)
    size_t w16_off;      // into the bf16 weight copies (elements)
};

std::vector<Layer> make_layers(size_t &nparams, size_t &nw16)
{
    std::vector<Layer> L;
    auto add = [&](int cin, int cout, bool relu) { L.push_back(Layer{cin, cout, relu, 0, 0, 0}); };
    int prev = kInCh;
    for (int l = 0; l < kLevels; l++) {
        add(prev, kCh[l], true);
        add(kCh[l], kCh[l], true);
        prev = kCh[l];
    }
    for (int l = kLevels - 2; l >= 0; l--) {
        add(kCh[l + 1] + kCh[l], kCh[l], true);
        add(kCh[l], kCh[l], true);
    }
    add(kCh[0], kOutCh, false);
    nparams = 0;
    nw16 = 0;
    for (auto &x : L) {
        x.w_off = nparams;
        nparams += (size_t)x.cout * 9 * x.cin;
        x.b_off = nparams;
        nparams += x.cout;
        x.w16_off = nw16;
        nw16 += (size_t)x.cout * 9 * x.cin;
    }
    return L;
}

// splitmix64 + Box-Muller: the same initial weights on every host
struct InitRng {
    uint64_t s;
    uint64_t next()
    {
        uint64_t z = (s += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    double uniform() { return ((next() >> 11) + 0.5) * (1.0 / 9007199254740992.0); }
    double normal() { return std::sqrt(-2.0 * std::log(uniform())) * std::cos(6.283185307179586 * uniform()); }
};

// One forward tensor of the network: level, channels, offset in the
// activation pool (bf16 elements); its gradient has the same offset in the
// gradient pool.
struct Tensor {
    int level = 0, ch = 0;
    size_t off = 0;
};

}  // namespace

struct vvpt_denoiser {
    vvpt_ctx *ctx = nullptr;
    std::vector<Layer> layers;
    size_t nparams = 0, nw16 = 0;
    DevBuf params, grads, adam_m, adam_v, w16, wt16;
    int step = 0;
    // shape-dependent buffers
    int n = 0, h = 0, w = 0;
    bool with_grads = false;
    DevBuf acts, gacts, out_f32, target3, dout, loss, err;
    bool mma_sync = false; // warp-level mma.sync convolutions instead of tcgen05
    vvdn::ConvKernels conv_kind = vvdn::kConvAuto;
    // tensors: x[l], a[l], e[l]; u[l], b[l], d[l] (l < 4)
    // gskip[l]: gradient of e_l through the decoder's concat (gradient pool only)
    Tensor x[kLevels], a[kLevels], e[kLevels], u[kLevels - 1], b[kLevels - 1], d[kLevels - 1], gskip[kLevels - 1];
    bool weights_dirty = true;
};

namespace {

size_t level_pixels(const vvpt_denoiser *dn, int l) { return (size_t)dn->n * (dn->h >> l) * (dn->w >> l); }

vvpt_status ensure_shape(vvpt_denoiser *dn, int n, int h, int w, bool with_grads)
{
    vvpt_ctx *ctx = dn->ctx;
    if (dn->n == n && dn->h == h && dn->w == w && (dn->with_grads || !with_grads))
        return VVPT_OK;
    dn->n = n;
    dn->h = h;
    dn->w = w;
    dn->with_grads = with_grads || dn->with_grads;
    size_t off = 0;
    auto place = [&](Tensor &t, int level, int ch) {
        t.level = level;
        t.ch = ch;
        t.off = off;
        off += (level_pixels(dn, level) * ch + 127) & ~size_t(127); // 256-byte aligned
    };
    place(dn->x[0], 0, kInCh);
    for (int l = 0; l < kLevels; l++) {
        if (l > 0)
            place(dn->x[l], l, kCh[l - 1]);
        place(dn->a[l], l, kCh[l]);
        place(dn->e[l], l, kCh[l]);
    }
    for (int l = kLevels - 2; l >= 0; l--) {
        place(dn->u[l], l, kCh[l + 1] + kCh[l]);
        place(dn->b[l], l, kCh[l]);
        place(dn->d[l], l, kCh[l]);
        place(dn->gskip[l], l, kCh[l]);
    }
    const size_t p0 = level_pixels(dn, 0);
    VV_CUDA(dn->acts.reserve(off * sizeof(bf16)), "cudaMalloc denoiser activations");
    VV_CUDA(dn->out_f32.reserve(p0 * kOutCh * sizeof(float)), "cudaMalloc denoiser output");
    if (dn->with_grads) {
        VV_CUDA(dn->gacts.reserve(off * sizeof(bf16)), "cudaMalloc denoiser gradients");
        VV_CUDA(dn->target3.reserve(p0 * 3 * sizeof(float)), "cudaMalloc denoiser target");
        VV_CUDA(dn->dout.reserve(p0 * kOutCh * sizeof(bf16)), "cudaMalloc denoiser output gradient");
        VV_CUDA(dn->loss.reserve(sizeof(float)), "cudaMalloc loss");
    }
    return VVPT_OK;
}

bf16 *act(vvpt_denoiser *dn, const Tensor &t) { return dn->acts.as<bf16>() + t.off; }
bf16 *grad(vvpt_denoiser *dn, const Tensor &t) { return dn->gacts.as<bf16>() + t.off; }

void refresh_weights(vvpt_denoiser *dn, cudaStream_t s)
{
    if (!dn->weights_dirty)
        return;
    for (const Layer &L : dn->layers) {
        vvdn::to_bf16(dn->params.as<float>() + L.w_off, dn->w16.as<bf16>() + L.w16_off, (size_t)L.cout * 9 * L.cin, s);
        vvdn::transform_weights(dn->w16.as<bf16>() + L.w16_off, dn->wt16.as<bf16>() + L.w16_off, L.cout, L.cin, s);
    }
    dn->weights_dirty = false;
}

void conv_fwd(vvpt_denoiser *dn, int li, const bf16 *in, void *out, int level, bool out_f32, cudaStream_t s,
              float4 *rgba = nullptr)
{
    const Layer &L = dn->layers[li];
    vvdn::ConvArgs a{};
    a.in = in;
    a.cin = L.cin;
    a.wgt = dn->w16.as<bf16>() + L.w16_off;
    a.bias = dn->params.as<float>() + L.b_off;
    a.out = out;
    a.cout = L.cout;
    a.out_f32 = out_f32 ? 1 : 0;
    a.relu = L.relu ? 1 : 0;
    a.mask = nullptr;
    a.n = dn->n;
    a.h = dn->h >> level;
    a.wd = dn->w >> level;
    a.rgba = rgba;
    vvdn::conv3x3(a, s, dn->mma_sync ? nullptr : dn->err.as<uint32_t>(), dn->conv_kind);
}

// layer li over concat(upsample2(coarse), skip) without the concatenated
// tensor; false when only the unfused path takes the layer
bool conv_fwd_concat(vvpt_denoiser *dn, int li, const bf16 *coarse, int cc, const bf16 *skip, bf16 *out, int level,
                     cudaStream_t s)
{
    if (dn->mma_sync)
        return false;
    const Layer &L = dn->layers[li];
    vvdn::ConvArgs a{};
    a.in = skip;
    a.cin = L.cin;
    a.coarse = coarse;
    a.cc = cc;
    a.wgt = dn->w16.as<bf16>() + L.w16_off;
    a.bias = dn->params.as<float>() + L.b_off;
    a.out = out;
    a.cout = L.cout;
    a.relu = L.relu ? 1 : 0;
    a.n = dn->n;
    a.h = dn->h >> level;
    a.wd = dn->w >> level;
    return vvdn::conv3x3_concat(a, s, dn->err.as<uint32_t>(), dn->conv_kind);
}

// input gradient of layer li: din = conv(dout, w_t) * (mask > 0)
void conv_dgrad(vvpt_denoiser *dn, int li, const bf16 *dout, bf16 *din, const bf16 *mask, int level, cudaStream_t s)
{
    const Layer &L = dn->layers[li];
    vvdn::ConvArgs a{};
    a.in = dout;
    a.cin = L.cout;
    a.wgt = dn->wt16.as<bf16>() + L.w16_off;
    a.bias = nullptr;
    a.out = din;
    a.cout = L.cin;
    a.out_f32 = 0;
    a.relu = 0;
    a.mask = mask;
    a.n = dn->n;
    a.h = dn->h >> level;
    a.wd = dn->w >> level;
    vvdn::conv3x3(a, s, dn->mma_sync ? nullptr : dn->err.as<uint32_t>(), dn->conv_kind);
}

void conv_wgrad(vvpt_denoiser *dn, int li, const bf16 *dout, const bf16 *in, int level, cudaStream_t s)
{
    const Layer &L = dn->layers[li];
    vvdn::conv3x3_wgrad(dout, L.cout, in, L.cin, dn->n, dn->h >> level, dn->w >> level,
                        dn->grads.as<float>() + L.w_off, dn->grads.as<float>() + L.b_off, s,
                        dn->conv_kind == vvdn::kConvWgradTc ? dn->err.as<uint32_t>() : nullptr);
}

// inference (fuse_concat): the decoder's first convolution of a level reads
// concat(upsample(coarse), skip) straight from both tensors where the strip
// kernel takes it; training keeps the concatenated tensor for the weight
// gradient
// rgba (inference, tcgen05 kernels): the output layer writes the final RGBA
// frame there instead of out_f32
void forward(vvpt_denoiser *dn, const float *rad, const float *alb, const float *nrm, cudaStream_t s,
             bool fuse_concat = false, float *rgba = nullptr)
{
    refresh_weights(dn, s);
    const int n = dn->n;
    vvdn::pack_features(rad, alb, nrm, act(dn, dn->x[0]), (int)level_pixels(dn, 0), s);
    for (int l = 0; l < kLevels; l++) {
        if (l > 0)
            vvdn::avgpool2(act(dn, dn->e[l - 1]), act(dn, dn->x[l]), n, dn->h >> (l - 1), dn->w >> (l - 1),
                           kCh[l - 1], s);
        conv_fwd(dn, 2 * l, act(dn, dn->x[l]), act(dn, dn->a[l]), l, false, s);
        conv_fwd(dn, 2 * l + 1, act(dn, dn->a[l]), act(dn, dn->e[l]), l, false, s);
    }
    for (int l = kLevels - 2; l >= 0; l--) {
        const Tensor &coarse = l == kLevels - 2 ? dn->e[kLevels - 1] : dn->d[l + 1];
        const int li = 10 + 2 * (kLevels - 2 - l);
        if (!(fuse_concat && conv_fwd_concat(dn, li, act(dn, coarse), kCh[l + 1], act(dn, dn->e[l]),
                                             act(dn, dn->b[l]), l, s))) {
            vvdn::upcat(act(dn, coarse), kCh[l + 1], act(dn, dn->e[l]), kCh[l], act(dn, dn->u[l]), n, dn->h >> l,
                        dn->w >> l, s);
            conv_fwd(dn, li, act(dn, dn->u[l]), act(dn, dn->b[l]), l, false, s);
        }
        conv_fwd(dn, li + 1, act(dn, dn->b[l]), act(dn, dn->d[l]), l, false, s);
    }
    conv_fwd(dn, kLayers - 1, act(dn, dn->d[0]), dn->out_f32.as<float>(), 0, true, s,
             dn->mma_sync ? nullptr : reinterpret_cast<float4 *>(rgba));
}

void backward(vvpt_denoiser *dn, cudaStream_t s)
{
    const int n = dn->n;
    bf16 *gout = dn->dout.as<bf16>();
    // output layer
    conv_wgrad(dn, kLayers - 1, gout, act(dn, dn->d[0]), 0, s);
    conv_dgrad(dn, kLayers - 1, gout, grad(dn, dn->d[0]), act(dn, dn->d[0]), 0, s);
    // decoder, finest level first
    for (int l = 0; l <= kLevels - 2; l++) {
        const int li = 10 + 2 * (kLevels - 2 - l);
        conv_wgrad(dn, li + 1, grad(dn, dn->d[l]), act(dn, dn->b[l]), l, s);
        conv_dgrad(dn, li + 1, grad(dn, dn->d[l]), grad(dn, dn->b[l]), act(dn, dn->b[l]), l, s);
        conv_wgrad(dn, li, grad(dn, dn->b[l]), act(dn, dn->u[l]), l, s);
        conv_dgrad(dn, li, grad(dn, dn->b[l]), grad(dn, dn->u[l]), act(dn, dn->u[l]), l, s);
        // the coarse part goes to d_{l+1} (or e_4), already masked by the concat's mask
        const Tensor &coarse = l == kLevels - 2 ? dn->e[kLevels - 1] : dn->d[l + 1];
        vvdn::upcat_backward(grad(dn, dn->u[l]), kCh[l + 1], kCh[l], grad(dn, coarse), grad(dn, dn->gskip[l]), n,
                             dn->h >> l, dn->w >> l, s);
    }
    // encoder, coarsest level first
    for (int l = kLevels - 1; l >= 0; l--) {
        if (l < kLevels - 1)
            vvdn::pool_backward_combine(grad(dn, dn->gskip[l]), grad(dn, dn->x[l + 1]), act(dn, dn->e[l]),
                                        grad(dn, dn->e[l]), n, dn->h >> l, dn->w >> l, kCh[l], s);
        conv_wgrad(dn, 2 * l + 1, grad(dn, dn->e[l]), act(dn, dn->a[l]), l, s);
        conv_dgrad(dn, 2 * l + 1, grad(dn, dn->e[l]), grad(dn, dn->a[l]), act(dn, dn->a[l]), l, s);
        conv_wgrad(dn, 2 * l, grad(dn, dn->a[l]), act(dn, dn->x[l]), l, s);
        if (l > 0)
            conv_dgrad(dn, 2 * l, grad(dn, dn->a[l]), grad(dn, dn->x[l]), nullptr, l, s);
    }
}

// reads and clears the tcgen05 status word (stream-synchronous)
vvpt_status check_device_status(vvpt_denoiser *dn, cudaStream_t s)
{
    vvpt_ctx *ctx = dn->ctx;
    uint32_t e = 0;
    VV_CUDA(cudaMemcpyAsync(&e, dn->err.ptr, sizeof(e), cudaMemcpyDeviceToHost, s), "read denoiser status");
    VV_CUDA(cudaStreamSynchronize(s), "denoiser");
    if (e) {
        VV_CUDA(cudaMemsetAsync(dn->err.ptr, 0, sizeof(uint32_t), s), "clear denoiser status");
        return fail(ctx, VVPT_ERR_DEVICE, "denoiser: a tensor-core wait timed out");
    }
    return VVPT_OK;
}

vvpt_status check_shape(vvpt_ctx *ctx, uint32_t n, uint32_t w, uint32_t h)
{
    if (n == 0 || w == 0 || h == 0 || w % 16 || h % 16)
        return fail(ctx, VVPT_ERR_INVALID_ARG, "denoiser: width and height must be positive multiples of 16");
    if ((uint64_t)n * w * h > (1ull << 31) / kInCh)
        return fail(ctx, VVPT_ERR_INVALID_ARG, "denoiser: batch too large");
    return VVPT_OK;
}

// forward + loss + backward into dn->grads; loss returned on the host
vvpt_status loss_and_grads(vvpt_denoiser *dn, const vvpt_denoise_batch *bt, float *loss_out)
{
    vvpt_ctx *ctx = dn->ctx;
    if (!bt || !bt->radiance || !bt->albedo || !bt->normal || !bt->target)
        return fail(ctx, VVPT_ERR_INVALID_ARG, "denoiser: null batch buffer");
    vvpt_status st = check_shape(ctx, bt->count, bt->width, bt->height);
    if (st != VVPT_OK)
        return st;
    if ((st = ensure_shape(dn, (int)bt->count, (int)bt->height, (int)bt->width, true)) != VVPT_OK)
        return st;
    cudaStream_t s = vv_stream(ctx);
    const int p0 = (int)level_pixels(dn, 0);
    forward(dn, bt->radiance, bt->albedo, bt->normal, s);
    vvdn::pack_target(bt->target, dn->target3.as<float>(), p0, s);
    VV_CUDA(cudaMemsetAsync(dn->loss.ptr, 0, sizeof(float), s), "clear loss");
    vvdn::l1_loss(dn->out_f32.as<float>(), kOutCh, dn->target3.as<float>(), dn->dout.as<bf16>(), dn->loss.as<float>(),
                  p0, s);
    VV_CUDA(cudaMemsetAsync(dn->grads.ptr, 0, dn->nparams * sizeof(float), s), "clear gradients");
    backward(dn, s);
    VV_CUDA(cudaGetLastError(), "denoiser kernels");
    float l = 0.0f;
    VV_CUDA(cudaMemcpyAsync(&l, dn->loss.ptr, sizeof(float), cudaMemcpyDeviceToHost, s), "read loss");
    VV_CUDA(cudaStreamSynchronize(s), "denoiser step");
    if ((st = check_device_status(dn, s)) != VVPT_OK)
        return st;
    if (loss_out)
        *loss_out = l / (3.0f * (float)p0);
    return VVPT_OK;
}

}  // namespace

extern "C" {

VVPT_API vvpt_status vvpt_denoiser_create(vvpt_ctx *ctx, uint64_t seed, vvpt_denoiser **out)
{
    if (!ctx || !out)
        return fail(ctx, VVPT_ERR_INVALID_ARG, "null argument");
    *out = nullptr;
    std::lock_guard<std::mutex> lk(ctx->mu);
    cudaSetDevice(ctx->device);
    auto dn = new vvpt_denoiser();
    std::unique_ptr<vvpt_denoiser> guard(dn);
    dn->ctx = ctx;
    dn->layers = make_layers(dn->nparams, dn->nw16);
    // He initialisation for the ReLU layers, a small one for the output layer
    // (its rows beyond the 3 radiance channels stay zero)
    std::vector<float> p(dn->nparams, 0.0f);
    InitRng rng{seed * 0x2545F4914F6CDD1Dull + 1};
    for (const Layer &L : dn->layers) {
        const double std_ = L.relu ? std::sqrt(2.0 / (9.0 * L.cin)) : 0.1 * std::sqrt(1.0 / (9.0 * L.cin));
        const int rows = L.relu ? L.cout : 3;
        for (int co = 0; co < rows; co++)
            for (int k = 0; k < 9 * L.cin; k++)
                p[L.w_off + (size_t)co * 9 * L.cin + k] = (float)(std_ * rng.normal());
    }
    VV_CUDA(dn->params.alloc(dn->nparams * sizeof(float)), "cudaMalloc denoiser parameters");
    VV_CUDA(dn->grads.alloc(dn->nparams * sizeof(float)), "cudaMalloc denoiser gradients");
    VV_CUDA(dn->adam_m.alloc(dn->nparams * sizeof(float)), "cudaMalloc denoiser optimiser");
    VV_CUDA(dn->adam_v.alloc(dn->nparams * sizeof(float)), "cudaMalloc denoiser optimiser");
    VV_CUDA(dn->w16.alloc(dn->nw16 * sizeof(bf16)), "cudaMalloc denoiser weights");
    VV_CUDA(dn->err.alloc(sizeof(uint32_t)), "cudaMalloc denoiser status");
    VV_CUDA(dn->wt16.alloc(dn->nw16 * sizeof(bf16)), "cudaMalloc denoiser weights");
    cudaStream_t s = vv_stream(ctx);
    VV_CUDA(cudaMemcpyAsync(dn->params.ptr, p.data(), p.size() * sizeof(float), cudaMemcpyHostToDevice, s),
            "upload parameters");
    VV_CUDA(cudaMemsetAsync(dn->err.ptr, 0, sizeof(uint32_t), s), "clear denoiser status");
    VV_CUDA(cudaMemsetAsync(dn->adam_m.ptr, 0, dn->nparams * sizeof(float), s), "clear optimiser");
    VV_CUDA(cudaMemsetAsync(dn->adam_v.ptr, 0, dn->nparams * sizeof(float), s), "clear optimiser");
    VV_CUDA(cudaStreamSynchronize(s), "denoiser create");
    *out = guard.release();
    return VVPT_OK;
}

VVPT_API vvpt_status vvpt_denoiser_destroy(vvpt_denoiser *dn)
{
    if (!dn)
        return VVPT_ERR_INVALID_ARG;
    cudaSetDevice(dn->ctx->device);
    cudaStreamSynchronize(vv_stream(dn->ctx));
    delete dn;
    return VVPT_OK;
}

VVPT_API vvpt_status vvpt_denoiser_num_params(vvpt_denoiser *dn, uint64_t *out)
{
    if (!dn || !out)
        return VVPT_ERR_INVALID_ARG;
    *out = dn->nparams;
    return VVPT_OK;
}

VVPT_API vvpt_status vvpt_denoiser_get_params(vvpt_denoiser *dn, float *host, uint64_t n)
{
    if (!dn || !host || n != dn->nparams)
        return fail(dn ? dn->ctx : nullptr, VVPT_ERR_INVALID_ARG, "parameter count mismatch");
    vvpt_ctx *ctx = dn->ctx;
    std::lock_guard<std::mutex> lk(ctx->mu);
    VV_CUDA(cudaMemcpy(host, dn->params.ptr, n * sizeof(float), cudaMemcpyDeviceToHost), "read parameters");
    return VVPT_OK;
}

VVPT_API vvpt_status vvpt_denoiser_set_params(vvpt_denoiser *dn, const float *host, uint64_t n)
{
    if (!dn || !host || n != dn->nparams)
        return fail(dn ? dn->ctx : nullptr, VVPT_ERR_INVALID_ARG, "parameter count mismatch");
    vvpt_ctx *ctx = dn->ctx;
    std::lock_guard<std::mutex> lk(ctx->mu);
    VV_CUDA(cudaMemcpy(dn->params.ptr, host, n * sizeof(float), cudaMemcpyHostToDevice), "write parameters");
    dn->weights_dirty = true;
    return VVPT_OK;
}

VVPT_API vvpt_status vvpt_denoiser_gradients(vvpt_denoiser *dn, const vvpt_denoise_batch *batch, float *grads_host,
                                             uint64_t n, float *loss)
{
    if (!dn || !grads_host || n != dn->nparams)
        return fail(dn ? dn->ctx : nullptr, VVPT_ERR_INVALID_ARG, "parameter count mismatch");
    vvpt_ctx *ctx = dn->ctx;
    std::lock_guard<std::mutex> lk(ctx->mu);
    cudaSetDevice(ctx->device);
    vvpt_status st = loss_and_grads(dn, batch, loss);
    if (st != VVPT_OK)
        return st;
    VV_CUDA(cudaMemcpy(grads_host, dn->grads.ptr, n * sizeof(float), cudaMemcpyDeviceToHost), "read gradients");
    return VVPT_OK;
}

VVPT_API vvpt_status vvpt_denoiser_train_step(vvpt_denoiser *dn, const vvpt_denoise_batch *batch, float lr,
                                              float *loss)
{
    if (!dn)
        return VVPT_ERR_INVALID_ARG;
    vvpt_ctx *ctx = dn->ctx;
    std::lock_guard<std::mutex> lk(ctx->mu);
    cudaSetDevice(ctx->device);
    vvpt_status st = loss_and_grads(dn, batch, loss);
    if (st != VVPT_OK)
        return st;
    cudaStream_t s = vv_stream(ctx);
    dn->step++;
    vvdn::adam(dn->params.as<float>(), dn->grads.as<float>(), dn->adam_m.as<float>(), dn->adam_v.as<float>(),
               dn->nparams, lr, 0.9f, 0.999f, 1e-8f, dn->step, s);
    dn->weights_dirty = true;
    VV_CUDA(cudaGetLastError(), "adam");
    return VVPT_OK;
}

VVPT_API vvpt_status vvpt_denoiser_set_kernels(vvpt_denoiser *dn, int kind)
{
    if (!dn || kind < VVPT_DENOISER_TCGEN05 || kind > VVPT_DENOISER_TCGEN05_WGRAD)
        return VVPT_ERR_INVALID_ARG;
    dn->mma_sync = kind == VVPT_DENOISER_MMA_SYNC;
    dn->conv_kind = kind == VVPT_DENOISER_TCGEN05_TILES        ? vvdn::kConvTiles
                    : kind == VVPT_DENOISER_TCGEN05_PERSISTENT ? vvdn::kConvPersistent
                    : kind == VVPT_DENOISER_TCGEN05_UNFUSED    ? vvdn::kConvNoFusion
                    : kind == VVPT_DENOISER_TCGEN05_WGRAD      ? vvdn::kConvWgradTc
                                                               : vvdn::kConvAuto;
    return VVPT_OK;
}

VVPT_API vvpt_status vvpt_denoiser_inject_wait_timeout(vvpt_denoiser *dn)
{
    if (!dn)
        return VVPT_ERR_INVALID_ARG;
    vvdn::inject_wait_timeout();
    return VVPT_OK;
}

VVPT_API vvpt_status vvpt_denoiser_apply(vvpt_denoiser *dn, const float *radiance, const float *albedo,
                                         const float *normal, float *out, uint32_t width, uint32_t height)
{
    if (!dn || !radiance || !albedo || !normal || !out)
        return fail(dn ? dn->ctx : nullptr, VVPT_ERR_INVALID_ARG, "null argument");
    vvpt_ctx *ctx = dn->ctx;
    std::lock_guard<std::mutex> lk(ctx->mu);
    cudaSetDevice(ctx->device);
    vvpt_status st = check_shape(ctx, 1, width, height);
    if (st != VVPT_OK)
        return st;
    if ((st = ensure_shape(dn, 1, (int)height, (int)width, false)) != VVPT_OK)
        return st;
    cudaStream_t s = vv_stream(ctx);
    const bool fused_out = !dn->mma_sync && (reinterpret_cast<uintptr_t>(out) & 15) == 0;
    forward(dn, radiance, albedo, normal, s, true, fused_out ? out : nullptr);
    if (!fused_out)
        vvdn::unpack_output(dn->out_f32.as<float>(), kOutCh, out, (int)(width * height), s);
    VV_CUDA(cudaGetLastError(), "denoiser kernels");
    return check_device_status(dn, s);
}

}  // extern "C"
