// Denoiser kernels (denoise_kernels.cuh). The convolutions are implicit GEMMs
// on the BF16 tensor cores with FP32 accumulators: tcgen05 MMAs into TMEM
// (the strip kernel, TMA-fed, for layers whose weights fit in shared memory;
// per-tile kernels for the rest), and the warp-level mma.sync m16n8k16 kernels
// (operand tiles read with ldmatrix) kept as a cross-check.
#include <algorithm>
#include <atomic>

#include <cuda.h>
#include <cudaTypedefs.h>

#include "denoise_kernels.cuh"

namespace vvdn {

namespace {

constexpr int kTileC = 64;  // channels per weight-gradient block tile

__device__ __forceinline__ uint32_t smem_addr(const void *p)
{
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void ldsm_x4(uint32_t addr, uint32_t &r0, uint32_t &r1, uint32_t &r2, uint32_t &r3)
{
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0, %1, %2, %3}, [%4];\n"
                 : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
                 : "r"(addr));
}

__device__ __forceinline__ void ldsm_x4_t(uint32_t addr, uint32_t &r0, uint32_t &r1, uint32_t &r2, uint32_t &r3)
{
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0, %1, %2, %3}, [%4];\n"
                 : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
                 : "r"(addr));
}

__device__ __forceinline__ void mma_bf16(float (&c)[4], uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3,
                                         uint32_t b0, uint32_t b1)
{
    asm volatile("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0, %1, %2, %3}, {%4, %5, %6, %7}, "
                 "{%8, %9}, {%0, %1, %2, %3};\n"
                 : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
                 : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

// Asynchronous 16-byte global -> shared copy; src_bytes = 0 writes zeros
// (padding, channels past cin, rows past cout).
__device__ __forceinline__ void cp_async16(void *smem, const void *gmem, bool valid)
{
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(smem_addr(smem)), "l"(gmem),
                 "r"(valid ? 16 : 0));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N)); }

// Forward tile: 256 threads = 8 warps; block tile 128 pixels x BN output
// channels (BN = 64: warps 4 x 2 of 32 x 32; BN = 32: warps 8 x 1 of 16 x 32,
// for the 32- and 16-channel layers). K runs over (tap, 32-channel chunk)
// with a 3-stage cp.async pipeline.
constexpr int kBM = 128, kBK = 32, kStages = 3, kLds = kBK + 8;

template <int BN, int WM>
__global__ void __launch_bounds__(256) k_conv3x3(ConvArgs a)
{
    constexpr int WN = 32;                // channels per warp
    constexpr int WARPS_M = kBM / WM;     // 4 or 8
    constexpr int MT = WM / 16, NT = WN / 8;
    static_assert(WARPS_M * (BN / WN) == 8, "8 warps");
    __shared__ __align__(128) bf16 sA[kStages][kBM][kLds];
    __shared__ __align__(128) bf16 sB[kStages][BN][kLds];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int wm = warp % WARPS_M, wn = warp / WARPS_M;
    const long P = (long)a.n * a.h * a.wd;
    const long p0 = (long)blockIdx.x * kBM;
    const int c0 = blockIdx.y * BN;
    const int nchunks = (a.cin + kBK - 1) / kBK;
    const int KT = 9 * nchunks;
    // A loads: row tid / 2, two 8-channel vectors starting at (tid % 2) * 16
    const int ar = tid >> 1, av = (tid & 1) * 16;
    const long ap = p0 + ar;
    int an = 0, ay = 0, ax = 0;
    if (ap < P) {
        an = (int)(ap / ((long)a.h * a.wd));
        const int rem = (int)(ap - (long)an * a.h * a.wd);
        ay = rem / a.wd;
        ax = rem - ay * a.wd;
    }
    // B loads: row tid / 4, one 8-channel vector at (tid % 4) * 8 (BN * 4 threads)
    const int br = tid >> 2, bv = (tid & 3) * 8;
    const int bc = c0 + br;

    auto load_stage = [&](int stage, int kt) {
        const int tap = kt / nchunks, ci0 = (kt - tap * nchunks) * kBK;
        const int yy = ay + tap / 3 - 1, xx = ax + tap % 3 - 1;
        const bool pix_ok = ap < P && yy >= 0 && yy < a.h && xx >= 0 && xx < a.wd;
        const long pix = pix_ok ? (((long)an * a.h + yy) * a.wd + xx) : 0;
#pragma unroll
        for (int v = 0; v < 2; v++) {
            const int ci = ci0 + av + 8 * v;
            const bool ok = pix_ok && ci < a.cin;
            cp_async16(&sA[stage][ar][av + 8 * v], ok ? (const void *)(a.in + pix * a.cin + ci) : (const void *)a.in,
                       ok);
        }
        if (br < BN) {
            const int ci = ci0 + bv;
            const bool okb = bc < a.cout && ci < a.cin;
            cp_async16(&sB[stage][br][bv], okb ? (const void *)(a.wgt + ((long)bc * 9 + tap) * a.cin + ci)
                                               : (const void *)a.wgt,
                       okb);
        }
    };

    float acc[MT][NT][4];
#pragma unroll
    for (int i = 0; i < MT; i++)
#pragma unroll
        for (int j = 0; j < NT; j++)
            acc[i][j][0] = acc[i][j][1] = acc[i][j][2] = acc[i][j][3] = 0.0f;

#pragma unroll
    for (int s = 0; s < kStages - 1; s++) {
        if (s < KT)
            load_stage(s, s);
        cp_async_commit();
    }
    for (int kt = 0; kt < KT; kt++) {
        cp_async_wait<kStages - 2>();
        __syncthreads();
        // refill the stage consumed in the previous iteration
        const int nk = kt + kStages - 1;
        if (nk < KT)
            load_stage(nk % kStages, nk);
        cp_async_commit();
        const int st = kt % kStages;
#pragma unroll
        for (int ks = 0; ks < kBK; ks += 16) {
            uint32_t af[MT][4], bfr[NT / 2][4];
#pragma unroll
            for (int mt = 0; mt < MT; mt++)
                ldsm_x4(smem_addr(&sA[st][wm * WM + mt * 16 + (lane & 15)][ks + (lane >> 4) * 8]), af[mt][0],
                        af[mt][1], af[mt][2], af[mt][3]);
#pragma unroll
            for (int j = 0; j < NT / 2; j++)
                ldsm_x4(smem_addr(&sB[st][wn * WN + 16 * j + (lane & 7) + ((lane >> 4) << 3)]
                                      [ks + ((lane >> 3) & 1) * 8]),
                        bfr[j][0], bfr[j][1], bfr[j][2], bfr[j][3]);
#pragma unroll
            for (int mt = 0; mt < MT; mt++)
#pragma unroll
                for (int j = 0; j < NT / 2; j++) {
                    mma_bf16(acc[mt][2 * j], af[mt][0], af[mt][1], af[mt][2], af[mt][3], bfr[j][0], bfr[j][1]);
                    mma_bf16(acc[mt][2 * j + 1], af[mt][0], af[mt][1], af[mt][2], af[mt][3], bfr[j][2], bfr[j][3]);
                }
        }
    }
    cp_async_wait<0>();
    // epilogue: c0,c1 at (row g, cols 2t, 2t+1), c2,c3 at row g + 8
    const int g = lane >> 2, t = lane & 3;
#pragma unroll
    for (int mt = 0; mt < MT; mt++)
#pragma unroll
        for (int half = 0; half < 2; half++) {
            const long p = p0 + wm * WM + mt * 16 + g + half * 8;
            if (p >= P)
                continue;
#pragma unroll
            for (int j = 0; j < NT; j++) {
                const int col = c0 + wn * WN + 8 * j + 2 * t;
                if (col >= a.cout)
                    continue;
                float v0 = acc[mt][j][2 * half], v1 = acc[mt][j][2 * half + 1];
                if (a.bias) {
                    v0 += a.bias[col];
                    v1 += a.bias[col + 1];
                }
                if (a.relu) {
                    v0 = fmaxf(v0, 0.0f);
                    v1 = fmaxf(v1, 0.0f);
                }
                const long o = p * a.cout + col;
                if (a.mask) {
                    const __nv_bfloat162 m = *reinterpret_cast<const __nv_bfloat162 *>(a.mask + o);
                    if (!(__bfloat162float(m.x) > 0.0f))
                        v0 = 0.0f;
                    if (!(__bfloat162float(m.y) > 0.0f))
                        v1 = 0.0f;
                }
                if (a.out_f32)
                    *reinterpret_cast<float2 *>(reinterpret_cast<float *>(a.out) + o) = make_float2(v0, v1);
                else
                    *reinterpret_cast<__nv_bfloat162 *>(reinterpret_cast<bf16 *>(a.out) + o) =
                        __floats2bfloat162_rn(v0, v1);
            }
        }
}

// Weight gradient for one tap: block tile BM output channels x 64 input
// channels, K = a slice of pixels in steps of 32 through a 3-stage cp.async
// pipeline. BM = 64: warp w owns output channels [16w, 16w + 16) and all 64
// input channels; BM = 32 (layers of at most 32 output channels): warp w
// owns output channels 16 (w & 1) and input channels 32 (w >> 1). Partial
// sums are added to dw with atomics.
constexpr int kWgK = 32, kWgStages = 3;
template <int BM>
__global__ void __launch_bounds__(128) k_conv3x3_wgrad(const bf16 *__restrict__ dout, int cout,
                                                       const bf16 *__restrict__ in, int cin, int n, int h, int w,
                                                       float *dw, long slice)
{
    constexpr int NT = BM == 64 ? 8 : 4; // n-tiles of 8 input channels per warp
    __shared__ __align__(16) bf16 Ds[kWgStages][kWgK][kTileC + 8]; // [pixel][cout]
    __shared__ __align__(16) bf16 Xs[kWgStages][kWgK][kTileC + 8]; // [pixel][cin]
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int tap = blockIdx.y % 9;
    const int tiles_ci = (cin + kTileC - 1) / kTileC;
    const int ct = blockIdx.y / 9;
    const int co0 = (ct / tiles_ci) * BM, ci0 = (ct % tiles_ci) * kTileC;
    const long P = (long)n * h * w;
    const long pbeg = (long)blockIdx.x * slice, pend = min(P, pbeg + slice);
    const int dy = tap / 3 - 1, dx = tap % 3 - 1;
    const int wm = BM == 64 ? warp * 16 : (warp & 1) * 16; // warp's output-channel offset in the tile
    const int wn = BM == 64 ? 0 : (warp >> 1) * 32;        // warp's input-channel offset in the tile
    // load mapping: row = tid / 4 (pixel), group = (tid % 4) * 16 channels
    const int lr = tid >> 2, lg = (tid & 3) * 16;
    float acc[NT][4];
#pragma unroll
    for (int j = 0; j < NT; j++)
        acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.0f;
    const int nsteps = (int)((pend - pbeg + kWgK - 1) / kWgK);
    auto load = [&](int step) {
        const int st = step % kWgStages;
        const long p = pbeg + (long)step * kWgK + lr;
        const bool ok = p < pend;
        int pn = 0, py = 0, px = 0;
        if (ok) {
            pn = (int)(p / ((long)h * w));
            const int rem = (int)(p - (long)pn * h * w);
            py = rem / w;
            px = rem - py * w;
        }
        const int co = co0 + lg, ci = ci0 + lg;
        const bool dok = ok && co < cout && lg < BM;
        const bf16 *ds = dok ? dout + p * cout + co : dout;
        cp_async16(&Ds[st][lr][lg], ds, dok);
        cp_async16(&Ds[st][lr][lg + 8], dok ? ds + 8 : dout, dok);
        const int yy = py + dy, xx = px + dx;
        const bool xok = ok && yy >= 0 && yy < h && xx >= 0 && xx < w && ci < cin;
        const bf16 *xs = xok ? in + (((long)pn * h + yy) * w + xx) * cin + ci : in;
        cp_async16(&Xs[st][lr][lg], xs, xok);
        cp_async16(&Xs[st][lr][lg + 8], xok ? xs + 8 : in, xok);
    };
    for (int st = 0; st < kWgStages - 1; st++) {
        if (st < nsteps)
            load(st);
        cp_async_commit();
    }
    for (int step = 0; step < nsteps; step++) {
        cp_async_wait<kWgStages - 2>();
        __syncthreads();
        const int st = step % kWgStages;
#pragma unroll
        for (int ks = 0; ks < kWgK; ks += 16) {
            // A[m = cout][k = pixel] from Ds[k][m] (transposed load)
            uint32_t a0, a1, a2, a3;
            ldsm_x4_t(smem_addr(&Ds[st][ks + (lane & 7) + ((lane >> 4) << 3)][wm + ((lane >> 3) & 1) * 8]), a0, a1,
                      a2, a3);
#pragma unroll
            for (int j = 0; j < NT / 2; j++) {
                // B[k = pixel][n = cin] from Xs[k][n] (transposed load): two n-tiles
                uint32_t b0, b1, b2, b3;
                ldsm_x4_t(smem_addr(&Xs[st][ks + (lane & 7) + ((lane >> 3) & 1) * 8][wn + 16 * j + (lane >> 4) * 8]),
                          b0, b1, b2, b3);
                mma_bf16(acc[2 * j], a0, a1, a2, a3, b0, b1);
                mma_bf16(acc[2 * j + 1], a0, a1, a2, a3, b2, b3);
            }
        }
        // the stage refilled next was read two steps ago; the barrier above
        // ordered those reads
        if (step + kWgStages - 1 < nsteps)
            load(step + kWgStages - 1);
        cp_async_commit();
    }
    cp_async_wait<0>();
    const int g = lane >> 2, t = lane & 3;
#pragma unroll
    for (int half = 0; half < 2; half++) {
        const int co = co0 + wm + g + half * 8;
        if (co >= cout)
            continue;
#pragma unroll
        for (int j = 0; j < NT; j++) {
            const int ci = ci0 + wn + 8 * j + 2 * t;
            if (ci >= cin)
                continue;
            float *d = dw + ((long)co * 9 + tap) * cin + ci;
            atomicAdd(d, acc[j][2 * half]);
            atomicAdd(d + 1, acc[j][2 * half + 1]);
        }
    }
}

// The layout kernels below move 8 channels (16 bytes) per thread: channel
// counts are multiples of 8, so every access is one aligned 128-bit load or
// store and a warp covers 512 consecutive bytes. Index arithmetic is 32-bit
// (element counts stay below 2^31; the host checks).
__device__ __forceinline__ void unpack8(const uint4 &v, float (&f)[8])
{
    const __nv_bfloat162 *h = reinterpret_cast<const __nv_bfloat162 *>(&v);
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const float2 t = __bfloat1622float2(h[k]);
        f[2 * k] = t.x;
        f[2 * k + 1] = t.y;
    }
}

__device__ __forceinline__ uint4 pack8(const float (&f)[8])
{
    uint4 v;
    __nv_bfloat162 *h = reinterpret_cast<__nv_bfloat162 *>(&v);
#pragma unroll
    for (int k = 0; k < 4; k++)
        h[k] = __floats2bfloat162_rn(f[2 * k], f[2 * k + 1]);
    return v;
}

__device__ __forceinline__ uint4 ld16(const bf16 *p) { return __ldg(reinterpret_cast<const uint4 *>(p)); }
__device__ __forceinline__ void st16(bf16 *p, const uint4 &v) { *reinterpret_cast<uint4 *>(p) = v; }

// dbias[c] += sum_p dout[p][c]: a thread sums 8 channels (one 16-byte load
// per pixel) over a strided set of pixels, the block reduces its pixel lanes
// in shared memory and adds one value per channel.
constexpr int kBiasThreads = 256;
__global__ void __launch_bounds__(kBiasThreads) k_bias_grad(const bf16 *dout, int cout, long P, float *dbias)
{
    __shared__ float red[kBiasThreads * 8];
    const int G = cout >> 3, lanes = kBiasThreads / G;
    const int g = threadIdx.x % G, r = threadIdx.x / G;
    float acc[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    if (r < lanes) {
        for (long p = (long)blockIdx.x * lanes + r; p < P; p += (long)gridDim.x * lanes) {
            float v[8];
            unpack8(ld16(dout + p * cout + 8 * g), v);
#pragma unroll
            for (int k = 0; k < 8; k++)
                acc[k] += v[k];
        }
    }
#pragma unroll
    for (int k = 0; k < 8; k++)
        red[threadIdx.x * 8 + k] = acc[k];
    __syncthreads();
    for (int c = threadIdx.x; c < cout; c += kBiasThreads) {
        float sum = 0.0f;
        for (int q = 0; q < lanes; q++)
            sum += red[(q * G + (c >> 3)) * 8 + (c & 7)];
        atomicAdd(dbias + c, sum);
    }
}

__global__ void k_transform_weights(const bf16 *w, bf16 *wt, int cout, int cin)
{
    const long total = (long)cout * 9 * cin;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x) {
        const int ci = (int)(i % cin);
        const int tap = (int)((i / cin) % 9);
        const int co = (int)(i / ((long)cin * 9));
        wt[((long)ci * 9 + (8 - tap)) * cout + co] = w[i];
    }
}

__global__ void k_to_bf16(const float *src, bf16 *dst, size_t n)
{
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        dst[i] = __float2bfloat16_rn(src[i]);
}

__global__ void k_pack_features(const float4 *rad, const float4 *alb, const float4 *nrm, bf16 *x, int npix)
{
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < npix; p += gridDim.x * blockDim.x) {
        const float4 r = rad[p], a = alb[p], q = nrm[p];
        __align__(16) bf16 v[16];
        v[0] = __float2bfloat16_rn(log1pf(fmaxf(r.x, 0.0f)));
        v[1] = __float2bfloat16_rn(log1pf(fmaxf(r.y, 0.0f)));
        v[2] = __float2bfloat16_rn(log1pf(fmaxf(r.z, 0.0f)));
        v[3] = __float2bfloat16_rn(a.x);
        v[4] = __float2bfloat16_rn(a.y);
        v[5] = __float2bfloat16_rn(a.z);
        v[6] = __float2bfloat16_rn(q.x);
        v[7] = __float2bfloat16_rn(q.y);
        v[8] = __float2bfloat16_rn(q.z);
#pragma unroll
        for (int k = 9; k < 16; k++)
            v[k] = __float2bfloat16_rn(0.0f);
        uint4 *dst = reinterpret_cast<uint4 *>(x + (long)p * 16);
        dst[0] = *reinterpret_cast<const uint4 *>(&v[0]);
        dst[1] = *reinterpret_cast<const uint4 *>(&v[8]);
    }
}

__global__ void k_pack_target(const float4 *t, float *t3, int npix)
{
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < npix; p += gridDim.x * blockDim.x) {
        const float4 v = t[p];
        t3[3 * p] = log1pf(fmaxf(v.x, 0.0f));
        t3[3 * p + 1] = log1pf(fmaxf(v.y, 0.0f));
        t3[3 * p + 2] = log1pf(fmaxf(v.z, 0.0f));
    }
}

__global__ void k_avgpool2(const bf16 *in, bf16 *out, int n, int h, int w, int c)
{
    const unsigned ho = h / 2, wo = w / 2, g = c / 8;
    const unsigned total = (unsigned)n * ho * wo * g;
    for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
        const unsigned cg = i % g, q = i / g;
        const unsigned x = q % wo, y = (q / wo) % ho, b = q / (wo * ho);
        const size_t base = (((size_t)b * h + 2 * y) * w + 2 * x) * c + 8 * cg, row = (size_t)w * c;
        float a[8], t[8];
        unpack8(ld16(in + base), a);
        unpack8(ld16(in + base + c), t);
#pragma unroll
        for (int k = 0; k < 8; k++)
            a[k] += t[k];
        unpack8(ld16(in + base + row), t);
#pragma unroll
        for (int k = 0; k < 8; k++)
            a[k] += t[k];
        unpack8(ld16(in + base + row + c), t);
#pragma unroll
        for (int k = 0; k < 8; k++)
            a[k] = 0.25f * (a[k] + t[k]);
        st16(out + (size_t)i * 8, pack8(a));
    }
}

__global__ void k_upcat(const bf16 *coarse, int cc, const bf16 *skip, int cs, bf16 *out, int n, int h, int w)
{
    const unsigned gc = cc / 8, gt = (cc + cs) / 8;
    const unsigned total = (unsigned)n * h * w * gt;
    for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
        const unsigned cg = i % gt, p = i / gt;
        uint4 v;
        if (cg < gc) {
            const unsigned x = p % w, y = (p / w) % h, b = p / (w * h);
            v = ld16(coarse + (((size_t)b * (h / 2) + y / 2) * (w / 2) + x / 2) * cc + 8 * cg);
        } else {
            v = ld16(skip + (size_t)p * cs + 8 * (cg - gc));
        }
        st16(out + (size_t)i * 8, v);
    }
}

__global__ void k_upcat_backward_coarse(const bf16 *dcat, int cc, int cs, bf16 *dcoarse, int n, int h, int w)
{
    const int ct = cc + cs;
    const unsigned ho = h / 2, wo = w / 2, g = cc / 8;
    const unsigned total = (unsigned)n * ho * wo * g;
    for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
        const unsigned cg = i % g, q = i / g;
        const unsigned x = q % wo, y = (q / wo) % ho, b = q / (wo * ho);
        const size_t base = (((size_t)b * h + 2 * y) * w + 2 * x) * ct + 8 * cg, row = (size_t)w * ct;
        float a[8], t[8];
        unpack8(ld16(dcat + base), a);
        unpack8(ld16(dcat + base + ct), t);
#pragma unroll
        for (int k = 0; k < 8; k++)
            a[k] += t[k];
        unpack8(ld16(dcat + base + row), t);
#pragma unroll
        for (int k = 0; k < 8; k++)
            a[k] += t[k];
        unpack8(ld16(dcat + base + row + ct), t);
#pragma unroll
        for (int k = 0; k < 8; k++)
            a[k] += t[k];
        st16(dcoarse + (size_t)i * 8, pack8(a));
    }
}

__global__ void k_upcat_backward_skip(const bf16 *dcat, int cc, int cs, bf16 *dskip, unsigned npix)
{
    const unsigned g = cs / 8, gt = (cc + cs) / 8, gc = cc / 8;
    const unsigned total = npix * g;
    for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
        const unsigned cg = i % g, p = i / g;
        st16(dskip + (size_t)i * 8, ld16(dcat + ((size_t)p * gt + gc + cg) * 8));
    }
}

__global__ void k_pool_backward_combine(const bf16 *dskip, const bf16 *dpooled, const bf16 *e, bf16 *de, int n, int h,
                                        int w, int c)
{
    const unsigned g = c / 8;
    const unsigned total = (unsigned)n * h * w * g;
    for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
        const unsigned cg = i % g, p = i / g;
        const unsigned x = p % w, y = (p / w) % h, b = p / (w * h);
        float v[8], t[8], m[8];
        unpack8(ld16(dpooled + (((size_t)b * (h / 2) + y / 2) * (w / 2) + x / 2) * c + 8 * cg), v);
#pragma unroll
        for (int k = 0; k < 8; k++)
            v[k] *= 0.25f;
        if (dskip) {
            unpack8(ld16(dskip + (size_t)i * 8), t);
#pragma unroll
            for (int k = 0; k < 8; k++)
                v[k] += t[k];
        }
        unpack8(ld16(e + (size_t)i * 8), m);
#pragma unroll
        for (int k = 0; k < 8; k++)
            if (!(m[k] > 0.0f))
                v[k] = 0.0f;
        st16(de + (size_t)i * 8, pack8(v));
    }
}

__global__ void k_l1_loss(const float *out, int cout, const float *t3, bf16 *dout, float *loss_sum, int npix)
{
    float local = 0.0f;
    const float scale = 1.0f / (3.0f * (float)npix);
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < npix; p += gridDim.x * blockDim.x) {
        for (int c = 0; c < cout; c++) {
            float g = 0.0f;
            if (c < 3) {
                const float d = out[(long)p * cout + c] - t3[3 * p + c];
                local += fabsf(d);
                g = d > 0.0f ? scale : (d < 0.0f ? -scale : 0.0f);
            }
            dout[(long)p * cout + c] = __float2bfloat16_rn(g);
        }
    }
    for (int o = 16; o > 0; o >>= 1)
        local += __shfl_xor_sync(0xffffffffu, local, o);
    if ((threadIdx.x & 31) == 0)
        atomicAdd(loss_sum, local);
}

__global__ void k_adam(float *p, const float *g, float *m, float *v, size_t n, float lr, float b1, float b2, float eps,
                       float c1, float c2)
{
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const float gi = g[i];
        const float mi = b1 * m[i] + (1.0f - b1) * gi;
        const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    }
}

__global__ void k_unpack_output(const float *y, int cout, float4 *out, int npix)
{
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < npix; p += gridDim.x * blockDim.x) {
        const float *v = y + (long)p * cout;
        out[p] = make_float4(expm1f(fmaxf(v[0], 0.0f)), expm1f(fmaxf(v[1], 0.0f)), expm1f(fmaxf(v[2], 0.0f)), 1.0f);
    }
}

int grid_for(long n, int block = 256)
{
    return (int)std::max<long>(1, std::min<long>((n + block - 1) / block, 152L * 16));
}


// ---------------------------------------------------------------------------
// tcgen05 convolution (5th-generation tensor cores, accumulator in TMEM).
//
// CTA = 128 threads, tile = 128 consecutive pixels of one image row (UMMA
// M = 128: pixel i of the tile is TMEM lane i) x all output channels (N =
// cout <= 256, one accumulator of N f32 columns). For each 32-channel chunk
// of the input the CTA stages a halo of 3 rows x 130 pixels once in shared
// memory; every one of the 9 taps is then an MMA over a shifted view of it
// (the operand descriptor starts 16 bytes per pixel and one halo row further),
// so the input is read once per chunk instead of once per tap. Layout, K-major
// without swizzle: for each halo row and 8-channel group the 130 pixels are
// consecutive 16-byte rows, so 8 consecutive pixels form a core matrix (SBO
// 128 B between pixel groups, LBO 130 x 16 B between channel groups). The
// weights of one (chunk, tap) step go to one of 4 stages. One thread issues
// the MMAs (two m128 nN k16 per step) and commits each step to its stage's
// mbarrier; refills wait on the mbarrier of the step two back (MMAs complete
// in issue order). Waits are bounded by the global timer; on a timeout the
// kernel records an error, stops issuing and still frees its TMEM.
constexpr int kTcM = 128, kTcBK = 32, kTcKC = kTcBK / 8, kTcBStages = 4, kTcHaloPx = kTcM + 2;
constexpr int kTcHaloRow = kTcKC * kTcHaloPx * 16;  // one halo row: 4 channel groups x 130 pixels x 16 B
constexpr int kTcHaloAlloc = 25088;                 // rounded up to 1 KB multiples
constexpr unsigned long long kTcWaitNs = 2000000000ull;

__host__ __device__ constexpr int tc_smem_bytes(int N) { return 2 * kTcHaloAlloc + kTcBStages * N * kTcBK * 2; }

__device__ __forceinline__ unsigned long long globaltimer()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity)
{
    const unsigned long long t0 = globaltimer();
    for (;;) {
        uint32_t done;
        asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                     "selp.u32 %0, 1, 0, p;\n\t}\n"
                     : "=r"(done)
                     : "r"(bar), "r"(parity)
                     : "memory");
        if (done)
            return true;
        if (globaltimer() - t0 > kTcWaitNs)
            return false;
    }
}

// shared-memory matrix descriptor: start, LBO, SBO (16-byte units),
// version 1, no swizzle
__device__ __forceinline__ uint64_t umma_desc(uint32_t addr, uint32_t lbo, uint32_t sbo)
{
    return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

__device__ __forceinline__ void tmem_ld16(uint32_t addr, uint32_t (&r)[16])
{
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, "
                 "%14, %15}, [%16];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                   "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
                   "=r"(r[15])
                 : "r"(addr));
    asm volatile("tcgen05.wait::ld.sync.aligned;");
}

// Epilogue of one pixel row x 16 channels: bias, ReLU, mask, store (bf16, or
// f32 for the output layer).
__device__ __forceinline__ void store_row16(const ConvArgs &a, long p, int c, const uint32_t (&r)[16])
{
    float v[16];
#pragma unroll
    for (int k = 0; k < 16; k++) {
        v[k] = __uint_as_float(r[k]);
        if (a.bias)
            v[k] += a.bias[c + k];
        if (a.relu)
            v[k] = fmaxf(v[k], 0.0f);
    }
    if (a.rgba) {
        // the output unpacking of the frame, in the epilogue (k_unpack_output)
        if (c == 0)
            a.rgba[p] = make_float4(expm1f(fmaxf(v[0], 0.0f)), expm1f(fmaxf(v[1], 0.0f)), expm1f(fmaxf(v[2], 0.0f)),
                                    1.0f);
        return;
    }
    const long o = p * a.cout + c;
    if (a.mask) {
        __align__(16) bf16 m[16];
        *reinterpret_cast<uint4 *>(&m[0]) = *reinterpret_cast<const uint4 *>(a.mask + o);
        *reinterpret_cast<uint4 *>(&m[8]) = *reinterpret_cast<const uint4 *>(a.mask + o + 8);
#pragma unroll
        for (int k = 0; k < 16; k++)
            if (!(__bfloat162float(m[k]) > 0.0f))
                v[k] = 0.0f;
    }
    if (a.out_f32) {
        float4 *dst = reinterpret_cast<float4 *>(reinterpret_cast<float *>(a.out) + o);
#pragma unroll
        for (int k = 0; k < 4; k++)
            dst[k] = make_float4(v[4 * k], v[4 * k + 1], v[4 * k + 2], v[4 * k + 3]);
    } else {
        __align__(16) __nv_bfloat162 hh[8];
#pragma unroll
        for (int k = 0; k < 8; k++)
            hh[k] = __floats2bfloat162_rn(v[2 * k], v[2 * k + 1]);
        uint4 *dst = reinterpret_cast<uint4 *>(reinterpret_cast<bf16 *>(a.out) + o);
        dst[0] = *reinterpret_cast<const uint4 *>(&hh[0]);
        dst[1] = *reinterpret_cast<const uint4 *>(&hh[4]);
    }
}

__global__ void __launch_bounds__(128) k_conv3x3_tc(ConvArgs a, int ncols, uint32_t *err)
{
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ uint32_t tmem_holder;
    __shared__ __align__(8) uint64_t mbar[kTcBStages];
    __shared__ int abort_flag;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int tiles_x = (a.wd + kTcM - 1) / kTcM;
    const int tx = blockIdx.x % tiles_x;
    const int y = (blockIdx.x / tiles_x) % a.h;
    const int nb = blockIdx.x / (tiles_x * a.h);
    const int x0 = tx * kTcM;
    const int N = (a.cout + 15) & ~15;
    const int bstage_bytes = N * kTcBK * 2;
    const int nchunks = (a.cin + kTcBK - 1) / kTcBK;
    const int S = 9 * nchunks;
    uint8_t *halo[2] = {smem, smem + kTcHaloAlloc};
    uint8_t *bst = smem + 2 * kTcHaloAlloc;
    const uint32_t sbase = smem_addr(smem);

    if (tid == 0) {
        for (int st = 0; st < kTcBStages; st++)
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&mbar[st])));
        abort_flag = 0;
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(&tmem_holder)),
                     "r"(ncols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    const uint32_t tmem = tmem_holder;
    // D f32, A/B bf16, both K-major, N >> 3, M >> 4
    const uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(kTcM >> 4) << 24);

    auto load_step = [&](int st) {
        const int c = st / 9, tap = st - c * 9, ci0 = c * kTcBK;
        if (tap == 0) {
            // halo of chunk c: 3 rows x 130 pixels x 4 channel groups
            uint8_t *h = halo[c & 1];
            for (int i = tid; i < 3 * kTcKC * kTcHaloPx; i += 128) {
                const int px = i % kTcHaloPx, kc = (i / kTcHaloPx) % kTcKC, hr = i / (kTcHaloPx * kTcKC);
                const int yy = y + hr - 1, xx = x0 - 1 + px, ci = ci0 + 8 * kc;
                const bool ok = yy >= 0 && yy < a.h && xx >= 0 && xx < a.wd && ci < a.cin;
                const bf16 *src = ok ? a.in + (((long)nb * a.h + yy) * a.wd + xx) * a.cin + ci : a.in;
                cp_async16(h + ((hr * kTcKC + kc) * kTcHaloPx + px) * 16, src, ok);
            }
        }
        uint8_t *b = bst + (st % kTcBStages) * bstage_bytes;
        for (int i = tid; i < N * kTcKC; i += 128) {
            const int n = i / kTcKC, kc = i - n * kTcKC, ci = ci0 + 8 * kc;
            const bool ok = n < a.cout && ci < a.cin;
            const bf16 *src = ok ? a.wgt + ((long)n * 9 + tap) * a.cin + ci : a.wgt;
            cp_async16(b + (n >> 3) * (kTcKC * 128) + kc * 128 + (n & 7) * 16, src, ok);
        }
    };

    // prologue: steps 0 and 1
    for (int st = 0; st < 2; st++) {
        if (st < S)
            load_step(st);
        cp_async_commit();
    }
    for (int st = 0; st < S; st++) {
        cp_async_wait<1>(); // this thread's copies of step st landed
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        if (abort_flag)
            break;
        if (tid == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;");
            const int c = st / 9, tap = st - c * 9, dy = tap / 3, dx = tap % 3;
            const uint32_t a_addr = sbase + (c & 1) * kTcHaloAlloc + dy * kTcHaloRow + dx * 16;
            const uint32_t b_addr = sbase + 2 * kTcHaloAlloc + (st % kTcBStages) * bstage_bytes;
#pragma unroll
            for (int j = 0; j < kTcBK / 16; j++) {
                const uint64_t ad = umma_desc(a_addr + j * 2 * kTcHaloPx * 16, kTcHaloPx * 16, 128);
                const uint64_t bd = umma_desc(b_addr + j * 2 * 128, 128, kTcKC * 128);
                const uint32_t accumulate = (st > 0 || j > 0) ? 1u : 0u;
                asm volatile("{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                             "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem),
                             "l"(ad), "l"(bd), "r"(idesc), "r"(accumulate));
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                smem_addr(&mbar[st % kTcBStages])));
        }
        // step st + 2 reuses the weight stage of step st - 2 and, at a chunk
        // start, the halo of chunk (st + 2) / 9 - 2: both done once step st - 2
        // is (in-order completion)
        const int nx = st + 2;
        if (nx < S) {
            if (st >= 2) {
                const int prev = st - 2;
                if (!mbar_wait(smem_addr(&mbar[prev % kTcBStages]), (prev / kTcBStages) & 1))
                    atomicOr(&abort_flag, 1);
            }
            load_step(nx);
        }
        cp_async_commit();
    }
    cp_async_wait<0>();
    if (!abort_flag && S > 0) {
        const int last = S - 1;
        if (!mbar_wait(smem_addr(&mbar[last % kTcBStages]), (last / kTcBStages) & 1))
            atomicOr(&abort_flag, 1);
    }
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    if (!abort_flag) {
        const int x = x0 + warp * 32 + lane;
        const long p = ((long)nb * a.h + y) * a.wd + x;
        for (int c = 0; c < N; c += 16) {
            uint32_t r[16];
            asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, "
                         "%12, %13, %14, %15}, [%16];"
                         : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
                           "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
                           "=r"(r[14]), "=r"(r[15])
                         : "r"(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c));
            asm volatile("tcgen05.wait::ld.sync.aligned;");
            if (x >= a.wd || c >= a.cout)
                continue;
            store_row16(a, p, c, r);
        }
    } else if (tid == 0) {
        atomicOr(err, 1u);
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(ncols));
}

// Chunk-batched variant for N <= 128 output channels: a stage holds the halo
// and the weights of all 9 taps of one 32-channel chunk, so a chunk is one
// barrier and 18 back-to-back MMAs; two stages alternate (the next chunk's
// copies overlap this chunk's MMAs). Same layouts, waits and error handling
// as k_conv3x3_tc.

// one stage when the layer has a single chunk, else two
// halo of `rows` output rows: rows + 2 halo rows, rounded up to 1 KB
__host__ __device__ constexpr int tc_chunk_halo_bytes(int rows) { return ((rows + 2) * kTcHaloRow + 1023) / 1024 * 1024; }

__host__ __device__ constexpr int tc_chunk_smem_bytes(int N, int nchunks, int rows)
{
    return (nchunks > 1 ? 2 : 1) * (tc_chunk_halo_bytes(rows) + 9 * N * kTcBK * 2);
}

// output rows per CTA of the chunk kernel: the chunk's weights are staged once
// for all of them (4 rows up to 64 output channels, else 2: two stages fit)
inline int tc_chunk_rows(int N) { return N <= 64 ? 4 : 2; }

__global__ void __launch_bounds__(128) k_conv3x3_tc_chunk(ConvArgs a, int ncols, int nacc, int rows, uint32_t *err)
{
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ uint32_t tmem_holder;
    __shared__ __align__(8) uint64_t mbar[2];
    __shared__ int abort_flag;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int tiles_x = (a.wd + kTcM - 1) / kTcM;
    const int yblocks = (a.h + rows - 1) / rows;
    const int tx = blockIdx.x % tiles_x;
    const int y0 = (blockIdx.x / tiles_x) % yblocks * rows;
    const int nb = blockIdx.x / (tiles_x * yblocks);
    const int x0 = tx * kTcM;
    const int N = (a.cout + 15) & ~15;
    const int tap_bytes = N * kTcBK * 2;
    const int halo_alloc = tc_chunk_halo_bytes(rows);
    const int stage_bytes = halo_alloc + 9 * tap_bytes;
    const int nchunks = (a.cin + kTcBK - 1) / kTcBK;
    const uint32_t sbase = smem_addr(smem);

    if (tid == 0) {
        for (int st = 0; st < 2; st++)
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&mbar[st])));
        abort_flag = 0;
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(&tmem_holder)),
                     "r"(ncols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    const uint32_t tmem = tmem_holder;
    const uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(kTcM >> 4) << 24);

    auto load_chunk = [&](int c) {
        uint8_t *h = smem + (c & 1) * stage_bytes;
        uint8_t *bw = h + halo_alloc;
        const int ci0 = c * kTcBK;
        for (int i = tid; i < (rows + 2) * kTcKC * kTcHaloPx; i += 128) {
            const int px = i % kTcHaloPx, kc = (i / kTcHaloPx) % kTcKC, hr = i / (kTcHaloPx * kTcKC);
            const int yy = y0 + hr - 1, xx = x0 - 1 + px, ci = ci0 + 8 * kc;
            const bool ok = yy >= 0 && yy < a.h && xx >= 0 && xx < a.wd && ci < a.cin;
            const bf16 *src = ok ? a.in + (((long)nb * a.h + yy) * a.wd + xx) * a.cin + ci : a.in;
            cp_async16(h + ((hr * kTcKC + kc) * kTcHaloPx + px) * 16, src, ok);
        }
        for (int i = tid; i < 9 * N * kTcKC; i += 128) {
            const int kc = i % kTcKC, n = (i / kTcKC) % N, tap = i / (kTcKC * N), ci = ci0 + 8 * kc;
            const bool ok = n < a.cout && ci < a.cin;
            const bf16 *src = ok ? a.wgt + ((long)n * 9 + tap) * a.cin + ci : a.wgt;
            cp_async16(bw + tap * tap_bytes + (n >> 3) * (kTcKC * 128) + kc * 128 + (n & 7) * 16, src, ok);
        }
    };

    load_chunk(0);
    cp_async_commit();
    for (int c = 0; c < nchunks; c++) {
        cp_async_wait<0>(); // this thread's copies of chunk c landed
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        if (abort_flag)
            break;
        if (tid == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;");
            const uint32_t h_addr = sbase + (c & 1) * stage_bytes, b_addr = h_addr + halo_alloc;
            // output row r of the block, tap t: accumulator r * nacc + t % nacc
            // (independent chains); the chunk's weights serve all rows
            for (int r = 0; r < rows; r++) {
#pragma unroll
                for (int j = 0; j < kTcBK / 16; j++) {
#pragma unroll
                    for (int tap = 0; tap < 9; tap++) {
                        const int dy = tap / 3, dx = tap % 3;
                        const uint64_t ad = umma_desc(h_addr + (r + dy) * kTcHaloRow + dx * 16 +
                                                          j * 2 * kTcHaloPx * 16,
                                                      kTcHaloPx * 16, 128);
                        const uint64_t bd = umma_desc(b_addr + tap * tap_bytes + j * 2 * 128, 128, kTcKC * 128);
                        const uint32_t accumulate = (c > 0 || j > 0 || tap >= nacc) ? 1u : 0u;
                        const uint32_t dst = tmem + (uint32_t)((r * nacc + (tap & (nacc - 1))) * N);
                        asm volatile("{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                                     "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(dst),
                                     "l"(ad), "l"(bd), "r"(idesc), "r"(accumulate));
                    }
                }
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                smem_addr(&mbar[c & 1])));
        }
        // chunk c + 1 goes to the stage chunk c - 1 was read from; the MMAs of
        // chunk c are queued behind it meanwhile
        if (c + 1 < nchunks) {
            if (c >= 1 && !mbar_wait(smem_addr(&mbar[(c - 1) & 1]), ((c - 1) >> 1) & 1))
                atomicOr(&abort_flag, 1);
            load_chunk(c + 1);
        }
        cp_async_commit();
    }
    cp_async_wait<0>();
    if (!abort_flag && nchunks > 0) {
        const int last = nchunks - 1;
        if (!mbar_wait(smem_addr(&mbar[last & 1]), (last >> 1) & 1))
            atomicOr(&abort_flag, 1);
    }
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    if (!abort_flag) {
        const int x = x0 + warp * 32 + lane;
        for (int rr = 0; rr < rows && y0 + rr < a.h; rr++) {
            const long p = ((long)nb * a.h + y0 + rr) * a.wd + x;
            const uint32_t lane_base = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(rr * nacc * N);
            for (int c = 0; c < N; c += 16) {
                uint32_t r[16];
                tmem_ld16(lane_base + (uint32_t)c, r);
                for (int q = 1; q < nacc; q++) {
                    uint32_t t[16];
                    tmem_ld16(lane_base + (uint32_t)(q * N + c), t);
#pragma unroll
                    for (int k = 0; k < 16; k++)
                        r[k] = __float_as_uint(__uint_as_float(r[k]) + __uint_as_float(t[k]));
                }
                if (x >= a.wd || c >= a.cout)
                    continue;
                store_row16(a, p, c, r);
            }
        }
    } else if (tid == 0) {
        atomicOr(err, 1u);
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(ncols));
}

// Strip kernel: TMA-fed, weights resident, persistent over runs of rows.
//
// A unit of work is a 128-pixel-wide column of one image and a run of
// consecutive output rows (a segment); a CTA runs its units one after the
// other. The weights of the whole layer (9 x N x cin bf16) are loaded once and
// stay in shared memory. Input rows arrive by TMA into a ring of `ring` slots,
// each one halo row of 130 pixels x cin channels; the tensor map zero-fills
// pixels and rows outside the image, which is the convolution's zero padding.
// Output row i of a segment reads halo rows i, i + 1, i + 2, so every output
// row needs one new halo row (the input is read once, not three times).
// Slot layout (K-major, no swizzle): per 8-channel group the 130 pixels are
// consecutive 16-byte rows (one TMA box of 8 channels x 130 pixels), groups
// kStKCBytes apart; a tap (dy, dx) of output row i is the operand starting at
// slot(i + dy) + 16 dx (SBO 128 B between 8-pixel groups, LBO kStKCBytes
// between channel groups). Two TMEM accumulators alternate between output
// rows; each holds `nacc` partial sums (taps spread over independent MMA
// chains) that the drain adds. The roles (k_conv3x3_strip below) are warp
// specialised: a producer warp, an MMA warp and four drain warps, linked by
// mbarriers only. Halo rows and output rows are counted over the CTA's whole
// run, so slot and accumulator phases carry across units. Every wait is
// bounded by the global timer; on a timeout the kernel records an error, the
// other roles stop at their next wait, copies and MMAs in flight are waited
// for (bounded) and the TMEM is freed.
constexpr int kStKCBytes = 2176; // 130 pixels x 16 B, padded to a multiple of 128 B
constexpr int kStHaloPx = kTcM + 2;
// at least the three halo rows one output row reads; three slots (no row
// prefetched ahead) are taken when they let more CTAs share an SM
constexpr int kStMaxRing = 8, kStMinRing = 3;

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count));
}

// Bounded wait that also gives up once another role has aborted.
__device__ __forceinline__ bool mbar_wait_role(uint32_t bar, uint32_t parity, const volatile int *abort_flag)
{
    const unsigned long long t0 = globaltimer();
    for (;;) {
        uint32_t done;
        asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                     "selp.u32 %0, 1, 0, p;\n\t}\n"
                     : "=r"(done)
                     : "r"(bar), "r"(parity)
                     : "memory");
        if (done)
            return true;
        if (*abort_flag || globaltimer() - t0 > kTcWaitNs)
            return false;
    }
}

__device__ __forceinline__ void mbar_arrive(uint32_t bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ void umma_commit(uint32_t bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar));
}

// 224 threads: warps 0-3 drain accumulators (TMEM lane quarter = warp),
// warp 4 loads halo rows by TMA, warp 5 issues the MMAs, warp 6 fills the
// upsampled channels of a fused upsample + concat input (a.coarse). The roles
// run ahead of each other as far as the ring (`ring` halo-row slots) and the
// two accumulators allow, synchronised only by mbarriers:
//   full[s]   the halo row in slot s is complete: TMA bytes landed (producer)
//             and, fused, the upsampled channels stored (warp 6) -> MMA
//   empty[s]  the MMAs that read slot s completed (MMA commit -> producer)
//   acc_full[b]  row accumulator b is complete (MMA commit -> drain)
//   acc_empty[b] the four drain warps have read accumulator b (drain -> MMA)
constexpr int kStThreads = 224;

__global__ void __launch_bounds__(kStThreads) k_conv3x3_strip(ConvArgs a, const __grid_constant__ CUtensorMap tmap,
                                                              int ncols, int nacc, int ring, int segs, int seg_rows,
                                                              uint32_t *err, int withhold_acc_full)
{
    extern __shared__ __align__(1024) uint8_t smem_raw[];
    __shared__ uint32_t tmem_holder;
    __shared__ __align__(8) uint64_t full[kStMaxRing], empty[kStMaxRing];
    __shared__ __align__(8) uint64_t acc_full[2], acc_empty[2];
    __shared__ int abort_flag;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int tiles_x = (a.wd + kTcM - 1) / kTcM;
    const int units = a.n * tiles_x * segs;
    const int KC = a.cin >> 3;
    const int N = (a.cout + 15) & ~15;
    const int slot_bytes = KC * kStKCBytes;
    const int tap_bytes = N * a.cin * 2;
    const uint32_t half_cols = (uint32_t)ncols >> 1;
    const uint32_t raw = smem_addr(smem_raw);
    const uint32_t ring_base = (raw + 1023u) & ~1023u;
    const uint32_t w_base = ring_base + (uint32_t)(ring * slot_bytes);
    uint8_t *w_ptr = smem_raw + (w_base - raw);
    const volatile int *abort_v = &abort_flag;

    const int CG = a.cc >> 3;  // channel groups filled by warp 6 (upsampled coarse input)
    if (tid == 0) {
        for (int r = 0; r < ring; r++) {
            mbar_init(&full[r], CG ? 2 : 1);
            mbar_init(&empty[r], 1);
        }
        for (int k = 0; k < 2; k++) {
            mbar_init(&acc_full[k], 1);
            mbar_init(&acc_empty[k], 4);
        }
        abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(&tmem_holder)),
                     "r"(ncols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    for (int i = tid; i < 9 * N * KC; i += kStThreads) {
        const int kc = i % KC, n = (i / KC) % N, tap = i / (KC * N);
        const bool ok = n < a.cout;
        const bf16 *src = ok ? a.wgt + ((long)n * 9 + tap) * a.cin + 8 * kc : a.wgt;
        cp_async16(w_ptr + tap * tap_bytes + (n >> 3) * (KC * 128) + kc * 128 + (n & 7) * 16, src, ok);
    }
    cp_async_commit();
    cp_async_wait<0>();
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    const uint32_t tmem = tmem_holder;

    if (warp == 6) {
        // ---- upsampled channels of a fused concat input: fine pixel x of
        // halo row y reads coarse pixel (x >> 1, y >> 1). 16-byte cp.async
        // copies (consecutive lanes on consecutive channel groups of a coarse
        // pixel), one commit group per row; a row is published (fence to the
        // async proxy, arrive on its full barrier) once `lag` newer rows are
        // in flight, lag <= ring - 3 so the MMA warp can always release the
        // slot this warp waits for.
        if (CG) {
            const int hc = a.h >> 1, wc = a.wd >> 1;
            const int npc = kStHaloPx * CG, dp = 32 / CG, dg = 32 % CG;
            const int lag = min(2, ring - 3);
            int slot = 0, phase = 0, pub_slot = 0, pending = 0;
            auto publish = [&]() {
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                __syncwarp();
                if (lane == 0)
                    mbar_arrive(smem_addr(&full[pub_slot]));
                pub_slot = pub_slot + 1 == ring ? 0 : pub_slot + 1;
                pending--;
            };
            bool ok = true;
            for (int u = blockIdx.x; u < units && ok; u += gridDim.x) {
                const int sg = u % segs, tx = (u / segs) % tiles_x, nb = u / (segs * tiles_x);
                const int x0 = tx * kTcM, ya = sg * seg_rows;
                const int nout = min(a.h, ya + seg_rows) - ya;
                if (nout <= 0)
                    continue;
                for (int h = 0; h < nout + 2 && ok; h++) {
                    bool w = true;
                    if (lane == 0)
                        w = mbar_wait_role(smem_addr(&empty[slot]), (uint32_t)(phase ^ 1), abort_v);
                    ok = __shfl_sync(0xffffffffu, w, 0);
                    if (!ok)
                        break;
                    const int yy = ya - 1 + h;
                    const bool row_ok = yy >= 0 && yy < a.h;
                    const bf16 *crow = a.coarse + ((long)nb * hc + (row_ok ? yy >> 1 : 0)) * wc * a.cc;
                    uint8_t *dst = smem_raw + (ring_base - raw) + slot * slot_bytes;
                    int pp = lane / CG, g = lane - (lane / CG) * CG;
                    for (int idx = lane; idx < npc; idx += 32) {
                        const int xx = x0 - 1 + pp;
                        const bool in = row_ok && xx >= 0 && xx < a.wd;
                        cp_async16(dst + g * kStKCBytes + pp * 16, in ? crow + (long)(xx >> 1) * a.cc + 8 * g : a.coarse,
                                   in);
                        g += dg;
                        pp += dp;
                        if (g >= CG) {
                            g -= CG;
                            pp++;
                        }
                    }
                    cp_async_commit();
                    pending++;
                    if (++slot == ring) {
                        slot = 0;
                        phase ^= 1;
                    }
                    if (pending > lag) {
                        if (lag <= 0)
                            cp_async_wait<0>();
                        else if (lag == 1)
                            cp_async_wait<1>();
                        else
                            cp_async_wait<2>();
                        publish();
                    }
                }
            }
            cp_async_wait<0>();
            while (pending > 0)
                publish();
            if (!ok)
                abort_flag = 1;
        }
    } else if (warp == 4) {
        // ---- producer: one TMA row (the KC - CG boxes of 8 channels x 130
        // pixels of `in`) per halo row
        if (lane == 0) {
            const uint64_t tmap_ptr = reinterpret_cast<uint64_t>(&tmap);
            const uint32_t row_tx = (uint32_t)((KC - CG) * kStHaloPx * 16);
            int slot = 0, phase = 0, issued = 0;
            int last_phase[kStMaxRing];
            for (int r = 0; r < kStMaxRing; r++)
                last_phase[r] = -1;
            for (int u = blockIdx.x; u < units && !*abort_v; u += gridDim.x) {
                const int sg = u % segs, tx = (u / segs) % tiles_x, nb = u / (segs * tiles_x);
                const int x0 = tx * kTcM, ya = sg * seg_rows;
                const int nout = min(a.h, ya + seg_rows) - ya;
                if (nout <= 0)
                    continue;
                for (int h = 0; h < nout + 2; h++) {
                    if (!mbar_wait_role(smem_addr(&empty[slot]), (uint32_t)(phase ^ 1), abort_v)) {
                        abort_flag = 1;
                        break;
                    }
                    const uint32_t bar = smem_addr(&full[slot]);
                    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(row_tx)
                                 : "memory");
                    const uint32_t dst = ring_base + (uint32_t)(slot * slot_bytes);
                    for (int kc = CG; kc < KC; kc++)
                        asm volatile("cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes "
                                     "[%0], [%1, {%2, %3, %4, %5}], [%6];" ::"r"(dst + (uint32_t)(kc * kStKCBytes)),
                                     "l"(tmap_ptr), "r"(8 * (kc - CG)), "r"(x0 - 1), "r"(ya - 1 + h), "r"(nb),
                                     "r"(bar)
                                     : "memory");
                    last_phase[slot] = phase;
                    issued++;
                    if (++slot == ring) {
                        slot = 0;
                        phase ^= 1;
                    }
                }
            }
            // every copy issued has landed before the CTA exits
            for (int r = 0; r < ring; r++)
                if (last_phase[r] >= 0 && !mbar_wait(smem_addr(&full[r]), (uint32_t)last_phase[r]))
                    abort_flag = 1;
        }
    } else if (warp == 5) {
        // ---- MMA issue: 9 taps x cin / 16 steps per output row
        if (lane == 0) {
            const uint32_t idesc =
                (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(kTcM >> 4) << 24);
            const uint64_t a_hi = umma_desc(0, kStKCBytes, 128), b_hi = umma_desc(0, 128, (uint32_t)(KC * 128));
            const uint32_t a_lo_base = ring_base >> 4, a_lo_slot = (uint32_t)slot_bytes >> 4;
            const uint32_t b_lo_base = w_base >> 4, b_lo_tap = (uint32_t)tap_bytes >> 4;
            int row_slot = 0;            // slot of the unit's halo row i
            int wait_slot = 0, wait_phase = 0, waited = 0; // next halo row to see complete
            int gi = 0;                  // output rows so far
            int halo = 0;                // halo rows of earlier units
            bool ok = true;
            for (int u = blockIdx.x; u < units && ok; u += gridDim.x) {
                const int sg = u % segs;
                const int ya = sg * seg_rows;
                const int nout = min(a.h, ya + seg_rows) - ya;
                if (nout <= 0)
                    continue;
                for (int i = 0; i < nout && ok; i++, gi++) {
                    while (ok && waited < halo + i + 3) {
                        ok = mbar_wait_role(smem_addr(&full[wait_slot]), (uint32_t)wait_phase, abort_v);
                        if (ok) {
                            waited++;
                            if (++wait_slot == ring) {
                                wait_slot = 0;
                                wait_phase ^= 1;
                            }
                        }
                    }
                    const int b = gi & 1;
                    if (ok)
                        ok = mbar_wait_role(smem_addr(&acc_empty[b]), (uint32_t)(((gi >> 1) & 1) ^ 1), abort_v);
                    if (!ok)
                        break;
                    asm volatile("tcgen05.fence::after_thread_sync;");
                    const uint32_t acc = tmem + (uint32_t)b * half_cols;
                    uint32_t slot_lo[3];
#pragma unroll
                    for (int dy = 0; dy < 3; dy++) {
                        int sl = row_slot + dy;
                        sl = sl >= ring ? sl - ring : sl;
                        slot_lo[dy] = a_lo_base + (uint32_t)sl * a_lo_slot;
                    }
                    for (int j = 0; j < KC / 2; j++) {
#pragma unroll
                        for (int tap = 0; tap < 9; tap++) {
                            const int dy = tap / 3, dx = tap % 3;
                            const uint64_t ad =
                                a_hi | (uint64_t)(slot_lo[dy] + (uint32_t)dx + (uint32_t)j * (2 * kStKCBytes / 16));
                            const uint64_t bd =
                                b_hi | (uint64_t)(b_lo_base + (uint32_t)tap * b_lo_tap + (uint32_t)j * (2 * 128 / 16));
                            const uint32_t accumulate = (j > 0 || tap >= nacc) ? 1u : 0u;
                            const uint32_t dst = acc + (uint32_t)((tap & (nacc - 1)) * N);
                            asm volatile("{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                                         "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(dst),
                                         "l"(ad), "l"(bd), "r"(idesc), "r"(accumulate));
                        }
                    }
                    // (withhold_acc_full: a diagnostic launch that never signals
                    // the drain warps, whose bounded waits then run out)
                    if (!withhold_acc_full)
                        umma_commit(smem_addr(&acc_full[b]));
                    // halo row i is not read by later rows of the unit
                    umma_commit(smem_addr(&empty[row_slot]));
                    row_slot = row_slot + 1 == ring ? 0 : row_slot + 1;
                }
                if (!ok)
                    break;
                // the unit's last two halo rows
                for (int k = 0; k < 2; k++) {
                    umma_commit(smem_addr(&empty[row_slot]));
                    row_slot = row_slot + 1 == ring ? 0 : row_slot + 1;
                }
                halo += nout + 2;
            }
            if (!ok)
                abort_flag = 1;
            // the MMAs of the last row issued are complete before TMEM is freed
            if (gi > 0 && !mbar_wait(smem_addr(&acc_full[(gi - 1) & 1]), (uint32_t)(((gi - 1) >> 1) & 1)))
                abort_flag = 1;
        }
    } else {
        // ---- drain: warp w reads TMEM lanes 32w..32w+31 (pixels x0 + 32w + lane)
        int gi = 0;
        bool ok = true;
        for (int u = blockIdx.x; u < units && ok; u += gridDim.x) {
            const int sg = u % segs, tx = (u / segs) % tiles_x, nb = u / (segs * tiles_x);
            const int x0 = tx * kTcM, ya = sg * seg_rows;
            const int nout = min(a.h, ya + seg_rows) - ya;
            if (nout <= 0)
                continue;
            for (int i = 0; i < nout; i++, gi++) {
                const int b = gi & 1;
                ok = mbar_wait_role(smem_addr(&acc_full[b]), (uint32_t)((gi >> 1) & 1), abort_v);
                ok = __all_sync(0xffffffffu, ok);
                if (!ok)
                    break;
                asm volatile("tcgen05.fence::after_thread_sync;");
                const int x = x0 + warp * 32 + lane;
                const long p = ((long)nb * a.h + ya + i) * a.wd + x;
                const uint32_t acc = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)b * half_cols;
                for (int c = 0; c < N; c += 16) {
                    uint32_t r[16];
                    tmem_ld16(acc + (uint32_t)c, r);
                    for (int q = 1; q < nacc; q++) {
                        uint32_t t[16];
                        tmem_ld16(acc + (uint32_t)(q * N + c), t);
#pragma unroll
                        for (int k = 0; k < 16; k++)
                            r[k] = __float_as_uint(__uint_as_float(r[k]) + __uint_as_float(t[k]));
                    }
                    if (c + 16 >= N) {
                        // the accumulator is read: hand it back to the MMA warp
                        asm volatile("tcgen05.fence::before_thread_sync;");
                        __syncwarp();
                        if (lane == 0)
                            mbar_arrive(smem_addr(&acc_empty[b]));
                    }
                    if (x < a.wd && c < a.cout)
                        store_row16(a, p, c, r);
                }
            }
        }
        if (!ok)
            abort_flag = 1;
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    if (abort_flag && tid == 0)
        atomicOr(err, 1u);
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(ncols));
}

// Weight gradient on the tcgen05 tensor cores, one tap per CTA:
// dW_tap[co][ci] = sum_p dout[p][co] * in[p shifted by the tap][ci], a GEMM
// with M = 128 output channels (zero rows past cout), N = up to 128 input
// channels, K = a slice of pixels. Both operands are MN-major as they lie in
// NHWC memory (8 consecutive channels of a pixel are 16 contiguous bytes): a
// K chunk of 64 pixels is staged as [channel group][pixel][16 B], i.e. core
// matrices of 8 channels x 8 pixels, K groups 128 B apart (LBO) and channel
// groups 64 x 16 B apart (SBO). Three stages of cp.async copies; thread 0
// issues four m128 nN k16 MMAs per chunk and commits each stage to its
// mbarrier, refills wait for the MMAs of the stage's previous chunk. The
// accumulator (one TMEM column per input channel, lane = output channel) is
// added to dw with atomics. Waits are bounded as in the other tcgen05
// kernels.
constexpr int kWtK = 64, kWtStages = 3, kWtM = 128;

__host__ __device__ constexpr int wt_stage_bytes(int N) { return kWtK * (kWtM + N) * 2; }

__global__ void __launch_bounds__(128) k_conv3x3_wgrad_tc(const bf16 *__restrict__ dout, int cout,
                                                          const bf16 *__restrict__ in, int cin, int n, int h, int w,
                                                          float *dw, long slice, int ntile, int ncols, uint32_t *err)
{
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ uint32_t tmem_holder;
    __shared__ __align__(8) uint64_t mbar[kWtStages];
    __shared__ int abort_flag;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int tap = blockIdx.y % 9;
    const int tiles_ci = (cin + ntile - 1) / ntile;
    const int ct = blockIdx.y / 9;
    const int co0 = (ct / tiles_ci) * kWtM, ci0 = (ct % tiles_ci) * ntile;
    const int N = min(ntile, (cin - ci0 + 15) & ~15);
    const long P = (long)n * h * w;
    const long pbeg = (long)blockIdx.x * slice, pend = min(P, pbeg + slice);
    const int dy = tap / 3 - 1, dx = tap % 3 - 1;
    const int nchunks = (int)((pend - pbeg + kWtK - 1) / kWtK);
    const int stage_bytes = wt_stage_bytes(ntile);
    const uint32_t sbase = smem_addr(smem);

    if (tid == 0) {
        for (int st = 0; st < kWtStages; st++)
            mbar_init(&mbar[st], 1);
        abort_flag = 0;
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(&tmem_holder)),
                     "r"(ncols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    const uint32_t tmem = tmem_holder;
    // D f32, A/B bf16, A and B MN-major (bits 15, 16), N >> 3, M >> 4
    const uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | (1u << 15) | (1u << 16) |
                           ((uint32_t)(N >> 3) << 17) | ((uint32_t)(kWtM >> 4) << 24);

    // A rows past cout stay zero: cleared once, never loaded
    const int ga = (min(cout - co0, kWtM) + 7) / 8; // A channel groups with data
    for (int i = tid; i < kWtStages * (kWtM / 8 - ga) * kWtK; i += 128) {
        const int st = i / ((kWtM / 8 - ga) * kWtK), r = i % ((kWtM / 8 - ga) * kWtK);
        *reinterpret_cast<uint4 *>(smem + st * stage_bytes + (ga * kWtK + r) * 16) = make_uint4(0u, 0u, 0u, 0u);
    }
    // thread -> one pixel of the chunk (its position decoded once) and every
    // other channel group
    const int lpx = tid & (kWtK - 1), lhalf = tid / kWtK;
    auto load_chunk = [&](int c) {
        uint8_t *a_s = smem + (c % kWtStages) * stage_bytes;
        uint8_t *b_s = a_s + kWtK * kWtM * 2;
        const long p = pbeg + (long)c * kWtK + lpx;
        const bool pok = p < pend;
        bool xok = false;
        long q = 0;
        if (pok) {
            const int pn = (int)(p / ((long)h * w));
            const int rem = (int)(p - (long)pn * h * w);
            const int y = rem / w;
            const int yy = y + dy, xx = rem - y * w + dx;
            xok = yy >= 0 && yy < h && xx >= 0 && xx < w;
            q = ((long)pn * h + yy) * w + xx;
        }
        for (int g = lhalf; g < ga; g += 2) {
            const int co = co0 + 8 * g;
            const bool ok = pok && co < cout;
            cp_async16(a_s + g * (kWtK * 16) + lpx * 16, ok ? dout + p * cout + co : dout, ok);
        }
        for (int g = lhalf; g < N / 8; g += 2) {
            const int ci = ci0 + 8 * g;
            const bool ok = xok && ci < cin;
            cp_async16(b_s + g * (kWtK * 16) + lpx * 16, ok ? in + q * cin + ci : in, ok);
        }
    };

    for (int st = 0; st < kWtStages - 1; st++) {
        if (st < nchunks)
            load_chunk(st);
        cp_async_commit();
    }
    for (int c = 0; c < nchunks; c++) {
        cp_async_wait<kWtStages - 2>(); // this thread's copies of chunk c landed
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        if (abort_flag)
            break;
        if (tid == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;");
            const uint32_t a_addr = sbase + (uint32_t)((c % kWtStages) * stage_bytes);
            const uint32_t b_addr = a_addr + (uint32_t)(kWtK * kWtM * 2);
#pragma unroll
            for (int j = 0; j < kWtK / 16; j++) {
                // K step j: pixels 16 j .. 16 j + 15 = two K groups of 8
                const uint64_t ad = umma_desc(a_addr + (uint32_t)(j * 256), 128, kWtK * 16);
                const uint64_t bd = umma_desc(b_addr + (uint32_t)(j * 256), 128, kWtK * 16);
                const uint32_t accumulate = (c > 0 || j > 0) ? 1u : 0u;
                asm volatile("{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                             "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem),
                             "l"(ad), "l"(bd), "r"(idesc), "r"(accumulate));
            }
            umma_commit(smem_addr(&mbar[c % kWtStages]));
        }
        // chunk c + 2 reuses the stage of chunk c - 1
        const int nx = c + kWtStages - 1;
        if (nx < nchunks) {
            if (c >= 1) {
                const int prev = c - 1;
                if (!mbar_wait(smem_addr(&mbar[prev % kWtStages]), (uint32_t)((prev / kWtStages) & 1)))
                    atomicOr(&abort_flag, 1);
            }
            load_chunk(nx);
        }
        cp_async_commit();
    }
    cp_async_wait<0>();
    if (!abort_flag && nchunks > 0) {
        const int last = nchunks - 1;
        if (!mbar_wait(smem_addr(&mbar[last % kWtStages]), (uint32_t)((last / kWtStages) & 1)))
            atomicOr(&abort_flag, 1);
    }
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    if (!abort_flag && nchunks > 0) {
        const int co = co0 + warp * 32 + lane;
        for (int c = 0; c < N; c += 16) {
            uint32_t r[16];
            tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c, r);
            if (co >= cout)
                continue;
            float *d = dw + ((long)co * 9 + tap) * cin + ci0 + c;
#pragma unroll
            for (int k = 0; k < 16; k++)
                if (ci0 + c + k < cin)
                    atomicAdd(d + k, __uint_as_float(r[k]));
        }
    } else if (abort_flag && tid == 0) {
        atomicOr(err, 1u);
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(ncols));
}

}  // namespace

namespace {

std::atomic<bool> g_inject_wait_timeout{false};

PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder()
{
    static PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            p = nullptr;
        return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }();
    return fn;
}

struct StripPlan {
    int ring = 0, smem = 0, grid = 0, segs = 0, seg_rows = 0, ncols = 0, nacc = 1, per_sm = 1;
};

// Occupancy first (up to 4 CTAs per SM, bounded by shared memory and by the
// 512 TMEM columns of an SM), then the deepest ring that fits; the rows of
// every 128-pixel column are cut into segments so that one wave of CTAs
// covers the layer.
#ifndef VVPT_STRIP_FUSED_ONE_CTA
#define VVPT_STRIP_FUSED_ONE_CTA 0
#endif
bool plan_strip(const ConvArgs &a, StripPlan &pl)
{
    if (a.cin % 16 || a.cin < 16 || a.cout > 256 || a.cout < 1 || (reinterpret_cast<uintptr_t>(a.in) & 15))
        return false;
    if (a.cc && (a.cc % 8 || a.cc >= a.cin || a.h % 2 || a.wd % 2 || (reinterpret_cast<uintptr_t>(a.coarse) & 15)))
        return false;
    static int nsm = 0, sm_smem = 0, optin = 0, reserved = 0;
    if (!nsm) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
        cudaDeviceGetAttribute(&sm_smem, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
        cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
        cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, dev);
    }
    if (!tensor_map_encoder())
        return false;
    const int N = (a.cout + 15) & ~15;
    const int wbytes = 9 * N * a.cin * 2, slot = (a.cin / 8) * kStKCBytes;
    int ncols = 32;
    while (ncols < 2 * N)
        ncols <<= 1;
    constexpr int kStatic = 2048; // mbarriers, TMEM address, flags (1 KB aligned)
    for (int c = (a.cc && VVPT_STRIP_FUSED_ONE_CTA) ? 1 : 4; c >= 1; c--) {
        if (c * ncols > 512)
            continue;
        const int dyn = std::min(optin - kStatic, sm_smem / c - reserved - kStatic);
        const int ring = std::min(kStMaxRing, (dyn - 1024 - wbytes) / slot);
        if (ring < kStMinRing)
            continue;
        const long cols = (long)a.n * ((a.wd + kTcM - 1) / kTcM);
        const long ctas = (long)nsm * c;
        int segs = (int)std::max<long>(1, std::min<long>(a.h, ctas / std::max<long>(1, cols)));
        const int seg_rows = (a.h + segs - 1) / segs;
        segs = (a.h + seg_rows - 1) / seg_rows;
        // accumulators per row: as many independent MMA chains (1, 2 or 4) as
        // the SM's TMEM leaves room for at this occupancy
        int nacc = 1, tcols = ncols;
        for (int q = 4; q >= 2; q >>= 1) {
            int cq = 32;
            while (cq < 2 * q * N)
                cq <<= 1;
            if (c * cq <= 512) {
                nacc = q;
                tcols = cq;
                break;
            }
        }
        pl.ring = ring;
        pl.smem = dyn;
        pl.segs = segs;
        pl.seg_rows = seg_rows;
        pl.ncols = tcols;
        pl.nacc = nacc;
        pl.per_sm = c;
        pl.grid = (int)std::min<long>(cols * segs, ctas);
        return true;
    }
    return false;
}

// rank-4 map over the NHWC input {C, W, H, N} (the cin - cc channels of `in`);
// box = 8 channels x 130 pixels
bool encode_input_map(const ConvArgs &a, CUtensorMap &m)
{
    const int c = a.cin - a.cc;
    const cuuint64_t dims[4] = {(cuuint64_t)c, (cuuint64_t)a.wd, (cuuint64_t)a.h, (cuuint64_t)a.n};
    const cuuint64_t strides[3] = {(cuuint64_t)c * 2, (cuuint64_t)a.wd * c * 2, (cuuint64_t)a.h * a.wd * c * 2};
    const cuuint32_t box[4] = {8, (cuuint32_t)kStHaloPx, 1, 1};
    const cuuint32_t estr[4] = {1, 1, 1, 1};
    return tensor_map_encoder()(&m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<bf16 *>(a.in), dims, strides, box,
                                estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                                CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

}  // namespace

namespace {

// The strip kernel for `a` when it takes the layer; false (nothing launched)
// otherwise. A fused upsample + concat input is taken only where two or more
// CTAs share an SM: the warp that copies the upsampled channels keeps up
// there, while with one CTA per SM (level 1, 219 KB of weights and ring) the
// unfused path measured faster (0.47 vs 0.57 ms at 1920 x 1080).
bool launch_strip(const ConvArgs &a, cudaStream_t s, uint32_t *err, ConvKernels kind)
{
    StripPlan pl;
    CUtensorMap tmap;
    // A fused layer (upsample + concat in the kernel) needs two CTAs per SM
    // to pay: at one (the half-resolution decoder input, whose weights leave
    // room for one) it took 581 us against 450 us for the separate
    // upsample-concat and convolution at 3840 x 2160.
    if (!err || kind == kConvTiles || !plan_strip(a, pl) || (a.cc && pl.per_sm < 2 && !VVPT_STRIP_FUSED_ONE_CTA) ||
        !encode_input_map(a, tmap))
        return false;
    if (kind == kConvPersistent)
        pl.grid = std::min(pl.grid, 16);
    static int attr_smem = 0;
    if (pl.smem > attr_smem) {
        cudaFuncSetAttribute(k_conv3x3_strip, cudaFuncAttributeMaxDynamicSharedMemorySize, pl.smem);
        cudaFuncSetAttribute(k_conv3x3_strip, cudaFuncAttributePreferredSharedMemoryCarveout,
                             cudaSharedmemCarveoutMaxShared);
        attr_smem = pl.smem;
    }
    const int withhold = g_inject_wait_timeout.exchange(false) ? 1 : 0;
    k_conv3x3_strip<<<pl.grid, kStThreads, pl.smem, s>>>(a, tmap, pl.ncols, pl.nacc, pl.ring, pl.segs, pl.seg_rows,
                                                         err, withhold);
    return true;
}

}  // namespace

void inject_wait_timeout() { g_inject_wait_timeout.store(true); }

bool conv3x3_concat(const ConvArgs &a, cudaStream_t s, uint32_t *err, ConvKernels kind)
{
    return kind != kConvNoFusion && a.coarse && a.cc > 0 && launch_strip(a, s, err, kind);
}

void conv3x3(const ConvArgs &a_in, cudaStream_t s, uint32_t *err, ConvKernels kind)
{
    ConvArgs a = a_in;
    a.coarse = nullptr;
    a.cc = 0;
    const long P = (long)a.n * a.h * a.wd;
    if (launch_strip(a, s, err, kind))
        return;
    if (err && a.cout <= 256) {
        static bool attr_set = false;
        if (!attr_set) {
            cudaFuncSetAttribute(k_conv3x3_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, tc_smem_bytes(256));
            cudaFuncSetAttribute(k_conv3x3_tc_chunk, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 std::max(tc_chunk_smem_bytes(128, 2, tc_chunk_rows(128)),
                                          tc_chunk_smem_bytes(64, 2, tc_chunk_rows(64))));
            attr_set = true;
        }
        const int N = (a.cout + 15) & ~15;
        int ncols = 32;
        while (ncols < N)
            ncols <<= 1;
        const long tiles = (long)a.n * a.h * ((a.wd + kTcM - 1) / kTcM);
        if (N <= 128) {
            // several output rows per CTA, one accumulator (one MMA chain)
            // per row
            const int rows = tc_chunk_rows(N);
            const int smem = tc_chunk_smem_bytes(N, (a.cin + kTcBK - 1) / kTcBK, rows);
            int cols = 32;
            while (cols < rows * N)
                cols <<= 1;
            const long blocks = (long)a.n * ((a.h + rows - 1) / rows) * ((a.wd + kTcM - 1) / kTcM);
            k_conv3x3_tc_chunk<<<(unsigned)blocks, 128, smem, s>>>(a, cols, 1, rows, err);
        }
        else
            k_conv3x3_tc<<<(unsigned)tiles, 128, tc_smem_bytes(N), s>>>(a, ncols, err);
        return;
    }
    // 32-wide channel tiles where they leave fewer channels of the last tile
    // empty than 64-wide ones (16, 32, 80, 96, 160, 224 channels)
    const int waste64 = (a.cout + 63) / 64 * 64 - a.cout, waste32 = (a.cout + 31) / 32 * 32 - a.cout;
    if (waste32 < waste64) {
        dim3 grid((unsigned)((P + kBM - 1) / kBM), (unsigned)((a.cout + 31) / 32));
        k_conv3x3<32, 16><<<grid, 256, 0, s>>>(a);
    } else {
        dim3 grid((unsigned)((P + kBM - 1) / kBM), (unsigned)((a.cout + 63) / 64));
        k_conv3x3<64, 32><<<grid, 256, 0, s>>>(a);
    }
}

void conv3x3_wgrad(const bf16 *dout, int cout, const bf16 *in, int cin, int n, int h, int w, float *dw, float *dbias,
                   cudaStream_t s, uint32_t *err)
{
    const long P = (long)n * h * w;
    if (err) {
        // tcgen05: 128 output channels x up to 128 input channels per tap and slice
        const int ntile = std::min(128, (cin + 15) & ~15);
        int ncols = 32;
        while (ncols < ntile)
            ncols <<= 1;
        const int tiles = ((cout + kWtM - 1) / kWtM) * ((cin + ntile - 1) / ntile);
        long slices = std::max<long>(1, (152L * 4) / (9L * tiles));
        long slice = (P + slices - 1) / slices;
        slice = std::max<long>(kWtK, (slice + kWtK - 1) / kWtK * kWtK);
        slices = (P + slice - 1) / slice;
        const int smem = kWtStages * wt_stage_bytes(ntile);
        static bool attr_set = false;
        if (!attr_set) {
            cudaFuncSetAttribute(k_conv3x3_wgrad_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 kWtStages * wt_stage_bytes(128));
            attr_set = true;
        }
        dim3 grid((unsigned)slices, (unsigned)(9 * tiles));
        k_conv3x3_wgrad_tc<<<grid, 128, smem, s>>>(dout, cout, in, cin, n, h, w, dw, slice, ntile, ncols, err);
    } else {
        wgrad_mma_sync(dout, cout, in, cin, n, h, w, dw, s);
    }
    if (dbias) {
        // channel counts are multiples of 8 up to 256: 1-32 groups per pixel lane
        const int lanes = kBiasThreads / (cout / 8);
        const long blocks = std::min<long>(152L * 4, (P + 16L * lanes - 1) / (16L * lanes));
        k_bias_grad<<<(unsigned)std::max<long>(blocks, 1), kBiasThreads, 0, s>>>(dout, cout, P, dbias);
    }
}

void wgrad_mma_sync(const bf16 *dout, int cout, const bf16 *in, int cin, int n, int h, int w, float *dw,
                    cudaStream_t s)
{
    const long P = (long)n * h * w;
    const int bm = cout <= 32 ? 32 : 64;
    const int tiles = ((cout + bm - 1) / bm) * ((cin + kTileC - 1) / kTileC);
    // about 8 blocks per SM over all taps and tiles (each block's K loop is
    // latency-bound; more blocks keep more copies and MMAs in flight)
    long slices = std::max<long>(1, (152L * 8) / (9L * tiles));
    long slice = (P + slices - 1) / slices;
    slice = std::max<long>(kWgK, (slice + kWgK - 1) / kWgK * kWgK);
    slices = (P + slice - 1) / slice;
    dim3 grid((unsigned)slices, (unsigned)(9 * tiles));
    if (bm == 32)
        k_conv3x3_wgrad<32><<<grid, 128, 0, s>>>(dout, cout, in, cin, n, h, w, dw, slice);
    else
        k_conv3x3_wgrad<64><<<grid, 128, 0, s>>>(dout, cout, in, cin, n, h, w, dw, slice);
}

void transform_weights(const bf16 *w, bf16 *wt, int cout, int cin, cudaStream_t s)
{
    k_transform_weights<<<grid_for((long)cout * 9 * cin), 256, 0, s>>>(w, wt, cout, cin);
}

void to_bf16(const float *src, bf16 *dst, size_t n, cudaStream_t s)
{
    k_to_bf16<<<grid_for((long)n), 256, 0, s>>>(src, dst, n);
}

void pack_features(const float *radiance, const float *albedo, const float *normal, bf16 *x, int npix, cudaStream_t s)
{
    k_pack_features<<<grid_for(npix), 256, 0, s>>>(reinterpret_cast<const float4 *>(radiance),
                                                   reinterpret_cast<const float4 *>(albedo),
                                                   reinterpret_cast<const float4 *>(normal), x, npix);
}

void pack_target(const float *target, float *t3, int npix, cudaStream_t s)
{
    k_pack_target<<<grid_for(npix), 256, 0, s>>>(reinterpret_cast<const float4 *>(target), t3, npix);
}

// 8-channel groups of a layout kernel, indexed in 32 bits by the kernels: the
// denoiser's batch limit (n x h x w <= 2^27 pixels, at most 80 channels at
// full resolution) keeps every count below 2^31
static long groups8(long pixels, int c) { return pixels * (c / 8); }

void avgpool2(const bf16 *in, bf16 *out, int n, int h, int w, int c, cudaStream_t s)
{
    k_avgpool2<<<grid_for(groups8((long)n * (h / 2) * (w / 2), c)), 256, 0, s>>>(in, out, n, h, w, c);
}

void upcat(const bf16 *coarse, int cc, const bf16 *skip, int cs, bf16 *out, int n, int h, int w, cudaStream_t s)
{
    k_upcat<<<grid_for(groups8((long)n * h * w, cc + cs)), 256, 0, s>>>(coarse, cc, skip, cs, out, n, h, w);
}

void upcat_backward(const bf16 *dcat, int cc, int cs, bf16 *dcoarse, bf16 *dskip, int n, int h, int w, cudaStream_t s)
{
    k_upcat_backward_coarse<<<grid_for(groups8((long)n * (h / 2) * (w / 2), cc)), 256, 0, s>>>(dcat, cc, cs, dcoarse,
                                                                                                n, h, w);
    if (dskip)
        k_upcat_backward_skip<<<grid_for(groups8((long)n * h * w, cs + cc)), 256, 0, s>>>(dcat, cc, cs, dskip,
                                                                                          (unsigned)((long)n * h * w));
}

void pool_backward_combine(const bf16 *dskip, const bf16 *dpooled, const bf16 *e, bf16 *de, int n, int h, int w, int c,
                           cudaStream_t s)
{
    k_pool_backward_combine<<<grid_for(groups8((long)n * h * w, c)), 256, 0, s>>>(dskip, dpooled, e, de, n, h, w, c);
}

void l1_loss(const float *out, int cout, const float *t3, bf16 *dout, float *loss_sum, int npix, cudaStream_t s)
{
    k_l1_loss<<<grid_for(npix), 256, 0, s>>>(out, cout, t3, dout, loss_sum, npix);
}

void adam(float *p, const float *g, float *m, float *v, size_t n, float lr, float b1, float b2, float eps, int t,
          cudaStream_t s)
{
    const float c1 = 1.0f - powf(b1, (float)t), c2 = 1.0f - powf(b2, (float)t);
    k_adam<<<grid_for((long)n), 256, 0, s>>>(p, g, m, v, n, lr, b1, b2, eps, c1, c2);
}

void unpack_output(const float *y, int cout, float *out_rgba, int npix, cudaStream_t s)
{
    k_unpack_output<<<grid_for(npix), 256, 0, s>>>(y, cout, reinterpret_cast<float4 *>(out_rgba), npix);
}

}  // namespace vvdn
