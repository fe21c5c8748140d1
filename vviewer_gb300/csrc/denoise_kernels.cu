// Denoiser kernels (denoise_kernels.cuh). The convolutions are implicit GEMMs
// on the BF16 tensor cores through warp-level mma.sync m16n8k16 with FP32
// accumulators; operand tiles are staged in shared memory and read with
// ldmatrix.
#include <algorithm>

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

// 16 bf16 (two 16-byte vectors) or zeros
__device__ __forceinline__ void load16(const bf16 *src, bool ok, bf16 *dst)
{
    uint4 v0 = make_uint4(0, 0, 0, 0), v1 = v0;
    if (ok) {
        v0 = *reinterpret_cast<const uint4 *>(src);
        v1 = *reinterpret_cast<const uint4 *>(src + 8);
    }
    *reinterpret_cast<uint4 *>(dst) = v0;
    *reinterpret_cast<uint4 *>(dst + 8) = v1;
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

// Weight gradient for one tap: block tile 64 output channels x 64 input
// channels, K = a slice of pixels in steps of 32. Warp w owns output
// channels [16w, 16w + 16). Partial sums are added to dw with atomics.
constexpr int kWgK = 32;
__global__ void __launch_bounds__(128) k_conv3x3_wgrad(const bf16 *__restrict__ dout, int cout,
                                                       const bf16 *__restrict__ in, int cin, int n, int h, int w,
                                                       float *dw, long slice)
{
    __shared__ __align__(16) bf16 Ds[kWgK][kTileC + 8]; // [pixel][cout]
    __shared__ __align__(16) bf16 Xs[kWgK][kTileC + 8]; // [pixel][cin]
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int tap = blockIdx.y % 9;
    const int tiles_ci = (cin + kTileC - 1) / kTileC;
    const int ct = blockIdx.y / 9;
    const int co0 = (ct / tiles_ci) * kTileC, ci0 = (ct % tiles_ci) * kTileC;
    const long P = (long)n * h * w;
    const long pbeg = (long)blockIdx.x * slice, pend = min(P, pbeg + slice);
    const int dy = tap / 3 - 1, dx = tap % 3 - 1;
    // load mapping: row = tid / 4 (pixel), group = (tid % 4) * 16 channels
    const int lr = tid >> 2, lg = (tid & 3) * 16;
    float acc[8][4];
#pragma unroll
    for (int j = 0; j < 8; j++)
        acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.0f;
    for (long pb = pbeg; pb < pend; pb += kWgK) {
        const long p = pb + lr;
        bool ok = p < pend;
        int pn = 0, py = 0, px = 0;
        if (ok) {
            pn = (int)(p / ((long)h * w));
            const int rem = (int)(p - (long)pn * h * w);
            py = rem / w;
            px = rem - py * w;
        }
        const int co = co0 + lg, ci = ci0 + lg;
        load16(dout + p * cout + co, ok && co < cout, &Ds[lr][lg]);
        const int yy = py + dy, xx = px + dx;
        const bool xok = ok && yy >= 0 && yy < h && xx >= 0 && xx < w && ci < cin;
        load16(in + (((long)pn * h + yy) * w + xx) * cin + ci, xok, &Xs[lr][lg]);
        __syncthreads();
#pragma unroll
        for (int ks = 0; ks < kWgK; ks += 16) {
            // A[m = cout][k = pixel] from Ds[k][m] (transposed load)
            uint32_t a0, a1, a2, a3;
            ldsm_x4_t(smem_addr(&Ds[ks + (lane & 7) + ((lane >> 4) << 3)][warp * 16 + ((lane >> 3) & 1) * 8]), a0, a1,
                      a2, a3);
#pragma unroll
            for (int j = 0; j < 4; j++) {
                // B[k = pixel][n = cin] from Xs[k][n] (transposed load): two n-tiles
                uint32_t b0, b1, b2, b3;
                ldsm_x4_t(smem_addr(&Xs[ks + (lane & 7) + ((lane >> 3) & 1) * 8][16 * j + (lane >> 4) * 8]), b0, b1,
                          b2, b3);
                mma_bf16(acc[2 * j], a0, a1, a2, a3, b0, b1);
                mma_bf16(acc[2 * j + 1], a0, a1, a2, a3, b2, b3);
            }
        }
        __syncthreads();
    }
    const int g = lane >> 2, t = lane & 3;
#pragma unroll
    for (int half = 0; half < 2; half++) {
        const int co = co0 + warp * 16 + g + half * 8;
        if (co >= cout)
            continue;
#pragma unroll
        for (int j = 0; j < 8; j++) {
            const int ci = ci0 + 8 * j + 2 * t;
            if (ci >= cin)
                continue;
            float *d = dw + ((long)co * 9 + tap) * cin + ci;
            atomicAdd(d, acc[j][2 * half]);
            atomicAdd(d + 1, acc[j][2 * half + 1]);
        }
    }
}

__global__ void k_bias_grad(const bf16 *dout, int cout, long P, float *dbias)
{
    // one block per 8 channels-group x pixel slice; simple strided sums
    const int c = blockIdx.y * blockDim.x + threadIdx.x;
    if (c >= cout)
        return;
    float s = 0.0f;
    for (long p = blockIdx.x; p < P; p += gridDim.x)
        s += __bfloat162float(dout[p * cout + c]);
    atomicAdd(dbias + c, s);
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
    const int ho = h / 2, wo = w / 2;
    const long total = (long)n * ho * wo * c;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x) {
        const int ch = (int)(i % c);
        const long q = i / c;
        const int x = (int)(q % wo), y = (int)((q / wo) % ho), b = (int)(q / ((long)wo * ho));
        const long base = (((long)b * h + 2 * y) * w + 2 * x) * c + ch;
        const float s = __bfloat162float(in[base]) + __bfloat162float(in[base + c]) +
                        __bfloat162float(in[base + (long)w * c]) + __bfloat162float(in[base + (long)w * c + c]);
        out[i] = __float2bfloat16_rn(0.25f * s);
    }
}

__global__ void k_upcat(const bf16 *coarse, int cc, const bf16 *skip, int cs, bf16 *out, int n, int h, int w)
{
    const int ct = cc + cs;
    const long total = (long)n * h * w * ct;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x) {
        const int ch = (int)(i % ct);
        const long p = i / ct;
        if (ch < cc) {
            const int x = (int)(p % w), y = (int)((p / w) % h), b = (int)(p / ((long)w * h));
            out[i] = coarse[(((long)b * (h / 2) + y / 2) * (w / 2) + x / 2) * cc + ch];
        } else {
            out[i] = skip[p * cs + (ch - cc)];
        }
    }
}

__global__ void k_upcat_backward_coarse(const bf16 *dcat, int cc, int cs, bf16 *dcoarse, int n, int h, int w)
{
    const int ct = cc + cs, ho = h / 2, wo = w / 2;
    const long total = (long)n * ho * wo * cc;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x) {
        const int ch = (int)(i % cc);
        const long q = i / cc;
        const int x = (int)(q % wo), y = (int)((q / wo) % ho), b = (int)(q / ((long)wo * ho));
        const long base = (((long)b * h + 2 * y) * w + 2 * x) * ct + ch;
        const float s = __bfloat162float(dcat[base]) + __bfloat162float(dcat[base + ct]) +
                        __bfloat162float(dcat[base + (long)w * ct]) + __bfloat162float(dcat[base + (long)w * ct + ct]);
        dcoarse[i] = __float2bfloat16_rn(s);
    }
}

__global__ void k_upcat_backward_skip(const bf16 *dcat, int cc, int cs, bf16 *dskip, long npix)
{
    const int ct = cc + cs;
    const long total = npix * cs;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x) {
        const int ch = (int)(i % cs);
        const long p = i / cs;
        dskip[i] = dcat[p * ct + cc + ch];
    }
}

__global__ void k_pool_backward_combine(const bf16 *dskip, const bf16 *dpooled, const bf16 *e, bf16 *de, int n, int h,
                                        int w, int c)
{
    const long total = (long)n * h * w * c;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x) {
        const int ch = (int)(i % c);
        const long p = i / c;
        const int x = (int)(p % w), y = (int)((p / w) % h), b = (int)(p / ((long)w * h));
        float v = 0.25f * __bfloat162float(dpooled[(((long)b * (h / 2) + y / 2) * (w / 2) + x / 2) * c + ch]);
        if (dskip)
            v += __bfloat162float(dskip[i]);
        if (!(__bfloat162float(e[i]) > 0.0f))
            v = 0.0f;
        de[i] = __float2bfloat16_rn(v);
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
constexpr int kTcHaloBytes = 3 * kTcHaloRow;        // 24,960 B
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
            float v[16];
#pragma unroll
            for (int k = 0; k < 16; k++) {
                v[k] = __uint_as_float(r[k]);
                if (a.bias)
                    v[k] += a.bias[c + k];
                if (a.relu)
                    v[k] = fmaxf(v[k], 0.0f);
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
    } else if (tid == 0) {
        atomicOr(err, 1u);
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(ncols));
}

}  // namespace

void conv3x3(const ConvArgs &a, cudaStream_t s, uint32_t *err)
{
    const long P = (long)a.n * a.h * a.wd;
    if (err && a.cout <= 256) {
        static bool attr_set = false;
        if (!attr_set) {
            cudaFuncSetAttribute(k_conv3x3_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, tc_smem_bytes(256));
            attr_set = true;
        }
        const int N = (a.cout + 15) & ~15;
        int ncols = 32;
        while (ncols < N)
            ncols <<= 1;
        const long tiles = (long)a.n * a.h * ((a.wd + kTcM - 1) / kTcM);
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
                   cudaStream_t s)
{
    const long P = (long)n * h * w;
    const int tiles = ((cout + kTileC - 1) / kTileC) * ((cin + kTileC - 1) / kTileC);
    // about 4 blocks per SM over all taps and tiles
    long slices = std::max<long>(1, (152L * 4) / (9L * tiles));
    long slice = (P + slices - 1) / slices;
    slice = std::max<long>(kWgK, (slice + kWgK - 1) / kWgK * kWgK);
    slices = (P + slice - 1) / slice;
    dim3 grid((unsigned)slices, (unsigned)(9 * tiles));
    k_conv3x3_wgrad<<<grid, 128, 0, s>>>(dout, cout, in, cin, n, h, w, dw, slice);
    if (dbias) {
        dim3 gb((unsigned)std::min<long>(P, 1024), (unsigned)((cout + 127) / 128));
        k_bias_grad<<<gb, 128, 0, s>>>(dout, cout, P, dbias);
    }
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

void avgpool2(const bf16 *in, bf16 *out, int n, int h, int w, int c, cudaStream_t s)
{
    k_avgpool2<<<grid_for((long)n * (h / 2) * (w / 2) * c), 256, 0, s>>>(in, out, n, h, w, c);
}

void upcat(const bf16 *coarse, int cc, const bf16 *skip, int cs, bf16 *out, int n, int h, int w, cudaStream_t s)
{
    k_upcat<<<grid_for((long)n * h * w * (cc + cs)), 256, 0, s>>>(coarse, cc, skip, cs, out, n, h, w);
}

void upcat_backward(const bf16 *dcat, int cc, int cs, bf16 *dcoarse, bf16 *dskip, int n, int h, int w, cudaStream_t s)
{
    k_upcat_backward_coarse<<<grid_for((long)n * (h / 2) * (w / 2) * cc), 256, 0, s>>>(dcat, cc, cs, dcoarse, n, h, w);
    if (dskip)
        k_upcat_backward_skip<<<grid_for((long)n * h * w * cs), 256, 0, s>>>(dcat, cc, cs, dskip, (long)n * h * w);
}

void pool_backward_combine(const bf16 *dskip, const bf16 *dpooled, const bf16 *e, bf16 *de, int n, int h, int w, int c,
                           cudaStream_t s)
{
    k_pool_backward_combine<<<grid_for((long)n * h * w * c), 256, 0, s>>>(dskip, dpooled, e, de, n, h, w, c);
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
