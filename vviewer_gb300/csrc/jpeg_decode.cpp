// Baseline JPEG decoding for model textures (host code).
//
// vengine loads textures through stb_image (AssimpLoadModel.cpp:
// assimpLoadTextureData), which reads JPEG as well as PNG. This decoder
// covers the sequential Huffman processes of ITU-T T.81 (SOF0 baseline and
// SOF1 extended, 8-bit samples): one component (grey) or three (YCbCr, JFIF),
// sampling factors of 1 or 2, restart intervals. The steps follow the
// standard: Huffman decoding per F.2.2 (MINCODE / MAXCODE / VALPTR tables),
// dequantisation, the 8 x 8 inverse DCT of A.3.3 in double precision as two
// separable passes, level shift, rounding to nearest and clamping to 8-bit
// samples; chroma upsampling by 2 with the triangle filter (3/4 of the
// nearest sample, 1/4 of the next nearest, edges repeated); the JFIF YCbCr to
// RGB matrix. The tests compare it with a Python restatement of the same
// steps (tests/jpeg_reference.py) and with the coefficients their encoder
// wrote.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "vvpt.h"

namespace {

constexpr double kPi = 3.14159265358979323846;

const int kZigzag[64] = {0,  1,  8,  16, 9,  2,  3,  10, 17, 24, 32, 25, 18, 11, 4,  5,  12, 19, 26, 33, 40, 48,
                         41, 34, 27, 20, 13, 6,  7,  14, 21, 28, 35, 42, 49, 56, 57, 50, 43, 36, 29, 22, 15, 23,
                         30, 37, 44, 51, 58, 59, 52, 45, 38, 31, 39, 46, 53, 60, 61, 54, 47, 55, 62, 63};

struct Huffman {
    bool present = false;
    int maxcode[18], mincode[17], valptr[17];
    std::vector<uint8_t> symbols;
    void build(const uint8_t *counts, const uint8_t *syms, int n)
    {
        symbols.assign(syms, syms + n);
        int code = 0, k = 0;
        for (int len = 1; len <= 16; len++) {
            maxcode[len] = -1;
            mincode[len] = 0;
            valptr[len] = 0;
            const int c = counts[len - 1];
            if (c) {
                valptr[len] = k;
                mincode[len] = code;
                code += c;
                k += c;
                maxcode[len] = code - 1;
            }
            code <<= 1;
        }
        present = true;
    }
};

struct Component {
    int id, h, v, tq;
    int bx, by; // blocks per row / column (MCU-padded)
    std::vector<int32_t> coef; // [by][bx][64], zigzag order
};

struct Failure {
    vvpt_status st;
};

[[noreturn]] void fail(vvpt_status st) { throw Failure{st}; }

// Entropy-coded segment reader: byte stuffing (FF 00) removed; a marker ends the data.
struct Bits {
    const uint8_t *d;
    size_t n, pos;
    uint32_t acc = 0;
    int cnt = 0;
    int marker = -1;
    int byte()
    {
        if (marker >= 0)
            return 0;
        if (pos + 1 >= n)
            fail(VVPT_ERR_INVALID_ARG);
        const int b = d[pos];
        if (b == 0xFF) {
            const int nx = d[pos + 1];
            if (nx == 0x00) {
                pos += 2;
                return 0xFF;
            }
            marker = nx;
            return 0;
        }
        pos++;
        return b;
    }
    int bit()
    {
        if (cnt == 0) {
            acc = (uint32_t)byte();
            cnt = 8;
        }
        cnt--;
        return (int)((acc >> cnt) & 1u);
    }
    int bits(int k)
    {
        int v = 0;
        for (int i = 0; i < k; i++)
            v = (v << 1) | bit();
        return v;
    }
    int decode(const Huffman &h)
    {
        int code = bit(), len = 1;
        while (len <= 16 && code > h.maxcode[len]) {
            code = (code << 1) | bit();
            len++;
        }
        if (len > 16)
            fail(VVPT_ERR_INVALID_ARG);
        const int idx = h.valptr[len] + code - h.mincode[len];
        if (idx < 0 || idx >= (int)h.symbols.size())
            fail(VVPT_ERR_INVALID_ARG);
        return h.symbols[idx];
    }
    void restart()
    {
        cnt = 0;
        if (marker < 0) {
            while (pos + 1 < n && !(d[pos] == 0xFF && d[pos + 1] >= 0xD0 && d[pos + 1] <= 0xD7))
                pos++;
            if (pos + 1 >= n)
                fail(VVPT_ERR_INVALID_ARG);
            marker = d[pos + 1];
        }
        if (marker < 0xD0 || marker > 0xD7)
            fail(VVPT_ERR_INVALID_ARG);
        pos += 2;
        marker = -1;
    }
};

int extend(int v, int t) { return (t && v < (1 << (t - 1))) ? v - (1 << t) + 1 : v; }

struct Frame {
    int w = 0, h = 0, hmax = 1, vmax = 1, mcux = 0, mcuy = 0;
    std::vector<Component> comps;
    double qt[4][64];
    bool qt_present[4] = {false, false, false, false};
    bool scanned = false;
};

void parse(const uint8_t *d, size_t n, Frame &f, bool header_only)
{
    if (n < 4 || d[0] != 0xFF || d[1] != 0xD8)
        fail(VVPT_ERR_INVALID_ARG);
    size_t pos = 2;
    Huffman huff[2][4];
    int restart_interval = 0;
    while (pos < n) {
        if (pos + 1 >= n || d[pos] != 0xFF)
            fail(VVPT_ERR_INVALID_ARG);
        const int marker = d[pos + 1];
        pos += 2;
        if (marker == 0xD8 || marker == 0x01 || (marker >= 0xD0 && marker <= 0xD7))
            continue;
        if (marker == 0xD9)
            break;
        if (pos + 2 > n)
            fail(VVPT_ERR_INVALID_ARG);
        const size_t len = ((size_t)d[pos] << 8) | d[pos + 1];
        if (len < 2 || pos + len > n)
            fail(VVPT_ERR_INVALID_ARG);
        const uint8_t *seg = d + pos + 2;
        const size_t sl = len - 2;
        pos += len;
        if (marker == 0xDB) { // DQT
            size_t k = 0;
            while (k < sl) {
                const int pq = seg[k] >> 4, tq = seg[k] & 15;
                k++;
                if (tq > 3 || k + (pq ? 128 : 64) > sl)
                    fail(VVPT_ERR_INVALID_ARG);
                for (int i = 0; i < 64; i++) {
                    const double v = pq ? (double)((seg[k + 2 * i] << 8) | seg[k + 2 * i + 1]) : (double)seg[k + i];
                    f.qt[tq][kZigzag[i]] = v;
                }
                f.qt_present[tq] = true;
                k += pq ? 128 : 64;
            }
        } else if (marker == 0xC4) { // DHT
            size_t k = 0;
            while (k < sl) {
                if (k + 17 > sl)
                    fail(VVPT_ERR_INVALID_ARG);
                const int tc = seg[k] >> 4, th = seg[k] & 15;
                int total = 0;
                for (int i = 0; i < 16; i++)
                    total += seg[k + 1 + i];
                if (tc > 1 || th > 3 || k + 17 + total > sl)
                    fail(VVPT_ERR_INVALID_ARG);
                huff[tc][th].build(seg + k + 1, seg + k + 17, total);
                k += 17 + total;
            }
        } else if (marker == 0xC0 || marker == 0xC1) { // SOF0 / SOF1
            if (sl < 6)
                fail(VVPT_ERR_INVALID_ARG);
            if (seg[0] != 8)
                fail(VVPT_ERR_UNSUPPORTED);
            f.h = (seg[1] << 8) | seg[2];
            f.w = (seg[3] << 8) | seg[4];
            const int nc = seg[5];
            if ((nc != 1 && nc != 3) || f.w == 0 || f.h == 0 || (uint64_t)f.w * f.h > (1ull << 28) ||
                sl < (size_t)(6 + 3 * nc))
                fail(nc == 1 || nc == 3 ? VVPT_ERR_INVALID_ARG : VVPT_ERR_UNSUPPORTED);
            f.comps.assign(nc, Component());
            f.hmax = f.vmax = 1;
            for (int c = 0; c < nc; c++) {
                Component &cp = f.comps[c];
                cp.id = seg[6 + 3 * c];
                cp.h = seg[7 + 3 * c] >> 4;
                cp.v = seg[7 + 3 * c] & 15;
                cp.tq = seg[8 + 3 * c];
                if (cp.h < 1 || cp.h > 2 || cp.v < 1 || cp.v > 2 || cp.tq > 3)
                    fail(VVPT_ERR_UNSUPPORTED);
                f.hmax = std::max(f.hmax, cp.h);
                f.vmax = std::max(f.vmax, cp.v);
            }
            f.mcux = (f.w + 8 * f.hmax - 1) / (8 * f.hmax);
            f.mcuy = (f.h + 8 * f.vmax - 1) / (8 * f.vmax);
            if (header_only)
                return;
            for (Component &cp : f.comps) {
                cp.bx = f.mcux * cp.h;
                cp.by = f.mcuy * cp.v;
                cp.coef.assign((size_t)cp.bx * cp.by * 64, 0);
            }
        } else if (marker == 0xC2 || marker == 0xC3 || (marker >= 0xC5 && marker <= 0xCF && marker != 0xC8 &&
                                                          marker != 0xCC)) {
            fail(VVPT_ERR_UNSUPPORTED); // progressive, lossless or arithmetic-coded
        } else if (marker == 0xDD) { // DRI
            if (sl < 2)
                fail(VVPT_ERR_INVALID_ARG);
            restart_interval = (seg[0] << 8) | seg[1];
        } else if (marker == 0xDA) { // SOS
            if (f.comps.empty() || sl < 1)
                fail(VVPT_ERR_INVALID_ARG);
            const int ns = seg[0];
            if (ns < 1 || ns > 3 || sl < (size_t)(1 + 2 * ns + 3))
                fail(VVPT_ERR_INVALID_ARG);
            Component *sc[3];
            const Huffman *dct[3], *act[3];
            for (int j = 0; j < ns; j++) {
                const int cid = seg[1 + 2 * j], tb = seg[2 + 2 * j];
                sc[j] = nullptr;
                for (Component &cp : f.comps)
                    if (cp.id == cid)
                        sc[j] = &cp;
                const int td = tb >> 4, ta = tb & 15;
                if (!sc[j] || td > 3 || ta > 3 || !huff[0][td].present || !huff[1][ta].present)
                    fail(VVPT_ERR_INVALID_ARG);
                dct[j] = &huff[0][td];
                act[j] = &huff[1][ta];
            }
            Bits b{d, n, pos};
            int pred[3] = {0, 0, 0};
            // a non-interleaved scan codes the component's own blocks (A.2.2)
            int ubx = 0, uby = 0;
            if (ns == 1) {
                const Component &c = *sc[0];
                ubx = ((int)std::ceil((double)f.w * c.h / f.hmax) + 7) / 8;
                uby = ((int)std::ceil((double)f.h * c.v / f.vmax) + 7) / 8;
            }
            const long total = ns == 1 ? (long)ubx * uby : (long)f.mcux * f.mcuy;
            for (long m = 0; m < total; m++) {
                if (restart_interval && m && m % restart_interval == 0) {
                    b.restart();
                    pred[0] = pred[1] = pred[2] = 0;
                }
                auto block = [&](int j, int yb, int xb) {
                    Component &c = *sc[j];
                    int32_t *blk = &c.coef[((size_t)yb * c.bx + xb) * 64];
                    const int t = b.decode(*dct[j]);
                    if (t > 16)
                        fail(VVPT_ERR_INVALID_ARG);
                    pred[j] += t ? extend(b.bits(t), t) : 0;
                    blk[0] = pred[j];
                    for (int k = 1; k < 64;) {
                        const int rs = b.decode(*act[j]);
                        const int r = rs >> 4, s = rs & 15;
                        if (s == 0) {
                            if (r != 15)
                                break;
                            k += 16;
                            continue;
                        }
                        k += r;
                        if (k > 63)
                            fail(VVPT_ERR_INVALID_ARG);
                        blk[k] = extend(b.bits(s), s);
                        k++;
                    }
                };
                if (ns == 1) {
                    block(0, (int)(m / ubx), (int)(m % ubx));
                } else {
                    const int my = (int)(m / f.mcux), mx = (int)(m % f.mcux);
                    for (int j = 0; j < ns; j++)
                        for (int yy = 0; yy < sc[j]->v; yy++)
                            for (int xx = 0; xx < sc[j]->h; xx++)
                                block(j, my * sc[j]->v + yy, mx * sc[j]->h + xx);
                }
            }
            // continue at the marker that ended the scan
            pos = b.pos;
            while (pos + 1 < n && !(d[pos] == 0xFF && d[pos + 1] != 0x00 && d[pos + 1] != 0xFF))
                pos++;
            f.scanned = true;
        }
        // APPn, COM and the rest: skipped
    }
    if (f.comps.empty() || !f.scanned)
        fail(VVPT_ERR_INVALID_ARG);
}

// Sample plane of one component: inverse DCT of every block, rounded and
// clamped to 8-bit samples, kept as doubles.
std::vector<double> plane_of(const Frame &f, const Component &c)
{
    if (!f.qt_present[c.tq])
        fail(VVPT_ERR_INVALID_ARG);
    double C[8][8];
    for (int x = 0; x < 8; x++)
        for (int u = 0; u < 8; u++)
            C[x][u] = 0.5 * (u == 0 ? 1.0 / std::sqrt(2.0) : 1.0) * std::cos((2 * x + 1) * u * kPi / 16.0);
    const int W = c.bx * 8;
    std::vector<double> out((size_t)c.by * 8 * W);
    const double *q = f.qt[c.tq];
    for (int by = 0; by < c.by; by++)
        for (int bx = 0; bx < c.bx; bx++) {
            const int32_t *blk = &c.coef[((size_t)by * c.bx + bx) * 64];
            double F[64], T[64];
            for (int i = 0; i < 64; i++)
                F[kZigzag[i]] = blk[i] * q[kZigzag[i]];
            // T[u][y] = sum_v F[u][v] C[y][v]  (u: row frequency, v: column)
            for (int u = 0; u < 8; u++)
                for (int y = 0; y < 8; y++) {
                    double s = 0.0;
                    for (int v = 0; v < 8; v++)
                        s += F[u * 8 + v] * C[y][v];
                    T[u * 8 + y] = s;
                }
            for (int x = 0; x < 8; x++)
                for (int y = 0; y < 8; y++) {
                    double s = 0.0;
                    for (int u = 0; u < 8; u++)
                        s += C[x][u] * T[u * 8 + y];
                    const double px = std::floor(s + 128.5);
                    out[(size_t)(by * 8 + x) * W + bx * 8 + y] = px < 0.0 ? 0.0 : (px > 255.0 ? 255.0 : px);
                }
        }
    return out;
}

// Doubles a plane along one axis with the triangle filter.
std::vector<double> upsample2(const std::vector<double> &p, int rows, int cols, bool vertical)
{
    const int orows = vertical ? 2 * rows : rows, ocols = vertical ? cols : 2 * cols;
    std::vector<double> o((size_t)orows * ocols);
    if (vertical) {
        for (int r = 0; r < rows; r++) {
            const int rp = r > 0 ? r - 1 : 0, rn = r + 1 < rows ? r + 1 : rows - 1;
            for (int c = 0; c < cols; c++) {
                const double a = p[(size_t)r * cols + c];
                o[(size_t)(2 * r) * cols + c] = 0.75 * a + 0.25 * p[(size_t)rp * cols + c];
                o[(size_t)(2 * r + 1) * cols + c] = 0.75 * a + 0.25 * p[(size_t)rn * cols + c];
            }
        }
    } else {
        for (int r = 0; r < rows; r++)
            for (int c = 0; c < cols; c++) {
                const int cp = c > 0 ? c - 1 : 0, cn = c + 1 < cols ? c + 1 : cols - 1;
                const double a = p[(size_t)r * cols + c];
                o[(size_t)r * ocols + 2 * c] = 0.75 * a + 0.25 * p[(size_t)r * cols + cp];
                o[(size_t)r * ocols + 2 * c + 1] = 0.75 * a + 0.25 * p[(size_t)r * cols + cn];
            }
    }
    return o;
}

uint8_t to_u8(double v)
{
    const double r = std::floor(v + 0.5);
    return (uint8_t)(r < 0.0 ? 0.0 : (r > 255.0 ? 255.0 : r));
}

}  // namespace

extern "C" VVPT_API vvpt_status vvpt_jpeg_decode(const uint8_t *data, uint64_t size, uint32_t *width,
                                                 uint32_t *height, uint32_t *channels, uint8_t *rgba,
                                                 uint64_t rgba_bytes)
{
    if (!data || !width || !height || !channels)
        return VVPT_ERR_INVALID_ARG;
    try {
        Frame f;
        parse(data, (size_t)size, f, rgba == nullptr);
        if (f.comps.empty())
            return VVPT_ERR_INVALID_ARG;
        *width = (uint32_t)f.w;
        *height = (uint32_t)f.h;
        *channels = (uint32_t)f.comps.size();
        if (!rgba)
            return VVPT_OK;
        if (rgba_bytes < (uint64_t)f.w * f.h * 4)
            return VVPT_ERR_INVALID_ARG;
        std::vector<std::vector<double>> planes;
        std::vector<int> pcols;
        for (const Component &c : f.comps) {
            std::vector<double> p = plane_of(f, c);
            int rows = c.by * 8, cols = c.bx * 8;
            if (c.v < f.vmax) {
                p = upsample2(p, rows, cols, true);
                rows *= 2;
            }
            if (c.h < f.hmax) {
                p = upsample2(p, rows, cols, false);
                cols *= 2;
            }
            planes.push_back(std::move(p));
            pcols.push_back(cols);
        }
        for (int y = 0; y < f.h; y++)
            for (int x = 0; x < f.w; x++) {
                uint8_t *o = rgba + ((size_t)y * f.w + x) * 4;
                o[3] = 255;
                if (planes.size() == 1) {
                    const uint8_t g = (uint8_t)planes[0][(size_t)y * pcols[0] + x];
                    o[0] = o[1] = o[2] = g;
                    continue;
                }
                const double Y = planes[0][(size_t)y * pcols[0] + x];
                const double cb = planes[1][(size_t)y * pcols[1] + x] - 128.0;
                const double cr = planes[2][(size_t)y * pcols[2] + x] - 128.0;
                o[0] = to_u8(Y + 1.402 * cr);
                o[1] = to_u8(Y - 0.344136 * cb - 0.714136 * cr);
                o[2] = to_u8(Y + 1.772 * cb);
            }
        return VVPT_OK;
    } catch (const Failure &e) {
        return e.st;
    } catch (...) {
        return VVPT_ERR_INVALID_ARG;
    }
}
