"""A small baseline JPEG encoder for the decoder's tests (no JPEG library in
this environment). Forward DCT in float64, quantisation by a scaled table,
zigzag order, Huffman tables built from the image's own symbol counts
(Huffman code lengths, canonical codes, one code point kept free so that
no code is all ones), byte stuffing, optional restart intervals, greyscale
or YCbCr at 4:4:4 or 4:2:0 (chroma averaged over 2 x 2)."""
from __future__ import annotations

import heapq
import math
import struct

import numpy as np

ZIGZAG = np.array([
    0, 1, 8, 16, 9, 2, 3, 10, 17, 24, 32, 25, 18, 11, 4, 5, 12, 19, 26, 33, 40, 48, 41, 34, 27, 20, 13, 6, 7, 14,
    21, 28, 35, 42, 49, 56, 57, 50, 43, 36, 29, 22, 15, 23, 30, 37, 44, 51, 58, 59, 52, 45, 38, 31, 39, 46, 53, 60,
    61, 54, 47, 55, 62, 63], dtype=np.int64)


def _dct_matrix():
    c = np.zeros((8, 8))
    for x in range(8):
        for u in range(8):
            cu = 1.0 / math.sqrt(2.0) if u == 0 else 1.0
            c[x, u] = 0.5 * cu * math.cos((2 * x + 1) * u * math.pi / 16.0)
    return c


_C = _dct_matrix()


def _blocks(plane, by, bx):
    p = np.zeros((by * 8, bx * 8))
    h, w = plane.shape
    p[:h, :w] = plane
    p[h:, :w] = plane[h - 1:h, :]
    p[:, w:] = p[:, w - 1:w]
    return p.reshape(by, 8, bx, 8).transpose(0, 2, 1, 3)


def _quantise(blocks, q):
    f = np.einsum("xu,abxy,yv->abuv", _C, blocks - 128.0, _C)
    return np.rint(f / q).astype(np.int64).reshape(blocks.shape[0], blocks.shape[1], 64)[..., ZIGZAG]


def _category(v):
    return 0 if v == 0 else int(abs(int(v))).bit_length()


def _code_lengths(freq: dict) -> dict:
    """Huffman code lengths of the symbols, with one extra symbol kept back
    (so the all-ones code of the longest length stays unused)."""
    items = [(f, i, [s]) for i, (s, f) in enumerate(freq.items())]
    items.append((0, len(items), [None]))
    heapq.heapify(items)
    lengths = {s: 0 for s in freq}
    lengths[None] = 0
    if len(items) == 1:
        return {s: 1 for s in freq}
    k = len(items)
    while len(items) > 1:
        fa, _, a = heapq.heappop(items)
        fb, _, b = heapq.heappop(items)
        for s in a + b:
            lengths[s] += 1
        heapq.heappush(items, (fa + fb, k, a + b))
        k += 1
    del lengths[None]
    if max(lengths.values()) > 16:
        return {s: 8 for s in freq}
    return lengths


def _table(freq: dict):
    lengths = _code_lengths(freq)
    syms = sorted(lengths, key=lambda s: (lengths[s], s))
    counts = [0] * 16
    for s in syms:
        counts[lengths[s] - 1] += 1
    codes, code, prev = {}, 0, 0
    for s in syms:
        code <<= lengths[s] - prev
        prev = lengths[s]
        codes[s] = (code, lengths[s])
        code += 1
    return counts, syms, codes


class _Writer:
    def __init__(self):
        self.out = bytearray()
        self.acc = 0
        self.n = 0

    def put(self, value, length):
        for i in range(length - 1, -1, -1):
            self.acc = (self.acc << 1) | ((value >> i) & 1)
            self.n += 1
            if self.n == 8:
                self.out.append(self.acc)
                if self.acc == 0xFF:
                    self.out.append(0)
                self.acc = 0
                self.n = 0

    def flush(self):
        if self.n:
            self.put((1 << (8 - self.n)) - 1, 8 - self.n)


def encode_jpeg(rgb: np.ndarray, quality: float = 1.0, subsample: bool | tuple = True, restart: int = 0,
                return_coefficients: bool = False):
    """rgb: H x W x 3 (or H x W for grey) uint8. quality scales a flat-ish
    quantisation table (1.0: steps of 1-3). subsample: True for 4:2:0, False
    for 4:4:4, or the luma sampling factors (h, v), e.g. (2, 1) for 4:2:2.
    With return_coefficients also the quantised coefficients per component
    ([block row, block column, 64], zigzag order) and the quantisation table
    (8 x 8)."""
    img = np.asarray(rgb, dtype=np.float64)
    grey = img.ndim == 2
    h, w = img.shape[:2]
    q = np.maximum(1.0, np.rint((1.0 + np.add.outer(np.arange(8), np.arange(8)) / 7.0) * quality))
    if grey:
        planes = [img]
        samp = [(1, 1)]
    else:
        r, g, b = img[..., 0], img[..., 1], img[..., 2]
        y = 0.299 * r + 0.587 * g + 0.114 * b
        cb = -0.168736 * r - 0.331264 * g + 0.5 * b + 128.0
        cr = 0.5 * r - 0.418688 * g - 0.081312 * b + 128.0
        if subsample:
            sh, sv = (2, 2) if subsample is True else subsample

            def half(p):
                hh, ww = (h + sv - 1) // sv, (w + sh - 1) // sh
                pp = np.pad(p, ((0, sv * hh - h), (0, sh * ww - w)), mode="edge")
                return pp.reshape(hh, sv, ww, sh).mean(axis=(1, 3))
            planes = [y, half(cb), half(cr)]
            samp = [(sh, sv), (1, 1), (1, 1)]
        else:
            planes = [y, cb, cr]
            samp = [(1, 1)] * 3
    hmax = max(s[0] for s in samp)
    vmax = max(s[1] for s in samp)
    mcux, mcuy = (w + 8 * hmax - 1) // (8 * hmax), (h + 8 * vmax - 1) // (8 * vmax)
    coefs = [_quantise(_blocks(p, mcuy * sv, mcux * sh), q) for p, (sh, sv) in zip(planes, samp)]
    # MCU order of the blocks: (component, block row, block column)
    order = []
    for my in range(mcuy):
        for mx in range(mcux):
            for c, (sh, sv) in enumerate(samp):
                for yy in range(sv):
                    for xx in range(sh):
                        order.append((c, my * sv + yy, mx * sh + xx, my * mcux + mx))
    # symbol statistics (luma tables 0, chroma tables 1)
    dcf, acf = [{}, {}], [{}, {}]
    pred = [0] * len(planes)
    last_mcu = -1
    seq = []
    for c, by, bx, m in order:
        if restart and m != last_mcu and m and m % restart == 0:
            pred = [0] * len(planes)
        last_mcu = m
        blk = coefs[c][by, bx]
        t = min(c, 1)
        d = int(blk[0]) - pred[c]
        pred[c] = int(blk[0])
        dcf[t][_category(d)] = dcf[t].get(_category(d), 0) + 1
        syms = []
        run = 0
        last_nz = max([k for k in range(1, 64) if blk[k] != 0], default=0)
        for k in range(1, last_nz + 1):
            v = int(blk[k])
            if v == 0:
                run += 1
                continue
            while run > 15:
                syms.append((0xF0, 0, 0))
                run -= 16
            s = _category(v)
            syms.append(((run << 4) | s, v, s))
            run = 0
        if last_nz < 63:
            syms.append((0x00, 0, 0))
        for sym, _, _ in syms:
            acf[t][sym] = acf[t].get(sym, 0) + 1
        seq.append((c, t, m, d, syms))
    ntab = 1 if grey else 2
    tables = [(_table(dcf[t]), _table(acf[t])) for t in range(ntab)]
    out = bytearray(b"\xff\xd8")

    def seg(marker, payload):
        out.extend(struct.pack(">BBH", 0xFF, marker, len(payload) + 2))
        out.extend(payload)

    qb = bytes([0]) + bytes(int(v) for v in q.reshape(64)[ZIGZAG])
    seg(0xDB, qb)
    sof = struct.pack(">BHHB", 8, h, w, len(planes))
    for c, (sh, sv) in enumerate(samp):
        sof += bytes([c + 1, (sh << 4) | sv, 0])
    seg(0xC0, sof)
    for t in range(ntab):
        for tc, (counts, syms, _) in ((0, tables[t][0]), (1, tables[t][1])):
            seg(0xC4, bytes([(tc << 4) | t]) + bytes(counts) + bytes(syms))
    if restart:
        seg(0xDD, struct.pack(">H", restart))
    sos = bytes([len(planes)])
    for c in range(len(planes)):
        t = min(c, 1)
        sos += bytes([c + 1, (t << 4) | t])
    sos += bytes([0, 63, 0])
    seg(0xDA, sos)
    wr = _Writer()
    last_mcu = -1
    rst = 0
    for c, t, m, d, syms in seq:
        if restart and m != last_mcu and m and m % restart == 0:
            wr.flush()
            out.extend(wr.out)
            wr.out = bytearray()
            out.extend(bytes([0xFF, 0xD0 + (rst & 7)]))
            rst += 1
        last_mcu = m
        dcodes, acodes = tables[t][0][2], tables[t][1][2]
        s = _category(d)
        wr.put(*dcodes[s])
        if s:
            wr.put(d if d > 0 else d + (1 << s) - 1, s)
        for sym, v, s in syms:
            wr.put(*acodes[sym])
            if s:
                wr.put(v if v > 0 else v + (1 << s) - 1, s)
    wr.flush()
    out.extend(wr.out)
    out.extend(b"\xff\xd9")
    if return_coefficients:
        return bytes(out), coefs, q
    return bytes(out)
