"""Baseline JPEG decoding in Python: the test restatement that libvvpt's
host decoder (vviewer_gb300/csrc/jpeg_decode.cpp) is compared with, and the
coefficient decoder the tests check against their encoder.

It covers the sequential Huffman processes of ITU-T T.81 (SOF0 baseline and
SOF1 extended, 8-bit samples), one component (grey) or three (YCbCr, JFIF),
any sampling factors of 1 or 2, and restart intervals. The steps follow the
standard: Huffman decoding per F.2.2, dequantisation, and an 8 x 8 inverse
DCT (separable, float64, level-shifted, rounded to nearest and clamped to
8-bit samples). Chroma upsampling by 2 uses the triangle filter (3/4 near +
1/4 far sample). YCbCr to RGB uses the JFIF matrix. Progressive and
arithmetic-coded files raise ValueError.
"""
from __future__ import annotations

import math

import numpy as np

# zigzag order: index k of the coefficient stream -> position in the 8x8 block (row-major)
_ZIGZAG = np.array([
    0, 1, 8, 16, 9, 2, 3, 10, 17, 24, 32, 25, 18, 11, 4, 5, 12, 19, 26, 33, 40, 48, 41, 34, 27, 20, 13, 6, 7, 14,
    21, 28, 35, 42, 49, 56, 57, 50, 43, 36, 29, 22, 15, 23, 30, 37, 44, 51, 58, 59, 52, 45, 38, 31, 39, 46, 53, 60,
    61, 54, 47, 55, 62, 63], dtype=np.int64)


def _idct_matrix() -> np.ndarray:
    """C[x, u] = c(u) / 2 * cos((2x + 1) u pi / 16), c(0) = 1/sqrt(2): f = C F C^T."""
    c = np.zeros((8, 8))
    for x in range(8):
        for u in range(8):
            cu = 1.0 / math.sqrt(2.0) if u == 0 else 1.0
            c[x, u] = 0.5 * cu * math.cos((2 * x + 1) * u * math.pi / 16.0)
    return c


_C = _idct_matrix()


class _Huffman:
    """Decoding tables of one Huffman table (T.81 F.2.2.3: MINCODE, MAXCODE, VALPTR)."""

    def __init__(self, counts, symbols):
        self.symbols = list(symbols)
        self.maxcode = [-1] * 17
        self.mincode = [0] * 17
        self.valptr = [0] * 17
        code = 0
        k = 0
        for length in range(1, 17):
            n = counts[length - 1]
            if n:
                self.valptr[length] = k
                self.mincode[length] = code
                code += n
                k += n
                self.maxcode[length] = code - 1
            code <<= 1


class _Bits:
    """Entropy-coded segment reader: byte stuffing (FF 00) removed; a marker ends the data."""

    def __init__(self, data: bytes, pos: int):
        self.data = data
        self.pos = pos
        self.acc = 0
        self.n = 0
        self.marker = None

    def _byte(self) -> int:
        if self.marker is not None:
            return 0
        if self.pos + 1 >= len(self.data):
            raise ValueError("JPEG: entropy-coded data runs past the end of the file")
        b = self.data[self.pos]
        if b == 0xFF:
            nxt = self.data[self.pos + 1]
            if nxt == 0x00:
                self.pos += 2
                return 0xFF
            self.marker = nxt
            return 0
        self.pos += 1
        return b

    def bit(self) -> int:
        if self.n == 0:
            self.acc = self._byte()
            self.n = 8
        self.n -= 1
        return (self.acc >> self.n) & 1

    def bits(self, k: int) -> int:
        v = 0
        for _ in range(k):
            v = (v << 1) | self.bit()
        return v

    def decode(self, h: _Huffman) -> int:
        code = self.bit()
        length = 1
        while length <= 16 and code > h.maxcode[length]:
            code = (code << 1) | self.bit()
            length += 1
        if length > 16:
            raise ValueError("JPEG: bad Huffman code")
        return h.symbols[h.valptr[length] + code - h.mincode[length]]

    def restart(self) -> None:
        """Skips to the RSTn marker that ends the interval and resets the bit buffer."""
        self.n = 0
        if self.marker is None:
            while not (self.data[self.pos] == 0xFF and 0xD0 <= self.data[self.pos + 1] <= 0xD7):
                self.pos += 1
                if self.pos + 1 >= len(self.data):
                    raise ValueError("JPEG: restart marker missing")
            self.marker = self.data[self.pos + 1]
        if not 0xD0 <= self.marker <= 0xD7:
            raise ValueError("JPEG: restart marker expected")
        self.pos += 2
        self.marker = None


def _extend(v: int, t: int) -> int:
    """T.81 F.2.2.1 EXTEND."""
    return v - (1 << t) + 1 if t and v < (1 << (t - 1)) else v


def _upsample2(plane: np.ndarray, axis: int) -> np.ndarray:
    """Doubles a plane along one axis with the triangle filter: each output
    sample is 3/4 of its nearest input sample plus 1/4 of the next nearest
    (edge samples repeated), kept in float."""
    p = np.moveaxis(plane, axis, 0)
    prev = np.concatenate([p[:1], p[:-1]], axis=0)
    nxt = np.concatenate([p[1:], p[-1:]], axis=0)
    out = np.empty((2 * p.shape[0],) + p.shape[1:], dtype=np.float64)
    out[0::2] = 0.75 * p + 0.25 * prev
    out[1::2] = 0.75 * p + 0.25 * nxt
    return np.moveaxis(out, 0, axis)


def decode_jpeg_coefficients(data: bytes, what: str = "JPEG"):
    """Entropy-decoded frame: (frame, quantisation tables). frame["comps"][i]["coef"] holds each
    component's quantised coefficients per block, in zigzag order: [block row, block column, 64].
    Every malformed file raises ValueError."""
    try:
        return _parse(data, what)
    except (IndexError, KeyError, StopIteration, OverflowError) as e:
        raise ValueError(f"{what}: corrupt JPEG ({type(e).__name__})") from e


def _parse(data: bytes, what: str):
    if data[:2] != b"\xff\xd8":
        raise ValueError(f"{what}: not a JPEG file")
    pos = 2
    qt = {}
    huff = {}
    frame = None
    restart_interval = 0
    planes = None
    while pos < len(data):
        if data[pos] != 0xFF or pos + 1 >= len(data):
            raise ValueError(f"{what}: marker expected at byte {pos}")
        marker = data[pos + 1]
        pos += 2
        if marker in (0xD8, 0x01) or 0xD0 <= marker <= 0xD7:
            continue
        if marker == 0xD9:  # EOI
            break
        if pos + 2 > len(data):
            raise ValueError(f"{what}: file ends inside a marker segment")
        seg_len = (data[pos] << 8) | data[pos + 1]
        if seg_len < 2 or pos + seg_len > len(data):
            raise ValueError(f"{what}: marker segment runs past the end of the file")
        seg = data[pos + 2:pos + seg_len]
        pos += seg_len
        if marker == 0xDB:  # DQT
            k = 0
            while k < len(seg):
                pq, tq = seg[k] >> 4, seg[k] & 15
                k += 1
                if pq:
                    vals = np.frombuffer(seg[k:k + 128], dtype=">u2").astype(np.float64)
                    k += 128
                else:
                    vals = np.frombuffer(seg[k:k + 64], dtype=np.uint8).astype(np.float64)
                    k += 64
                q = np.zeros(64)
                q[_ZIGZAG] = vals
                qt[tq] = q.reshape(8, 8)
        elif marker == 0xC4:  # DHT
            k = 0
            while k < len(seg):
                tc, th = seg[k] >> 4, seg[k] & 15
                counts = list(seg[k + 1:k + 17])
                n = sum(counts)
                huff[(tc, th)] = _Huffman(counts, seg[k + 17:k + 17 + n])
                k += 17 + n
        elif marker in (0xC0, 0xC1):  # SOF0 / SOF1
            if seg[0] != 8:
                raise ValueError(f"{what}: {seg[0]}-bit samples are not supported")
            h, w, nc = (seg[1] << 8) | seg[2], (seg[3] << 8) | seg[4], seg[5]
            if nc not in (1, 3) or h == 0 or w == 0 or h * w > (1 << 28):
                raise ValueError(f"{what}: {nc} components / {w}x{h} not supported")
            comps = []
            for c in range(nc):
                cid, hv, tq = seg[6 + 3 * c], seg[7 + 3 * c], seg[8 + 3 * c]
                comps.append({"id": cid, "h": hv >> 4, "v": hv & 15, "tq": tq})
            hmax = max(c["h"] for c in comps)
            vmax = max(c["v"] for c in comps)
            if any(c["h"] not in (1, 2) or c["v"] not in (1, 2) for c in comps):
                raise ValueError(f"{what}: sampling factors other than 1 and 2 are not supported")
            mcux, mcuy = (w + 8 * hmax - 1) // (8 * hmax), (h + 8 * vmax - 1) // (8 * vmax)
            for c in comps:
                c["coef"] = np.zeros((mcuy * c["v"], mcux * c["h"], 64), dtype=np.int32)
            frame = {"h": h, "w": w, "comps": comps, "hmax": hmax, "vmax": vmax, "mcux": mcux, "mcuy": mcuy}
        elif marker in (0xC2, 0xC3, 0xC5, 0xC6, 0xC7, 0xC9, 0xCA, 0xCB, 0xCD, 0xCE, 0xCF):
            raise ValueError(f"{what}: progressive, lossless or arithmetic-coded JPEG is not supported")
        elif marker == 0xDD:  # DRI
            restart_interval = (seg[0] << 8) | seg[1]
        elif marker == 0xDA:  # SOS
            if frame is None:
                raise ValueError(f"{what}: scan before frame header")
            ns = seg[0]
            scomps = []
            for j in range(ns):
                cid, tables = seg[1 + 2 * j], seg[2 + 2 * j]
                comp = next(c for c in frame["comps"] if c["id"] == cid)
                scomps.append((comp, huff[(0, tables >> 4)], huff[(1, tables & 15)]))
            bits = _Bits(data, pos)
            pred = [0] * ns
            single = ns == 1
            if single:  # a non-interleaved scan codes the component's own blocks (A.2.2)
                comp = scomps[0][0]
                bx = (math.ceil(frame["w"] * comp["h"] / frame["hmax"]) + 7) // 8
                by = (math.ceil(frame["h"] * comp["v"] / frame["vmax"]) + 7) // 8
                units = [(comp, 0, y, x) for y in range(by) for x in range(bx)]
            total_mcus = len(units) if single else frame["mcux"] * frame["mcuy"]
            for m in range(total_mcus):
                if restart_interval and m and m % restart_interval == 0:
                    bits.restart()
                    pred = [0] * ns
                if single:
                    blocks = [(0, units[m][2], units[m][3])]
                else:
                    my, mx = divmod(m, frame["mcux"])
                    blocks = [(j, my * c["v"] + yy, mx * c["h"] + xx)
                              for j, (c, _, _) in enumerate(scomps) for yy in range(c["v"]) for xx in range(c["h"])]
                for j, yb, xb in blocks:
                    comp, dct, act = scomps[j]
                    blk = comp["coef"][yb, xb]
                    t = bits.decode(dct)
                    diff = _extend(bits.bits(t), t) if t else 0
                    pred[j] += diff
                    blk[0] = pred[j]
                    k = 1
                    while k < 64:
                        rs = bits.decode(act)
                        r, s = rs >> 4, rs & 15
                        if s == 0:
                            if r != 15:
                                break
                            k += 16
                            continue
                        k += r
                        if k > 63:
                            raise ValueError(f"{what}: AC coefficient index out of range")
                        blk[k] = _extend(bits.bits(s), s)
                        k += 1
            # continue at the marker that ended the scan
            pos = bits.pos
            while pos + 1 < len(data) and not (data[pos] == 0xFF and data[pos + 1] not in (0x00, 0xFF)):
                pos += 1
            planes = True
        else:  # APPn, COM and the rest
            continue
    if frame is None or planes is None:
        raise ValueError(f"{what}: no image data")
    return frame, qt


def decode_jpeg(data: bytes, what: str = "JPEG") -> tuple[np.ndarray, int]:
    """(H x W x 4 uint8 RGBA, channels in the file: 1 or 3) of a baseline or
    extended-sequential Huffman JPEG. Raises ValueError otherwise."""
    frame, qt = decode_jpeg_coefficients(data, what)
    if any(c["tq"] not in qt for c in frame["comps"]):
        raise ValueError(f"{what}: quantisation table missing")
    out = []
    for c in frame["comps"]:
        coef = c["coef"].astype(np.float64)
        ny, nx = coef.shape[:2]
        f = np.zeros((ny, nx, 64))
        f[..., _ZIGZAG] = coef
        f = f.reshape(ny, nx, 8, 8) * qt[c["tq"]]
        px = np.clip(np.floor(np.einsum("xu,abuv,yv->abxy", _C, f, _C) + 128.5), 0.0, 255.0)
        plane = px.transpose(0, 2, 1, 3).reshape(ny * 8, nx * 8)
        if c["v"] < frame["vmax"]:
            plane = _upsample2(plane, 0)
        if c["h"] < frame["hmax"]:
            plane = _upsample2(plane, 1)
        out.append(plane[:frame["h"], :frame["w"]])
    h, w = frame["h"], frame["w"]
    rgba = np.full((h, w, 4), 255, dtype=np.uint8)
    if len(out) == 1:
        g = out[0].astype(np.uint8)
        rgba[..., 0] = rgba[..., 1] = rgba[..., 2] = g
        return rgba, 1
    y, cb, cr = out[0], out[1] - 128.0, out[2] - 128.0
    rgb = np.stack([y + 1.402 * cr, y - 0.344136 * cb - 0.714136 * cr, y + 1.772 * cb], axis=-1)
    rgba[..., :3] = np.clip(np.floor(rgb + 0.5), 0, 255).astype(np.uint8)
    return rgba, 3
