"""JPEG texture decoding for model import, through libvvpt's host decoder
(`vvpt_jpeg_decode`, vviewer_gb300/csrc/jpeg_decode.cpp).

vengine loads textures through stb_image (AssimpLoadModel.cpp:assimpLoadTextureData), which reads
JPEG as well as PNG. The native decoder covers the sequential Huffman processes of ITU-T T.81
(baseline and extended, 8-bit samples, grey or YCbCr with sampling factors 1 and 2, restart
intervals); progressive, lossless, arithmetic-coded and 12-bit files raise ValueError, and the model
loader then leaves the slot untextured with a warning, as the reference does when stb_image fails.
Results can differ from stb_image's integer IDCT and upsampling by a unit in the last place of some
texels.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as N


def decode_jpeg(data: bytes, what: str = "JPEG") -> tuple[np.ndarray, int]:
    """(H x W x 4 uint8 RGBA, channels in the file: 1 or 3). Raises
    ValueError for files the decoder does not take."""
    lib = N.load()
    buf = np.frombuffer(bytes(data), dtype=np.uint8)
    w, h, ch = C.c_uint32(0), C.c_uint32(0), C.c_uint32(0)
    st = lib.vvpt_jpeg_decode(buf.ctypes.data, buf.size, C.byref(w), C.byref(h), C.byref(ch), None, 0)
    if st == N.VVPT_OK:
        rgba = np.empty((h.value, w.value, 4), dtype=np.uint8)
        st = lib.vvpt_jpeg_decode(buf.ctypes.data, buf.size, C.byref(w), C.byref(h), C.byref(ch),
                                  rgba.ctypes.data, rgba.nbytes)
    if st != N.VVPT_OK:
        kind = "not supported (progressive, lossless, arithmetic-coded or 12-bit)" \
            if st == 8 else "malformed or not a JPEG file"
        raise ValueError(f"{what}: {kind} ({N.STATUS_NAMES.get(st, st)})")
    return rgba, int(ch.value)
