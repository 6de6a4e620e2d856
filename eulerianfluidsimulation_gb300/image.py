"""8-bit grey images for the 2D scene import (Scene2D::loadImage, src/simulation/data/Scene2D.cpp:87-121).

The reference reads the image with stb_image (nothings/stb, an un-vendored submodule of the reference tree with
no pinned commit) as `stbi_load(path, &w, &h, &n, 1)`: any supported file becomes one 8-bit grey channel, rows
top to bottom. This module restates that conversion for the formats a scene image comes in:

- PNG (every colour type, bit depths 1-16, Adam7 interlacing);
- binary netpbm (P5 grey, P6 RGB; maxval up to 255, samples taken as stored);
- BMP (uncompressed 8-bit palette, 24-bit and 32-bit, rows bottom-up or top-down).

stb_image's published conversions, followed here: RGB (and the RGB of RGBA) to grey is the integer luma
(77 R + 150 G + 29 B) >> 8, computed at the image's own bit depth; grey and alpha keeps the grey; 16-bit
samples become 8-bit by their high byte, after the colour conversion; grey PNGs of 1, 2 and 4 bits are
scaled to 8 bits (x 255, x 85, x 17); palette indices are looked up, not scaled.
"""
import struct
import zlib

import numpy as np

_PNG_MAGIC = b"\x89PNG\r\n\x1a\n"
_GREY_SCALE = {1: 255, 2: 85, 4: 17, 8: 1}


def _luma(r, g, b):
    return (r.astype(np.int64) * 77 + g.astype(np.int64) * 150 + b.astype(np.int64) * 29) >> 8


def _to_grey(px, channels, bits):
    """(H, W, channels) samples at `bits` per sample -> (H, W) uint8, as stbi_load(..., 1)."""
    if channels in (1, 2):
        y = px[..., 0].astype(np.int64)
    else:
        y = _luma(px[..., 0], px[..., 1], px[..., 2])
    if bits == 16:
        y = y >> 8
    return (y & 0xFF).astype(np.uint8)


# ---- PNG -------------------------------------------------------------------------------------------------------
def _paeth(a, b, c):
    p = a + b - c
    pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
    if pa <= pb and pa <= pc:
        return a
    return b if pb <= pc else c


def _unfilter(data, pos, rows, row_bytes, bpp):
    """The filtered scanlines of one (sub)image starting at data[pos]; returns (rows x row_bytes uint8, next pos)."""
    out = np.zeros((rows, row_bytes), np.uint8)
    prev = np.zeros(row_bytes, np.int64)
    for y in range(rows):
        ftype = data[pos]
        line = np.frombuffer(data, np.uint8, row_bytes, pos + 1).astype(np.int64)
        pos += 1 + row_bytes
        if ftype == 0:
            cur = line
        elif ftype == 2:
            cur = (line + prev) & 0xFF
        elif ftype in (1, 3, 4):
            cur = np.zeros(row_bytes, np.int64)
            for i in range(row_bytes):
                a = cur[i - bpp] if i >= bpp else 0
                if ftype == 1:
                    pred = a
                elif ftype == 3:
                    pred = (a + prev[i]) >> 1
                else:
                    pred = _paeth(a, prev[i], prev[i - bpp] if i >= bpp else 0)
                cur[i] = (line[i] + pred) & 0xFF
        else:
            raise ValueError(f"PNG: unknown filter type {ftype}")
        out[y] = cur
        prev = cur
    return out, pos


def _samples(raw, width, channels, bits):
    """Unfiltered scanlines (rows x row_bytes) -> (rows, width, channels) integer samples."""
    rows = raw.shape[0]
    if bits == 8:
        return raw[:, :width * channels].reshape(rows, width, channels).astype(np.int64)
    if bits == 16:
        b = raw[:, :width * channels * 2].reshape(rows, width * channels, 2).astype(np.int64)
        return ((b[..., 0] << 8) | b[..., 1]).reshape(rows, width, channels)
    # 1, 2 or 4 bits: samples packed from the most significant bit of each byte
    bitsarr = np.unpackbits(raw, axis=1)[:, :width * channels * bits]
    vals = bitsarr.reshape(rows, width * channels, bits)
    weights = 1 << np.arange(bits - 1, -1, -1)
    return (vals.astype(np.int64) * weights).sum(-1).reshape(rows, width, channels)


def _read_png(data):
    pos = 8
    ihdr = None
    palette = None
    idat = []
    while pos < len(data):
        length, ctype = struct.unpack(">I4s", data[pos:pos + 8])
        body = data[pos + 8:pos + 8 + length]
        pos += 12 + length
        if ctype == b"IHDR":
            ihdr = struct.unpack(">IIBBBBB", body)
        elif ctype == b"PLTE":
            palette = np.frombuffer(body, np.uint8).reshape(-1, 3).astype(np.int64)
        elif ctype == b"IDAT":
            idat.append(body)
        elif ctype == b"IEND":
            break
    if ihdr is None:
        raise ValueError("PNG: no IHDR chunk")
    width, height, bits, ctype, _, _, interlace = ihdr
    channels = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}[ctype]
    raw = zlib.decompress(b"".join(idat))
    bpp = max(1, channels * bits // 8)

    def sub(w, h, p):
        row_bytes = (w * channels * bits + 7) // 8
        lines, p = _unfilter(raw, p, h, row_bytes, bpp)
        return _samples(lines, w, channels, bits), p

    if interlace == 0:
        px, _ = sub(width, height, 0)
    else:
        # Adam7: seven passes of (x0, y0, dx, dy)
        px = np.zeros((height, width, channels), np.int64)
        p = 0
        for x0, y0, dx, dy in ((0, 0, 8, 8), (4, 0, 8, 8), (0, 4, 4, 8), (2, 0, 4, 4), (0, 2, 2, 4), (1, 0, 2, 2),
                               (0, 1, 1, 2)):
            w = (width - x0 + dx - 1) // dx if width > x0 else 0
            h = (height - y0 + dy - 1) // dy if height > y0 else 0
            if w == 0 or h == 0:
                continue
            part, p = sub(w, h, p)
            px[y0::dy, x0::dx][:h, :w] = part
    if ctype == 3:
        if palette is None:
            raise ValueError("PNG: palette image without PLTE")
        rgb = palette[px[..., 0]]
        return _to_grey(rgb, 3, 8)
    if ctype == 0 and bits < 8:
        return (px[..., 0] * _GREY_SCALE[bits]).astype(np.uint8)
    return _to_grey(px, channels, bits)


# ---- netpbm -------------------------------------------------------------------------------------------------------
def _read_pnm(data):
    kind = data[:2]
    fields, pos = [], 2
    while len(fields) < 3:
        while data[pos:pos + 1].isspace():
            pos += 1
        if data[pos:pos + 1] == b"#":
            while data[pos:pos + 1] not in (b"\n", b""):
                pos += 1
            continue
        start = pos
        while not data[pos:pos + 1].isspace():
            pos += 1
        fields.append(int(data[start:pos]))
    pos += 1   # the single whitespace after maxval
    width, height, maxval = fields
    if maxval > 255:
        raise ValueError("netpbm: 16-bit samples are not supported")
    channels = 1 if kind == b"P5" else 3
    px = np.frombuffer(data, np.uint8, width * height * channels, pos).reshape(height, width, channels)
    return _to_grey(px, channels, 8)


# ---- BMP ----------------------------------------------------------------------------------------------------------
def _read_bmp(data):
    offset = struct.unpack("<I", data[10:14])[0]
    hsize = struct.unpack("<I", data[14:18])[0]
    width, height = struct.unpack("<ii", data[18:26])
    bits = struct.unpack("<H", data[28:30])[0]
    compression = struct.unpack("<I", data[30:34])[0] if hsize >= 40 else 0
    if compression not in (0, 3):
        raise ValueError("BMP: compressed images are not supported")
    flip = height > 0
    height = abs(height)
    stride = (width * bits + 31) // 32 * 4
    rows = np.frombuffer(data, np.uint8, stride * height, offset).reshape(height, stride)
    if bits == 8:
        ncol = struct.unpack("<I", data[46:50])[0] if hsize >= 40 else 0
        ncol = ncol or 256
        pal = np.frombuffer(data, np.uint8, ncol * 4, 14 + hsize).reshape(ncol, 4).astype(np.int64)
        rgb = pal[rows[:, :width].astype(np.int64)][..., [2, 1, 0]]
    elif bits in (24, 32):
        c = bits // 8
        bgr = rows[:, :width * c].reshape(height, width, c).astype(np.int64)
        rgb = bgr[..., [2, 1, 0]]
    else:
        raise ValueError(f"BMP: {bits}-bit images are not supported")
    grey = _to_grey(rgb, 3, 8)
    return grey[::-1] if flip else grey


def read_grey8(path):
    """The image at `path` as stbi_load(path, ..., 1) gives it: (height, width) uint8, row 0 the top row."""
    with open(path, "rb") as fh:
        data = fh.read()
    if data[:8] == _PNG_MAGIC:
        return _read_png(data)
    if data[:2] in (b"P5", b"P6"):
        return _read_pnm(data)
    if data[:2] == b"BM":
        return _read_bmp(data)
    raise ValueError(f"{path}: not a PNG, binary netpbm or BMP image")
