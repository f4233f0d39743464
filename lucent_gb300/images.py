"""Image decoding for model textures.

The reference decodes a model's images with the browser (createImageBitmap,
src/loaders/model.ts:43-72) into 8-bit RGBA, unpremultiplied, without colour
conversion. This build decodes PNG (all colour types, bit depths 1-16,
palettes with transparency, Adam7 interlacing): chunks and inflate here,
scanline unfiltering in the native library (lucent_png_unfilter). Other
formats raise ImageDecodeError, and the model loader drops the maps that use
them with the reference's warning, as model.ts does for an image the browser
cannot decode.
"""
import ctypes as C
import struct
import zlib

import numpy as np

from . import _native as N

PNG_SIGNATURE = b"\x89PNG\r\n\x1a\n"
CHANNELS = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}  # colour type -> samples per pixel
ADAM7 = ((0, 0, 8, 8), (4, 0, 8, 8), (0, 4, 4, 8), (2, 0, 4, 4), (0, 2, 2, 4), (1, 0, 2, 2), (0, 1, 1, 2))


class ImageDecodeError(ValueError):
    pass


def _unfilter(raw, rows, row_bytes, bpp):
    out = np.empty(rows * row_bytes, np.uint8)
    if rows and row_bytes:
        src = np.frombuffer(raw, np.uint8, count=rows * (row_bytes + 1))
        N.check(N.lib().lucent_png_unfilter(N.ptr(src, C.c_uint8), rows, row_bytes, bpp, N.ptr(out, C.c_uint8)))
    return out.reshape(rows, row_bytes)


def _samples(rows_u8, width, depth, channels):
    """Unpacked samples [rows, width * channels] as uint16 (values 0..2^depth-1)."""
    n = width * channels
    if depth == 8:
        return rows_u8[:, :n].astype(np.uint16)
    if depth == 16:
        v = rows_u8[:, :2 * n].reshape(rows_u8.shape[0], n, 2).astype(np.uint16)
        return (v[:, :, 0] << 8) | v[:, :, 1]
    bits = np.unpackbits(rows_u8, axis=1).reshape(rows_u8.shape[0], -1, depth)
    weights = (1 << np.arange(depth - 1, -1, -1)).astype(np.uint16)
    return (bits.astype(np.uint16) * weights).sum(axis=2, dtype=np.uint16)[:, :n]


def decode_png(data) -> np.ndarray:
    """PNG bytes -> uint8 RGBA [height, width, 4] (row 0 = top)."""
    data = bytes(data)
    if not data.startswith(PNG_SIGNATURE):
        raise ImageDecodeError("not a PNG file")
    at, ihdr, plte, trns, idat = 8, None, None, None, []
    while at + 8 <= len(data):
        length, kind = struct.unpack_from(">I4s", data, at)
        body = data[at + 8:at + 8 + length]
        if len(body) != length:
            raise ImageDecodeError("truncated PNG chunk")
        if kind == b"IHDR":
            ihdr = struct.unpack(">IIBBBBB", body)
        elif kind == b"PLTE":
            plte = np.frombuffer(body, np.uint8).reshape(-1, 3)
        elif kind == b"tRNS":
            trns = body
        elif kind == b"IDAT":
            idat.append(body)
        elif kind == b"IEND":
            break
        at += 12 + length
    if ihdr is None or not idat:
        raise ImageDecodeError("PNG without IHDR or IDAT")
    width, height, depth, ctype, method, filt, interlace = ihdr
    if ctype not in CHANNELS or depth not in (1, 2, 4, 8, 16) or method or filt or interlace > 1 or not width or not height:
        raise ImageDecodeError("unsupported PNG header %s" % (ihdr,))
    if ctype == 3 and plte is None:
        raise ImageDecodeError("palette PNG without PLTE")
    try:
        raw = zlib.decompress(b"".join(idat))
    except zlib.error as e:
        raise ImageDecodeError("bad PNG data: %s" % e)
    ch = CHANNELS[ctype]
    bpp = max(1, ch * depth // 8)
    samples = np.zeros((height, width * ch), np.uint16)
    passes = ADAM7 if interlace else ((0, 0, 1, 1),)
    pos = 0
    for x0, y0, dx, dy in passes:
        w = (width - x0 + dx - 1) // dx
        h = (height - y0 + dy - 1) // dy
        if w <= 0 or h <= 0:
            continue
        row_bytes = (w * ch * depth + 7) // 8
        need = h * (row_bytes + 1)
        if pos + need > len(raw):
            raise ImageDecodeError("PNG data too short")
        rows = _unfilter(raw[pos:pos + need], h, row_bytes, bpp)
        pos += need
        s = _samples(rows, w, depth, ch).reshape(h, w, ch)
        samples.reshape(height, width, ch)[y0::dy, x0::dx] = s
    s = samples.reshape(height, width, ch)
    if ctype == 3:
        idx = s[:, :, 0].astype(np.intp)
        if idx.max() >= plte.shape[0]:
            raise ImageDecodeError("palette index out of range")
        alpha = np.full(plte.shape[0], 255, np.uint8)
        if trns is not None:
            a = np.frombuffer(trns, np.uint8)[: plte.shape[0]]
            alpha[: a.size] = a
        return np.concatenate([plte[idx], alpha[idx][:, :, None]], axis=2)
    maxv = (1 << depth) - 1
    to8 = lambda v: ((v.astype(np.uint32) * 255 + maxv // 2) // maxv).astype(np.uint8) if depth != 8 else v.astype(np.uint8)
    out = np.empty((height, width, 4), np.uint8)
    if ctype in (0, 4):
        g = to8(s[:, :, 0])
        out[:, :, 0] = out[:, :, 1] = out[:, :, 2] = g
        out[:, :, 3] = to8(s[:, :, 1]) if ctype == 4 else 255
        if ctype == 0 and trns is not None and len(trns) >= 2:
            key = struct.unpack(">H", trns[:2])[0]
            out[:, :, 3] = np.where(s[:, :, 0] == key, 0, 255)
    else:
        out[:, :, :3] = to8(s[:, :, :3])
        out[:, :, 3] = to8(s[:, :, 3]) if ctype == 6 else 255
        if ctype == 2 and trns is not None and len(trns) >= 6:
            key = np.array(struct.unpack(">HHH", trns[:6]), np.uint16)
            out[:, :, 3] = np.where((s[:, :, :3] == key).all(axis=2), 0, 255)
    return out


def decode_image(data, mime_type="") -> np.ndarray:
    """Decoded RGBA8 [h, w, 4] of an encoded image, or ImageDecodeError."""
    data = bytes(data)
    if data.startswith(PNG_SIGNATURE):
        return decode_png(data)
    raise ImageDecodeError("cannot decode %s images in this build" % (mime_type or "these"))


def encode_png(rgba: np.ndarray) -> bytes:
    """Minimal PNG writer (RGBA8, filter 0): writes test fixtures and texture dumps."""
    rgba = np.ascontiguousarray(rgba, np.uint8)
    h, w = rgba.shape[:2]
    raw = b"".join(b"\x00" + rgba[y].tobytes() for y in range(h))

    def chunk(kind, body):
        return struct.pack(">I", len(body)) + kind + body + struct.pack(">I", zlib.crc32(kind + body) & 0xFFFFFFFF)

    return (PNG_SIGNATURE + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, 6, 0, 0, 0)) +
            chunk(b"IDAT", zlib.compress(raw)) + chunk(b"IEND", b""))
