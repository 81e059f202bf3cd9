"""A small PNG encoder for the loader tests (written from the PNG
specification): every colour type and bit depth, a chosen filter per
scanline, optional Adam7 interlacing, optional PLTE and tRNS chunks."""
import struct
import zlib

import numpy as np

ADAM7 = [(0, 0, 8, 8), (4, 0, 8, 8), (0, 4, 4, 8), (2, 0, 4, 4), (0, 2, 2, 4), (1, 0, 2, 2), (0, 1, 1, 2)]
CHANNELS = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}


def _chunk(typ, body):
    return struct.pack(">I", len(body)) + typ + body + struct.pack(">I", zlib.crc32(typ + body) & 0xFFFFFFFF)


def _pack_row(samples, depth):
    """samples: 1-D int array of one scanline's samples."""
    if depth == 8:
        return samples.astype(np.uint8).tobytes()
    if depth == 16:
        return samples.astype(">u2").tobytes()
    bits = np.zeros(len(samples) * depth, np.uint8)
    for k in range(depth):
        bits[k::depth] = (samples >> (depth - 1 - k)) & 1
    return np.packbits(bits).tobytes()


def _filter(raw, prev, bpp, ft):
    raw = np.frombuffer(raw, np.uint8).astype(np.int32)
    prev = np.frombuffer(prev, np.uint8).astype(np.int32)
    n = len(raw)
    left = np.concatenate([np.zeros(bpp, np.int32), raw[:-bpp]]) if n > bpp else np.zeros(n, np.int32)
    upleft = np.concatenate([np.zeros(bpp, np.int32), prev[:-bpp]]) if n > bpp else np.zeros(n, np.int32)
    if ft == 0:
        out = raw
    elif ft == 1:
        out = raw - left
    elif ft == 2:
        out = raw - prev
    elif ft == 3:
        out = raw - ((left + prev) >> 1)
    else:
        p = left + prev - upleft
        pa, pb, pc = np.abs(p - left), np.abs(p - prev), np.abs(p - upleft)
        pred = np.where((pa <= pb) & (pa <= pc), left, np.where(pb <= pc, prev, upleft))
        out = raw - pred
    return bytes([ft]) + (out & 0xFF).astype(np.uint8).tobytes()


def encode(samples, color_type, depth, palette=None, trns=None, interlace=False, filters=(0, 1, 2, 3, 4)):
    """samples: (h, w, channels) ints in [0, 2^depth)."""
    h, w, ch = samples.shape
    assert ch == CHANNELS[color_type]
    bpp = max(1, depth * ch // 8)
    stream = b""
    passes = ADAM7 if interlace else [(0, 0, 1, 1)]
    row_no = 0
    for x0, y0, dx, dy in passes:
        sub = samples[y0::dy, x0::dx]
        if sub.size == 0:
            continue
        prev = bytes((sub.shape[1] * ch * depth + 7) // 8)
        for y in range(sub.shape[0]):
            raw = _pack_row(sub[y].reshape(-1), depth)
            stream += _filter(raw, prev, bpp, filters[row_no % len(filters)])
            prev = raw
            row_no += 1
    out = b"\x89PNG\r\n\x1a\n" + _chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, depth, color_type, 0, 0,
                                                              1 if interlace else 0))
    if palette is not None:
        out += _chunk(b"PLTE", np.asarray(palette, np.uint8).tobytes())
    if trns is not None:
        out += _chunk(b"tRNS", trns)
    out += _chunk(b"IDAT", zlib.compress(stream)) + _chunk(b"IEND", b"")
    return out
