"""Test images written from scratch (PNG per ISO 15948, Radiance RGBE), with
every feature the texture decoders handle: colour types, bit depths,
palettes with transparency, Adam7 interlacing, all five scanline filters,
stored and compressed deflate blocks, flat and run-length RGBE scanlines."""
from __future__ import annotations

import struct
import zlib

import numpy as np

_ADAM7 = [(0, 0, 8, 8), (4, 0, 8, 8), (0, 4, 4, 8), (2, 0, 4, 4), (0, 2, 2, 4), (1, 0, 2, 2), (0, 1, 1, 2)]


def _chunk(tag: bytes, body: bytes) -> bytes:
    return struct.pack(">I", len(body)) + tag + body + struct.pack(">I", zlib.crc32(tag + body) & 0xFFFFFFFF)


def _pack_row(samples: np.ndarray, depth: int) -> bytes:
    """One row of samples (already interleaved) at the bit depth."""
    if depth == 16:
        return samples.astype(">u2").tobytes()
    if depth == 8:
        return samples.astype(np.uint8).tobytes()
    out, acc, nb = bytearray(), 0, 0
    for v in samples.tolist():
        acc = (acc << depth) | int(v)
        nb += depth
        if nb == 8:
            out.append(acc)
            acc, nb = 0, 0
    if nb:
        out.append(acc << (8 - nb))
    return bytes(out)


def _paeth(a, b, c):
    p = a + b - c
    pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
    if pa <= pb and pa <= pc:
        return a
    return b if pb <= pc else c


def _filter_rows(rows: list[bytes], bpp: int, first_filter: int) -> bytes:
    out = bytearray()
    prev = bytes(len(rows[0])) if rows else b""
    for y, r in enumerate(rows):
        ft = (first_filter + y) % 5
        f = bytearray([ft])
        for x in range(len(r)):
            a = r[x - bpp] if x >= bpp else 0
            b = prev[x]
            c = prev[x - bpp] if x >= bpp else 0
            pred = [0, a, b, (a + b) >> 1, _paeth(a, b, c)][ft]
            f.append((r[x] - pred) & 0xFF)
        out += f
        prev = r
    return bytes(out)


def write_png(path: str, samples: np.ndarray, color_type: int, depth: int, interlace: bool = False,
              palette: np.ndarray | None = None, trns: bytes | None = None, level: int = 9, first_filter: int = 0):
    """samples: (H, W, C) integer samples (palette indices for colour type 3)."""
    h, w, ch = samples.shape
    ihdr = struct.pack(">IIBBBBB", w, h, depth, color_type, 0, 0, 1 if interlace else 0)
    bpp = max(1, ch * depth // 8)
    raw = b""
    passes = _ADAM7 if interlace else [(0, 0, 1, 1)]
    for k, (x0, y0, dx, dy) in enumerate(passes):
        sub = samples[y0::dy, x0::dx]
        if sub.shape[0] == 0 or sub.shape[1] == 0:
            continue
        rows = [_pack_row(sub[y].reshape(-1), depth) for y in range(sub.shape[0])]
        raw += _filter_rows(rows, bpp, first_filter + k)
    data = b"\x89PNG\r\n\x1a\n" + _chunk(b"IHDR", ihdr)
    if palette is not None:
        data += _chunk(b"PLTE", np.asarray(palette, np.uint8).tobytes())
    if trns is not None:
        data += _chunk(b"tRNS", trns)
    z = zlib.compress(raw, level)
    # split the stream over several IDAT chunks
    step = max(1, len(z) // 3)
    for i in range(0, len(z), step):
        data += _chunk(b"IDAT", z[i:i + step])
    data += _chunk(b"IEND", b"")
    with open(path, "wb") as f:
        f.write(data)


def write_rgbe(path: str, rgbe: np.ndarray, rle: bool = True):
    """rgbe: (H, W, 4) uint8 mantissas and exponents."""
    h, w, _ = rgbe.shape
    out = bytearray(b"#?RADIANCE\n# test image\nFORMAT=32-bit_rle_rgbe\n\n")
    out += f"-Y {h} +X {w}\n".encode()
    for y in range(h):
        row = rgbe[y]
        if not rle:
            out += row.astype(np.uint8).tobytes()
            continue
        out += bytes([2, 2, w >> 8, w & 255])
        for c in range(4):
            v = row[:, c].astype(np.uint8).tolist()
            x = 0
            while x < w:
                run = 1
                while x + run < w and run < 127 and v[x + run] == v[x]:
                    run += 1
                if run >= 3:
                    out += bytes([128 + run, v[x]])
                    x += run
                else:
                    n = 1
                    while x + n < w and n < 128 and not (x + n + 2 < w and v[x + n] == v[x + n + 1] == v[x + n + 2]):
                        n += 1
                    out += bytes([n]) + bytes(v[x:x + n])
                    x += n
    with open(path, "wb") as f:
        f.write(bytes(out))
