"""TGA files written independently of the library's writer, for testing its reader: every
layout TGAImage::read_tga_file accepts (tgaimage.cpp:40-143) — 8/24/32 bits, raw or
run-length, bottom-left or top-left origin, right-to-left columns — with a chunking that
differs from the library's own encoder (raw chunks of up to 3 pixels, runs of 2 or more)."""
from __future__ import annotations

import struct

import numpy as np


def encode(img: np.ndarray, rle: bool, top_left: bool = True, right_left: bool = False) -> bytes:
    """File bytes whose decoded TGAImage buffer is `img` ((h, w, bpp) uint8, row 0 first)."""
    h, w, bpp = img.shape
    rows = img if top_left else img[::-1]
    rows = rows[:, ::-1] if right_left else rows
    desc = (0x20 if top_left else 0) | (0x10 if right_left else 0)
    typ = (11 if rle else 3) if bpp == 1 else (10 if rle else 2)
    head = struct.pack("<BBBHHBHHHHBB", 0, 0, typ, 0, 0, 0, 0, 0, w, h, bpp * 8, desc)
    px = np.ascontiguousarray(rows).reshape(-1, bpp)
    if not rle:
        return head + px.tobytes()
    out = bytearray(head)
    i, n = 0, len(px)
    while i < n:
        j = i + 1
        while j < n and j - i < 128 and (px[j] == px[i]).all():
            j += 1
        if j - i >= 2:
            out.append(128 + (j - i) - 1)
            out += px[i].tobytes()
            i = j
        else:
            k = min(3, n - i)
            out.append(k - 1)
            out += px[i:i + k].tobytes()
            i += k
    return bytes(out)


def runs_image(h: int, w: int, bpp: int, seed: int) -> np.ndarray:
    """Random image with long runs of equal pixels (exercises both chunk kinds)."""
    rng = np.random.default_rng(seed)
    img = rng.integers(0, 256, (h, w, bpp), dtype=np.uint8)
    flat = img.reshape(-1, bpp)
    for _ in range(max(1, (h * w) // 40)):
        a = int(rng.integers(0, h * w))
        flat[a:a + int(rng.integers(2, 300))] = flat[a]
    return img
