"""Regenerate the golden fixtures in this directory from the reference tree.

Run in a checkout where the Ascent sources are readable (default path
/root/reference, override with GVR_REFERENCE_ROOT). Tests read only the
committed .npz files.

apcomp_volume_partial.npz
    The reference's baseline image of its partial-compositing test
    (src/tests/_baseline_images/apcomp/apcomp_volume_partial.png, produced by
    src/tests/apcomp/t_apcomp_volume_partials.cpp:16-57), decoded to RGBA
    uint8 rows as stored in the PNG (top row first).
"""
from __future__ import annotations

import os
import struct
import zlib
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REF = Path(os.environ.get("GVR_REFERENCE_ROOT", "/root/reference"))


def decode_png(data: bytes) -> np.ndarray:
    """Minimal decoder for non-interlaced PNGs: 8-bit RGB/RGBA or palette
    images of 1/2/4/8-bit indices with tRNS transparency (filters 0-4)."""
    assert data[:8] == b"\x89PNG\r\n\x1a\n", "not a PNG"
    pos, idat, hdr, plte, trns = 8, b"", None, None, b""
    while pos < len(data):
        ln, typ = struct.unpack(">I4s", data[pos:pos + 8])
        chunk = data[pos + 8:pos + 8 + ln]
        pos += 12 + ln
        if typ == b"IHDR":
            hdr = struct.unpack(">IIBBBBB", chunk)
        elif typ == b"PLTE":
            plte = np.frombuffer(chunk, dtype=np.uint8).reshape(-1, 3)
        elif typ == b"tRNS":
            trns = chunk
        elif typ == b"IDAT":
            idat += chunk
        elif typ == b"IEND":
            break
    w, h, depth, ctype, _, _, interlace = hdr
    assert interlace == 0 and ctype in (2, 3, 6)
    assert depth == 8 or ctype == 3
    ch = {6: 4, 2: 3, 3: 1}[ctype]
    raw = zlib.decompress(idat)
    stride = (w * ch * depth + 7) // 8
    bpp = max(1, ch * depth // 8)
    out = np.zeros((h, stride), dtype=np.uint8)
    prev = np.zeros(stride, dtype=np.int32)
    for y in range(h):
        f = raw[y * (stride + 1)]
        line = np.frombuffer(raw, dtype=np.uint8, count=stride, offset=y * (stride + 1) + 1).astype(np.int32)
        cur = np.zeros(stride, dtype=np.int32)
        if f == 0:
            cur = line
        elif f == 2:
            cur = (line + prev) & 255
        else:
            for x in range(stride):
                a = cur[x - bpp] if x >= bpp else 0
                b = prev[x]
                c = prev[x - bpp] if x >= bpp else 0
                if f == 1:
                    p = a
                elif f == 3:
                    p = (a + b) // 2
                else:
                    pa, pb, pc = abs(b - c), abs(a - c), abs(a + b - 2 * c)
                    p = a if (pa <= pb and pa <= pc) else (b if pb <= pc else c)
                cur[x] = (line[x] + p) & 255
        out[y] = cur
        prev = cur
    if ctype == 3:
        per = 8 // depth
        idx = np.zeros((h, stride * per), dtype=np.int32)
        for k in range(per):
            idx[:, k::per] = (out >> (8 - depth * (k + 1))) & ((1 << depth) - 1)
        idx = idx[:, :w]
        alpha = np.full(len(plte), 255, np.uint8)
        alpha[:len(trns)] = np.frombuffer(trns, dtype=np.uint8)
        rgba = np.concatenate([plte, alpha[:, None]], axis=1)
        return rgba[idx]
    img = out.reshape(h, w, ch)
    if ch == 3:
        img = np.concatenate([img, np.full((h, w, 1), 255, np.uint8)], axis=2)
    return img


def main() -> None:
    png = REF / "src/tests/_baseline_images/apcomp/apcomp_volume_partial.png"
    img = decode_png(png.read_bytes())
    np.savez_compressed(HERE / "apcomp_volume_partial.npz", rgba=img,
                        source=np.array(str(png.relative_to(REF))))
    print("wrote apcomp_volume_partial.npz", img.shape)


if __name__ == "__main__":
    main()
