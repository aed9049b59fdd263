"""PNG output of a rendered canvas, as Ascent writes it.

encode_canvas follows PNGEncoder::Encode(const float*)
(src/libs/png_utils/ascent_png_encoder.cpp:77-118): rows are flipped (the
canvas has y up, PNG rows run top down) and every channel is converted with
a truncating cast of value * 255. The file is an 8-bit RGBA PNG written with
zlib (the encoding itself is host-side post-processing, outside the hot path).
"""
from __future__ import annotations

import struct
import zlib
from pathlib import Path

import numpy as np


def canvas_to_rgba8(rgba: np.ndarray) -> np.ndarray:
    """(H, W, 4) float canvas (row 0 = bottom) -> (H, W, 4) uint8, row 0 = top."""
    x = np.asarray(rgba, dtype=np.float32)[::-1]
    x = np.clip(x * np.float32(255.0), 0.0, 255.0)
    return x.astype(np.uint8)


def _chunk(tag: bytes, data: bytes) -> bytes:
    return struct.pack(">I", len(data)) + tag + data + struct.pack(">I", zlib.crc32(tag + data) & 0xFFFFFFFF)


def encode_rgba8(img: np.ndarray) -> bytes:
    h, w, _ = img.shape
    raw = b"".join(b"\x00" + img[y].tobytes() for y in range(h))
    return (b"\x89PNG\r\n\x1a\n" + _chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, 6, 0, 0, 0)) +
            _chunk(b"IDAT", zlib.compress(raw, 6)) + _chunk(b"IEND", b""))


def save_canvas(path, rgba: np.ndarray) -> Path:
    """Write a float canvas as `path` (".png" appended when missing)."""
    p = Path(path)
    if p.suffix.lower() != ".png":
        p = p.with_name(p.name + ".png")
    p.parent.mkdir(parents=True, exist_ok=True)
    p.write_bytes(encode_rgba8(canvas_to_rgba8(rgba)))
    return p
