"""PNG output of a rendered canvas, as Ascent writes it.

The pixel conversion follows PNGEncoder::Encode(const float*)
(src/libs/png_utils/ascent_png_encoder.cpp:77-118): rows are flipped (the
canvas has y up, PNG rows run top down) and every channel is converted with
a truncating cast of value * 255. A canvas that lives on the GPU is
converted there (gvr_canvas_to_rgba8), so only its 4 bytes per pixel come
back to the host; a host canvas is converted with numpy. The file is an
8-bit RGBA PNG written with zlib (the deflate is host-side).
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


def canvas_to_rgba8_device(rgba):
    """canvas_to_rgba8 on the GPU: a (H, W, 4) float32 CUDA tensor -> a
    (H, W, 4) uint8 CUDA tensor, row 0 = top, stream-ordered on the tensor's
    current stream (gvr_canvas_to_rgba8)."""
    import ctypes as C

    import torch

    from . import _native as N
    if rgba.dtype != torch.float32 or not rgba.is_cuda or rgba.dim() != 3 or rgba.shape[2] != 4:
        raise ValueError("canvas must be a (H, W, 4) float32 CUDA tensor")
    src = rgba.contiguous()
    h, w, _ = src.shape
    out = torch.empty((h, w, 4), dtype=torch.uint8, device=src.device)
    stream = torch.cuda.current_stream(src.device).cuda_stream
    N.call("gvr_canvas_to_rgba8", C.c_void_p(src.data_ptr()), int(w), int(h),
           C.c_void_p(out.data_ptr()), N.MEM_DEVICE, C.c_void_p(stream))
    return out


def _chunk(tag: bytes, data: bytes) -> bytes:
    return struct.pack(">I", len(data)) + tag + data + struct.pack(">I", zlib.crc32(tag + data) & 0xFFFFFFFF)


def encode_rgba8(img: np.ndarray) -> bytes:
    h, w, _ = img.shape
    raw = b"".join(b"\x00" + img[y].tobytes() for y in range(h))
    return (b"\x89PNG\r\n\x1a\n" + _chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, 6, 0, 0, 0)) +
            _chunk(b"IDAT", zlib.compress(raw, 6)) + _chunk(b"IEND", b""))


def save_canvas(path, rgba) -> Path:
    """Write a float canvas — a numpy array, or a CUDA tensor converted on
    the device — as `path` (".png" appended when missing)."""
    p = Path(path)
    if p.suffix.lower() != ".png":
        p = p.with_name(p.name + ".png")
    p.parent.mkdir(parents=True, exist_ok=True)
    if isinstance(rgba, np.ndarray):
        img = canvas_to_rgba8(rgba)
    else:
        img = canvas_to_rgba8_device(rgba).cpu().numpy()
    p.write_bytes(encode_rgba8(img))
    return p
