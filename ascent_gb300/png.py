"""PNG output of a rendered canvas, as Ascent writes it.

The pixel conversion follows PNGEncoder::Encode(const float*)
(src/libs/png_utils/ascent_png_encoder.cpp:77-118): rows are flipped (the
canvas has y up, PNG rows run top down) and every channel is converted with
a truncating cast of value * 255. A canvas that lives on the GPU is
converted there (gvr_canvas_to_rgba8), so only its 4 bytes per pixel come
back to the host; a host canvas is converted with numpy. The file is an
8-bit RGBA PNG written with zlib (the deflate is host-side).

decode_png reads PNGs back to RGBA8 (the role of PNGDecoder::Decode,
src/libs/png_utils/ascent_png_decoder.cpp), for comparing written images and
for reading colour-bar images.
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


# default colour bar positions of the reference's Annotator (Annotator.cpp:15-24):
# {xmin, xmax, ymin, ymax} in screen coordinates, one per plot with a table
DEFAULT_COLOR_BAR_BOXES = ((0.84, 0.92, 0.1, 0.8), (0.84, 0.92, -0.8, -0.1),
                           (-0.8, -0.72, 0.1, 0.8), (-0.8, -0.72, -0.8, -0.1))


def draw_color_bar(canvas, lut, box=DEFAULT_COLOR_BAR_BOXES[0], fg=(1.0, 1.0, 1.0, 1.0)):
    """Draw a colour bar's body into a float canvas in place
    (gvr_canvas_color_bar): a (H, W, 4) float32 numpy array or CUDA tensor,
    the colour table as (n, 4) RGBA rows, box = (xmin, xmax, ymin, ymax) in
    screen coordinates. Labels and ticks are not drawn."""
    import ctypes as C

    from . import _native as N
    lut = np.ascontiguousarray(lut, dtype=np.float32).reshape(-1, 4)
    b = (C.c_float * 4)(*[float(x) for x in box])
    f = (C.c_float * 4)(*[float(x) for x in fg])
    if isinstance(canvas, np.ndarray):
        if canvas.dtype != np.float32 or canvas.ndim != 3 or canvas.shape[2] != 4 or not canvas.flags.c_contiguous:
            raise ValueError("canvas must be a C-contiguous (H, W, 4) float32 array")
        h, w, _ = canvas.shape
        N.call("gvr_canvas_color_bar", C.c_void_p(canvas.ctypes.data), w, h, N.fptr(lut), lut.shape[0], b, f,
               N.MEM_HOST, None)
        return canvas
    import torch
    if canvas.dtype != torch.float32 or not canvas.is_cuda or canvas.dim() != 3 or canvas.shape[2] != 4 \
            or not canvas.is_contiguous():
        raise ValueError("canvas must be a contiguous (H, W, 4) float32 CUDA tensor")
    h, w, _ = canvas.shape
    stream = torch.cuda.current_stream(canvas.device).cuda_stream
    N.call("gvr_canvas_color_bar", C.c_void_p(canvas.data_ptr()), w, h, N.fptr(lut), lut.shape[0], b, f,
           N.MEM_DEVICE, C.c_void_p(stream))
    return canvas


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


def decode_png(data: bytes) -> np.ndarray:
    """(H, W, 4) uint8 RGBA of a non-interlaced PNG, top row first: 8-bit
    grey, RGB or RGBA, or palette images of 1/2/4/8-bit indices with tRNS
    transparency (row filters 0-4)."""
    if data[:8] != b"\x89PNG\r\n\x1a\n":
        raise ValueError("not a PNG")
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
    if hdr is None:
        raise ValueError("PNG without IHDR")
    w, h, depth, ctype, _, _, interlace = hdr
    if interlace != 0 or ctype not in (0, 2, 3, 6) or (depth != 8 and ctype != 3):
        raise ValueError(f"unsupported PNG: colour type {ctype}, depth {depth}, interlace {interlace}")
    ch = {0: 1, 6: 4, 2: 3, 3: 1}[ctype]
    raw = zlib.decompress(idat)
    stride = (w * ch * depth + 7) // 8
    bpp = max(1, ch * depth // 8)
    out = np.zeros((h, stride), dtype=np.uint8)
    prev = np.zeros(stride, dtype=np.int32)
    for y in range(h):
        f = raw[y * (stride + 1)]
        line = np.frombuffer(raw, dtype=np.uint8, count=stride, offset=y * (stride + 1) + 1).astype(np.int32)
        if f == 0:
            cur = line
        elif f == 2:
            cur = (line + prev) & 255
        else:
            cur = np.zeros(stride, dtype=np.int32)
            for x in range(stride):
                a = cur[x - bpp] if x >= bpp else 0
                b = prev[x]
                c = prev[x - bpp] if x >= bpp else 0
                if f == 1:
                    pr = a
                elif f == 3:
                    pr = (a + b) // 2
                else:  # Paeth
                    pa, pb, pc = abs(b - c), abs(a - c), abs(a + b - 2 * c)
                    pr = a if (pa <= pb and pa <= pc) else (b if pb <= pc else c)
                cur[x] = (line[x] + pr) & 255
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
    if ch == 1:
        img = np.repeat(img, 3, axis=2)
    if img.shape[2] == 3:
        img = np.concatenate([img, np.full((h, w, 1), 255, np.uint8)], axis=2)
    return img
