"""Partial compositing on the device.

`PartialCompositor` mirrors vtkh's PartialCompositor<VolumePartial<float>>
(vtkh/compositing/PartialCompositor.hpp, PartialCompositor.cpp:494-547):
`composite(partial_images)` takes a list of per-image partial arrays and
returns one record per pixel, blended front to back in depth order, in the
reference's output order (single-record pixels first, then blended pixels,
each in pixel order). The work runs in gvr_composite_partials: records are
grouped by pixel with a histogram of pixel ids and a bucket scatter (a
device radix sort when the ids are sparse), each pixel's records are ordered
by (depth, input position) and blended in FP32 by one thread per pixel.

Host partials are numpy structured arrays of `PARTIAL_DTYPE` (the 24-byte
VolumePartial<float> record). Device partials are torch int32 tensors of
shape (n, 6) holding the same records: column 0 the pixel id, columns 1-5
the bits of depth, r, g, b, alpha (`to_device` / `from_device` convert).
"""
from __future__ import annotations

import ctypes as C
from typing import Sequence

import numpy as np

from . import _native as N

PARTIAL_DTYPE = np.dtype([("pixel_id", "<i4"), ("depth", "<f4"), ("rgb", "<f4", (3,)),
                          ("alpha", "<f4")])
assert PARTIAL_DTYPE.itemsize == 24


def _stream_ptr(stream) -> int:
    if stream is None:
        import torch
        return torch.cuda.current_stream().cuda_stream
    return int(getattr(stream, "cuda_stream", stream))


def composite_partials(partials: np.ndarray) -> np.ndarray:
    """Composite one concatenated host array of partials (the body of
    PartialCompositor::composite after merge)."""
    parts = np.ascontiguousarray(partials, dtype=PARTIAL_DTYPE)
    out = np.empty(len(parts), dtype=PARTIAL_DTYPE)
    n_out = C.c_int64(0)
    N.call("gvr_composite_partials", parts.ctypes.data if len(parts) else None, len(parts),
           out.ctypes.data if len(out) else None, C.byref(n_out), N.MEM_HOST, None)
    return out[:n_out.value]


def composite_partials_device(partials, stream=None):
    """Composite partials held on the device as an (n, 6) int32 torch tensor;
    returns a new (n_out, 6) int32 tensor on the same device."""
    import torch
    if partials.dtype != torch.int32 or partials.dim() != 2 or partials.shape[1] != 6:
        raise N.GvrError(N.GVR_ERR_INVALID_ARGUMENT, "device partials must be an (n, 6) int32 tensor")
    if not partials.is_cuda:
        raise N.GvrError(N.GVR_ERR_INVALID_ARGUMENT, "device partials must be a CUDA tensor")
    parts = partials.contiguous()
    out = torch.empty_like(parts)
    n_out = C.c_int64(0)
    n = parts.shape[0]
    N.call("gvr_composite_partials", parts.data_ptr() if n else None, n,
           out.data_ptr() if n else None, C.byref(n_out), N.MEM_DEVICE, C.c_void_p(_stream_ptr(stream)))
    return out[:n_out.value]


def composite_partials_device_async(partials, pixel_lo: int, pixel_hi: int, out=None, n_out=None,
                                    stream=None):
    """Composite device partials whose pixel ids lie in [pixel_lo, pixel_hi]
    with no host synchronisation (gvr_composite_partials_async). Returns
    (out, n_out): an (n, 6) int32 tensor of which the first n_out rows are
    the result, and n_out as a one-element int64 CUDA tensor (-1 if a record
    was outside the range). Reading n_out waits for the work."""
    import torch
    if partials.dtype != torch.int32 or partials.dim() != 2 or partials.shape[1] != 6 or not partials.is_cuda:
        raise N.GvrError(N.GVR_ERR_INVALID_ARGUMENT, "device partials must be an (n, 6) int32 CUDA tensor")
    parts = partials.contiguous()
    if out is None:
        out = torch.empty_like(parts)
    if n_out is None:
        n_out = torch.zeros(1, dtype=torch.int64, device=parts.device)
    n = parts.shape[0]
    N.call("gvr_composite_partials_async", parts.data_ptr() if n else None, n, int(pixel_lo), int(pixel_hi),
           out.data_ptr() if n else None, n_out.data_ptr(), C.c_void_p(_stream_ptr(stream)))
    return out, n_out


def to_device(partials: np.ndarray, device="cuda"):
    import torch
    raw = np.ascontiguousarray(partials, dtype=PARTIAL_DTYPE).view(np.int32).reshape(-1, 6)
    return torch.from_numpy(raw.copy()).to(device)


def from_device(t) -> np.ndarray:
    raw = np.ascontiguousarray(t.cpu().numpy(), dtype=np.int32)
    return raw.reshape(-1).view(PARTIAL_DTYPE).copy()


class PartialCompositor:
    """The reference's PartialCompositor for VolumePartial<float>.

    composite(partial_images) concatenates the images (merge,
    PartialCompositor.cpp:244-325) and composites them
    (composite_partials :331-490). The exchange between MPI ranks that
    vtkh adds under VTKH_PARALLEL (redistribute :521-529, collect :540-546)
    is not part of this single-GPU compositor.
    """

    def composite(self, partial_images: Sequence[np.ndarray]) -> np.ndarray:
        images = [np.asarray(p, dtype=PARTIAL_DTYPE) for p in partial_images]
        merged = np.concatenate(images) if images else np.zeros(0, PARTIAL_DTYPE)
        return composite_partials(merged)


def zbuffer_composite(rgba_images, depth_images, stream=None):
    """Z-buffer compositing of opaque canvases (gvr_zbuffer_composite):
    Renderer::Composite in Z_BUFFER_SURFACE mode (vtkh/rendering/
    Renderer.cpp:111-142, ImageCompositor.hpp:49-76). Inputs are lists of
    (H, W, 4) / (H, W) float32 arrays, all numpy (host) or all CUDA tensors
    (device, stream-ordered on `stream` or the current stream); returns the
    composited (rgba, depth) on the same side. The result is the opaque
    canvas a volume pass draws over (Scene.render_over)."""
    n = len(rgba_images)
    if n == 0 or n != len(depth_images):
        raise N.GvrError(N.GVR_ERR_INVALID_ARGUMENT, "need as many depth images as colour images (>= 1)")
    on_device = not isinstance(rgba_images[0], np.ndarray)
    if on_device:
        import torch
        cols = [c.contiguous() for c in rgba_images]
        deps = [d.contiguous() for d in depth_images]
        if any(c.dtype != torch.float32 or not c.is_cuda for c in cols + deps):
            raise N.GvrError(N.GVR_ERR_INVALID_ARGUMENT, "device images must be float32 CUDA tensors")
        h, w = cols[0].shape[0], cols[0].shape[1]
        if any(tuple(c.shape) != (h, w, 4) for c in cols) or any(tuple(d.shape) != (h, w) for d in deps):
            raise N.GvrError(N.GVR_ERR_INVALID_ARGUMENT, "images must share one (H, W) size")
        out = torch.empty_like(cols[0])
        out_d = torch.empty_like(deps[0])
        cp = (C.c_void_p * n)(*[c.data_ptr() for c in cols])
        dp = (C.c_void_p * n)(*[d.data_ptr() for d in deps])
        N.call("gvr_zbuffer_composite", n, cp, dp, w, h, C.c_void_p(out.data_ptr()),
               C.c_void_p(out_d.data_ptr()), N.MEM_DEVICE, C.c_void_p(_stream_ptr(stream)))
        return out, out_d
    cols = [np.ascontiguousarray(c, dtype=np.float32) for c in rgba_images]
    deps = [np.ascontiguousarray(d, dtype=np.float32) for d in depth_images]
    h, w = cols[0].shape[0], cols[0].shape[1]
    if any(c.shape != (h, w, 4) for c in cols) or any(d.shape != (h, w) for d in deps):
        raise N.GvrError(N.GVR_ERR_INVALID_ARGUMENT, "images must share one (H, W) size")
    out = np.zeros((h, w, 4), np.float32)
    out_d = np.zeros((h, w), np.float32)
    cp = (C.c_void_p * n)(*[c.ctypes.data for c in cols])
    dp = (C.c_void_p * n)(*[d.ctypes.data for d in deps])
    N.call("gvr_zbuffer_composite", n, cp, dp, w, h, C.c_void_p(out.ctypes.data),
           C.c_void_p(out_d.ctypes.data), N.MEM_HOST, None)
    return out, out_d
