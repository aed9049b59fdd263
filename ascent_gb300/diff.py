"""Differentiable volume render of one uniform domain as a torch.autograd.Function.

`VolumeRender.apply(field, lut, cameras, origin, spacing, params)` returns the
RGBA images of all cameras, (V, H, W, 4) float32 on the field's device. The
forward pass (gvr_diff_render_forward) keeps transmittance checkpoints every
64 samples; the backward pass (gvr_diff_render_backward) re-marches each
64-sample segment from its checkpoint and returns dL/dfield (same shape as
the field) and dL/dlut (lut_size x 4). Both run as hand-written CUDA kernels
behind the C ABI; there is no PyTorch fallback.
"""
from __future__ import annotations

import ctypes as C

import torch

from . import _native as N


def _geom(field: torch.Tensor, origin, spacing):
    nz, ny, nx = field.shape
    dims = (C.c_int * 3)(nx, ny, nz)
    o = (C.c_double * 3)(*map(float, origin))
    s = (C.c_double * 3)(*map(float, spacing))
    return dims, o, s


def workspace_per_ray(field_shape, spacing, sample_dist: float) -> int:
    """Floats per ray of the training workspace (transmittance checkpoints
    every 64 samples + the scalar of every sample)."""
    nz, ny, nx = field_shape
    n = C.c_int()
    N.call("gvr_diff_workspace", (C.c_int * 3)(nx, ny, nz), (C.c_double * 3)(*map(float, spacing)),
           float(sample_dist), C.byref(n))
    return n.value


class VolumeRender(torch.autograd.Function):
    """Images of `cameras` rendered from (field, lut); differentiable in both."""

    @staticmethod
    def forward(ctx, field, lut, cameras, origin, spacing, params):
        if not (field.is_cuda and lut.is_cuda):
            raise N.GvrError(N.GVR_ERR_UNSUPPORTED, "field and lut must be CUDA tensors")
        field = field.contiguous().float()
        lut = lut.contiguous().float()
        if lut.dim() != 2 or lut.shape[1] != 4:
            raise N.GvrError(N.GVR_ERR_INVALID_ARGUMENT, "lut must be (n, 4)")
        params.lut_size = lut.shape[0]
        v, h, w = len(cameras), params.height, params.width
        cams = (N.Camera * v)(*cameras)
        dims, o, s = _geom(field, origin, spacing)
        per_ray = workspace_per_ray(field.shape, spacing, params.sample_dist)
        rgba = torch.empty((v, h, w, 4), dtype=torch.float32, device=field.device)
        need_ws = bool(ctx.needs_input_grad[0] or ctx.needs_input_grad[1])
        ckpt = torch.empty((v * h * w * per_ray if need_ws else 1,), dtype=torch.float32,
                           device=field.device)
        stream = C.c_void_p(torch.cuda.current_stream(field.device).cuda_stream)
        N.call("gvr_diff_render_forward", C.c_void_p(field.data_ptr()), dims, o, s, cams, v,
               C.byref(params), C.c_void_p(lut.data_ptr()), C.c_void_p(rgba.data_ptr()),
               C.c_void_p(ckpt.data_ptr()) if need_ws else None, stream)
        ctx.save_for_backward(field, lut, ckpt)
        ctx.cams = cams
        ctx.geom = (origin, spacing)
        ctx.params = params
        return rgba

    @staticmethod
    def backward(ctx, grad_rgba):
        field, lut, ckpt = ctx.saved_tensors
        origin, spacing = ctx.geom
        dims, o, s = _geom(field, origin, spacing)
        g = grad_rgba.contiguous().float()
        gfield = torch.zeros_like(field)
        glut = torch.zeros_like(lut)
        stream = C.c_void_p(torch.cuda.current_stream(field.device).cuda_stream)
        N.call("gvr_diff_render_backward", C.c_void_p(field.data_ptr()), dims, o, s, ctx.cams,
               len(ctx.cams), C.byref(ctx.params), C.c_void_p(lut.data_ptr()),
               C.c_void_p(g.data_ptr()), C.c_void_p(ckpt.data_ptr()), C.c_void_p(gfield.data_ptr()),
               C.c_void_p(glut.data_ptr()), stream)
        return gfield, glut, None, None, None, None


def render(field, lut, cameras, origin, spacing, width, height, sample_dist, scalar_range):
    """Convenience wrapper: build the params and apply VolumeRender."""
    import numpy as np
    p = N.make_params(width, height, sample_dist, scalar_range, np.zeros((2, 4), np.float32),
                      lut_filter=N.LUT_LINEAR, alpha_cull=0.0, early_term=1.0)
    return VolumeRender.apply(field, lut, list(cameras), tuple(origin), tuple(spacing), p)
