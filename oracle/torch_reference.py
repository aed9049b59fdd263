"""Dense PyTorch reference of the differentiable render, for gradient checks.

TEST INFRASTRUCTURE ONLY (like the rest of oracle/): it restates, with
ordinary differentiable torch operations in float64, the render that
gvr_diff_render_forward computes — the pinhole rays the reference's
partials_to_canvas inverts (src/libs/vtkh/rendering/VolumeRenderer.cpp:
303-344), samples t0 + k * dt inside the grid's bounds, trilinear
interpolation of node values, a linearly interpolated transfer function and
the front-to-back emission-absorption blend — so that torch.autograd gives
FP64 gradients to compare the hand-written adjoint with. It pads every ray
to the longest one and is meant for small grids and images.
"""
from __future__ import annotations

import math

import torch


def _rays(cam, width, height, dtype):
    o = torch.tensor(list(cam.position), dtype=dtype)
    look = torch.tensor(list(cam.look_at), dtype=dtype) - o
    look = look / look.norm()
    up = torch.tensor(list(cam.up), dtype=dtype)
    ru = torch.linalg.cross(look, up)
    ru = ru / ru.norm()
    rv = torch.linalg.cross(ru, look)
    rv = rv / rv.norm()
    fov_y = float(cam.fov_y)
    fov_x = fov_y
    if width != height:
        vd = math.tan(0.5 * fov_y * math.pi / 180.0)
        fov_x = 2.0 * math.atan(width / height * vd) * 180.0 / math.pi
    thx = math.tan(fov_x * math.pi / 180.0 * 0.5)
    thy = math.tan(fov_y * math.pi / 180.0 * 0.5)
    dxs, dys = 2 * thx / width, 2 * thy / height
    if cam.zoom > 0:
        dxs /= cam.zoom
        dys /= cam.zoom
    xoff, yoff = cam.xpan * width * 0.5, cam.ypan * height * 0.5
    j, i = torch.meshgrid(torch.arange(height, dtype=dtype), torch.arange(width, dtype=dtype),
                          indexing="ij")
    fx = dxs * (i - width / 2 - xoff)
    fy = dys * (j - height / 2 - yoff)
    d = look + ru * fx[..., None] + rv * fy[..., None]
    d = d / d.norm(dim=-1, keepdim=True)
    return o, d.reshape(-1, 3)


def render(field, lut, cameras, origin, spacing, width, height, sample_dist, scalar_range):
    """field (nz, ny, nx) and lut (n, 4) float64 tensors (may require grad);
    returns (V, H, W, 4)."""
    dtype = field.dtype
    nz, ny, nx = field.shape
    dims = torch.tensor([nx, ny, nz])
    org = torch.tensor([float(x) for x in origin], dtype=dtype)
    sp = torch.tensor([float(x) for x in spacing], dtype=dtype)
    # bounds follow the kernels' float32 geometry
    org32 = org.float().double().to(dtype)
    hi = (org32 + (dims.to(dtype) - 1) * sp.float().double().to(dtype))
    lo = org32
    flat = field.reshape(-1)
    n_lut = lut.shape[0]
    smin, smax = float(scalar_range[0]), float(scalar_range[1])
    inv_range = 1.0 / (smax - smin) if smax > smin else 0.0
    images = []
    for cam in cameras:
        o, d = _rays(cam, width, height, dtype)
        inv = 1.0 / torch.where(d == 0, torch.full_like(d, 1e-300), d)
        ta = (lo - o) * inv
        tb = (hi - o) * inv
        t0 = torch.clamp(torch.minimum(ta, tb).amax(dim=1), min=0.0)
        t1 = torch.maximum(ta, tb).amin(dim=1)
        hit = t1 > t0
        nmax = int(torch.ceil(((t1 - t0).clamp(min=0) / sample_dist).max()).item()) + 1 if hit.any() else 1
        k = torch.arange(nmax, dtype=dtype)
        t = t0[:, None] + k[None, :] * float(sample_dist)
        valid = (t < t1[:, None]) & hit[:, None]
        pos = o + t[..., None] * d[:, None, :]
        g = (pos - org) / sp
        c = torch.floor(g).clamp(min=0)
        c = torch.minimum(c, (dims - 2).to(dtype))
        w = g - c
        ci = c.long()
        base = (ci[..., 2] * ny + ci[..., 1]) * nx + ci[..., 0]
        base = torch.where(valid, base, torch.zeros_like(base))
        sy, sz = nx, nx * ny
        def at(off):
            return flat[base + off]
        wx, wy, wz = w[..., 0], w[..., 1], w[..., 2]
        c00 = at(0) + wx * (at(1) - at(0))
        c10 = at(sy) + wx * (at(sy + 1) - at(sy))
        c01 = at(sz) + wx * (at(sz + 1) - at(sz))
        c11 = at(sz + sy) + wx * (at(sz + sy + 1) - at(sz + sy))
        c0 = c00 + wy * (c10 - c00)
        c1 = c01 + wy * (c11 - c01)
        v = c0 + wz * (c1 - c0)
        s = ((v - smin) * inv_range).clamp(0.0, 1.0)
        x = s * (n_lut - 1)
        i0 = torch.floor(x).clamp(max=n_lut - 2).long()
        wl = (x - i0.to(dtype))[..., None]
        col = lut[i0] + wl * (lut[i0 + 1] - lut[i0])
        a = torch.where(valid, col[..., 3], torch.zeros_like(col[..., 3]))
        rgb = col[..., :3]
        one_m = 1.0 - a
        T = torch.cumprod(torch.cat([torch.ones_like(one_m[:, :1]), one_m[:, :-1]], dim=1), dim=1)
        wgt = T * a
        out_rgb = (wgt[..., None] * rgb).sum(dim=1)
        out_a = 1.0 - torch.prod(one_m, dim=1)
        img = torch.cat([out_rgb, out_a[:, None]], dim=1).reshape(height, width, 4)
        images.append(img)
    return torch.stack(images)
