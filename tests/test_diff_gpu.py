"""Adjoint of the march + composite (gvr_diff_render_backward) against FP64
autograd through the dense PyTorch reference, and against central finite
differences of the CUDA forward itself."""
import numpy as np
import pytest
import torch

from ascent_gb300 import diff as D
from ascent_gb300 import scene as S
from ascent_gb300 import workloads as W
from oracle import torch_reference as TR

pytestmark = pytest.mark.gpu


def problem(n=32, size=(40, 32), views=3, lut_n=256, seed=0):
    wl = W.plain_small(n=n, width=size[0], height=size[1], seed=seed)
    d = wl.domains[0]
    pt = np.array([[30 + 70 * i, 40 + 30 * i] for i in range(views)], np.float32)
    cams = S.cinema_cameras(wl.bounds, pt)
    x = np.linspace(0, 1, lut_n)
    lut = np.stack([x, 0.5 + 0.3 * np.sin(6 * x), 1 - x, 0.25 * x ** 1.5], 1).astype(np.float32)
    sd = S.sample_distance(wl.bounds, int(np.ceil(np.sqrt(3) * (n - 1) / 0.5)))
    return wl, d, cams, lut, sd


def test_forward_matches_fp64_reference():
    wl, d, cams, lut, sd = problem()
    f = torch.from_numpy(d.field).cuda()
    img = D.render(f, torch.from_numpy(lut).cuda(), cams, d.origin, d.spacing, 40, 32, sd, wl.scalar_range)
    ref = TR.render(torch.from_numpy(d.field).double(), torch.from_numpy(lut).double(), cams, d.origin,
                    d.spacing, 40, 32, sd, wl.scalar_range)
    np.testing.assert_allclose(img.cpu().numpy(), ref.numpy(), atol=2e-4)
    assert ref[..., 3].max() > 0.2


def test_gradients_match_fp64_autograd():
    wl, d, cams, lut, sd = problem()
    rng = np.random.default_rng(5)
    target = torch.from_numpy(rng.uniform(0, 0.5, (3, 32, 40, 4)).astype(np.float32))
    f = torch.from_numpy(d.field).cuda().requires_grad_(True)
    lt = torch.from_numpy(lut).cuda().requires_grad_(True)
    img = D.render(f, lt, cams, d.origin, d.spacing, 40, 32, sd, wl.scalar_range)
    loss = ((img - target.cuda()) ** 2).sum()
    loss.backward()
    fr = torch.from_numpy(d.field).double().requires_grad_(True)
    lr = torch.from_numpy(lut).double().requires_grad_(True)
    ref = TR.render(fr, lr, cams, d.origin, d.spacing, 40, 32, sd, wl.scalar_range)
    ((ref - target.double()) ** 2).sum().backward()
    gf, gl = f.grad.cpu().double(), lt.grad.cpu().double()
    ef = (gf - fr.grad).norm() / fr.grad.norm()
    el = (gl - lr.grad).norm() / lr.grad.norm()
    assert fr.grad.norm() > 0 and lr.grad.norm() > 0
    assert ef < 2e-3 and el < 2e-3, (float(ef), float(el))


def test_directional_finite_differences_of_the_cuda_forward():
    wl, d, cams, lut, sd = problem(n=24, size=(32, 24), views=2, lut_n=64, seed=3)
    rng = np.random.default_rng(7)
    target = torch.from_numpy(rng.uniform(0, 0.5, (2, 24, 32, 4)).astype(np.float32)).cuda()
    f0 = torch.from_numpy(d.field).cuda()
    l0 = torch.from_numpy(lut).cuda()

    def loss(f, lt):
        img = D.render(f, lt, cams, d.origin, d.spacing, 32, 24, sd, wl.scalar_range)
        return ((img.double() - target.double()) ** 2).sum()

    f = f0.clone().requires_grad_(True)
    lt = l0.clone().requires_grad_(True)
    loss(f, lt).backward()
    uf = torch.from_numpy(rng.normal(size=d.field.shape).astype(np.float32)).cuda()
    ul = torch.from_numpy(rng.normal(size=lut.shape).astype(np.float32)).cuda()
    # The loss is piecewise smooth (linear LUT interpolation and trilinear
    # cells have kinks), so central differences along a direction that moves
    # every node carry an O(h) kink error: 5% here; the exact check is the
    # comparison with FP64 autograd above.
    h = 1e-3
    fd_f = (loss(f0 + h * uf, l0) - loss(f0 - h * uf, l0)) / (2 * h)
    fd_l = (loss(f0, l0 + h * ul) - loss(f0, l0 - h * ul)) / (2 * h)
    an_f = (f.grad.double() * uf.double()).sum()
    an_l = (lt.grad.double() * ul.double()).sum()
    assert abs(float(fd_f - an_f)) <= 5e-2 * abs(float(an_f)), (float(fd_f), float(an_f))
    assert abs(float(fd_l - an_l)) <= 5e-2 * abs(float(an_l)), (float(fd_l), float(an_l))
    # single nodes with the largest gradients
    flat = f.grad.reshape(-1)
    for idx in torch.topk(flat.abs(), 4).indices.tolist():
        e = torch.zeros_like(f0).reshape(-1)
        e[idx] = 1.0
        e = e.reshape(f0.shape)
        hh = 1e-2
        fd = (loss(f0 + hh * e, l0) - loss(f0 - hh * e, l0)) / (2 * hh)
        an = float(flat[idx])
        assert abs(float(fd) - an) <= 5e-2 * abs(an), (idx, float(fd), an)


def test_gradient_descent_step_reduces_loss():
    wl, d, cams, lut, sd = problem(n=24, size=(32, 32), views=2, lut_n=64)
    gt = torch.from_numpy(d.field).cuda()
    lt = torch.from_numpy(lut).cuda()
    with torch.no_grad():
        target = D.render(gt, lt, cams, d.origin, d.spacing, 32, 32, sd, wl.scalar_range)
    noise = torch.randn(gt.shape, generator=torch.Generator("cuda").manual_seed(1), device="cuda")
    f = (gt + 0.05 * noise).requires_grad_(True)
    opt = torch.optim.Adam([f], lr=0.01)
    losses = []
    for _ in range(5):
        opt.zero_grad()
        img = D.render(f, lt, cams, d.origin, d.spacing, 32, 32, sd, wl.scalar_range)
        loss = ((img - target) ** 2).sum()
        loss.backward()
        opt.step()
        losses.append(float(loss.detach()))
    assert losses[-1] < losses[0]
