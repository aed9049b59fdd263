"""The dense FP64 PyTorch reference used to check the adjoint kernel agrees
with the C oracle's forward, and its autograd passes finite differences."""
import numpy as np
import torch

from ascent_gb300 import _native as N
from ascent_gb300 import scene as S
from ascent_gb300 import workloads as W
from oracle import oracle as O
from oracle import torch_reference as TR


def smooth_lut(n, seed=0):
    rng = np.random.default_rng(seed)
    return np.clip(np.cumsum(rng.uniform(0, 0.2, (n, 4)), 0) / 3, 0, 1).astype(np.float32)


def test_torch_reference_matches_oracle_forward():
    wl = W.plain_small(n=20, width=24, height=20)
    d = wl.domains[0]
    cams = S.cinema_cameras(wl.bounds, np.array([[30, 60], [-100, 120]], np.float32))
    lut = smooth_lut(16)
    sd = S.sample_distance(wl.bounds, 40)
    p = N.make_params(24, 20, sd, wl.scalar_range, lut, lut_filter=N.LUT_LINEAR, alpha_cull=0.0,
                      early_term=1.0)
    osc = O.OracleScene(64)
    osc.add_uniform(d.dims, d.origin, d.spacing, d.field)
    ref = TR.render(torch.from_numpy(d.field).double(), torch.from_numpy(lut).double(), cams,
                    d.origin, d.spacing, 24, 20, sd, wl.scalar_range)
    for v, cam in enumerate(cams):
        o, _, _ = osc.render(cam, p)
        np.testing.assert_allclose(ref[v].numpy(), o, atol=1e-6)


def test_torch_reference_gradcheck():
    wl = W.plain_small(n=6, width=6, height=5)
    d = wl.domains[0]
    cams = S.cinema_cameras(wl.bounds, np.array([[20, 70]], np.float32))
    sd = S.sample_distance(wl.bounds, 12)
    field = torch.from_numpy(d.field).double().requires_grad_(True)
    lut = torch.from_numpy(smooth_lut(6, 1)).double().requires_grad_(True)

    def f(fld, lt):
        return TR.render(fld, lt, cams, d.origin, d.spacing, 6, 5, sd, wl.scalar_range)

    assert torch.autograd.gradcheck(f, (field, lut), eps=1e-6, atol=1e-5, rtol=1e-3)
