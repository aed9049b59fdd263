"""Z-buffer compositing of opaque canvases (Renderer::Composite in
Z_BUFFER_SURFACE mode, vtkh/rendering/Renderer.cpp:111-142 with
ImageCompositor::ZBufferComposite, ImageCompositor.hpp:49-76) and the mixed
scene it feeds: opaque surface renders composited by depth, then the volume
drawn over the result (Scene.cpp:154-212).

CPU: the oracle's C restatement against an independent numpy statement of
the same rules, and the C ABI's argument checks. GPU: the device compositor
bit for bit against the oracle (host and device buffers), and two opaque
canvases plus a volume against the oracle's pipeline.
"""
import ctypes as C

import numpy as np
import pytest

from ascent_gb300 import _native as N
from ascent_gb300 import volume as V
from ascent_gb300 import workloads as W
from oracle import oracle as O

from conftest import assert_parity
from test_canvas import canvas_for


def numpy_zbuffer(cols, deps):
    """Image::Init -> ZBufferComposite over images 1.. -> ImageToCanvas."""
    def u8(c):
        return np.clip(c.astype(np.float32) * np.float32(255.0), 0, 255).astype(np.uint8)
    px = u8(cols[0])
    d = np.abs(deps[0]).astype(np.float32)
    for c, dk in zip(cols[1:], deps[1:]):
        dk = np.abs(dk).astype(np.float32)
        take = ~((dk > 1.0) | (d < dk))
        d = np.where(take, dk, d)
        px = np.where(take[..., None], u8(c), px)
    return px.astype(np.float32) * np.float32(1.0 / 255.0), d


def random_canvases(n, h, w, seed):
    rng = np.random.default_rng(seed)
    cols, deps = [], []
    for _ in range(n):
        c = rng.uniform(0, 1, (h, w, 4)).astype(np.float32)
        d = rng.choice(np.array([0.25, 0.5, 0.75, 1.0, 1.5, -0.5], np.float32), (h, w))
        d = np.where(rng.uniform(size=(h, w)) < 0.5, d, rng.uniform(0, 1.2, (h, w))).astype(np.float32)
        cols.append(c)
        deps.append(d)
    return cols, deps


@pytest.mark.parametrize("n", [1, 2, 5])
def test_oracle_zbuffer_rules(n):
    cols, deps = random_canvases(n, 17, 23, seed=n)
    o, od = O.zbuffer_composite(cols, deps)
    e, ed = numpy_zbuffer(cols, deps)
    np.testing.assert_array_equal(o, e)
    np.testing.assert_array_equal(od, ed)


def test_zbuffer_argument_checks():
    cols, deps = random_canvases(1, 4, 4, 0)
    cp = (C.c_void_p * 1)(cols[0].ctypes.data)
    dp = (C.c_void_p * 1)(deps[0].ctypes.data)
    out = np.zeros((4, 4, 4), np.float32)
    od = np.zeros((4, 4), np.float32)
    f = N.lib().gvr_zbuffer_composite
    args = (cp, dp, 4, 4, C.c_void_p(out.ctypes.data), C.c_void_p(od.ctypes.data), N.MEM_HOST, None)
    assert f(0, *args) == N.GVR_ERR_INVALID_ARGUMENT
    assert f(65, *args) == N.GVR_ERR_INVALID_ARGUMENT
    assert f(1, cp, dp, 0, 4, *args[4:]) == N.GVR_ERR_INVALID_ARGUMENT
    assert f(1, cp, dp, 4, 4, None, C.c_void_p(od.ctypes.data), N.MEM_HOST, None) == N.GVR_ERR_INVALID_ARGUMENT
    assert f(1, *args[:-2], 7, None) == N.GVR_ERR_INVALID_ARGUMENT


@pytest.mark.gpu
@pytest.mark.parametrize("n", [1, 3, 8])
def test_device_zbuffer_bit_exact(n):
    import torch
    from ascent_gb300 import compositing as CP
    cols, deps = random_canvases(n, 61, 97, seed=10 + n)
    o, od = O.zbuffer_composite(cols, deps)
    h, hd = CP.zbuffer_composite(cols, deps)
    np.testing.assert_array_equal(h, o)
    np.testing.assert_array_equal(hd, od)
    g, gd = CP.zbuffer_composite([torch.from_numpy(c).cuda() for c in cols],
                                 [torch.from_numpy(d).cuda() for d in deps])
    torch.cuda.synchronize()
    np.testing.assert_array_equal(g.cpu().numpy(), o)
    np.testing.assert_array_equal(gd.cpu().numpy(), od)


@pytest.mark.gpu
def test_two_surfaces_then_volume_matches_oracle():
    """Two opaque surface canvases (one slanted through the volume, one
    nearer on part of the image) composited by depth, then the volume drawn
    over the result, against the oracle doing the same two steps."""
    from ascent_gb300 import compositing as CP
    from ascent_gb300 import scene as S
    wl = W.plain_small(n=40, width=96, height=72, parts=(2, 1, 1))
    cam = V.workload_camera(wl)
    p = V.workload_params(wl)
    a, ad = canvas_for(wl, cam, p, seed=1)
    b, bd = canvas_for(wl, cam, p, seed=2)
    b = b[:, ::-1].copy()          # ramp the other way
    bd = bd[:, ::-1].copy()
    bd[:, : p.width // 3] = 1.0    # nothing drawn on the left third
    b[:, : p.width // 3] = 0.0
    zc, zd = CP.zbuffer_composite([a, b], [ad, bd])
    oc, od = O.zbuffer_composite([a, b], [ad, bd])
    np.testing.assert_array_equal(zc, oc)
    np.testing.assert_array_equal(zd, od)
    with S.Scene(0) as sc:
        V.load_workload(sc, wl)
        g, gd = sc.render_over(cam, p, zc, zd)
    osc = O.OracleScene(64)
    for d in wl.domains:
        osc.add_uniform(d.dims, d.origin, d.spacing, d.field)
    o, o_d, _ = osc.render_over(O.workload_camera(wl), O.workload_params(wl), oc, od)
    assert_parity(g, o)
    assert np.mean(np.abs(gd - o_d) <= 2e-4) >= 0.999
    # both surfaces show somewhere, and the volume changed the image
    assert (zd < 1.0).mean() > 0.3 and np.abs(g - zc).max() > 0.05
