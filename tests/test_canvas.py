"""Volume pass of a mixed scene: rendering over an opaque canvas
(gvr_render_volume_over), against the oracle's or_render_over.

The canvas depth is an image-space depth (0.5 z_ndc + 0.5) made here from a
ramp of eye-space distances across the image, so that the opaque "surface"
cuts through the volume on part of the image and lies behind it elsewhere.
"""
import numpy as np
import pytest

from ascent_gb300 import volume as V
from ascent_gb300 import workloads as W
from oracle import oracle as O

from conftest import assert_parity


def canvas_for(wl, cam, params, seed=0):
    """Opaque canvas: colour of an opaque surface, image depth of eye
    distances ramping from 0.8 to 1.2 times the distance to the volume
    centre (left to right)."""
    h, w = params.height, params.width
    b = np.asarray(wl.bounds, dtype=np.float64)
    centre = np.array([(b[0] + b[1]) / 2, (b[2] + b[3]) / 2, (b[4] + b[5]) / 2])
    dist = np.linalg.norm(centre - np.asarray(cam.position, dtype=np.float64))
    n, f = float(cam.near_plane), float(cam.far_plane)
    ze = dist * (0.8 + 0.4 * (np.arange(w) + 0.5) / w)[None, :].repeat(h, axis=0)
    zn = (f + n) / (f - n) - 2 * f * n / ((f - n) * ze)
    depth = (0.5 * zn + 0.5).astype(np.float32)
    rng = np.random.default_rng(seed)
    rgba = np.empty((h, w, 4), np.float32)
    rgba[..., :3] = rng.uniform(0.2, 0.8, 3).astype(np.float32)
    rgba[..., 3] = 1.0
    # a band with nothing drawn (depth 1, transparent)
    rgba[: h // 4] = 0.0
    depth[: h // 4] = 1.0
    return rgba, depth


def oracle_of(wl, precision=64):
    osc = O.OracleScene(precision)
    for d in wl.domains:
        osc.add_uniform(d.dims, d.origin, d.spacing, d.field)
    return osc


@pytest.mark.parametrize("parts", [(1, 1, 1), (2, 1, 2)])
def test_oracle_empty_canvas_equals_plain_render(parts):
    wl = W.plain_small(n=20, width=40, height=32, parts=parts)
    cam = V.workload_camera(wl)
    p = V.workload_params(wl)
    osc = oracle_of(wl)
    a, ad, an = osc.render(cam, p)
    e = np.zeros_like(a)
    b, bd, bn = osc.render_over(cam, p, e, np.full(ad.shape, p.clear_depth, np.float32))
    np.testing.assert_array_equal(a, b)
    np.testing.assert_array_equal(ad, bd)
    assert an == bn


def test_oracle_canvas_in_front_hides_the_volume():
    wl = W.plain_small(n=20, width=40, height=32, parts=(2, 1, 1))
    cam = V.workload_camera(wl)
    p = V.workload_params(wl)
    osc = oracle_of(wl)
    rgba, depth = canvas_for(wl, cam, p)
    depth[:] = 0.02  # just beyond the near plane: in front of everything
    out, od, n = osc.render_over(cam, p, rgba, depth)
    assert n == 0
    np.testing.assert_array_equal(out, rgba)
    np.testing.assert_array_equal(od, depth)


@pytest.mark.gpu
@pytest.mark.parametrize("parts", [(1, 1, 1), (2, 2, 1)])
def test_render_over_matches_oracle(parts):
    from ascent_gb300 import scene as S
    wl = W.plain_small(n=32, width=96, height=80, parts=parts)
    cam = V.workload_camera(wl)
    p = V.workload_params(wl)
    rgba, depth = canvas_for(wl, cam, p, seed=len(parts))
    with S.Scene(0) as sc:
        V.load_workload(sc, wl)
        g, gd, gn = sc.render_over(cam, p, rgba, depth, count_samples=True)
        plain, plain_d = sc.render(cam, p)
    o, od, on = oracle_of(wl).render_over(cam, p, rgba, depth)
    assert_parity(g, o)
    assert np.mean(np.abs(gd - od) <= 2e-4) >= 0.999
    assert abs(gn - on) <= 2e-3 * max(on, 1)
    # the clamp removed samples: the canvas cuts through the volume
    _, _, full = oracle_of(wl).render(cam, p)
    assert on < full
    if p.quantize_uint8 == 0:
        # where the volume leaves no partial, the canvas is untouched
        empty = plain[..., 3] == 0
        np.testing.assert_array_equal(g[empty], rgba[empty])
        np.testing.assert_array_equal(gd[empty], depth[empty])


@pytest.mark.gpu
def test_render_over_empty_canvas_is_the_plain_render_and_device_in_place():
    import torch
    from ascent_gb300 import scene as S
    wl = W.plain_small(n=32, width=64, height=48, parts=(2, 1, 1))
    cam = V.workload_camera(wl)
    p = V.workload_params(wl)
    with S.Scene(0) as sc:
        V.load_workload(sc, wl)
        a, ad = sc.render(cam, p)
        b, bd = sc.render_over(cam, p, np.zeros_like(a), np.full(ad.shape, p.clear_depth, np.float32))
        np.testing.assert_array_equal(a, b)
        np.testing.assert_array_equal(ad, bd)
        rgba, depth = canvas_for(wl, cam, p)
        h, hd = sc.render_over(cam, p, rgba, depth)
        tr = torch.from_numpy(rgba).cuda()
        td = torch.from_numpy(depth).cuda()
        sc.render_over(cam, p, tr, td)
        torch.cuda.synchronize()
        np.testing.assert_array_equal(tr.cpu().numpy(), h)
        np.testing.assert_array_equal(td.cpu().numpy(), hd)


@pytest.mark.gpu
def test_render_over_hex_mesh_matches_oracle():
    from ascent_gb300 import scene as S
    wl = W.hex_mesh(n_cells=16, seed=2, width=80, height=72)
    cam = V.workload_camera(wl)
    p = V.workload_params(wl)
    rgba, depth = canvas_for(wl, cam, p, seed=4)
    h = wl.domains[0]
    with S.Scene(0) as sc:
        sc.add_hex(h.x, h.y, h.z, h.conn, h.field)
        g, gd = sc.render_over(cam, p, rgba, depth)
    osc = O.OracleScene(64)
    osc.add_hex(h.x, h.y, h.z, h.conn, h.field)
    o, od, on = osc.render_over(cam, p, rgba, depth)
    assert_parity(g, o)
    assert np.mean(np.abs(gd - od) <= 2e-4) >= 0.999
    _, _, full = osc.render(cam, p)
    assert on < full
