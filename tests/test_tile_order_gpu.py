"""Longest-first tile launch order (gvr_scene_set_tile_order(scene, 1)).

Before each render one kernel estimates every 16 x 16 tile's cost for the
view and writes a permutation of the tiles, longest first; the march then
takes its tiles in that order. The order changes no pixel: images, depths
and sample counts must equal the centre-first order exactly, every tile
must be written once (outputs are pre-filled with NaN on the device), on
centred, panned and inside-the-volume views, odd image sizes, the staged
march, a scene whose boxes lie off the image, and grids too large for the
order kernel (which keep the centre-first table).
"""
import ctypes as C

import numpy as np
import pytest

from ascent_gb300 import _native as N
from ascent_gb300 import scene as S
from ascent_gb300 import volume as V
from ascent_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def render_nan_filled(sc, cam, p):
    import torch
    rgba = torch.full((p.height, p.width, 4), float("nan"), dtype=torch.float32, device="cuda:0")
    depth = torch.full((p.height, p.width), float("nan"), dtype=torch.float32, device="cuda:0")
    n = C.c_uint64(0)
    st = C.c_void_p(torch.cuda.current_stream(0).cuda_stream)
    N.call("gvr_render_volume", sc.handle, C.byref(cam), C.byref(p), C.c_void_p(rgba.data_ptr()),
           C.c_void_p(depth.data_ptr()), N.MEM_DEVICE, st, C.byref(n))
    return rgba.cpu().numpy(), depth.cpu().numpy(), int(n.value)


def both_orders(sc, cam, p, staged=0):
    out = []
    for order in (0, 1):
        sc.set_tuning(packet_w=8, unroll=2, min_blocks=4, staged=staged, tile_order=order)
        out.append(render_nan_filled(sc, cam, p))
    a, b = out
    assert not np.isnan(a[0]).any() and not np.isnan(a[1]).any()
    np.testing.assert_array_equal(a[0], b[0])
    np.testing.assert_array_equal(a[1], b[1])
    assert a[2] == b[2]
    return a


@pytest.mark.parametrize("parts,size", [(None, (96, 80)), ((2, 2, 2), (128, 96)),
                                        ((3, 1, 2), (77, 131)), ((1, 2, 1), (1, 1)),
                                        ((2, 1, 1), (17, 300))])
def test_longest_first_equals_centre_first(parts, size):
    wl = W.plain_small(n=49, width=size[0], height=size[1], parts=parts)
    cam = V.workload_camera(wl)
    p = V.workload_params(wl)
    with S.Scene(0) as sc:
        V.load_workload(sc, wl)
        a = both_orders(sc, cam, p)
    if size[0] > 1:
        assert a[0][..., 3].max() > 0.05


def test_panned_inside_and_off_image_views():
    wl = W.plain_small(n=64, width=150, height=110, parts=(2, 2, 1))
    p = V.workload_params(wl)
    panned = V.workload_camera(wl)
    panned.xpan, panned.ypan, panned.zoom = 0.6, -0.3, 1.7
    inside = S.camera_reset_to_bounds(wl.bounds)
    c = 0.5 * (wl.bounds[4] + wl.bounds[5])
    inside.position[0] += 0.11
    inside.position[2] = c + 0.13 * (wl.bounds[5] - wl.bounds[4])
    away = V.workload_camera(wl)
    away.xpan = 5.0           # every box off the image: all costs are zero
    with S.Scene(0) as sc:
        V.load_workload(sc, wl)
        for cam in (panned, inside, away):
            both_orders(sc, cam, p)


def test_staged_march_with_longest_first():
    wl = W.plain_small(n=65, width=128, height=96, parts=(2, 2, 2))
    cam = V.workload_camera(wl)
    p = V.workload_params(wl)
    with S.Scene(0) as sc:
        V.load_workload(sc, wl)
        both_orders(sc, cam, p, staged=1)
        assert sc.staging_failures() == 0


def test_grid_beyond_the_order_kernel_keeps_the_centre_table():
    """3600 x 3520 pixels are 225 x 220 = 49500 tiles, more than the order
    kernel sorts (49152): the render falls back to the centre-first table."""
    wl = W.plain_small(n=33, width=3600, height=3520)
    cam = V.workload_camera(wl)
    p = V.workload_params(wl)
    with S.Scene(0) as sc:
        V.load_workload(sc, wl)
        both_orders(sc, cam, p)


def test_tile_order_argument_checks():
    with S.Scene(0) as sc:
        with pytest.raises(N.GvrError):
            N.call("gvr_scene_set_tile_order", sc.handle, 2)
    assert N.lib().gvr_scene_set_tile_order(None, 1) == N.GVR_ERR_INVALID_ARGUMENT
