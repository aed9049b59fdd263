"""The shared-memory staged march (gvr_scene_set_staging(scene, 1)).

Per 16 x 16 tile and slab of ray distance, the bricks the tile's rays cross
are copied into shared memory with bulk async copies and read there;
domains are taken in one front-to-back order per view. Its images, depths
and sample counts must equal the L1-gather march exactly (same per-sample
arithmetic, same compositing order), on single and split domains, uneven
domain sizes, scenes with empty bricks, an opaque canvas, a camera inside
the volume and a camera on a domain boundary plane, and stay within the
parity bar of the FP64 oracle. No bounded wait may give up.
"""
import numpy as np
import pytest

from ascent_gb300 import scene as S
from ascent_gb300 import volume as V
from ascent_gb300 import workloads as W
from oracle import oracle as O

from conftest import assert_parity

pytestmark = pytest.mark.gpu


def both(sc, cam, p, over=None):
    """Gather march and slab-staged march; the layer-staged march (mode 2)
    must equal the gather march too."""
    out = []
    for staged in (0, 1, 2):
        sc.set_tuning(packet_w=8, unroll=1, min_blocks=3, staged=staged)
        if over is None:
            out.append(sc.render(cam, p, count_samples=True))
        else:
            out.append(sc.render_over(cam, p, over[0], over[1], count_samples=True))
    assert_same(out[0], out[2])
    return out[:2]


def assert_same(a, b):
    np.testing.assert_array_equal(a[0], b[0])
    np.testing.assert_array_equal(a[1], b[1])
    assert a[2] == b[2]


@pytest.mark.parametrize("parts,size", [(None, (96, 80)), ((2, 2, 2), (128, 96)),
                                        ((3, 1, 2), (77, 131)), ((1, 2, 1), (256, 256))])
def test_staged_equals_gather(parts, size):
    wl = W.plain_small(n=65, width=size[0], height=size[1], parts=parts)
    cam = V.workload_camera(wl)
    p = V.workload_params(wl)
    with S.Scene(0) as sc:
        V.load_workload(sc, wl)
        g, st = both(sc, cam, p)
        assert_same(g, st)
        assert sc.staging_failures() == 0
    assert st[0][..., 3].max() > 0.1


def test_staged_matches_oracle_and_large_grid():
    """A 193^3-node field in 8 domains at 384^2 (many slabs per tile), against
    the gather march exactly and the FP64 oracle within the bar."""
    wl = W.plain_large(n_cells=192, width=384, height=384)
    cam = V.workload_camera(wl)
    p = V.workload_params(wl)
    with S.Scene(0) as sc:
        V.load_workload(sc, wl)
        g, st = both(sc, cam, p)
        assert sc.staging_failures() == 0
    assert_same(g, st)
    osc = O.OracleScene(64)
    for d in wl.domains:
        osc.add_uniform(d.dims, d.origin, d.spacing, d.field)
    o, _, _ = osc.render(O.workload_camera(wl), O.workload_params(wl))
    assert_parity(st[0], o)


def test_staged_cinema_views_of_uneven_domains():
    """37 domains of uneven sizes seen from a Cinema sweep: every view's
    image equals the gather march's."""
    wl = W.cinema_batch(n_domains=37, box_cells=128, seed=7, width=96, height=96, n_phi=4, n_theta=3)
    cams = S.cinema_cameras(wl.bounds, wl.phi_theta)
    p = V.workload_params(wl)
    with S.Scene(0) as sc:
        V.load_workload(sc, wl)
        for cam in cams:
            g, st = both(sc, cam, p)
            assert_same(g, st)
        assert sc.staging_failures() == 0


def test_staged_with_empty_bricks_and_a_canvas():
    """A transfer function with zero opacity over the lower half of the range
    (empty bricks are skipped without a copy), and the same volume drawn over
    an opaque canvas."""
    from test_canvas import canvas_for
    wl = W.plain_small(n=81, width=120, height=100, parts=(2, 1, 2))
    x = np.linspace(0.0, 1.0, 64)
    wl.alpha_pos, wl.alpha = x, np.where(x < 0.55, 0.0, 0.4 * (x - 0.55) / 0.45)
    cam = V.workload_camera(wl)
    p = V.workload_params(wl)
    with S.Scene(0) as sc:
        V.load_workload(sc, wl)
        g, st = both(sc, cam, p)
        assert_same(g, st)
        rgba, depth = canvas_for(wl, cam, p, seed=3)
        g2, st2 = both(sc, cam, p, over=(rgba, depth))
        assert_same(g2, st2)
        assert sc.staging_failures() == 0


def test_staged_camera_inside_and_on_a_split_plane():
    wl = W.plain_small(n=64, width=90, height=70, parts=(2, 2, 1))
    p = V.workload_params(wl)
    # reset camera only: it looks along -z from x = y = centre, the planes
    # where the domains meet
    on_plane = S.camera_reset_to_bounds(wl.bounds)
    inside = S.camera_reset_to_bounds(wl.bounds)
    c = 0.5 * (wl.bounds[4] + wl.bounds[5])
    inside.position[0] += 0.11
    inside.position[1] -= 0.07
    inside.position[2] = c + 0.13 * (wl.bounds[5] - wl.bounds[4])
    with S.Scene(0) as sc:
        V.load_workload(sc, wl)
        for cam in (on_plane, inside):
            g, st = both(sc, cam, p)
            assert_same(g, st)
        assert sc.staging_failures() == 0


def test_staging_falls_back_where_it_does_not_apply():
    """A scene holding a hexahedral domain renders with the gather march
    whatever the staging switch says."""
    hw = W.hex_mesh(n_cells=10, seed=3, width=48, height=40)
    h = hw.domains[0]
    cam = V.workload_camera(hw)
    p = V.workload_params(hw)
    with S.Scene(0) as sc:
        sc.add_hex(h.x, h.y, h.z, h.conn, h.field)
        g, st = both(sc, cam, p)
        assert_same(g, st)
