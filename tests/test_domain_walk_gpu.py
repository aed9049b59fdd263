"""The one-loop domain walk (render_ray_unified in gvr_march.cu): rays over
two or more uniform vertex domains in 8^3-cell bricks, at most 16 domains,
sample every domain they cross in one loop. Its images must equal the
shared-memory staged march's exactly (an independent implementation of the
same per-domain order, sample positions and blend) and stay within the
parity bar of the FP64 oracle, at the 16-domain limit and past it (18
domains take the per-domain loop), for a camera outside and inside the
volume, with an opaque canvas that ends rays part-way, and in the batch
kernel.
"""
import numpy as np
import pytest

from ascent_gb300 import scene as S
from ascent_gb300 import volume as V
from ascent_gb300 import workloads as W
from oracle import oracle as O

from conftest import assert_parity

pytestmark = pytest.mark.gpu


def oracle_scene(wl):
    osc = O.OracleScene(64)
    for d in wl.domains:
        osc.add_uniform(d.dims, d.origin, d.spacing, d.field)
    return osc


def inside_camera(wl):
    cam = S.camera_reset_to_bounds(wl.bounds)
    c = 0.5 * (wl.bounds[4] + wl.bounds[5])
    cam.position[0] += 0.07
    cam.position[1] -= 0.05
    cam.position[2] = c + 0.21 * (wl.bounds[5] - wl.bounds[4])
    return cam


@pytest.mark.parametrize("parts", [(2, 1, 1), (4, 2, 2), (3, 3, 2)])
@pytest.mark.parametrize("where", ["outside", "inside"])
def test_domain_walk_equals_staged_and_oracle(parts, where):
    wl = W.plain_small(n=73, width=120, height=104, parts=parts)
    assert len(wl.domains) == parts[0] * parts[1] * parts[2]
    cam = V.workload_camera(wl) if where == "outside" else inside_camera(wl)
    p = V.workload_params(wl)
    with S.Scene(0) as sc:
        V.load_workload(sc, wl)
        out = []
        for staged in (0, 1):
            sc.set_tuning(packet_w=4, unroll=4, min_blocks=4, staged=staged)
            out.append(sc.render(cam, p, count_samples=True))
        assert sc.staging_failures() == 0
    (g, gd, gn), (s, sd, sn) = out
    np.testing.assert_array_equal(g, s)
    np.testing.assert_array_equal(gd, sd)
    assert gn == sn
    ocam = O.workload_camera(wl) if where == "outside" else cam
    o, _, _ = oracle_scene(wl).render(ocam, O.workload_params(wl))
    assert_parity(g, o)
    assert g[..., 3].max() > 0.05


def test_domain_walk_over_a_canvas():
    from test_canvas import canvas_for
    wl = W.plain_small(n=57, width=96, height=80, parts=(2, 2, 2))
    cam = V.workload_camera(wl)
    p = V.workload_params(wl)
    rgba, depth = canvas_for(wl, cam, p, seed=11)
    with S.Scene(0) as sc:
        V.load_workload(sc, wl)
        out = []
        for staged in (0, 1):
            sc.set_tuning(packet_w=8, unroll=2, min_blocks=4, staged=staged)
            out.append(sc.render_over(cam, p, rgba, depth, count_samples=True))
    np.testing.assert_array_equal(out[0][0], out[1][0])
    np.testing.assert_array_equal(out[0][1], out[1][1])
    assert out[0][2] == out[1][2]


def test_domain_walk_in_the_batch_kernel():
    """The batch kernel takes the one-loop walk for tiles whose domain mask
    has two or more domains: its views equal the per-view renders and the
    oracle's."""
    wl = W.plain_small(n=57, width=72, height=64, parts=(2, 2, 2))
    cams = S.cinema_cameras(wl.bounds, W.cinema_angles(2, 2))
    p = V.workload_params(wl)
    with S.Scene(0) as sc:
        V.load_workload(sc, wl)
        rgba, depth, n = sc.render_batch(cams, p, count_samples=True)
        total = 0
        for v, cam in enumerate(cams):
            g, gd, gn = sc.render(cam, p, count_samples=True)
            np.testing.assert_array_equal(rgba[v], g)
            np.testing.assert_array_equal(depth[v], gd)
            total += gn
        assert n == total
    ocams = O.cinema_cameras(wl.bounds, W.cinema_angles(2, 2))
    osc = oracle_scene(wl)
    op = O.workload_params(wl)
    for v in range(len(cams)):
        o, _, _ = osc.render(ocams[v], op)
        assert_parity(rgba[v], o)
