"""Batched multi-view path: one persistent, graph-replayed launch over a device
work queue of (view, tile) items must give, for every view, the image the
plain single-view path gives (per-tile domain culling only drops domains a
ray cannot hit), and match the oracle."""
import numpy as np
import pytest

from ascent_gb300 import _native as N
from ascent_gb300 import scene as S
from ascent_gb300 import volume as V
from ascent_gb300 import workloads as W
from oracle import oracle as O

from conftest import assert_parity

pytestmark = pytest.mark.gpu


def small_cinema(n_phi=3, n_theta=3, size=96):
    wl = W.cinema_batch(n_domains=9, box_cells=96, seed=11, width=size, height=size,
                        n_phi=n_phi, n_theta=n_theta)
    cams = S.cinema_cameras(wl.bounds, wl.phi_theta)
    p = V.workload_params(wl)
    return wl, cams, p


def test_batch_equals_per_view_renders_and_counts():
    wl, cams, p = small_cinema()
    assert p.quantize_uint8 == 0
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


def test_batch_matches_oracle():
    wl, cams, p = small_cinema(2, 2, 80)
    with S.Scene(0) as sc:
        V.load_workload(sc, wl)
        rgba, _ = sc.render_batch(cams, p)
    osc = O.OracleScene(64)
    for d in wl.domains:
        osc.add_uniform(d.dims, d.origin, d.spacing, d.field)
    for v, cam in enumerate(cams):
        o, _, _ = osc.render(cam, p)
        assert_parity(rgba[v], o)
    assert rgba[..., 3].max() > 0.1


def test_graph_is_reused_and_rebuilt_on_change():
    import torch
    wl, cams, p = small_cinema(2, 3, 64)
    with S.Scene(0) as sc:
        V.load_workload(sc, wl)
        out = (torch.empty((6, 64, 64, 4), device="cuda"), torch.empty((6, 64, 64), device="cuda"))
        a, _ = sc.render_batch(cams, p, device_out=True, out=out)
        a = a.clone()
        sc.render_batch(cams, p, device_out=True, out=out)
        torch.cuda.synchronize()
        assert sc.batch_graph_builds == 1
        assert torch.equal(out[0], a)
        for tpi in (2, 5):
            sc.set_batch_granularity(tpi)
            sc.render_batch(cams, p, device_out=True, out=out)
            torch.cuda.synchronize()
            assert torch.equal(out[0], a)
        assert sc.batch_graph_builds == 3
        # new cameras reuse the graph (views are uploaded before the replay)
        cams2 = S.cinema_cameras(wl.bounds, np.array([[10, 20], [30, 40]] * 3, np.float32))
        b, _ = sc.render_batch(cams2, p, device_out=True, out=out)
        torch.cuda.synchronize()
        assert sc.batch_graph_builds == 3
        g, _ = sc.render(cams2[1], p)
        np.testing.assert_array_equal(b[1].cpu().numpy(), g)
        with pytest.raises(N.GvrError):
            sc.set_batch_granularity(0)


def test_batch_host_outputs_many_domains_and_uneven_views():
    wl = W.cinema_batch(n_domains=37, box_cells=128, seed=4, width=72, height=40, n_phi=3, n_theta=2)
    cams = S.cinema_cameras(wl.bounds, wl.phi_theta)
    p = V.workload_params(wl)
    with S.Scene(0) as sc:
        V.load_workload(sc, wl)
        assert sc.num_domains == 37
        rgba, depth = sc.render_batch(cams, p)
        for v in (0, 3, 5):
            g, gd = sc.render(cams[v], p)
            np.testing.assert_array_equal(rgba[v], g)
            np.testing.assert_array_equal(depth[v], gd)


def test_batch_with_hex_and_uniform_domains():
    """A scene of a uniform domain beside a hexahedral one, batched over four
    views: each view equals the single-view render and the oracle."""
    hw = W.hex_mesh(n_cells=10, seed=6, width=72, height=64)
    h = hw.domains[0]
    # a uniform block next to the hex mesh (which spans the unit cube)
    n = 12
    rng = np.random.default_rng(3)
    field = rng.uniform(0.2, 1.0, (n + 1, n + 1, n + 1)).astype(np.float32)
    origin, spacing = (1.0, 0.0, 0.0), (1.0 / n,) * 3
    bounds = np.array([0, 2, 0, 1, 0, 1.0])
    cams = S.cinema_cameras(bounds, W.cinema_angles(2, 2))
    p = V.workload_params(hw)
    p.scalar_min, p.scalar_max = 0.0, 1.0
    with S.Scene(0) as sc:
        sc.add_hex(h.x, h.y, h.z, h.conn, h.field)
        sc.add_uniform(field, origin, spacing)
        rgba, depth = sc.render_batch(cams, p)
        for v, cam in enumerate(cams):
            g, gd = sc.render(cam, p)
            np.testing.assert_array_equal(rgba[v], g)
            np.testing.assert_array_equal(depth[v], gd)
    osc = O.OracleScene(64)
    osc.add_hex(h.x, h.y, h.z, h.conn, h.field)
    osc.add_uniform(field.shape[::-1], origin, spacing, field)
    for v, cam in enumerate(cams):
        assert_parity(rgba[v], osc.render(cam, p)[0])
    assert rgba[..., 3].max() > 0.1


def test_cinema_shaped_batch_matches_oracle():
    """The batched configuration's shape: 37 uniform domains of uneven sizes
    (edges from {32, ..., 256} cells, seeded splits of a 256^3 box) and a
    4 x 2 Cinema sweep, against the FP64 oracle with the oracle's own
    cameras and parameters, at 128^2."""
    wl = W.cinema_batch(width=128, height=128, n_phi=4, n_theta=2)
    assert len(wl.domains) == 37
    assert len({d.dims for d in wl.domains}) > 5  # uneven
    cams = S.cinema_cameras(wl.bounds, wl.phi_theta)
    p = V.workload_params(wl)
    with S.Scene(0) as sc:
        V.load_workload(sc, wl)
        rgba, _ = sc.render_batch(cams, p)
    osc = O.OracleScene(64)
    for d in wl.domains:
        osc.add_uniform(d.dims, d.origin, d.spacing, d.field)
    ocams = O.cinema_cameras(wl.bounds, wl.phi_theta)
    op = O.workload_params(wl)
    for v in range(len(cams)):
        o, _, _ = osc.render(ocams[v], op)
        assert o[..., 3].max() > 0.1
        assert_parity(rgba[v], o)
