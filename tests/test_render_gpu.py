"""CUDA path vs the FP64 oracle, through the C ABI, on seeded inputs.

Bar (per pixel, per RGBA channel): |error| <= 2/255 on >= 99.9% of pixels
and mean absolute error <= 1e-3, against the oracle run with the same
parameters (same early termination). The error against the oracle with
early termination off is computed too and held to the same bar.
"""
import numpy as np
import pytest

from ascent_gb300 import _native as N
from ascent_gb300 import scene as S
from ascent_gb300 import volume as V
from ascent_gb300 import workloads as W
from oracle import oracle as O

from conftest import assert_parity, image_error

pytestmark = pytest.mark.gpu


def assert_depth(gd, od, atol=2e-4, frac=0.999):
    """Image depths agree on >= 99.9% of pixels (a partial right at the
    alpha cull threshold may exist on one side only)."""
    ok = np.abs(gd.astype(np.float64) - od) <= atol
    assert ok.mean() >= frac, (ok.mean(), np.abs(gd - od).max())


def oracle_scene(wl):
    osc = O.OracleScene(64)
    for d in wl.domains:
        osc.add_uniform(d.dims, d.origin, d.spacing, d.field)
    return osc


def render_both(wl, cam=None, **kw):
    """The product sets up its camera and parameters through the library, the
    oracle through its own restatement of the same host logic, so the
    comparison covers the set-up as well as the march."""
    ocam = O.workload_camera(wl) if cam is None else cam
    cam = cam or V.workload_camera(wl)
    p = V.workload_params(wl, **kw)
    op = O.workload_params(wl, **kw)
    with S.Scene(0) as sc:
        V.load_workload(sc, wl)
        g_rgba, g_depth, g_n = sc.render(cam, p, count_samples=True)
    o_rgba, o_depth, o_n = oracle_scene(wl).render(ocam, op)
    return (g_rgba, g_depth, g_n), (o_rgba, o_depth, o_n), p


def test_plain_small_single_domain():
    wl = W.plain_small(n=64, width=256, height=256)
    (g, gd, gn), (o, od, on), p = render_both(wl)
    assert p.quantize_uint8 == 1
    e = assert_parity(g, o)
    assert o[..., 3].max() > 0.2, "image must not be empty"
    assert abs(gn - on) <= 1e-3 * on, (gn, on)
    assert_depth(gd, od)


def test_plain_cpu_case_512():
    """The CPU-runnable plain case at its full size: 64^3, 512^2, 218 samples."""
    wl = W.plain_small()
    (g, gd, gn), (o, od, on), p = render_both(wl)
    assert_parity(g, o)
    (g2, _, _), (o2, _, _), _ = render_both(wl, early_term=1.0)
    assert_parity(g2, o2)
    assert_parity(g, o2)  # early termination at 0.99 stays within the bar


def test_multi_domain_composite_uint8_lut():
    wl = W.plain_small(n=49, width=200, height=150, parts=(2, 2, 2))
    (g, gd, gn), (o, od, on), p = render_both(wl)
    assert p.quantize_uint8 == 0
    assert_parity(g, o)
    assert abs(gn - on) <= 1e-3 * on
    assert_depth(gd, od)


def test_multi_domain_uneven_split_matches_single_domain_geometry():
    wl = W.plain_small(n=41, width=96, height=96, parts=(3, 1, 2))
    (g, _, _), (o, _, _), _ = render_both(wl)
    assert_parity(g, o)


@pytest.mark.parametrize("az,el,zoom", [(0, 0, 1.0), (135, -40, 1.0), (200, 70, 2.0), (30, 20, 0.5)])
def test_camera_variants(az, el, zoom):
    wl = W.plain_small(n=33, width=128, height=96, parts=(2, 1, 1))
    cam = S.camera_reset_to_bounds(wl.bounds)
    S.camera_azimuth(cam, az)
    S.camera_elevation(cam, el)
    cam.zoom = zoom
    (g, gd, _), (o, od, _), _ = render_both(wl, cam=cam)
    assert_parity(g, o)


def test_camera_inside_volume_and_looking_away():
    wl = W.plain_small(n=33, width=64, height=64)
    cam = S.camera_reset_to_bounds(wl.bounds)
    cam.position[:] = [0.5, 0.5, 0.5]
    cam.look_at[:] = [0.9, 0.6, 0.4]
    (g, _, _), (o, _, _), _ = render_both(wl, cam=cam)
    assert_parity(g, o)
    cam.position[:] = [0.5, 0.5, 3.0]
    cam.look_at[:] = [0.5, 0.5, 6.0]
    (g, gd, gn), (o, od, on), p = render_both(wl, cam=cam)
    assert gn == on == 0
    assert np.all(g == 0) and np.all(gd == p.clear_depth)


def test_odd_image_sizes_and_tiny_lut():
    wl = W.plain_small(n=20, width=37, height=1)
    (g, _, _), (o, _, _), _ = render_both(wl)
    assert_parity(g, o)
    wl = W.plain_small(n=20, width=1, height=1)
    (g, _, _), (o, _, _), _ = render_both(wl)
    assert_parity(g, o)
    wl = W.plain_small(n=24, width=45, height=33)
    lut = np.array([[0, 0, 1, 0.0], [1, 0.5, 0, 0.2]], np.float32)
    cam = V.workload_camera(wl)
    for filt in (N.LUT_NEAREST, N.LUT_LINEAR):
        p = N.make_params(45, 33, 0.01, wl.scalar_range, lut, lut_filter=filt)
        with S.Scene(0) as sc:
            V.load_workload(sc, wl)
            g, _ = sc.render(cam, p)
        o, _, _ = oracle_scene(wl).render(cam, p)
        assert_parity(g, o)


@pytest.mark.parametrize("parts", [(1, 1, 1), (2, 1, 2)])
def test_empty_space_skipping_is_exact(parts):
    """Bricks whose range maps to zero opacity are skipped; samples still count."""
    wl = W.plain_small(n=72, width=128, height=128, parts=parts)
    vr = V.workload_renderer(wl)
    lut = vr.lut(True)
    lut[: 600, 3] = 0.0  # transparent below s = 0.586
    cam = V.workload_camera(wl)
    p = N.make_params(128, 128, S.sample_distance(wl.bounds, 218), wl.scalar_range, lut)
    with S.Scene(0) as sc:
        V.load_workload(sc, wl)
        g, gd, gn = sc.render(cam, p, count_samples=True)
    o, od, on = oracle_scene(wl).render(cam, p)
    assert_parity(g, o)
    assert abs(gn - on) <= 1e-3 * on


def test_background_blend_and_depth_clear():
    wl = W.plain_small(n=24, width=64, height=48, parts=(1, 2, 1))
    cam = V.workload_camera(wl)
    p = V.workload_params(wl, render_bg=True, bg_color=(0.1, 0.2, 0.3, 1.0))
    p.clear_depth = 1.001
    with S.Scene(0) as sc:
        V.load_workload(sc, wl)
        g, gd = sc.render(cam, p)
    o, od, _ = oracle_scene(wl).render(cam, p)
    assert_parity(g, o)
    np.testing.assert_allclose(g[..., 3], 1.0, atol=1e-6)


def test_rectilinear_domain_matches_oracle():
    rng = np.random.default_rng(7)
    xs = [np.cumsum(np.r_[0.0, rng.uniform(0.5, 1.5, n - 1)]) for n in (30, 25, 35)]
    xs = [x / x[-1] for x in xs]
    c, s, a = W.blob_params(rng)
    f = W.blob_field(xs, c, s, a)
    lut = V.VolumeRenderer().lut(True)
    rp, rgb, ap, al = W.linear_ramp_tf()
    vr = V.VolumeRenderer()
    vr.set_color_table(V.TransferFunction(rp, rgb, ap, al))
    vr.set_num_samples(150)
    lut = vr.lut(True)
    b = np.array([0, 1, 0, 1, 0, 1.0])
    cam = S.camera_reset_to_bounds(b)
    S.camera_azimuth(cam, 40)
    S.camera_elevation(cam, 25)
    p = N.make_params(120, 100, S.sample_distance(b, 150), (float(f.min()), float(f.max())), lut)
    with S.Scene(0) as sc:
        sc.add_rectilinear(f, *xs)
        g, gd = sc.render(cam, p)
    osc = O.OracleScene(64)
    osc.add_rectilinear(*xs, f)
    o, od, _ = osc.render(cam, p)
    assert o[..., 3].max() > 0.1
    assert_parity(g, o)


def test_element_field_matches_oracle():
    rng = np.random.default_rng(9)
    cells = rng.uniform(0, 1, (15, 17, 19)).astype(np.float32)
    rp, rgb, ap, al = W.linear_ramp_tf(alpha_max=0.8)
    vr = V.VolumeRenderer()
    vr.set_color_table(V.TransferFunction(rp, rgb, ap, al))
    lut = vr.lut(True)
    sp = (1 / 19, 1 / 17, 1 / 15)
    b = np.array([0, 1, 0, 1, 0, 1.0])
    cam = S.camera_reset_to_bounds(b)
    S.camera_azimuth(cam, 10)
    p = N.make_params(80, 80, S.sample_distance(b, 100), (0.0, 1.0), lut)
    with S.Scene(0) as sc:
        sc.add_uniform(cells, (0, 0, 0), sp, association=N.ASSOC_ELEMENT)
        g, _ = sc.render(cam, p)
    osc = O.OracleScene(64)
    osc.add_uniform((20, 18, 16), (0, 0, 0), sp, cells, assoc=N.ASSOC_ELEMENT)
    o, _, _ = osc.render(cam, p)
    # nearest-cell lookups flip at cell faces under FP32 vs FP64 positions
    e = image_error(g, o)
    assert e["frac_within_2"] >= 0.99 and e["mae"] <= 2e-3, e


def test_float64_and_strided_device_input():
    import torch
    wl = W.plain_small(n=24, width=64, height=64)
    d = wl.domains[0]
    cam = V.workload_camera(wl)
    p = V.workload_params(wl)
    with S.Scene(0) as sc:
        sc.add_uniform(torch.from_numpy(d.field.astype(np.float64)).cuda(), d.origin, d.spacing)
        g64, _ = sc.render(cam, p)
    with S.Scene(0) as sc:
        sc.add_uniform(torch.from_numpy(d.field).cuda(), d.origin, d.spacing)
        g32, _ = sc.render(cam, p)
        t, _ = sc.render(cam, p, device_out=True)
        torch.cuda.synchronize()
        np.testing.assert_array_equal(t.cpu().numpy(), g32)
    np.testing.assert_array_equal(g64, g32)


def test_update_field_and_bounds_and_range():
    wl = W.plain_small(n=24, width=48, height=48, parts=(2, 1, 1))
    with S.Scene(0) as sc:
        V.load_workload(sc, wl)
        assert sc.num_domains == 2
        np.testing.assert_allclose(sc.bounds(), wl.bounds, atol=1e-6)
        lo, hi = sc.scalar_range()
        assert np.isclose(lo, wl.scalar_range[0]) and np.isclose(hi, wl.scalar_range[1])
        sc.update_field(1, wl.domains[1].field * 2)
        assert np.isclose(sc.scalar_range()[1], max(wl.domains[0].field.max(), 2 * wl.domains[1].field.max()))
        with pytest.raises(N.GvrError):
            sc.update_field(5, wl.domains[0].field)


def test_invalid_arguments_raise():
    wl = W.plain_small(n=16, width=16, height=16)
    with S.Scene(0) as sc:
        V.load_workload(sc, wl)
        cam = V.workload_camera(wl)
        p = V.workload_params(wl)
        p.sample_dist = 0.0
        with pytest.raises(N.GvrError):
            sc.render(cam, p)
        p = V.workload_params(wl)
        bad = cam.copy()
        bad.look_at[:] = list(bad.position)
        with pytest.raises(N.GvrError):
            sc.render(bad, p)
        with pytest.raises(N.GvrError):
            sc.add_uniform(np.zeros((1, 4, 4), np.float32), (0, 0, 0), (1, 1, 1))
        with pytest.raises(N.GvrError):
            sc.add_uniform(np.full((4, 4, 4), np.nan, np.float32), (0, 0, 0), (1, 1, 1))


def test_every_launch_shape_gives_the_same_image():
    from ascent_gb300 import tune
    wl = W.plain_small(n=57, width=100, height=84, parts=(2, 2, 1))
    cam = V.workload_camera(wl)
    p = V.workload_params(wl)
    with S.Scene(0) as sc:
        V.load_workload(sc, wl)
        ref = None
        for cand in tune.CANDIDATES + tune.STAGED_CANDIDATES:
            sc.set_tuning(**cand)
            g, gd, n = sc.render(cam, p, count_samples=True)
            if ref is None:
                ref = (g, gd, n)
                continue
            np.testing.assert_allclose(g, ref[0], rtol=0, atol=1e-6)
            np.testing.assert_array_equal(gd, ref[1])
            assert n == ref[2]
        out = tune.autotune(sc, cam, p, reps=1, use_cache=False)
        every = tune.CANDIDATES + tune.STAGED_CANDIDATES
        # the winning shape, then timed again with each tile launch order
        shape = {k: v for k, v in out["best"].items() if k != "tile_order"}
        assert shape in every and out["best"]["tile_order"] in (0, 1)
        assert len(out["ms"]) == len(every) + 2
        with pytest.raises(N.GvrError):
            sc.set_tuning(packet_w=5)


def test_image_sizes_in_turn_on_one_scene():
    """The march launches its tiles in a per-size order (nearest the image
    centre first); a scene rendering several sizes in turn keeps one order
    per size. Each image equals the one a fresh scene renders, and the
    oracle's."""
    wl = W.plain_small(n=40, width=64, height=64, parts=(2, 1, 2))
    cam = V.workload_camera(wl)
    sizes = [(45, 33), (64, 64), (17, 130), (45, 33)]

    def params_at(w, h):
        wl.width, wl.height = w, h
        return V.workload_params(wl)

    with S.Scene(0) as sc:
        V.load_workload(sc, wl)
        got = [sc.render(cam, params_at(w, h), count_samples=True) for w, h in sizes]
    for (w, h), (g, gd, n) in zip(sizes, got):
        p = params_at(w, h)
        with S.Scene(0) as fresh:
            V.load_workload(fresh, wl)
            f, fd, fn = fresh.render(cam, p, count_samples=True)
        np.testing.assert_array_equal(g, f)
        np.testing.assert_array_equal(gd, fd)
        assert n == fn
        o, od, on = oracle_scene(wl).render(cam, p)
        assert_parity(g, o)
    np.testing.assert_array_equal(got[0][0], got[3][0])


def test_update_fields_pipelined_equals_one_by_one():
    """gvr_scene_update_fields (two staging buffers, copy stream, device
    ranges) gives the scene of eight gvr_scene_update_field calls: same
    ranges, same image; host and device sources; mixed element-field and
    hex domains take the one-at-a-time path inside the same call."""
    import torch
    wl = W.plain_large(n_cells=64, width=96, height=80, seed=8)
    cam = V.workload_camera(wl)
    p = V.workload_params(wl)
    rng = np.random.default_rng(3)
    new = [(d.field * rng.uniform(0.5, 1.5)).astype(np.float32) for d in wl.domains]
    with S.Scene(0) as a, S.Scene(0) as b, S.Scene(0) as c:
        for sc in (a, b, c):
            V.load_workload(sc, wl)
        for i, f in enumerate(new):
            a.update_field(i, f)
        b.update_fields(range(len(new)), [torch.from_numpy(f).pin_memory() for f in new])
        c.update_fields(range(len(new)), [torch.from_numpy(f).cuda() for f in new])
        ia, _ = a.render(cam, p)
        for sc in (b, c):
            np.testing.assert_array_equal(sc.scalar_range(), a.scalar_range())
            for i in range(len(new)):
                np.testing.assert_array_equal(sc.bounds(i), a.bounds(i))
            im, _ = sc.render(cam, p)
            np.testing.assert_array_equal(im, ia)
        # a second call reuses the staging buffers
        b.update_fields(range(len(new)), [torch.from_numpy(f).pin_memory() for f in new[::-1]])
        for i, f in enumerate(new[::-1]):
            a.update_field(i, f)
        np.testing.assert_array_equal(b.render(cam, p)[0], a.render(cam, p)[0])
        bad = [f.copy() for f in new]
        bad[3][5] = np.nan
        with pytest.raises(N.GvrError):
            b.update_fields(range(len(bad)), bad)
    hw = W.hex_mesh(n_cells=6, seed=2, width=32, height=32)
    h = hw.domains[0]
    with S.Scene(0) as sc:
        sc.add_uniform(wl.domains[0].field, wl.domains[0].origin, wl.domains[0].spacing)
        sc.add_hex(h.x, h.y, h.z, h.conn, h.field)
        sc.update_fields([0, 1], [new[0], (h.field * 2).astype(np.float32)])
        assert sc.scalar_range()[1] >= float((h.field * 2).max()) - 1e-6
        # the same from device memory: the uniform domain takes the one-launch
        # bricking, the hex domain its own path
        sc.update_fields([0, 1], [torch.from_numpy(new[0]).cuda(),
                                  torch.from_numpy((h.field * 3).astype(np.float32)).cuda()])
        assert sc.scalar_range()[1] >= float((h.field * 3).max()) - 1e-6


@pytest.mark.parametrize("name", ["Viridis", "Jet", "black-body radiation"])
def test_named_preset_against_oracle(name):
    """A VTK-m preset named in the plot's colour table (with alpha points, as
    the reference's documentation asks of volume plots) renders within the
    bar of the oracle, which samples the same control points itself; the
    image differs from the default table's."""
    from ascent_gb300 import colortable as CT
    wl = W.plain_small(n=33, width=96, height=80, parts=(2, 1, 1))
    alpha = [{"type": "alpha", "position": 0.0, "alpha": 0.0},
             {"type": "alpha", "position": 1.0, "alpha": 0.6}]
    tf = CT.parse_color_table({"name": name, "control_points": alpha})
    wl.rgb_pos, wl.rgb, wl.alpha_pos, wl.alpha = tf.rgb_pos, tf.rgb, tf.alpha_pos, tf.alpha
    (g, _, _), (o, _, _), _ = render_both(wl)
    assert o[..., 3].max() > 0.2
    assert_parity(g, o)
    ctw = CT.parse_color_table({"control_points": alpha})
    wl.rgb_pos, wl.rgb, wl.alpha_pos, wl.alpha = ctw.rgb_pos, ctw.rgb, ctw.alpha_pos, ctw.alpha
    (g2, _, _), _, _ = render_both(wl)
    assert np.abs(g2 - g).max() > 0.05


def test_sixty_four_domains_and_the_limit():
    """The most domains one render composites (64: a 4 x 4 x 4 split), against
    the oracle; a 65th domain is refused with a clear error."""
    wl = W.plain_small(n=41, width=96, height=80, parts=(4, 4, 4))
    assert len(wl.domains) == 64
    (g, gd, gn), (o, od, on), _ = render_both(wl)
    assert_parity(g, o)
    assert abs(gn - on) <= 1e-3 * on
    assert_depth(gd, od)
    with S.Scene(0) as sc:
        V.load_workload(sc, wl)
        d = wl.domains[0]
        with pytest.raises(N.GvrError) as err:
            sc.add_uniform(d.field, d.origin, d.spacing)
        assert err.value.code == N.GVR_ERR_UNSUPPORTED


def test_two_node_domains():
    """Domains of a single cell (2 nodes per axis) side by side: the smallest
    bricks (one cell, padded) render like the oracle."""
    rng = np.random.default_rng(9)
    with S.Scene(0) as sc:
        osc = O.OracleScene(64)
        for i in range(3):
            for j in range(2):
                f = rng.uniform(0, 1, (2, 2, 2)).astype(np.float32)
                origin = (0.5 * i, 0.5 * j, 0.0)
                sc.add_uniform(f, origin, (0.5, 0.5, 0.5))
                osc.add_uniform((2, 2, 2), origin, (0.5, 0.5, 0.5), f)
        bounds = sc.bounds()
        cam = S.camera_reset_to_bounds(bounds)
        S.camera_azimuth(cam, 20.0)
        S.camera_elevation(cam, 25.0)
        x = np.linspace(0, 1, 64)
        lut = np.stack([x, 1 - x, 0.5 * np.ones_like(x), 0.05 * x], 1).astype(np.float32)
        p = N.make_params(64, 48, S.sample_distance(bounds, 200), (0.0, 1.0), lut)
        g, _, gn = sc.render(cam, p, count_samples=True)
    o, _, on = osc.render(cam, p)
    assert o[..., 3].max() > 0.05
    assert_parity(g, o)
    assert abs(gn - on) <= 1e-3 * on + 2
