"""Ascent actions end to end on the GPU: publish Blueprint data, execute
`add_scenes` with a volume plot, and check the PNGs against direct renders."""
import numpy as np
import pytest

from ascent_gb300 import Ascent, AscentError
from ascent_gb300 import _native as N
from ascent_gb300 import colortable as CT
from ascent_gb300 import png as PNG
from ascent_gb300 import scene as S
from ascent_gb300 import volume as V
from ascent_gb300 import workloads as W
from ascent_gb300.png import decode_png

pytestmark = pytest.mark.gpu

TF = {"control_points": [
    {"type": "rgb", "position": 0.0, "color": [0.0, 0.2, 1.0]},
    {"type": "rgb", "position": 1.0, "color": [1.0, 0.8, 0.0]},
    {"type": "alpha", "position": 0.0, "alpha": 0.0},
    {"type": "alpha", "position": 1.0, "alpha": 0.6}]}


def actions(renders, samples=120):
    return [{"action": "add_scenes", "scenes": {"s1": {
        "plots": {"p1": {"type": "volume", "field": "braid", "samples": samples, "color_table": TF}},
        "renders": renders}}}]


def direct(wl, render, samples=120):
    """The same image through the Scene API, as the plot would set it up."""
    with S.Scene(0) as sc:
        V.load_workload(sc, wl)
        vr = V.VolumeRenderer()
        vr.set_num_samples(samples)
        vr.set_color_table(CT.parse_color_table(TF))
        single = len(wl.domains) == 1 and not hasattr(wl.domains[0], "conn")
        p = vr.params(render["image_width"], render["image_height"], sc.bounds(), sc.scalar_range(),
                      single, render_bg=True, bg_color=(0.1, 0.1, 0.1, 1.0))
        cam = S.camera_reset_to_bounds(sc.bounds())
        S.camera_azimuth(cam, render["camera"]["azimuth"])
        S.camera_elevation(cam, render["camera"]["elevation"])
        rgba, _ = sc.render(cam, p)
    return PNG.canvas_to_rgba8(rgba)


@pytest.mark.parametrize("parts", [None, (2, 1, 2)])
def test_volume_plot_png_matches_direct_render(tmp_path, parts):
    wl = W.plain_small(n=33, width=8, height=8, parts=parts)
    a = Ascent()
    a.open({"default_dir": str(tmp_path), "exceptions": "forward"})
    a.publish(W.to_blueprint(wl))
    render = {"image_width": 96, "image_height": 80, "image_prefix": "vol_%04d", "bg_color": [0.1, 0.1, 0.1],
              "camera": {"azimuth": 40.0, "elevation": 15.0}}
    a.execute(actions({"r1": render}))
    info = a.info()
    assert len(info["images"]) == 1
    path = info["images"][0]["image_name"]
    assert path.endswith("vol_0100.png")
    got = decode_png(open(path, "rb").read())
    want = direct(wl, render)
    assert np.array_equal(got, want)
    a.close()


def test_cinema_render_writes_database(tmp_path):
    wl = W.cinema_batch(n_domains=5, box_cells=64, seed=2, width=8, height=8)
    a = Ascent()
    a.open({"default_dir": str(tmp_path), "exceptions": "forward"})
    a.publish(W.to_blueprint(wl))
    a.execute(actions({"c1": {"type": "cinema", "phi": 3, "theta": 2, "image_width": 48,
                              "image_height": 48, "db_name": "vol_db", "image_prefix": "img"}}))
    imgs = a.info()["images"]
    assert len(imgs) == 6
    db = tmp_path / "cinema_databases" / "vol_db"
    assert (db / "data.csv").read_text().startswith("phi,theta,time,FILE")
    assert (db / "1.5" / "-180_0_img.png").exists()
    # each cinema image equals a single-view render of its camera
    with S.Scene(0) as sc:
        V.load_workload(sc, wl)
        vr = V.VolumeRenderer()
        vr.set_num_samples(120)
        vr.set_color_table(CT.parse_color_table(TF))
        p = vr.params(48, 48, sc.bounds(), sc.scalar_range(), False, render_bg=True)
        cam = S.cinema_cameras(sc.bounds(), [[imgs[4]["phi"], imgs[4]["theta"]]])[0]
        rgba, _ = sc.render(cam, p)
    got = decode_png(open(imgs[4]["image_name"], "rb").read())
    assert np.array_equal(got, PNG.canvas_to_rgba8(rgba))


def test_hex_and_republish(tmp_path):
    wl = W.hex_mesh(n_cells=10, seed=1, width=8, height=8)
    a = Ascent()
    a.open({"default_dir": str(tmp_path), "exceptions": "forward"})
    bp = W.to_blueprint(wl)
    a.publish(bp)
    render = {"image_width": 64, "image_height": 64, "image_prefix": "hex",
              "camera": {"azimuth": 30.0, "elevation": 20.0}}
    a.execute(actions({"r": render}))
    first = decode_png(open(a.info()["images"][0]["image_name"], "rb").read())
    assert first[..., 3].max() > 0
    # a non-linear change (a linear one would be undone by the range normalisation)
    bp[0]["fields"]["braid"]["values"] = np.sqrt(np.abs(bp[0]["fields"]["braid"]["values"]))
    a.publish(bp)  # same mesh: fields are swapped in place
    a.execute(actions({"r": render}))
    second = decode_png(open(a.info()["images"][0]["image_name"], "rb").read())
    assert not np.array_equal(first, second)


def test_errors_are_caught_or_forwarded(tmp_path):
    wl = W.plain_small(n=16, width=8, height=8)
    a = Ascent()
    a.open({"default_dir": str(tmp_path)})
    a.publish(W.to_blueprint(wl))
    bad = [{"action": "add_scenes", "scenes": {"s": {"plots": {"p": {"type": "volume", "field": "nope"}}}}}]
    a.execute(bad)
    assert any("Unknown field" in e for e in a.info()["errors"])
    b = Ascent()
    b.open({"default_dir": str(tmp_path), "exceptions": "forward"})
    b.publish(W.to_blueprint(wl))
    with pytest.raises(AscentError):
        b.execute(bad)
    with pytest.raises(AscentError):
        b.execute([{"action": "add_scenes", "scenes": {"s": {"plots": {
            "p": {"type": "volume", "field": "braid", "bogus": 1}}}}}])
    with pytest.raises(N.GvrError):
        b.execute([{"action": "add_scenes", "scenes": {"s": {"plots": {
            "p": {"type": "volume", "field": "braid", "samples": 0}}}}}])


@pytest.mark.parametrize("size", [(1, 1), (37, 5), (256, 130)])
def test_device_png_conversion_equals_host(size):
    """gvr_canvas_to_rgba8 (device) and canvas_to_rgba8 (numpy) give the same
    bytes: flip, value * 255, clamp, truncation — also for values outside
    [0, 1] and on the exact steps k / 255."""
    import ctypes as C
    import torch
    from ascent_gb300 import _native as N
    w, h = size
    rng = np.random.default_rng(w * 1000 + h)
    img = rng.uniform(-0.2, 1.2, (h, w, 4)).astype(np.float32)
    steps = (np.arange(h * w * 4) % 256).astype(np.float32).reshape(h, w, 4) / np.float32(255.0)
    img[::2] = steps[::2]
    want = PNG.canvas_to_rgba8(img)
    got = PNG.canvas_to_rgba8_device(torch.from_numpy(img).cuda()).cpu().numpy()
    np.testing.assert_array_equal(got, want)
    out = np.empty((h, w, 4), np.uint8)
    N.call("gvr_canvas_to_rgba8", C.c_void_p(img.ctypes.data), w, h, C.c_void_p(out.ctypes.data),
           N.MEM_HOST, None)
    np.testing.assert_array_equal(out, want)
    with pytest.raises(N.GvrError):
        N.call("gvr_canvas_to_rgba8", C.c_void_p(img.ctypes.data), 0, h, C.c_void_p(out.ctypes.data),
               N.MEM_HOST, None)
