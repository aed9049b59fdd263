"""Host-side pieces of the Ascent front end: colour-table parsing, camera
keys, cinema angles and PNG output (no GPU needed)."""
import math
from pathlib import Path

import numpy as np
import pytest

from ascent_gb300 import _native as N
from ascent_gb300 import ascent as A
from ascent_gb300 import colortable as CT
from ascent_gb300 import png as PNG
from ascent_gb300 import scene as S
from ascent_gb300 import volume as V
from ascent_gb300.png import decode_png

GOLDEN = Path(__file__).resolve().parent / "golden"


def test_color_table_rules():
    # rgb points without a name clear the preset's colours
    t = CT.parse_color_table({"control_points": [
        {"type": "rgb", "position": 0.0, "color": [1, 0, 0]},
        {"type": "rgb", "position": 1.0, "color": [0, 0, 2.0]},
        {"type": "alpha", "position": 0.0, "alpha": -1.0},
        {"type": "alpha", "position": 1.0, "alpha": 0.5}]})
    assert list(t.rgb_pos) == [0.0, 1.0]
    np.testing.assert_allclose(t.rgb, [[1, 0, 0], [0, 0, 1]])  # clamped
    np.testing.assert_allclose(t.alpha, [0.0, 0.5])
    # with a name the preset colours stay and the point is added
    t2 = CT.parse_color_table({"name": "cool to warm", "control_points": [
        {"type": "rgb", "position": 0.5, "color": [0, 1, 0]}]})
    assert len(t2.rgb_pos) == 257 and [0, 1, 0] in t2.rgb.tolist()
    # reverse mirrors the colour points; an unknown name falls back to the
    # default with a message, as parse_color_table does
    warnings = []
    t3 = CT.parse_color_table({"name": "no such map", "reverse": "true"}, warn=warnings.append)
    assert warnings and np.allclose(t3.rgb[0], CT.preset("cool to warm")[1][-1])
    # a colour table without alpha points keeps the preset's opaque ends;
    # alpha points at other positions are added between them
    t4 = CT.parse_color_table({})
    assert list(t4.alpha_pos) == [0.0, 1.0] and list(t4.alpha) == [1.0, 1.0]
    t5 = CT.parse_color_table({"name": "Jet", "control_points": [
        {"type": "alpha", "position": 0.5, "alpha": 0.25}]})
    assert list(t5.alpha_pos) == [0.0, 0.5, 1.0] and list(t5.alpha) == [1.0, 0.25, 1.0]
    # rgb points clear the colours only: the opacity points stay
    assert list(t.alpha_pos) == [0.0, 1.0]
    # no colour_table node: VolumeRenderer's default opacity over the preset
    tf = V.TransferFunction.default()
    assert list(tf.alpha_pos) == [0.0, 1.0] and list(tf.alpha) == [0.5, 1.0]
    assert len(tf.rgb_pos) == 257


def test_preset_names_follow_string_equal():
    """Every VTK-m preset name is accepted ignoring case; near misses are not
    (string_equal compares length and characters, no trimming)."""
    names = CT.preset_names()
    assert len(names) == 18 and "Viridis" in names and "Cool to Warm" in names
    for n in names:
        assert CT.canonical_name(n.upper()) == n and CT.canonical_name(n.lower()) == n
    assert CT.canonical_name(" viridis") is None
    assert CT.canonical_name("grayscale") is None
    assert CT.canonical_name("cool2warm") is None


def test_cool_to_warm_matches_reference_color_bar():
    """The Moreland-generated "Cool to Warm" against the reference's own
    256-sample rendering of VTK-m's table (Actions/color_tables/vtkm/Cool to
    Warm.png): within 1/255 per channel everywhere, and its 8-bit rounding
    (A10) reproduces more of the bar's bytes than truncation does."""
    bars = np.load(GOLDEN / "vtkm_color_bars.npz")
    bar = bars["Cool to Warm"].astype(np.float64)
    pos, rgb = CT.preset("Cool to Warm")
    x = np.arange(256) / 255.0
    v = np.stack([np.interp(x, pos, rgb[:, c]) for c in range(3)], 1) * 255.0
    assert np.abs(v - bar).max() <= 1.0, np.abs(v - bar).max()
    rounded = (np.floor(v + 0.5) == bar).mean()
    truncated = (np.floor(v) == bar).mean()
    assert rounded > 0.9 and rounded > truncated, (rounded, truncated)


@pytest.mark.parametrize("name", sorted(np.load(GOLDEN / "vtkm_color_bars.npz").files))
def test_every_preset_samples_to_its_color_bar(name):
    """Each preset, sampled by the library at 256 entries through uint8
    (gvr_color_table_sample, rounding), equals the reference's colour bar
    byte for byte ("Cool to Warm", generated from the published method,
    within 1/255)."""
    bar = np.load(GOLDEN / "vtkm_color_bars.npz")[name].astype(np.int64)
    t = CT.parse_color_table({"name": name})
    lut = S.color_table_sample(t.rgb_pos, t.rgb, t.alpha_pos, t.alpha, 256, N.UINT8_ROUND)
    got = np.rint(lut[:, :3] * 255.0).astype(np.int64)
    tol = 1 if name == "Cool to Warm" else 0
    assert np.abs(got - bar).max() <= tol
    assert (lut[:, 3] == 1.0).all()  # presets are opaque


def test_cool_to_warm_is_diverging_through_white():
    pos, rgb = CT.preset("cool to warm")
    assert np.allclose(rgb[0], [59 / 255, 76 / 255, 192 / 255], atol=2e-3)
    assert np.allclose(rgb[-1], [180 / 255, 4 / 255, 38 / 255], atol=2e-3)
    mid = rgb[len(rgb) // 2]
    assert mid.min() > 0.8  # near white in the middle


def test_camera_keys_follow_parse_camera():
    b = np.array([0, 1, 0, 1, 0, 1.0])
    cam = S.camera_reset_to_bounds(b)
    A.apply_camera(cam, {"up": [0, 2, 0], "fov": 45, "zoom": 2.0, "ypan": 0.25,
                         "near_plane": 0.5, "far_plane": 9.0})
    assert cam.up[1] == 1.0 and cam.fov_y == 45.0
    assert abs(cam.zoom - 2.0) < 1e-6
    assert cam.xpan == 0.25 and cam.ypan == 0.0  # ypan lands in xpan, as in the reference
    assert cam.near_plane == 0.5 and cam.far_plane == 9.0
    c2 = S.camera_reset_to_bounds(b)
    A.apply_camera(c2, {"azimuth": 90})
    assert abs(c2.position[0] - 0.5) > 1.0 and abs(c2.position[2] - 0.5) < 1e-5


def test_cinema_angle_specs():
    a = A.cinema_angles({"phi": 4, "theta": 2})
    assert a.shape == (8, 2) and a[0].tolist() == [-180.0, 0.0] and a[1].tolist() == [-180.0, 90.0]
    b = A.cinema_angles({"phi_range": [0, 90], "dphi": 45, "theta_angles": [10, 20]})
    assert b[:, 0].tolist() == [0, 0, 45, 45, 90, 90]
    c = A.cinema_angles({"phi_theta_positions": [[1, 2], [3, 4]]})
    assert c.tolist() == [[1, 2], [3, 4]]
    with pytest.raises(A.AscentError):
        A.cinema_angles({"phi": 3})


def test_png_flip_and_truncation(tmp_path):
    img = np.zeros((3, 4, 4), np.float32)
    img[0, 0] = [1.0, 0.5, 0.2, 1.0]   # bottom-left of the canvas
    img[2, 3] = [0.999, 0.0, 0.0, 0.004]
    p = PNG.save_canvas(tmp_path / "x", img)
    back = decode_png(p.read_bytes())
    assert back.shape == (3, 4, 4)
    assert back[2, 0].tolist() == [255, 127, 51, 255]  # flipped to the bottom row, truncated
    assert back[0, 3].tolist() == [254, 0, 0, 1]


def test_ascent_requires_open_and_reports_errors():
    a = A.Ascent()
    with pytest.raises(A.AscentError):
        a.publish({})
    a.open({"exceptions": "forward"})
    with pytest.raises(A.AscentError):
        a.publish({"coordsets": {}})
    a2 = A.Ascent()
    a2.open()
    a2.execute([{"action": "add_scenes", "scenes": {}}])  # nothing published: caught
    assert a2.info()["errors"]
