"""Host-side pieces of the Ascent front end: colour-table parsing, camera
keys, cinema angles and PNG output (no GPU needed)."""
import math

import numpy as np
import pytest

from ascent_gb300 import _native as N
from ascent_gb300 import ascent as A
from ascent_gb300 import colortable as CT
from ascent_gb300 import png as PNG
from ascent_gb300 import scene as S
from golden.make_golden import decode_png


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
    assert len(t2.rgb_pos) == 33 and [0, 1, 0] in t2.rgb.tolist()
    # reverse mirrors the colour points; an unknown name falls back to the default
    warnings = []
    t3 = CT.parse_color_table({"name": "no such map", "reverse": "true"}, warn=warnings.append)
    assert warnings and np.allclose(t3.rgb[0], CT.preset("cool to warm")[1][-1])
    # the default table keeps VolumeRenderer's constructor opacity
    assert list(CT.parse_color_table({}).alpha) == [0.5]


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
