"""Colour bar body on the canvas (gvr_canvas_color_bar): the coloured part
of the bars Render::RenderScreenAnnotations draws for a plot's colour table
(vtkh/rendering/Render.cpp:205-227), at the Annotator's default positions
(Annotator.cpp:15-24) or a render's `color_bar_position`. Tick labels and
the field name (VTK-m text) are not drawn.

CPU: argument checks. GPU: the device drawing against a numpy statement of
the same rule (pixel rectangle of the box, table entry by position along
the long axis, opaque, outline in the foreground colour), on host and
device canvases, clipped and horizontal boxes; the Ascent front end draws
the bar only when a render asks for annotations."""
import ctypes as C

import numpy as np
import pytest

from ascent_gb300 import _native as N
from ascent_gb300 import png as PNG


def numpy_bar(canvas, lut, box, fg):
    out = canvas.copy()
    h, w, _ = out.shape

    b = [float(np.float32(v)) for v in box]   # the box as the C ABI receives it

    def px(v, n):   # exact in double
        return int(np.floor((v + 1.0) * 0.5 * n + 0.5))
    x0, x1 = max(0, px(b[0], w)), min(w, px(b[1], w))
    y0, y1 = max(0, px(b[2], h)), min(h, px(b[3], h))
    if x1 - x0 < 1 or y1 - y0 < 1:
        return out
    bw, bh = x1 - x0, y1 - y0
    vertical = (b[3] - b[2]) * h >= (b[1] - b[0]) * w
    lut = np.asarray(lut, np.float32).reshape(-1, 4)
    n = len(lut)
    for ly in range(bh):
        for lx in range(bw):
            if lx in (0, bw - 1) or ly in (0, bh - 1):
                c = np.asarray(fg, np.float32)
            else:
                t = np.float32((ly + 0.5) / bh if vertical else (lx + 0.5) / bw)
                e = lut[min(int(t * np.float32(n)), n - 1)]
                c = np.array([e[0], e[1], e[2], 1.0], np.float32)
            out[y0 + ly, x0 + lx] = c
    return out


def test_color_bar_argument_checks():
    canvas = np.zeros((8, 8, 4), np.float32)
    lut = np.zeros((16, 4), np.float32)
    f = N.lib().gvr_canvas_color_bar
    box = (C.c_float * 4)(-0.5, 0.5, -0.5, 0.5)
    fg = (C.c_float * 4)(1, 1, 1, 1)
    lp = N.fptr(lut)
    cv = C.c_void_p(canvas.ctypes.data)
    assert f(cv, 0, 8, lp, 16, box, fg, N.MEM_HOST, None) == N.GVR_ERR_INVALID_ARGUMENT
    assert f(cv, 8, 8, lp, 1, box, fg, N.MEM_HOST, None) == N.GVR_ERR_INVALID_ARGUMENT
    assert f(cv, 8, 8, lp, 16, (C.c_float * 4)(0.5, -0.5, 0, 1), fg, N.MEM_HOST, None) == N.GVR_ERR_INVALID_ARGUMENT
    assert f(cv, 8, 8, lp, 16, (C.c_float * 4)(0, float("nan"), 0, 1), fg, N.MEM_HOST, None) == \
        N.GVR_ERR_INVALID_ARGUMENT
    assert f(cv, 8, 8, lp, 16, box, fg, 9, None) == N.GVR_ERR_INVALID_ARGUMENT
    assert f(None, 8, 8, lp, 16, box, fg, N.MEM_HOST, None) == N.GVR_ERR_INVALID_ARGUMENT
    with pytest.raises(ValueError):
        PNG.draw_color_bar(np.zeros((8, 8, 3), np.float32), lut)


@pytest.mark.gpu
@pytest.mark.parametrize("box", [PNG.DEFAULT_COLOR_BAR_BOXES[0], PNG.DEFAULT_COLOR_BAR_BOXES[3],
                                 (-0.6, 0.6, -0.9, -0.8), (0.9, 1.4, -0.2, 0.7)])
def test_color_bar_matches_numpy_rule(box):
    import torch
    rng = np.random.default_rng(5)
    canvas = rng.uniform(0, 1, (90, 120, 4)).astype(np.float32)
    x = np.linspace(0, 1, 37)
    lut = np.stack([x, 1 - x, x * x, 0.2 * x], 1).astype(np.float32)
    fg = (0.3, 0.6, 0.9, 1.0)
    want = numpy_bar(canvas, lut, box, fg)
    got = PNG.draw_color_bar(canvas.copy(), lut, box, fg)
    np.testing.assert_array_equal(got, want)
    t = torch.from_numpy(canvas).cuda()
    PNG.draw_color_bar(t, lut, box, fg)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(t.cpu().numpy(), want)
    assert not np.array_equal(want, canvas)


@pytest.mark.gpu
def test_front_end_draws_the_bar_only_when_asked(tmp_path):
    from ascent_gb300 import Ascent
    from ascent_gb300 import workloads as W
    from ascent_gb300.png import decode_png
    wl = W.plain_small(n=33, width=8, height=8)
    tf = {"name": "Viridis", "control_points": [{"type": "alpha", "position": 0.0, "alpha": 0.0},
                                                 {"type": "alpha", "position": 1.0, "alpha": 0.5}]}

    def run(extra):
        a = Ascent()
        a.open({"default_dir": str(tmp_path), "exceptions": "forward"})
        a.publish(W.to_blueprint(wl))
        render = {"image_width": 128, "image_height": 96, "image_prefix": "cb_%04d"}
        render.update(extra)
        a.execute([{"action": "add_scenes", "scenes": {"s1": {
            "plots": {"p1": {"type": "volume", "field": "braid", "color_table": tf}},
            "renders": {"r1": render}}}}])
        img = decode_png(open(a.info()["images"][0]["image_name"], "rb").read())
        a.close()
        return img
    plain = run({})
    bar = run({"annotations": "true", "fg_color": [1.0, 0.0, 0.0]})
    diff = np.any(plain != bar, axis=-1)
    # PNG rows run top down; the default box spans x in [0.84, 0.92], y in [0.1, 0.8]
    ys, xs = np.nonzero(diff)
    assert diff.any() and xs.min() >= int(0.92 * 64) - 1 and xs.max() <= int(0.96 * 128) + 1
    assert ys.max() <= 96 // 2
    assert tuple(bar[ys.min(), xs.min()]) == (255, 0, 0, 255)   # outline in fg
    with pytest.raises(Exception):
        run({"annotations": "true", "color_bar_position": [0.1, 0.2, 0.3]})
