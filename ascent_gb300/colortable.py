"""Colour tables of the volume plot's `color_table` node.

parse_color_table follows Ascent's parse_color_table
(src/libs/ascent/runtimes/flow_filters/ascent_runtime_conduit_to_vtkm_parsing.cpp:199-305):
  - the default table is "cool to warm"; a `name` is accepted when it equals
    one of VTK-m's preset names ignoring case (is_valid_name / string_equal,
    :37-57, :176-197), otherwise the plot keeps "cool to warm" and a message
    says so (:220-234);
  - a preset brings its colours and its opacity points (0, 1) and (1, 1);
  - when `control_points` hold any `rgb` point and no `name` was given, the
    preset's colours are cleared so only the given points remain; its
    opacity points stay (ClearColors touches colours only);
  - rgb colours and alpha values are clamped to [0, 1];
  - a point at an existing position replaces the earlier one;
  - `reverse: "true"` mirrors the colour points (ReverseColors).
Presets:
  - "Cool to Warm" is built from the diverging colour map of K. Moreland,
    "Diverging Color Maps for Scientific Visualization" (ISVC 2009): linear
    interpolation in the Msh space derived from CIELAB between the end points
    (59, 76, 192) and (180, 4, 38), through white at the centre, sampled into
    257 RGB control points;
  - the other 17 presets are the reference's own 256-sample renderings of
    VTK-m's tables (src/docs/sphinx/Actions/color_tables/vtkm/<name>.png,
    decoded into data/vtkm_presets.npz by data/make_presets.py), as 256 RGB
    control points at positions i / 255.
A preset's opacity points (0, 1) and (1, 1) are assumed from the reference's
documentation (a volume plot given a colour table without alpha points
"will look exactly the same as a pseudocolor plot", Actions/Scenes.rst);
VTK-m's preset definitions are not part of the reference tree.
"""
from __future__ import annotations

import math
from pathlib import Path

import numpy as np

from .volume import TransferFunction

DEFAULT_NAME = "cool to warm"

# --- sRGB <-> CIELAB <-> Msh (D65 white), from the published formulas -------


def _srgb_to_linear(c):
    return c / 12.92 if c <= 0.04045 else ((c + 0.055) / 1.055) ** 2.4


def _linear_to_srgb(c):
    c = min(max(c, 0.0), 1.0)
    return 12.92 * c if c <= 0.0031308 else 1.055 * c ** (1 / 2.4) - 0.055


_WHITE = (0.95047, 1.0, 1.08883)


def _rgb_to_lab(rgb):
    r, g, b = (_srgb_to_linear(x) for x in rgb)
    X = 0.4124 * r + 0.3576 * g + 0.1805 * b
    Y = 0.2126 * r + 0.7152 * g + 0.0722 * b
    Z = 0.0193 * r + 0.1192 * g + 0.9505 * b

    def f(t):
        return t ** (1 / 3) if t > 0.008856 else 7.787 * t + 16 / 116

    fx, fy, fz = f(X / _WHITE[0]), f(Y / _WHITE[1]), f(Z / _WHITE[2])
    return 116 * fy - 16, 500 * (fx - fy), 200 * (fy - fz)


def _lab_to_rgb(lab):
    L, a, b = lab
    fy = (L + 16) / 116
    fx = fy + a / 500
    fz = fy - b / 200

    def finv(t):
        return t ** 3 if t ** 3 > 0.008856 else (t - 16 / 116) / 7.787

    X, Y, Z = finv(fx) * _WHITE[0], finv(fy) * _WHITE[1], finv(fz) * _WHITE[2]
    r = 3.2406 * X - 1.5372 * Y - 0.4986 * Z
    g = -0.9689 * X + 1.8758 * Y + 0.0415 * Z
    bb = 0.0557 * X - 0.2040 * Y + 1.0570 * Z
    return tuple(_linear_to_srgb(x) for x in (r, g, bb))


def _lab_to_msh(lab):
    L, a, b = lab
    M = math.sqrt(L * L + a * a + b * b)
    s = math.acos(L / M) if M > 0 else 0.0
    h = math.atan2(b, a)
    return M, s, h


def _msh_to_lab(msh):
    M, s, h = msh
    return M * math.cos(s), M * math.sin(s) * math.cos(h), M * math.sin(s) * math.sin(h)


def _adjust_hue(msh, m_unsat):
    M, s, h = msh
    if M >= m_unsat:
        return h
    spin = s * math.sqrt(m_unsat * m_unsat - M * M) / (M * math.sin(s))
    return h + spin if h > -math.pi / 3 else h - spin


def diverging(rgb1, rgb2, x):
    """Moreland's diverging interpolation between two sRGB colours at x in [0,1]."""
    m1 = _lab_to_msh(_rgb_to_lab(rgb1))
    m2 = _lab_to_msh(_rgb_to_lab(rgb2))
    if m1[1] > 0.05 and m2[1] > 0.05 and abs(m1[2] - m2[2]) > math.pi / 3:
        mmid = max(m1[0], m2[0], 88.0)
        if x < 0.5:
            m2 = (mmid, 0.0, 0.0)
            x = 2 * x
        else:
            m1 = (mmid, 0.0, 0.0)
            x = 2 * x - 1
    if m1[1] < 0.05 and m2[1] > 0.05:
        m1 = (m1[0], m1[1], _adjust_hue(m2, m1[0]))
    elif m2[1] < 0.05 and m1[1] > 0.05:
        m2 = (m2[0], m2[1], _adjust_hue(m1, m2[0]))
    msh = tuple((1 - x) * a + x * b for a, b in zip(m1, m2))
    return _lab_to_rgb(_msh_to_lab(msh))


def _cool_to_warm(n=257):
    c1 = (59 / 255, 76 / 255, 192 / 255)
    c2 = (180 / 255, 4 / 255, 38 / 255)
    xs = np.linspace(0, 1, n)
    return xs, np.array([diverging(c1, c2, float(x)) for x in xs])


# opacity points every preset brings (position -> alpha)
PRESET_ALPHA = {0.0: 1.0, 1.0: 1.0}

_DATA = Path(__file__).resolve().parent / "data" / "vtkm_presets.npz"
_bars: dict | None = None


def _color_bars() -> dict:
    global _bars
    if _bars is None:
        with np.load(_DATA) as d:
            _bars = {k: d[k] for k in d.files}
    return _bars


def preset_names() -> list:
    """VTK-m's preset names, as the reference accepts them."""
    return sorted(_color_bars())


def _string_equal(a: str, b: str) -> bool:
    """string_equal (conduit_to_vtkm_parsing.cpp:37-57): same length, equal
    ignoring case."""
    return len(a) == len(b) and a.lower() == b.lower()


def canonical_name(name: str) -> str | None:
    """The preset name `name` denotes, or None if the reference rejects it."""
    for k in preset_names():
        if _string_equal(k, str(name)):
            return k
    return None


def preset(name: str):
    """(positions, rgb) of a named preset, or None if the name is not one."""
    key = canonical_name(name)
    if key is None:
        return None
    if key == "Cool to Warm":
        return _cool_to_warm()
    bar = _color_bars()[key].astype(np.float64) / 255.0
    return np.arange(len(bar)) / (len(bar) - 1.0), bar


def parse_color_table(node: dict | None, warn=print) -> TransferFunction:
    """A TransferFunction from a volume plot's `color_table` node."""
    node = node or {}
    name = DEFAULT_NAME
    name_provided = "name" in node
    if name_provided:
        if preset(str(node["name"])) is not None:
            name = str(node["name"])
        else:
            warn(f"Invalid color table name '{node['name']}'. Defaulting to {DEFAULT_NAME}")
    pos, rgb = preset(name)
    colors = {float(p): tuple(float(c) for c in col) for p, col in zip(pos, rgb)}
    alphas = dict(PRESET_ALPHA)
    points = node.get("control_points", [])
    if isinstance(points, dict):
        points = list(points.values())
    if any(p.get("type") == "rgb" for p in points) and not name_provided:
        colors = {}
    for p in points:
        if "position" not in p:
            warn("Color map control point must have a position")
            continue
        x = float(p["position"])
        if x > 1.0 or x < 0.0:
            warn(f"Cannot add color map control point position {x}. Must be a normalized scalar.")
        if p.get("type") == "rgb":
            col = [min(1.0, max(0.0, float(c))) for c in list(p["color"])[:3]]
            colors[x] = tuple(col)
        elif p.get("type") == "alpha":
            alphas[x] = min(1.0, max(0.0, float(p["alpha"])))
        else:
            warn(f"Unknown color table control point type {p.get('type')}\n"
                 "Valid types are 'alpha' and 'rgb'")
    if str(node.get("reverse", "false")) == "true":
        colors = {1.0 - x: c for x, c in colors.items()}
    cx = np.array(sorted(colors))
    crgb = np.array([colors[x] for x in cx]).reshape(-1, 3)
    ax = np.array(sorted(alphas))
    av = np.array([alphas[x] for x in ax])
    return TransferFunction(cx, crgb, ax, av)
