"""Ascent-shaped front end for the volume plot: open / publish / execute / info / close.

The actions schema is Ascent's (`add_scenes` -> scenes -> plots of
`type: volume` and renders; src/libs/ascent/runtimes/ascent_main_runtime.cpp:
1571-1785 and flow_filters/ascent_runtime_rendering_filters.cpp), and the data
is Blueprint-shaped: one domain or a list / dict of domains, each a dict with
`coordsets`, `topologies`, `fields` (and optional `state/domain_id`), numpy
arrays or torch tensors as values. Supported meshes are those the volume
plot renders: uniform and rectilinear coordsets with uniform / rectilinear
topologies, and explicit coordsets with unstructured `hex` topologies.

What each part mirrors:
  plots        CreatePlot volume branch: samples, color_table, min/max_value
               (rendering_filters.cpp:1565-1831)
  renders      parse_render / parse_camera / parse_image_dims
               (rendering_filters.cpp:330-517, conduit_to_vtkm_parsing.cpp:59-174)
  cinema       CinemaManager phi/theta sweeps (rendering_filters.cpp:519-962),
               rendered in one batched launch
  images       RenderBackground + Save -> PNG (Render.cpp:279-312)
  info         the `images` list of Ascent::info (rendering_filters.cpp:2024-2062)
  errors       `exceptions: forward` raises, the default prints and continues
               (ascent.cpp:218-230)
Annotations: the reference draws them unless a render sets
`annotations: "false"`; this front end draws none unless a render sets
`annotations: "true"`, and then only the body of the volume plot's colour
bar (gvr_canvas_color_bar, at `color_bar_position` or the first default
position, in `fg_color`): the world annotations, tick labels and field name
are VTK-m text rendering, which is not part of this path.
"""
from __future__ import annotations

import math
import os
from pathlib import Path

import numpy as np

from . import _native as N
from . import colortable as CT
from . import png as PNG
from . import scene as S
from . import volume as V

VALID_PLOT_KEYS = {"type", "pipeline", "topology", "field", "points/radius", "points/radius_delta",
                   "min_value", "max_value", "samples", "color_table"}


class AscentError(RuntimeError):
    pass


def _arr(x):
    try:
        import torch
        if isinstance(x, torch.Tensor):
            return x
    except ImportError:  # pragma: no cover
        pass
    return np.asarray(x)


def _domains(data) -> list:
    if isinstance(data, dict) and "coordsets" in data:
        return [data]
    if isinstance(data, dict):
        return list(data.values())
    return list(data)


def _f(node, key, default):
    v = node.get(key, default)
    return float(v)


def _parse_image_dims(render: dict):
    """parse_image_dims (conduit_to_vtkm_parsing.cpp:72-87): 1024 x 1024 default."""
    return int(render.get("image_width", 1024)), int(render.get("image_height", 1024))


def apply_camera(cam: N.Camera, node: dict) -> N.Camera:
    """parse_camera (conduit_to_vtkm_parsing.cpp:91-174), applied in its order.
    Its `ypan` key writes into xpan (:136); that is kept."""
    if "look_at" in node:
        cam.look_at[:] = [float(x) for x in list(node["look_at"])[:3]]
    if "position" in node:
        cam.position[:] = [float(x) for x in list(node["position"])[:3]]
    if "up" in node:
        up = np.array([float(x) for x in list(node["up"])[:3]])
        n = np.linalg.norm(up)
        cam.up[:] = list(up / n if n > 0 else up)
    if "fov" in node:
        cam.fov_y = float(node["fov"])
    if "xpan" in node or "ypan" in node:
        xpan = float(node.get("xpan", 0.0))
        if "ypan" in node:
            xpan = float(node["ypan"])
        cam.xpan += xpan
        cam.ypan += 0.0
    if "zoom" in node:
        # zoom_to_vtkm_zoom gives log4(zoom); the camera's factor becomes 4^that
        cam.zoom *= float(4.0 ** (math.log(float(node["zoom"])) / math.log(4.0)))
    if "near_plane" in node:
        cam.near_plane = float(node["near_plane"])
    if "far_plane" in node:
        cam.far_plane = float(node["far_plane"])
    if "azimuth" in node:
        S.camera_azimuth(cam, float(node["azimuth"]))
    if "elevation" in node:
        S.camera_elevation(cam, float(node["elevation"]))
    return cam


def cinema_angles(render: dict) -> np.ndarray:
    """(phi, theta) pairs of a cinema render (CinemaManager, rendering_filters.cpp:548-677)."""
    if "phi_theta_positions" in render:
        pos = render["phi_theta_positions"]
        pts = [tuple(map(float, p)) for p in (pos.values() if isinstance(pos, dict) else pos)]
        for p in pts:
            if len(p) != 2:
                raise AscentError("Cinema camera phi_theta_positions must be an array of tuples")
        return np.array(pts, dtype=np.float32)

    def axis(name, lo_default, span):
        if name in render:
            n = int(render[name])
            inc = np.float32(span / float(n))
            return [np.float32(lo_default + inc * float(a)) for a in range(n)]
        if f"{name}_angles" in render:
            return [np.float32(x) for x in render[f"{name}_angles"]]
        rng = render.get(f"{name}_range")
        if rng is not None and f"d{name}" in render:
            if rng[0] >= rng[1]:
                raise AscentError(f"Cinema camera {name}_range[0] must be less that {name}_range[1]")
            inc = np.float32(render[f"d{name}"])
            n = int(math.floor((rng[1] - rng[0] + 1.0e-6) / inc)) + 1
            return [np.float32(rng[0] + inc * float(a)) for a in range(n)]
        if rng is not None and f"{name}_num_angles" in render:
            if rng[0] >= rng[1]:
                raise AscentError(f"Cinema camera {name}_range[0] must be less that {name}_range[1]")
            n = int(render[f"{name}_num_angles"])
            inc = np.float32((rng[1] - rng[0]) / float(n - 1))
            return [np.float32(rng[0] + inc * float(a)) for a in range(n)]
        raise AscentError(f"Cinema camera must specify {name} or {name}_range")

    phis = axis("phi", -180.0, 360.0)
    thetas = axis("theta", 0.0, 180.0)
    return np.array([(p, t) for p in phis for t in thetas], dtype=np.float32)


class Ascent:
    """In-situ entry point for the volume plot (Ascent::open/publish/execute/info/close)."""

    def __init__(self):
        self._options = {}
        self._data = None
        self._scenes = {}       # (topology, field) -> gvr Scene
        self._info = {"images": [], "actions": [], "errors": []}
        self._open = False

    # -- lifecycle -------------------------------------------------------
    def open(self, options: dict | None = None) -> None:
        self._options = dict(options or {})
        self._device = int(self._options.get("device", 0))
        self._dir = Path(self._options.get("default_dir", "."))
        self._open = True

    def close(self) -> None:
        for sc in self._scenes.values():
            sc.close()
        self._scenes = {}
        self._data = None
        self._open = False

    def info(self) -> dict:
        return self._info

    # -- data ------------------------------------------------------------
    def publish(self, data) -> None:
        self._guard(self._publish, data)

    def _publish(self, data) -> None:
        doms = _domains(data)
        if not doms:
            raise AscentError("publish: no domains")
        for d in doms:
            for key in ("coordsets", "topologies", "fields"):
                if key not in d:
                    raise AscentError(f"publish: domain is missing '{key}'")
        old = self._data
        self._data = doms
        # same mesh shapes and field keys: keep the device scenes, swap fields
        if old is not None and len(old) == len(doms) and self._scenes:
            try:
                for (topo, field), sc in self._scenes.items():
                    for i, d in enumerate(doms):
                        sc.update_field(i, self._field_values(d, field, topo))
                return
            except Exception:
                pass
        for sc in self._scenes.values():
            sc.close()
        self._scenes = {}

    def _cycle(self) -> int:
        d = self._data[0] if self._data else {}
        return int(d.get("state", {}).get("cycle", 0))

    def _time(self) -> float:
        d = self._data[0] if self._data else {}
        return float(d.get("state", {}).get("time", 0.0))

    def _field_values(self, dom, field, topo):
        f = dom["fields"][field]
        return _arr(f["values"])

    def _resolve_topology(self, field, topo):
        dom = self._data[0]
        if field not in dom["fields"]:
            known = ", ".join(dom["fields"].keys())
            raise AscentError(f"Unknown field '{field}'. Known fields: {known}")
        ftopo = dom["fields"][field].get("topology")
        if topo and ftopo and topo != ftopo:
            raise AscentError(f"field '{field}' lives on topology '{ftopo}', not '{topo}'")
        return ftopo or topo or next(iter(dom["topologies"]))

    def _scene_for(self, field, topo) -> S.Scene:
        key = (topo, field)
        if key in self._scenes:
            return self._scenes[key]
        sc = S.Scene(self._device)
        try:
            for dom in self._data:
                self._add_domain(sc, dom, field, topo)
        except Exception:
            sc.close()
            raise
        self._scenes[key] = sc
        return sc

    def _add_domain(self, sc: S.Scene, dom, field, topo_name):
        topo = dom["topologies"][topo_name]
        cset = dom["coordsets"][topo["coordset"]]
        fnode = dom["fields"][field]
        assoc = {"vertex": N.ASSOC_VERTEX, "element": N.ASSOC_ELEMENT}.get(fnode.get("association", "vertex"))
        if assoc is None:
            raise AscentError(f"field association '{fnode.get('association')}' is not supported")
        vals = _arr(fnode["values"])
        ctype = cset["type"]
        if ctype == "uniform":
            dims = cset["dims"]
            nx, ny, nz = int(dims["i"]), int(dims["j"]), int(dims.get("k", 1))
            if nz < 2:
                raise AscentError("the volume plot needs a 3D mesh")
            o = cset.get("origin", {})
            s = cset.get("spacing", {})
            origin = (_f(o, "x", 0), _f(o, "y", 0), _f(o, "z", 0))
            spacing = (_f(s, "dx", 1), _f(s, "dy", 1), _f(s, "dz", 1))
            shape = (nz, ny, nx) if assoc == N.ASSOC_VERTEX else (nz - 1, ny - 1, nx - 1)
            sc.add_uniform(vals.reshape(shape), origin, spacing, association=assoc)
        elif ctype == "rectilinear":
            xv = np.asarray(cset["values"]["x"], dtype=np.float64)
            yv = np.asarray(cset["values"]["y"], dtype=np.float64)
            zv = np.asarray(cset["values"]["z"], dtype=np.float64)
            shape = (len(zv), len(yv), len(xv))
            if assoc == N.ASSOC_ELEMENT:
                shape = tuple(n - 1 for n in shape)
            sc.add_rectilinear(vals.reshape(shape), xv, yv, zv, association=assoc)
        elif ctype == "explicit":
            if topo.get("type") != "unstructured" or topo.get("elements", {}).get("shape") != "hex":
                raise AscentError("explicit coordsets are rendered for unstructured hex topologies")
            v = cset["values"]
            conn = _arr(topo["elements"]["connectivity"])
            sc.add_hex(_arr(v["x"]), _arr(v["y"]), _arr(v["z"]), conn, vals, association=assoc)
        else:
            raise AscentError(f"coordset type '{ctype}' is not supported by the volume plot")

    # -- actions ---------------------------------------------------------
    def execute(self, actions) -> None:
        self._guard(self._execute, actions)

    def _guard(self, fn, *args):
        if not self._open:
            raise AscentError("Ascent is not open")
        try:
            fn(*args)
        except Exception as e:
            if self._options.get("exceptions", "catch") == "forward":
                raise
            msg = f"[ascent_gb300 error] {e}"
            self._info["errors"].append(msg)
            print(msg)

    def _execute(self, actions) -> None:
        if isinstance(actions, dict):
            actions = list(actions.values())
        self._info = {"images": [], "actions": actions, "errors": self._info.get("errors", [])}
        if self._data is None:
            raise AscentError("execute: nothing published")
        for act in actions:
            name = act.get("action")
            if name == "add_scenes":
                for sname, scene in act.get("scenes", {}).items():
                    self._run_scene(sname, scene)
            else:
                raise AscentError(f"action '{name}' is outside the volume-plot path")

    def _run_scene(self, sname, scene: dict) -> None:
        plots = scene.get("plots", {})
        vols = [(pn, p) for pn, p in plots.items() if p.get("type") == "volume"]
        others = [p.get("type") for p in plots.values() if p.get("type") != "volume"]
        if others:
            raise AscentError(f"plot types {others} are outside the volume-plot path")
        if len(vols) > 1:
            raise AscentError("A scene holds at most one volume plot")  # Scene.cpp:84-87
        if not vols:
            return
        pname, plot = vols[0]
        self._check_plot(plot)
        field = plot["field"]
        topo = self._resolve_topology(field, plot.get("topology"))
        sc = self._scene_for(field, topo)
        vr = V.VolumeRenderer()
        if "samples" in plot:
            vr.set_num_samples(int(plot["samples"]))
        if "color_table" in plot:
            vr.set_color_table(CT.parse_color_table(plot["color_table"]))
        vr.set_range(float(plot["min_value"]) if "min_value" in plot else None,
                     float(plot["max_value"]) if "max_value" in plot else None)
        bounds = sc.bounds()
        data_range = sc.scalar_range()
        single = sc.num_domains == 1 and not sc._hex_cells
        renders = scene.get("renders")
        if not renders:
            prefix = scene.get("image_prefix", scene.get("image_name", f"{sname}_%04d"))
            renders = {"default": {"image_prefix": prefix}}
        for rname, render in renders.items():
            self._run_render(sname, rname, render, sc, vr, bounds, data_range, single)

    def _check_plot(self, plot: dict) -> None:
        """CreatePlot::verify_params (rendering_filters.cpp:1565-1625)."""
        if "field" not in plot:
            raise AscentError("volume plot: missing required 'field'")

        def flat(node, prefix=""):
            for k, v in node.items():
                path = prefix + k
                if isinstance(v, dict) and path != "color_table":
                    yield from flat(v, path + "/")
                else:
                    yield path
        bad = [p for p in flat(plot) if p not in VALID_PLOT_KEYS]
        if bad:
            raise AscentError(f"volume plot: unknown parameters {bad}")

    def _image_name(self, render: dict, default: str) -> str:
        name = render.get("image_name", render.get("image_prefix", default))
        if "%" in name:
            name = name % self._cycle()
        return name

    def _params(self, vr, render, bounds, data_range, single):
        w, h = _parse_image_dims(render)
        bg = [0.0, 0.0, 0.0, 1.0]
        if "bg_color" in render:
            c = list(render["bg_color"])
            if len(c) != 3:
                raise AscentError("render/bg_color node must be an array of 3 values")
            bg = [float(c[0]), float(c[1]), float(c[2]), 1.0]
        render_bg = str(render.get("render_bg", "true")) != "false"
        return vr.params(w, h, bounds, data_range, single, render_bg=render_bg, bg_color=bg)

    def _color_bars(self, render: dict, vr, rgba) -> None:
        """The colour bar of the volume plot, when the render asks for
        annotations explicitly (RenderScreenAnnotations, Render.cpp:205-227;
        color_bar_position and fg_color parsing, rendering_filters.cpp:453-512)."""
        if str(render.get("annotations", "false")) != "true" or \
                str(render.get("screen_annotations", "true")) == "false":
            return
        box = PNG.DEFAULT_COLOR_BAR_BOXES[0]
        if "color_bar_position" in render:
            pos = np.asarray(render["color_bar_position"], dtype=np.float64).ravel()
            if pos.size == 0 or pos.size % 4 != 0:
                raise AscentError("render/color_bar_position must be an array of 4 values for each color bar")
            box = tuple(float(x) for x in pos[:4])
        fg = (1.0, 1.0, 1.0, 1.0)
        if "fg_color" in render:
            c = list(render["fg_color"])
            if len(c) != 3:
                raise AscentError("render/fg_color node must be an array of 3 values")
            fg = (float(c[0]), float(c[1]), float(c[2]), 1.0)
        tf = vr.tf
        lut = S.color_table_sample(tf.rgb_pos, tf.rgb, tf.alpha_pos, tf.alpha, V.LUT_SIZE, N.UINT8_NONE)
        if getattr(rgba, "dim", None) and rgba.dim() == 4:
            for img in rgba:
                PNG.draw_color_bar(img, lut, box, fg)
        else:
            PNG.draw_color_bar(rgba, lut, box, fg)

    def _run_render(self, sname, rname, render, sc, vr, bounds, data_range, single):
        params = self._params(vr, render, bounds, data_range, single)
        name = self._image_name(render, f"{sname}_{rname}_%04d")
        if render.get("type") == "cinema":
            self._run_cinema(sname, rname, render, sc, vr, params, bounds, name)
            return
        cam = S.camera_reset_to_bounds(bounds)
        if "camera" in render:
            apply_camera(cam, render["camera"])
        rgba, depth = sc.render(cam, params, device_out=True)
        self._color_bars(render, vr, rgba)
        path = PNG.save_canvas(self._dir / name, rgba)
        self._info["images"].append({"image_name": str(path), "image_width": params.width,
                                     "image_height": params.height, "camera": cam.as_dict(),
                                     "scene_bounds": list(map(float, bounds)), "scene": sname,
                                     "render": rname})

    def _run_cinema(self, sname, rname, render, sc, vr, params, bounds, name):
        angles = cinema_angles(render)
        cams = S.cinema_cameras(bounds, angles)
        db = render.get("db_name", name)
        base = self._dir / "cinema_databases" / db / f"{self._time():g}"
        rgba, _ = sc.render_batch(cams, params, device_out=True)
        self._color_bars(render, vr, rgba)
        lines = ["phi,theta,time,FILE"]
        for (phi, theta), img, cam in zip(angles, rgba, cams):
            fname = f"{_angle(phi)}_{_angle(theta)}_{name}.png"
            path = PNG.save_canvas(base / fname, img)
            lines.append(f"{_angle(phi)},{_angle(theta)},{self._time():g},{self._time():g}/{fname}")
            self._info["images"].append({"image_name": str(path), "image_width": params.width,
                                         "image_height": params.height, "camera": cam.as_dict(),
                                         "scene_bounds": list(map(float, bounds)), "scene": sname,
                                         "render": rname, "phi": float(phi), "theta": float(theta)})
        (self._dir / "cinema_databases" / db).mkdir(parents=True, exist_ok=True)
        (self._dir / "cinema_databases" / db / "data.csv").write_text("\n".join(lines) + "\n")


def _angle(a: float) -> str:
    """Angles in cinema file names: integers without a fraction."""
    a = float(a)
    return str(int(round(a))) if abs(a - round(a)) < 1e-6 else f"{a:g}"


def about() -> dict:
    return {"library": str(N.LIB_PATH), "version": N.lib().gvr_version(), "cwd": os.getcwd()}
