"""Host logic of the volume plot, mirroring vtkh::VolumeRenderer.

Reference: src/libs/vtkh/rendering/VolumeRenderer.cpp
  - defaults: 100 samples, alpha points (0, 0.02) and (0, 0.5)     :395-407
    added to the renderer's "Cool to Warm" table (Renderer.cpp:13)
  - CorrectOpacity: a' = 1 - (1 - a)^(10 / samples)                 :448-466
  - DoExecute: one structured domain -> RenderOneDomainPerRank,
    which round-trips the canvas through a uint8 vtkh::Image;
    otherwise RenderMultipleDomainsPerRank with a 1024-entry
    LUT sampled through uint8 (detail::convert_table)               :469-597, 65-90
  - PreExecute: sample distance = |bounds extent| / samples          :600-612
  - SetNumberOfSamples rejects samples < 1                           :622-629
The numeric work happens behind the C ABI (gvr_correct_opacity,
gvr_color_table_sample, gvr_sample_distance).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from . import _native as N
from . import scene as S

LUT_SIZE = 1024


@dataclass
class TransferFunction:
    rgb_pos: np.ndarray
    rgb: np.ndarray
    alpha_pos: np.ndarray
    alpha: np.ndarray

    @staticmethod
    def default() -> "TransferFunction":
        """The table of a volume plot without a `color_table` node: the
        renderer's "Cool to Warm" preset (Renderer.cpp:13) with its opacity
        points (0, 1) and (1, 1), to which VolumeRenderer's constructor adds
        alpha points (0, .02) and then (0, .5) (VolumeRenderer.cpp:402-405); a
        point added at an existing position replaces it, leaving (0, .5) and
        (1, 1)."""
        from . import colortable as CT
        pos, rgb = CT.preset(CT.DEFAULT_NAME)
        alphas = dict(CT.PRESET_ALPHA)
        alphas[0.0] = 0.02
        alphas[0.0] = 0.5
        ax = np.array(sorted(alphas))
        return TransferFunction(np.asarray(pos), np.asarray(rgb), ax, np.array([alphas[x] for x in ax]))


class VolumeRenderer:
    """Parameters of one volume plot; produces the camera-independent render params."""

    def __init__(self):
        self.num_samples = 100
        self.tf = TransferFunction.default()
        self.range = [None, None]
        self.early_term = 0.99
        self.lut_filter = N.LUT_NEAREST
        self.alpha_cull = 0.001

    def set_num_samples(self, n: int) -> None:
        if int(n) < 1:
            raise N.GvrError(N.GVR_ERR_INVALID_ARGUMENT, "Volume rendering samples must be greater than 0")
        self.num_samples = int(n)

    def set_color_table(self, tf: TransferFunction) -> None:
        self.tf = tf

    def set_range(self, lo=None, hi=None) -> None:
        self.range = [lo, hi]

    def resolve_range(self, data_range) -> tuple:
        lo = self.range[0] if self.range[0] is not None else data_range[0]
        hi = self.range[1] if self.range[1] is not None else data_range[1]
        return float(lo), float(hi)

    def lut(self, single_domain: bool) -> np.ndarray:
        corrected = S.correct_opacity(self.tf.alpha, self.num_samples)
        mode = N.UINT8_NONE if single_domain else N.UINT8_ROUND
        return S.color_table_sample(self.tf.rgb_pos, self.tf.rgb, self.tf.alpha_pos, corrected,
                                    LUT_SIZE, mode)

    def params(self, width: int, height: int, bounds, data_range, single_domain: bool, *,
               render_bg=False, bg_color=(0.0, 0.0, 0.0, 1.0), lut=None) -> N.RenderParams:
        if lut is None:
            lut = self.lut(single_domain)
        rng = self.resolve_range(data_range)
        return N.make_params(width, height, S.sample_distance(bounds, self.num_samples), rng, lut,
                             lut_filter=self.lut_filter, alpha_cull=self.alpha_cull,
                             early_term=self.early_term, quantize_uint8=single_domain,
                             render_bg=render_bg, bg_color=bg_color)


def workload_camera(wl) -> N.Camera:
    """Camera of a workload: reset to the scene bounds, then azimuth and elevation
    (the order parse_camera applies them, conduit_to_vtkm_parsing.cpp:164-174)."""
    cam = S.camera_reset_to_bounds(wl.bounds)
    if wl.azimuth:
        S.camera_azimuth(cam, wl.azimuth)
    if wl.elevation:
        S.camera_elevation(cam, wl.elevation)
    return cam


def workload_renderer(wl) -> VolumeRenderer:
    vr = VolumeRenderer()
    vr.set_num_samples(wl.samples)
    vr.set_color_table(TransferFunction(wl.rgb_pos, wl.rgb, wl.alpha_pos, wl.alpha))
    return vr


def workload_params(wl, **kw) -> N.RenderParams:
    vr = workload_renderer(wl)
    for k in ("early_term", "lut_filter"):
        if k in kw:
            setattr(vr, k, kw.pop(k))
    return vr.params(wl.width, wl.height, wl.bounds, wl.scalar_range, wl.single_domain, **kw)


def load_workload(scene: S.Scene, wl) -> None:
    for d in wl.domains:
        if hasattr(d, "conn"):
            scene.add_hex(d.x, d.y, d.z, d.conn, d.field)
        else:
            scene.add_uniform(d.field, d.origin, d.spacing)
