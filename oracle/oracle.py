"""ctypes binding of the CPU oracle (``oracle/gvr_oracle.c``).

TEST INFRASTRUCTURE ONLY: loaded by tests/, by ``__graft_entry__.smoke()``
to compare against, and by bench.py's CPU-baseline arm. The product library
never imports this module.

Two builds of one C source:
  precision=64 -> liboracle64.so, FP64 arithmetic (the accuracy oracle)
  precision=32 -> liboracle32.so, FP32 arithmetic (the timed CPU port)
and, when the reference sources are present at build time,
``_ref/libapcomp_ref.so``: the reference's own partial compositor.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

# ctypes mirrors of the gvr.h structs the oracle's C entry points take. They
# are declared here, not imported from the product package, so that the CPU
# arm of the benchmark never maps the product library. Structures of the
# same layout built elsewhere (the product binding's) are accepted too: the
# entry points take their address.


class Camera(C.Structure):
    _fields_ = [("position", C.c_float * 3), ("look_at", C.c_float * 3), ("up", C.c_float * 3),
                ("fov_y", C.c_float), ("zoom", C.c_float), ("xpan", C.c_float), ("ypan", C.c_float),
                ("near_plane", C.c_float), ("far_plane", C.c_float)]


class RenderParams(C.Structure):
    _fields_ = [("width", C.c_int), ("height", C.c_int), ("sample_dist", C.c_float),
                ("scalar_min", C.c_float), ("scalar_max", C.c_float),
                ("lut_rgba", C.POINTER(C.c_float)), ("lut_size", C.c_int), ("lut_filter", C.c_int),
                ("alpha_cull", C.c_float), ("early_term", C.c_float), ("quantize_uint8", C.c_int),
                ("render_bg", C.c_int), ("bg_color", C.c_float * 4), ("clear_depth", C.c_float)]


class ColorTable(C.Structure):
    _fields_ = [("n_rgb", C.c_int), ("rgb_pos", C.POINTER(C.c_double)), ("rgb", C.POINTER(C.c_double)),
                ("n_alpha", C.c_int), ("alpha_pos", C.POINTER(C.c_double)),
                ("alpha", C.POINTER(C.c_double))]


LUT_NEAREST, LUT_LINEAR = 0, 1
UINT8_NONE, UINT8_ROUND, UINT8_TRUNCATE = 0, 1, 2


def dptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def fptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_float))


def _addr(obj, kind) -> int:
    """Address of a struct laid out as `kind` (this module's or a same-layout mirror)."""
    if not isinstance(obj, C.Structure) or C.sizeof(obj) != C.sizeof(kind) or \
            [f[0] for f in type(obj)._fields_] != [f[0] for f in kind._fields_]:
        raise TypeError(f"expected a {kind.__name__} structure, got {type(obj).__name__}")
    return C.addressof(obj)


HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
REF = HERE / "_ref"

PARTIAL_DTYPE = np.dtype([("pixel_id", "<i4"), ("depth", "<f4"), ("rgb", "<f4", (3,)),
                          ("alpha", "<f4")])

_libs: dict = {}


def build(with_reference: bool | None = None) -> None:
    """make the oracle; also the apcomp reference when its sources exist
    (oracle/Makefile's REF, overridden by GVR_REFERENCE_ROOT)."""
    subprocess.run(["make", "-s", "-C", str(HERE), "all"], check=True)
    if with_reference is None:
        subprocess.run(["make", "-s", "-C", str(HERE), "ref-if-present"], check=True)
    elif with_reference:
        subprocess.run(["make", "-s", "-C", str(HERE), "ref"], check=True)


def load(precision: int = 64) -> C.CDLL:
    if precision in _libs:
        return _libs[precision]
    path = BUILD / f"liboracle{precision}.so"
    if not path.exists():
        build(with_reference=False)
    lib = C.CDLL(str(path))
    i, d, f, vp = C.c_int, C.c_double, C.c_float, C.c_void_p
    P = C.POINTER
    lib.or_correct_opacity.argtypes = [P(d), i, i, P(d)]
    lib.or_sample_distance.argtypes = [P(d), i]
    lib.or_sample_distance.restype = f
    # struct arguments are passed by address (void *): a Camera, RenderParams
    # or ColorTable of this module or any structure of the same layout
    lib.or_color_table_sample.argtypes = [vp, i, i, P(f)]
    lib.or_camera_reset_to_bounds.argtypes = [vp, P(d)]
    lib.or_camera_azimuth.argtypes = [vp, d]
    lib.or_camera_elevation.argtypes = [vp, d]
    lib.or_cinema_cameras.argtypes = [P(d), P(f), i, vp]
    lib.or_visibility_order.argtypes = [vp, P(d), i, P(i)]
    lib.or_composite_partials.argtypes = [i, P(i), vp, vp]
    lib.or_zbuffer_composite.argtypes = [i, P(vp), P(vp), i, i, P(f), P(f)]
    lib.or_scene_new.restype = vp
    lib.or_scene_free.argtypes = [vp]
    lib.or_scene_add_uniform.argtypes = [vp, P(i), P(d), P(d), P(f), i]
    lib.or_scene_add_rectilinear.argtypes = [vp, P(i), P(d), P(d), P(d), P(f), i]
    lib.or_scene_add_hex.argtypes = [vp, C.c_int64, P(f), P(f), P(f), C.c_int64, P(i), P(f), i]
    lib.or_hex_bvh.argtypes = [vp, i, vp, vp, vp, vp, vp, vp]
    lib.or_hex_locate.argtypes = [vp, i, P(f), i, P(i), P(f)]
    lib.or_render.argtypes = [vp, vp, vp, P(f), P(f), P(C.c_uint64)]
    lib.or_render_rows.argtypes = [vp, vp, vp, i, i, P(f), P(f), P(C.c_uint64)]
    lib.or_render_over.argtypes = [vp, vp, vp, P(f), P(f), P(C.c_uint64)]
    lib.or_num_threads.restype = i
    _libs[precision] = lib
    return lib


def load_apcomp_reference():
    """The reference's compiled partial compositor, or None if it was not built."""
    path = REF / "libapcomp_ref.so"
    if not path.exists():
        return None
    lib = C.CDLL(str(path))
    lib.ref_apcomp_composite.argtypes = [C.c_int, C.POINTER(C.c_int), C.c_void_p, C.c_void_p]
    lib.ref_apcomp_composite.restype = C.c_int
    return lib


def _ints(a):
    a = np.ascontiguousarray(a, dtype=np.int32)
    return a, a.ctypes.data_as(C.POINTER(C.c_int))


class OracleScene:
    """Domains as the oracle sees them; field arrays are kept alive here."""

    def __init__(self, precision: int = 64):
        self.lib = load(precision)
        self.handle = self.lib.or_scene_new()
        self._keep = []

    def add_uniform(self, dims, origin, spacing, field, assoc=0) -> int:
        dims_a, dims_p = _ints(dims)
        o = np.ascontiguousarray(origin, dtype=np.float64)
        s = np.ascontiguousarray(spacing, dtype=np.float64)
        f = np.ascontiguousarray(field, dtype=np.float32).ravel()
        self._keep += [dims_a, o, s, f]
        return self.lib.or_scene_add_uniform(self.handle, dims_p, dptr(o), dptr(s), fptr(f), int(assoc))

    def add_rectilinear(self, x, y, z, field, assoc=0) -> int:
        xs = [np.ascontiguousarray(c, dtype=np.float64) for c in (x, y, z)]
        dims_a, dims_p = _ints([len(c) for c in xs])
        f = np.ascontiguousarray(field, dtype=np.float32).ravel()
        self._keep += [dims_a, f, *xs]
        return self.lib.or_scene_add_rectilinear(self.handle, dims_p, dptr(xs[0]), dptr(xs[1]),
                                                 dptr(xs[2]), fptr(f), int(assoc))

    def add_hex(self, x, y, z, conn, field, assoc=0) -> int:
        xs = [np.ascontiguousarray(c, dtype=np.float32) for c in (x, y, z)]
        cn = np.ascontiguousarray(conn, dtype=np.int32).ravel()
        f = np.ascontiguousarray(field, dtype=np.float32).ravel()
        self._keep += [*xs, cn, f]
        self._ncells = getattr(self, "_ncells", {})
        did = self.lib.or_scene_add_hex(self.handle, len(xs[0]), fptr(xs[0]), fptr(xs[1]), fptr(xs[2]),
                                        len(cn) // 8, cn.ctypes.data_as(C.POINTER(C.c_int)), fptr(f),
                                        int(assoc))
        self._ncells[did] = len(cn) // 8
        return did

    def hex_bvh(self, dom: int) -> dict:
        n = self._ncells[dom]
        out = {"codes": np.zeros(n, np.uint32), "ids": np.zeros(n, np.uint32),
               "left": np.zeros(max(n - 1, 1), np.int32), "right": np.zeros(max(n - 1, 1), np.int32),
               "parent": np.zeros(max(2 * n - 1, 1), np.int32),
               "inner_box": np.zeros((max(n - 1, 1), 6), np.float32)}
        self.lib.or_hex_bvh(self.handle, dom, *[out[k].ctypes.data for k in
                            ("codes", "ids", "left", "right", "parent", "inner_box")])
        return out

    def hex_locate(self, dom: int, points):
        p = np.ascontiguousarray(points, dtype=np.float32).reshape(-1, 3)
        cells = np.zeros(len(p), np.int32)
        rst = np.zeros((len(p), 3), np.float32)
        self.lib.or_hex_locate(self.handle, dom, fptr(p), len(p), cells.ctypes.data_as(C.POINTER(C.c_int)),
                               fptr(rst))
        return cells, rst

    def render(self, cam: Camera, params: RenderParams):
        w, h = params.width, params.height
        rgba = np.zeros((h, w, 4), dtype=np.float32)
        depth = np.zeros((h, w), dtype=np.float32)
        n = C.c_uint64(0)
        rc = self.lib.or_render(self.handle, _addr(cam, Camera), _addr(params, RenderParams),
                                fptr(rgba), fptr(depth), C.byref(n))
        if rc != 0:
            raise RuntimeError(f"oracle render failed with status {rc}")
        return rgba, depth, int(n.value)

    def render_over(self, cam: Camera, params: RenderParams, canvas_rgba, canvas_depth):
        """Render over an opaque canvas (copies of the inputs are returned)."""
        rgba = np.array(canvas_rgba, dtype=np.float32, copy=True, order="C")
        depth = np.array(canvas_depth, dtype=np.float32, copy=True, order="C")
        n = C.c_uint64(0)
        rc = self.lib.or_render_over(self.handle, _addr(cam, Camera), _addr(params, RenderParams),
                                     fptr(rgba), fptr(depth), C.byref(n))
        if rc != 0:
            raise RuntimeError(f"oracle render failed with status {rc}")
        return rgba, depth, int(n.value)

    def render_rows(self, cam: Camera, params: RenderParams, row0: int, row1: int, rgba, depth) -> int:
        """Render rows [row0, row1) into caller buffers; returns the sample count."""
        n = C.c_uint64(0)
        rc = self.lib.or_render_rows(self.handle, _addr(cam, Camera), _addr(params, RenderParams),
                                     int(row0), int(row1), fptr(rgba), fptr(depth), C.byref(n))
        if rc != 0:
            raise RuntimeError(f"oracle render failed with status {rc}")
        return int(n.value)

    def close(self):
        if self.handle:
            self.lib.or_scene_free(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def composite_partials(images, precision: int = 64, reference: bool = False) -> np.ndarray:
    """Composite a list of PARTIAL_DTYPE arrays; reference=True uses apcomp."""
    counts_a, counts_p = _ints([len(im) for im in images])
    flat = np.ascontiguousarray(np.concatenate(images) if images else np.zeros(0, PARTIAL_DTYPE),
                                dtype=PARTIAL_DTYPE)
    out = np.zeros(max(len(flat), 1), dtype=PARTIAL_DTYPE)
    if reference:
        lib = load_apcomp_reference()
        if lib is None:
            raise RuntimeError("apcomp reference library was not built")
        n = lib.ref_apcomp_composite(len(images), counts_p, flat.ctypes.data, out.ctypes.data)
    else:
        n = load(precision).or_composite_partials(len(images), counts_p, flat.ctypes.data,
                                                  out.ctypes.data)
    return out[:n].copy()


def zbuffer_composite(rgba_images, depth_images):
    """Renderer::Composite in Z_BUFFER_SURFACE mode (or_zbuffer_composite):
    lists of (H, W, 4) / (H, W) float arrays -> the composited canvas."""
    cols = [np.ascontiguousarray(c, dtype=np.float32) for c in rgba_images]
    deps = [np.ascontiguousarray(d, dtype=np.float32) for d in depth_images]
    h, w = cols[0].shape[:2]
    out = np.zeros((h, w, 4), np.float32)
    out_d = np.zeros((h, w), np.float32)
    cp = (C.c_void_p * len(cols))(*[c.ctypes.data for c in cols])
    dp = (C.c_void_p * len(deps))(*[d.ctypes.data for d in deps])
    rc = load(64).or_zbuffer_composite(len(cols), cp, dp, w, h, fptr(out), fptr(out_d))
    if rc != 0:
        raise RuntimeError(f"oracle z-buffer composite failed with status {rc}")
    return out, out_d


def composite_partials_f32(images) -> np.ndarray:
    """FP32 restatement of PartialCompositor::composite in the reference's
    output order (vtkh/compositing/PartialCompositor.cpp:331-490): records
    sorted by (pixel_id, depth) with the input position as the final key;
    single-record pixels first, then blended pixels, each in pixel order;
    blend of VolumePartial::blend (VolumePartial.hpp:53-62) as separately
    rounded float32 operations (numpy never fuses a multiply-add).

    Vectorised over pixels: pass k blends every pixel's k-th record."""
    flat = (np.concatenate([np.asarray(im, PARTIAL_DTYPE) for im in images]) if len(images)
            else np.zeros(0, PARTIAL_DTYPE))
    n = len(flat)
    if n == 0:
        return np.zeros(0, PARTIAL_DTYPE)
    order = np.lexsort((np.arange(n), flat["depth"], flat["pixel_id"]))
    s = flat[order]
    pid = s["pixel_id"]
    head = np.ones(n, bool)
    head[1:] = pid[1:] != pid[:-1]
    starts = np.nonzero(head)[0]
    counts = np.diff(np.append(starts, n))
    seg = np.cumsum(head) - 1
    rank = np.arange(n) - starts[seg]
    res = s[starts].copy()
    rgb, a = res["rgb"].copy(), res["alpha"].copy()
    one = np.float32(1.0)
    for k in range(1, int(counts.max())):
        m = rank == k
        g = seg[m]
        o = s[m]
        live = (a[g] < one) & (o["alpha"] != np.float32(0.0))
        g, o = g[live], o[live]
        op = (one - a[g]).astype(np.float32)
        rgb[g] = (rgb[g] + (op[:, None] * o["rgb"]).astype(np.float32)).astype(np.float32)
        na = (a[g] + (op * o["alpha"]).astype(np.float32)).astype(np.float32)
        a[g] = np.minimum(na, one)
    res["rgb"], res["alpha"] = rgb, a
    return np.concatenate([res[counts == 1], res[counts > 1]])


HEX_FACES = np.array([[0, 3, 7, 4], [1, 2, 6, 5], [0, 1, 5, 4], [3, 2, 6, 7], [0, 1, 2, 3],
                      [4, 5, 6, 7]])


def hex_face_neighbors(conn) -> np.ndarray:
    """Face-neighbour table of a hex mesh, (n_cells, 6): the cell across each
    VTK hexahedron face (r=0, r=1, s=0, s=1, t=0, t=1), -1 on the boundary.
    Faces are identified by their three smallest node ids (two faces of a
    conforming mesh share at most an edge) and paired by a stable sort of
    the faces by that triple: a face takes the next face in the order when
    it has the same triple, else the previous one."""
    conn = np.asarray(conn, dtype=np.int64).reshape(-1, 8)
    nc = len(conn)
    trip = np.sort(conn[:, HEX_FACES], axis=2)[:, :, :3].reshape(-1, 3)
    order = np.lexsort((np.arange(6 * nc), trip[:, 2], trip[:, 1], trip[:, 0]))
    t = trip[order]
    same_next = np.zeros(6 * nc, bool)
    same_next[:-1] = (t[1:] == t[:-1]).all(axis=1)
    same_prev = np.zeros(6 * nc, bool)
    same_prev[1:] = same_next[:-1]
    other = np.full(6 * nc, -1, np.int64)
    idx = np.arange(6 * nc)
    other[same_prev] = order[idx[same_prev] - 1] // 6
    other[same_next] = order[idx[same_next] + 1] // 6
    nbr = np.full(6 * nc, -1, np.int64)
    nbr[order] = other
    return nbr.reshape(nc, 6).astype(np.int32)


def num_threads(precision: int = 32) -> int:
    return int(load(precision).or_num_threads())


# ---------------------------------------------------------------------------
# Render set-up restated on the oracle side: the camera, the opacity-corrected
# and sampled transfer function and the sample distance of a volume plot,
# built with the oracle's own C functions (never the product library's), so
# that a fault in the product's host set-up shows up as an image difference.
# ---------------------------------------------------------------------------

LUT_SIZE = 1024   # detail::convert_table samples 1024 entries (VolumeRenderer.cpp:65-90)


def correct_opacity(alpha, num_samples: int) -> np.ndarray:
    """VolumeRenderer::CorrectOpacity (VolumeRenderer.cpp:448-466)."""
    a = np.ascontiguousarray(alpha, dtype=np.float64)
    out = np.empty_like(a)
    if load(64).or_correct_opacity(dptr(a), a.size, int(num_samples), dptr(out)) != 0:
        raise ValueError("samples must be greater than 0")
    return out


def sample_distance(bounds, num_samples: int) -> float:
    """VolumeRenderer::PreExecute (VolumeRenderer.cpp:600-612)."""
    b = np.ascontiguousarray(bounds, dtype=np.float64)
    return float(load(64).or_sample_distance(dptr(b), int(num_samples)))


def color_table_sample(rgb_pos, rgb, alpha_pos, alpha, n: int = LUT_SIZE,
                       uint8_mode: int = UINT8_NONE) -> np.ndarray:
    """Sample control points to an (n, 4) float32 RGBA table; through uint8
    for the multi-domain path (VolumeRenderer.cpp:65-90)."""
    keep = [np.ascontiguousarray(x, dtype=np.float64) for x in (rgb_pos, rgb, alpha_pos, alpha)]
    t = ColorTable(len(keep[0]), dptr(keep[0]), dptr(keep[1]), len(keep[2]), dptr(keep[2]),
                   dptr(keep[3]))
    out = np.zeros((n, 4), np.float32)
    if load(64).or_color_table_sample(C.byref(t), int(n), int(uint8_mode), fptr(out)) != 0:
        raise ValueError("invalid colour table")
    return out


def camera_reset_to_bounds(bounds) -> Camera:
    b = np.ascontiguousarray(bounds, dtype=np.float64)
    cam = Camera()
    load(64).or_camera_reset_to_bounds(C.byref(cam), dptr(b))
    return cam


def cinema_cameras(bounds, phi_theta) -> list:
    """CinemaManager::create_cinema_cameras (rendering_filters.cpp:906-960)."""
    b = np.ascontiguousarray(bounds, dtype=np.float64)
    pt = np.ascontiguousarray(phi_theta, dtype=np.float32).reshape(-1, 2)
    out = (Camera * max(len(pt), 1))()
    load(64).or_cinema_cameras(dptr(b), fptr(pt), len(pt), out)
    cams = []
    for i in range(len(pt)):
        c = Camera()
        C.memmove(C.byref(c), C.byref(out[i]), C.sizeof(Camera))
        cams.append(c)
    return cams


def workload_camera(wl) -> Camera:
    """Reset to the scene bounds, then azimuth, then elevation (the order
    parse_camera applies them, conduit_to_vtkm_parsing.cpp:164-174)."""
    cam = camera_reset_to_bounds(wl.bounds)
    if wl.azimuth:
        load(64).or_camera_azimuth(C.byref(cam), float(wl.azimuth))
    if wl.elevation:
        load(64).or_camera_elevation(C.byref(cam), float(wl.elevation))
    return cam


def make_params(width, height, sample_dist, scalar_range, lut, *, lut_filter=LUT_NEAREST,
                alpha_cull=0.001, early_term=0.99, quantize_uint8=False, render_bg=False,
                bg_color=(0.0, 0.0, 0.0, 1.0), clear_depth=1.0) -> RenderParams:
    """RenderParams for the oracle; the LUT array is kept alive by the struct."""
    lut = np.ascontiguousarray(lut, dtype=np.float32).reshape(-1, 4)
    p = RenderParams()
    p.width, p.height = int(width), int(height)
    p.sample_dist = float(sample_dist)
    p.scalar_min, p.scalar_max = float(scalar_range[0]), float(scalar_range[1])
    p.lut_rgba = fptr(lut)
    p.lut_size = lut.shape[0]
    p.lut_filter = int(lut_filter)
    p.alpha_cull = float(alpha_cull)
    p.early_term = float(early_term)
    p.quantize_uint8 = int(bool(quantize_uint8))
    p.render_bg = int(bool(render_bg))
    for i in range(4):
        p.bg_color[i] = float(bg_color[i])
    p.clear_depth = float(clear_depth)
    p._lut_keepalive = lut  # noqa: SLF001
    return p


def workload_lut(wl, single_domain: bool | None = None) -> np.ndarray:
    """The plot's LUT: control points opacity-corrected for wl.samples, sampled
    at 1024 entries, in float on the one-domain path and through uint8
    (rounded) on the multi-domain path (VolumeRenderer.cpp:469-597, 65-90)."""
    single = wl.single_domain if single_domain is None else single_domain
    alpha = correct_opacity(wl.alpha, wl.samples)
    return color_table_sample(wl.rgb_pos, wl.rgb, wl.alpha_pos, alpha, LUT_SIZE,
                              UINT8_NONE if single else UINT8_ROUND)


def workload_params(wl, *, lut=None, single_domain: bool | None = None, **kw) -> RenderParams:
    """Render parameters of a workload's volume plot, set up by the oracle."""
    single = wl.single_domain if single_domain is None else single_domain
    if lut is None:
        lut = workload_lut(wl, single)
    kw.setdefault("quantize_uint8", single)
    return make_params(wl.width, wl.height, sample_distance(wl.bounds, wl.samples), wl.scalar_range,
                       lut, **kw)
