"""The C-ABI library loads, exports every declared entry point, and its host
logic (no device work) agrees with the CPU oracle."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

from ascent_gb300 import _native as N
from ascent_gb300 import scene as S
from oracle import oracle as O

ROOT = Path(__file__).resolve().parents[1]


def declared_symbols():
    txt = (ROOT / "include" / "gvr.h").read_text()
    return sorted(set(re.findall(r"GVR_API\s+[\w\s\*]*?\b(gvr_\w+)\s*\(", txt)))


def test_library_exports_every_declared_symbol():
    lib = N.lib()
    names = declared_symbols()
    assert len(names) >= 19
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert lib.gvr_version() == 1


def test_error_reporting():
    out = np.zeros(2)
    a = np.array([0.1, 0.2])
    rc = N.lib().gvr_correct_opacity(N.dptr(a), 2, 0, N.dptr(out))
    assert rc == N.GVR_ERR_INVALID_ARGUMENT
    assert "samples must be greater than 0" in N.lib().gvr_last_error().decode()
    with pytest.raises(N.GvrError):
        S.correct_opacity(a, -3)


def test_correct_opacity_matches_oracle_and_formula():
    a = np.linspace(0, 1, 33)
    for n in (1, 7, 100, 218, 1774):
        got = S.correct_opacity(a, n)
        ref = np.empty_like(a)
        O.load(64).or_correct_opacity(N.dptr(a), a.size, n, N.dptr(ref))
        np.testing.assert_array_equal(got, ref)
        ratio = np.float32(10.0) / np.float32(n)
        np.testing.assert_allclose(got, 1 - (1 - a) ** float(ratio), rtol=0, atol=1e-15)


def test_sample_distance_matches_oracle():
    for b, n in [((0, 1, 0, 1, 0, 1), 218), ((-3, 5, 0, 0.5, 2, 9), 100), ((0, 512, 0, 512, 0, 512), 1774)]:
        b = np.array(b, dtype=np.float64)
        assert S.sample_distance(b, n) == O.load(64).or_sample_distance(N.dptr(b), n)
    assert abs(S.sample_distance(np.array([0, 63, 0, 63, 0, 63.0]), 218) - np.sqrt(3) * 63 / 218) < 1e-5


@pytest.mark.parametrize("mode", [N.UINT8_NONE, N.UINT8_ROUND, N.UINT8_TRUNCATE])
def test_color_table_sample_matches_oracle(mode):
    rng = np.random.default_rng(0)
    rp = np.sort(np.unique(np.r_[0.0, rng.uniform(0, 1, 10), 1.0]))
    rgb = rng.uniform(0, 1, (len(rp), 3))
    ap = np.sort(np.unique(np.r_[0.1, rng.uniform(0.1, 0.9, 6)]))
    al = rng.uniform(0, 1, len(ap))
    got = S.color_table_sample(rp, rgb, ap, al, 1024, mode)
    t = N.ColorTable(len(rp), N.dptr(rp), N.dptr(rgb.ravel().copy()), len(ap), N.dptr(ap), N.dptr(al))
    rgb_keep = rgb.ravel().copy()
    t.rgb = N.dptr(rgb_keep)
    ref = np.empty((1024, 4), np.float32)
    assert O.load(64).or_color_table_sample(C.byref(t), 1024, mode, N.fptr(ref)) == 0
    np.testing.assert_allclose(got, ref, rtol=0, atol=1e-7)
    if mode != N.UINT8_NONE:
        assert np.all(np.abs(got * 255 - np.round(got * 255)) < 1e-4)


def test_color_table_rejects_unsorted_points():
    with pytest.raises(N.GvrError):
        S.color_table_sample([0.5, 0.2], [[0, 0, 0], [1, 1, 1]], [0.0], [1.0])


def _ocam(fn, *args):
    c = N.Camera()
    fn(C.byref(c), *args)
    return c


def test_cameras_match_oracle():
    b = np.array([-1.0, 3.0, 0.0, 2.0, -5.0, 1.0])
    got = S.camera_reset_to_bounds(b)
    ref = N.Camera()
    O.load(64).or_camera_reset_to_bounds(C.byref(ref), N.dptr(b))
    assert bytes(got) == bytes(ref)
    S.camera_azimuth(got, 30.0)
    S.camera_elevation(got, 20.0)
    O.load(64).or_camera_azimuth(C.byref(ref), 30.0)
    O.load(64).or_camera_elevation(C.byref(ref), 20.0)
    np.testing.assert_allclose(list(got.position), list(ref.position), rtol=1e-6)
    # elevation raises the camera, azimuth turns it about +y
    assert got.position[1] > got.look_at[1]


def test_cinema_cameras_match_oracle():
    b = np.array([0.0, 1.0, 0.0, 2.0, 0.0, 3.0])
    phis = np.linspace(-180, 180, 8, endpoint=False)
    thetas = np.linspace(0, 180, 8, endpoint=False)
    pt = np.array([(p, t) for p in phis for t in thetas], dtype=np.float32)
    got = S.cinema_cameras(b, pt)
    ref = (N.Camera * len(pt))()
    O.load(64).or_cinema_cameras(N.dptr(b), N.fptr(pt), len(pt), ref)
    for g, r in zip(got, ref):
        np.testing.assert_allclose(list(g.position), list(r.position), rtol=1e-5, atol=1e-5)
        np.testing.assert_allclose(list(g.up), list(r.up), rtol=1e-5, atol=1e-6)
        np.testing.assert_allclose(list(g.look_at), [0.5, 1.0, 1.5])
    radius = np.linalg.norm([1, 2, 3]) * 2.5 / 2
    for g in got:
        assert abs(np.linalg.norm(np.array(g.position) - [0.5, 1, 1.5]) - radius) < 1e-4


def test_visibility_order_matches_oracle():
    rng = np.random.default_rng(3)
    lo = rng.uniform(-5, 5, (37, 3))
    hi = lo + rng.uniform(0.1, 2, (37, 3))
    bounds = np.stack([lo[:, 0], hi[:, 0], lo[:, 1], hi[:, 1], lo[:, 2], hi[:, 2]], axis=1)
    cam = S.camera_reset_to_bounds(np.array([-5, 7, -5, 7, -5, 7.0]))
    got = S.visibility_order(cam, bounds)
    ref = np.zeros(37, np.int32)
    O.load(64).or_visibility_order(C.byref(cam), N.dptr(np.ascontiguousarray(bounds)), 37,
                                   ref.ctypes.data_as(C.POINTER(C.c_int)))
    np.testing.assert_array_equal(got, ref)
    assert sorted(got.tolist()) == list(range(37))


def test_canvas_conversion_rejects_bad_arguments_before_any_device_work():
    lib = N.lib()
    img = np.zeros((2, 3, 4), np.float32)
    out = np.zeros((2, 3, 4), np.uint8)
    cases = [(img.ctypes.data, 0, 2, out.ctypes.data, N.MEM_HOST, "image size"),
             (img.ctypes.data, 3, 2, None, N.MEM_HOST, "NULL"),
             (img.ctypes.data, 3, 2, out.ctypes.data, 7, "bad location")]
    for src, w, h, dst, loc, msg in cases:
        rc = lib.gvr_canvas_to_rgba8(C.c_void_p(src), w, h, C.c_void_p(dst), loc, None)
        assert rc == N.GVR_ERR_INVALID_ARGUMENT
        assert msg in lib.gvr_last_error().decode()


def test_device_png_conversion_wants_a_cuda_tensor():
    torch = pytest.importorskip("torch")
    from ascent_gb300 import png as PNG
    with pytest.raises(ValueError):
        PNG.canvas_to_rgba8_device(torch.zeros((2, 2, 4), dtype=torch.float32))


def test_scratch_trim_arguments():
    """gvr_scratch_trim needs no GPU for its argument checks; a device the
    library never used holds no pool (0 bytes reserved)."""
    with pytest.raises(N.GvrError):
        N.scratch_trim(-1, 0)
    assert N.scratch_trim(63, 0) == 0


@pytest.mark.parametrize("parts", [None, (2, 1, 2)])
def test_oracle_setup_equals_library_setup(parts):
    """The oracle builds the camera and render parameters of a workload with
    its own functions (no product library); on the same workload they equal
    the library's field for field, LUT included (float on the one-domain
    path, through uint8 on the multi-domain path)."""
    from ascent_gb300 import volume as V
    from ascent_gb300 import workloads as W
    wl = W.plain_small(n=24, width=40, height=30, parts=parts)
    assert bytes(O.workload_camera(wl)) == bytes(V.workload_camera(wl))
    op, pp = O.workload_params(wl), V.workload_params(wl)
    for f in ("width", "height", "sample_dist", "scalar_min", "scalar_max", "lut_size", "lut_filter",
              "alpha_cull", "early_term", "quantize_uint8", "render_bg", "clear_depth"):
        assert getattr(op, f) == getattr(pp, f), f
    n = op.lut_size * 4
    np.testing.assert_array_equal(np.ctypeslib.as_array(op.lut_rgba, (n,)),
                                  np.ctypeslib.as_array(pp.lut_rgba, (n,)))
    angles = W.cinema_angles(3, 2)
    assert [bytes(c) for c in O.cinema_cameras(wl.bounds, angles)] == \
           [bytes(c) for c in S.cinema_cameras(wl.bounds, angles)]
