"""Brick size as a scene setting (gvr_scene_set_brick_cells: 4, 8 or 16
cells per brick axis). The bricks hold the same node values whatever their
size, and the march interpolates the same corners with the same weights, so
images, depths and sample counts must be identical across sizes: plain and
empty-space-skipping walks, rectilinear and element fields, the batched
path; and within the bar of the FP64 oracle."""
import numpy as np
import pytest

from ascent_gb300 import _native as N
from ascent_gb300 import scene as S
from ascent_gb300 import volume as V
from ascent_gb300 import workloads as W
from oracle import oracle as O

from conftest import assert_parity

pytestmark = pytest.mark.gpu


def render_at(wl, cells, cam, p, batch_cams=None):
    with S.Scene(0, brick_cells=cells) as sc:
        V.load_workload(sc, wl)
        single = sc.render(cam, p, count_samples=True)
        batch = sc.render_batch(batch_cams, p, count_samples=True) if batch_cams else None
    return single, batch


@pytest.mark.parametrize("parts", [None, (2, 2, 2), (3, 1, 2)])
def test_images_identical_across_brick_sizes(parts):
    wl = W.plain_small(n=71, width=120, height=96, parts=parts)
    cam = V.workload_camera(wl)
    p = V.workload_params(wl)
    ref, _ = render_at(wl, 8, cam, p)
    for cells in (4, 16):
        got, _ = render_at(wl, cells, cam, p)
        np.testing.assert_array_equal(got[0], ref[0])
        np.testing.assert_array_equal(got[1], ref[1])
        assert got[2] == ref[2]
    osc = O.OracleScene(64)
    for d in wl.domains:
        osc.add_uniform(d.dims, d.origin, d.spacing, d.field)
    assert_parity(ref[0], osc.render(O.workload_camera(wl), O.workload_params(wl))[0])


def test_empty_bricks_and_batch_across_brick_sizes():
    """Zero opacity below the middle of the range: the brick walk skips
    empty bricks of each size; the batched views agree too."""
    wl = W.plain_small(n=97, width=100, height=100, parts=(2, 1, 2))
    x = np.linspace(0.0, 1.0, 64)
    wl.alpha_pos, wl.alpha = x, np.where(x < 0.5, 0.0, 0.5 * (x - 0.5))
    cam = V.workload_camera(wl)
    cams = S.cinema_cameras(wl.bounds, W.cinema_angles(2, 2))
    p = V.workload_params(wl)
    ref, refb = render_at(wl, 8, cam, p, cams)
    for cells in (4, 16):
        got, gotb = render_at(wl, cells, cam, p, cams)
        np.testing.assert_array_equal(got[0], ref[0])
        assert got[2] == ref[2]
        np.testing.assert_array_equal(gotb[0], refb[0])
        assert gotb[2] == refb[2]


def test_rectilinear_and_element_fields_across_brick_sizes():
    rng = np.random.default_rng(3)
    nx, ny, nz = 37, 29, 33
    x = np.cumsum(rng.uniform(0.5, 1.5, nx)) / 30
    y = np.cumsum(rng.uniform(0.5, 1.5, ny)) / 30
    z = np.cumsum(rng.uniform(0.5, 1.5, nz)) / 30
    f = rng.uniform(0, 1, (nz, ny, nx)).astype(np.float32)
    cells_f = rng.uniform(0, 1, (nz - 1, ny - 1, nx - 1)).astype(np.float32)
    bounds = [x[0], x[-1], y[0], y[-1], z[0], z[-1]]
    cam = S.camera_reset_to_bounds(bounds)
    S.camera_azimuth(cam, 25.0)
    lut = np.stack([np.linspace(0, 1, 256), np.full(256, 0.5), np.linspace(1, 0, 256),
                    np.linspace(0, 0.05, 256)], 1).astype(np.float32)
    p = N.make_params(80, 64, S.sample_distance(bounds, 150), (0.0, 1.0), lut)
    out = []
    for cells in (8, 4, 16):
        with S.Scene(0, brick_cells=cells) as sc:
            sc.add_rectilinear(f, x, y, z)
            out.append(sc.render(cam, p, count_samples=True))
    for o in out[1:]:
        np.testing.assert_array_equal(o[0], out[0][0])
        assert o[2] == out[0][2]
    assert out[0][0][..., 3].max() > 0.05
    # element fields are not bricked: the setting does not touch them
    with S.Scene(0, brick_cells=16) as sc:
        sc.add_uniform(cells_f, (0, 0, 0), (1 / 36, 1 / 28, 1 / 32), association=N.ASSOC_ELEMENT)
        e16 = sc.render(S.camera_reset_to_bounds(sc.bounds()), p)[0]
    with S.Scene(0) as sc:
        sc.add_uniform(cells_f, (0, 0, 0), (1 / 36, 1 / 28, 1 / 32), association=N.ASSOC_ELEMENT)
        e8 = sc.render(S.camera_reset_to_bounds(sc.bounds()), p)[0]
    np.testing.assert_array_equal(e16, e8)


def test_brick_size_argument_rules():
    wl = W.plain_small(n=16, width=16, height=16)
    with S.Scene(0) as sc:
        with pytest.raises(N.GvrError):
            sc.set_brick_cells(6)
        V.load_workload(sc, wl)
        with pytest.raises(N.GvrError):
            sc.set_brick_cells(4)   # after a vertex-field domain


def test_tuner_sweeps_brick_sizes():
    from ascent_gb300 import tune
    wl = W.plain_small(n=49, width=64, height=64, parts=(2, 1, 1))
    cam = V.workload_camera(wl)
    p = V.workload_params(wl)

    def build(cells):
        sc = S.Scene(0, brick_cells=cells)
        V.load_workload(sc, wl)
        return sc

    out = tune.autotune_bricks(build, cam, p, reps=1)
    sc = out["scene"]
    try:
        assert out["best"]["brick_cells"] in (4, 8, 16) and sc.brick_cells == out["best"]["brick_cells"]
        assert set(out["ms"]) == {"4", "8", "16"}
        img = sc.render(cam, p)[0]
    finally:
        sc.close()
    with S.Scene(0) as ref:
        V.load_workload(ref, wl)
        np.testing.assert_array_equal(img, ref.render(cam, p)[0])
