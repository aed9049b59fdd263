"""Hexahedral path on the GPU vs the CPU rebuild in the oracle.

Integer work is bit-exact: Morton codes, the leaf order (equal codes keep
cell order), Karras children and parents, and the refit boxes (min/max of
float32) must equal the oracle's arrays exactly. Point location must give the
oracle's cell except at points within 1e-3 (reference space) of a cell face,
where either neighbour is correct. Images meet the parity bar of the
structured path.
"""
import numpy as np
import pytest

from ascent_gb300 import _native as N
from ascent_gb300 import scene as S
from ascent_gb300 import volume as V
from ascent_gb300 import workloads as W
from oracle import oracle as O

from conftest import assert_parity

pytestmark = pytest.mark.gpu


def both_bvh(d):
    with S.Scene(0) as sc:
        did = sc.add_hex(d.x, d.y, d.z, d.conn, d.field)
        g = sc.hex_bvh(did)
    osc = O.OracleScene(64)
    oid = osc.add_hex(d.x, d.y, d.z, d.conn, d.field)
    return g, osc.hex_bvh(oid)


@pytest.mark.parametrize("n,seed", [(12, 3), (31, 4), (40, 5)])
def test_bvh_is_bit_exact_against_cpu_rebuild(n, seed):
    wl = W.hex_mesh(n_cells=n, seed=seed, width=8, height=8)
    g, o = both_bvh(wl.domains[0])
    for k in ("codes", "ids", "left", "right", "parent"):
        np.testing.assert_array_equal(g[k], o[k], err_msg=k)
    np.testing.assert_array_equal(g["inner_box"], o["inner_box"])


def test_bvh_ties_and_tiny_meshes():
    wl = W.hex_mesh(n_cells=3, seed=1, width=8, height=8)
    d = wl.domains[0]
    # duplicated cells give equal Morton codes: order must follow cell ids
    dup = W.HexDomain(d.x, d.y, d.z, np.concatenate([d.conn, d.conn[::-1], d.conn[:5]]), d.field)
    g, o = both_bvh(dup)
    for k in ("codes", "ids", "left", "right", "parent"):
        np.testing.assert_array_equal(g[k], o[k], err_msg=k)
    assert (np.diff(g["codes"].astype(np.int64)) == 0).any()
    for m in (1, 2):
        small = W.HexDomain(d.x, d.y, d.z, d.conn[:m].copy(), d.field)
        g, o = both_bvh(small)
        np.testing.assert_array_equal(g["codes"], o["codes"])
        np.testing.assert_array_equal(g["ids"], o["ids"])
        if m == 2:
            for k in ("left", "right", "parent"):
                np.testing.assert_array_equal(g[k], o[k], err_msg=k)


def test_locate_matches_oracle():
    wl = W.hex_mesh(n_cells=16, seed=7, width=8, height=8)
    d = wl.domains[0]
    rng = np.random.default_rng(0)
    pts = rng.uniform(-0.05, 1.05, size=(20000, 3)).astype(np.float32)
    with S.Scene(0) as sc:
        did = sc.add_hex(d.x, d.y, d.z, d.conn, d.field)
        gc, gr = sc.hex_locate(did, pts)
    osc = O.OracleScene(64)
    oid = osc.add_hex(d.x, d.y, d.z, d.conn, d.field)
    oc, orr = osc.hex_locate(oid, pts)
    assert (oc >= 0).mean() > 0.5
    margin = np.minimum(orr, 1 - orr).min(axis=1)
    clear = (oc < 0) | (margin > 1e-3)
    np.testing.assert_array_equal(gc[clear], oc[clear])
    amb = ~clear
    # near a face: the GPU's cell must contain the point too
    assert np.all(gr[amb & (gc >= 0)] > -2e-3) and np.all(gr[amb & (gc >= 0)] < 1 + 2e-3)
    inside = (oc >= 0) & (gc >= 0) & clear
    np.testing.assert_allclose(gr[inside], orr[inside], atol=5e-4)


def test_hex_render_matches_oracle():
    wl = W.hex_mesh(n_cells=20, seed=3, width=96, height=80)
    cam = V.workload_camera(wl)
    p = V.workload_params(wl)
    assert p.quantize_uint8 == 0  # unstructured input takes the multi-domain path
    with S.Scene(0) as sc:
        V.load_workload(sc, wl)
        g, gd, gn = sc.render(cam, p, count_samples=True)
    d = wl.domains[0]
    osc = O.OracleScene(64)
    osc.add_hex(d.x, d.y, d.z, d.conn, d.field)
    # the oracle's camera and parameters come from its own set-up functions
    o, od, on = osc.render(O.workload_camera(wl), O.workload_params(wl))
    assert o[..., 3].max() > 0.1
    assert_parity(g, o)
    assert abs(gn - on) <= 1e-3 * on


def test_mixed_uniform_and_hex_scene():
    wl = W.hex_mesh(n_cells=10, seed=2, width=8, height=8)
    d = wl.domains[0]
    x = d.x + np.float32(1.0)  # hex block at [1, 2] x [0, 1]^2
    uni = W.plain_small(n=17, width=8, height=8).domains[0]
    b = np.array([0.0, 2.0, 0.0, 1.0, 0.0, 1.0])
    cam = S.camera_reset_to_bounds(b)
    S.camera_azimuth(cam, 25)
    S.camera_elevation(cam, 15)
    vr = V.workload_renderer(wl)
    lo = min(uni.field.min(), d.field.min())
    hi = max(uni.field.max(), d.field.max())
    p = vr.params(100, 60, b, (lo, hi), single_domain=False)
    with S.Scene(0) as sc:
        sc.add_uniform(uni.field, uni.origin, uni.spacing)
        sc.add_hex(x, d.y, d.z, d.conn, d.field)
        g, gd = sc.render(cam, p)
    osc = O.OracleScene(64)
    osc.add_uniform(uni.dims, uni.origin, uni.spacing, uni.field)
    osc.add_hex(x, d.y, d.z, d.conn, d.field)
    o, od, _ = osc.render(cam, p)
    assert_parity(g, o)


def test_hex_update_field_and_errors():
    wl = W.hex_mesh(n_cells=6, seed=4, width=32, height=32)
    d = wl.domains[0]
    cam = V.workload_camera(wl)
    p = V.workload_params(wl)
    with S.Scene(0) as sc:
        did = sc.add_hex(d.x, d.y, d.z, d.conn, d.field)
        a, _ = sc.render(cam, p)
        sc.update_field(did, d.field * 0.5)
        assert np.isclose(sc.scalar_range()[1], d.field.max() * 0.5)
        sc.update_field(did, d.field)
        b, _ = sc.render(cam, p)
        np.testing.assert_array_equal(a, b)
        bad = d.conn.copy()
        bad[0, 0] = len(d.x) + 5
        with pytest.raises(N.GvrError, match="missing node"):
            sc.add_hex(d.x, d.y, d.z, bad, d.field)


def test_hex_element_field():
    wl = W.hex_mesh(n_cells=8, seed=6, width=64, height=48)
    d = wl.domains[0]
    cells = np.random.default_rng(1).uniform(0, 1, len(d.conn)).astype(np.float32)
    cam = V.workload_camera(wl)
    vr = V.workload_renderer(wl)
    p = vr.params(64, 48, wl.bounds, (0.0, 1.0), single_domain=False)
    with S.Scene(0) as sc:
        sc.add_hex(d.x, d.y, d.z, d.conn, cells, association=N.ASSOC_ELEMENT)
        g, _ = sc.render(cam, p)
    osc = O.OracleScene(64)
    osc.add_hex(d.x, d.y, d.z, d.conn, cells, assoc=N.ASSOC_ELEMENT)
    o, _, _ = osc.render(cam, p)
    from conftest import image_error
    e = image_error(g, o)
    # a sample right on a face may pick either neighbour's constant value
    assert e["frac_within_2"] >= 0.99 and e["mae"] <= 2e-3, e


def _rotated_cells(conn, seed):
    """The same mesh with every other cell's local node order rotated a
    quarter turn about t (still a valid VTK hexahedron), so neighbouring
    cells disagree on orientation."""
    rng = np.random.default_rng(seed)
    rot = np.array([1, 2, 3, 0, 5, 6, 7, 4])
    out = conn.copy()
    pick = rng.uniform(size=len(conn)) < 0.5
    out[pick] = conn[pick][:, rot]
    return out


@pytest.mark.parametrize("n,rotate", [(6, False), (17, False), (17, True)])
def test_face_neighbours_bit_exact(n, rotate):
    wl = W.hex_mesh(n_cells=n, seed=9, width=8, height=8)
    d = wl.domains[0]
    conn = _rotated_cells(d.conn, 2) if rotate else d.conn
    with S.Scene(0) as sc:
        did = sc.add_hex(d.x, d.y, d.z, conn, d.field)
        nbr, ms = sc.hex_neighbors(did)
    np.testing.assert_array_equal(nbr, O.hex_face_neighbors(conn))
    assert (nbr >= 0).sum() == 6 * n ** 3 - 6 * n * n and ms >= 0


def test_hex_render_rotated_cells_matches_oracle():
    """Face stepping with neighbours of another orientation (the guess across
    the face is then wrong and Newton or the LBVH must recover)."""
    wl = W.hex_mesh(n_cells=20, seed=4, width=96, height=80)
    d = wl.domains[0]
    conn = _rotated_cells(d.conn, 5)
    cam = V.workload_camera(wl)
    p = V.workload_params(wl)
    with S.Scene(0) as sc:
        sc.add_hex(d.x, d.y, d.z, conn, d.field)
        g, gd, gn = sc.render(cam, p, count_samples=True)
    osc = O.OracleScene(64)
    osc.add_hex(d.x, d.y, d.z, conn, d.field)
    o, od, on = osc.render(cam, p)
    assert o[..., 3].max() > 0.1
    assert_parity(g, o)
