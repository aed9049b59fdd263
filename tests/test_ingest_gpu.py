"""Bricking of contiguous float32 fields by the staged ingest kernel
(gvr_ingest.cu: runs of 16 bricks along x copied row by row into shared
memory, bricks written four nodes per lane and step) against the per-brick
gather kernel, which bricks float64 fields: a float32 field and its exact
float64 copy must give the same scalar range and the same image, on shapes
whose runs end early (x node counts 9, 129, 130 and 300), single-row and
single-layer domains, and from host and device memory. Non-finite values
anywhere in a field (first node, last node, a node shared by two bricks, an
interior node) must be refused by host and device publishes alike.
"""
import numpy as np
import pytest

from ascent_gb300 import _native as N
from ascent_gb300 import scene as S
from ascent_gb300 import volume as V
from ascent_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def random_workload(shape, seed=0, width=96, height=80):
    rng = np.random.default_rng(seed)
    f = rng.uniform(0.0, 1.0, shape).astype(np.float32)
    nz, ny, nx = shape
    sp = (1.0 / max(nx - 1, 1), 1.0 / max(ny - 1, 1), 1.0 / max(nz - 1, 1))
    wl = W.plain_small(n=9, width=width, height=height)
    wl.domains = [W.UniformDomain(f, (0.0, 0.0, 0.0), sp)]
    return wl


@pytest.mark.parametrize("shape", [(9, 9, 9), (17, 10, 129), (20, 13, 130), (11, 33, 300),
                                   (2, 5, 257), (40, 2, 140)])
def test_staged_bricking_equals_the_gather(shape):
    import torch
    wl = random_workload(shape, seed=sum(shape))
    d = wl.domains[0]
    cam = V.workload_camera(wl)
    p = V.workload_params(wl)
    with S.Scene(0) as a, S.Scene(0) as b:
        a.add_uniform(d.field, d.origin, d.spacing)                       # float32: staged
        b.add_uniform(d.field.astype(np.float64), d.origin, d.spacing)    # float64: gather
        np.testing.assert_array_equal(a.scalar_range(), b.scalar_range())
        np.testing.assert_array_equal(a.scalar_range(), [d.field.min(), d.field.max()])
        ia, da = a.render(cam, p)
        ib, db = b.render(cam, p)
        np.testing.assert_array_equal(ia, ib)
        np.testing.assert_array_equal(da, db)
        assert ia[..., 3].max() > 0.01
        # device-resident publish of the same values: the one-launch path
        a.update_fields([0], [torch.from_numpy(d.field).cuda()])
        np.testing.assert_array_equal(a.scalar_range(), b.scalar_range())
        np.testing.assert_array_equal(a.render(cam, p)[0], ib)


@pytest.mark.parametrize("value", [np.nan, np.inf, -np.inf])
@pytest.mark.parametrize("where", ["first", "last", "shared", "interior"])
def test_non_finite_values_are_refused(value, where):
    import torch
    shape = (20, 13, 130)
    wl = random_workload(shape, seed=3)
    d = wl.domains[0]
    idx = {"first": (0, 0, 0), "last": (19, 12, 129), "shared": (8, 8, 8), "interior": (11, 5, 77)}[where]
    bad = d.field.copy()
    bad[idx] = value
    with S.Scene(0) as sc:
        sc.add_uniform(d.field, d.origin, d.spacing)
        good = sc.scalar_range()
        with pytest.raises(N.GvrError):
            sc.update_fields([0], [bad])
        with pytest.raises(N.GvrError):
            sc.update_fields([0], [torch.from_numpy(bad).cuda()])
        sc.update_fields([0], [torch.from_numpy(d.field).cuda()])
        np.testing.assert_array_equal(sc.scalar_range(), good)
