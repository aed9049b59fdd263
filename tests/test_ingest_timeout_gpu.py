"""The staged ingest kernel's timeout path, run without faulting anything.

The kernel that bricks contiguous float32 fields waits for its own bulk
copies with a bounded wait (gvr_ingest.cu). GVR_STAGE_WAIT_POLLS=0 makes the
first wait give up at once; the kernel then sets the scene's flag, writes
the bricks with non-finite ranges, and waits a second, full-length time so
that its copies land before it exits. The host must report GVR_ERR_TIMEOUT
and an unknown (NaN) range, and a normal publish afterwards must restore
the scene exactly.
"""
import numpy as np
import pytest

from ascent_gb300 import _native as N
from ascent_gb300 import scene as S
from ascent_gb300 import volume as V
from ascent_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def test_staged_wait_timeout_reports_and_recovers(monkeypatch):
    wl = W.plain_small(n=40, width=64, height=48, parts=(2, 1, 1))
    cam = V.workload_camera(wl)
    p = V.workload_params(wl)
    fields = [np.ascontiguousarray(d.field, dtype=np.float32) for d in wl.domains]
    with S.Scene(0) as sc:
        V.load_workload(sc, wl)
        before, before_d = sc.render(cam, p)
        good_range = sc.scalar_range()
        assert np.isfinite(good_range).all()

        monkeypatch.setenv("GVR_STAGE_WAIT_POLLS", "0")
        with pytest.raises(N.GvrError) as err:
            sc.update_fields([0, 1], fields)
        assert err.value.code == N.GVR_ERR_TIMEOUT
        assert np.isnan(sc.scalar_range()).all()
        with pytest.raises(N.GvrError) as err:
            sc.update_field(0, fields[0])
        assert err.value.code == N.GVR_ERR_TIMEOUT
        assert np.isnan(sc.scalar_range()).all()

        # device-resident fields: all domains bricked by one launch
        import torch
        dev_fields = [torch.from_numpy(f).cuda() for f in fields]
        with pytest.raises(N.GvrError) as err:
            sc.update_fields([0, 1], dev_fields)
        assert err.value.code == N.GVR_ERR_TIMEOUT
        assert np.isnan(sc.scalar_range()).all()

        monkeypatch.delenv("GVR_STAGE_WAIT_POLLS")
        sc.update_fields([0, 1], dev_fields)
        np.testing.assert_array_equal(sc.scalar_range(), good_range)
        np.testing.assert_array_equal(sc.render(cam, p)[0], before)
        sc.update_fields([0, 1], fields)
        np.testing.assert_array_equal(sc.scalar_range(), good_range)
        after, after_d = sc.render(cam, p)
        assert np.array_equal(after, before) and np.array_equal(after_d, before_d)


def test_stage_wait_setting_out_of_range_falls_back(monkeypatch):
    """A malformed or negative setting keeps the default bound."""
    wl = W.plain_small(n=24, width=32, height=32)
    with S.Scene(0) as sc:
        V.load_workload(sc, wl)
        for v in ("-5", "abc", ""):
            monkeypatch.setenv("GVR_STAGE_WAIT_POLLS", v)
            sc.update_field(0, np.ascontiguousarray(wl.domains[0].field, dtype=np.float32))
        assert np.isfinite(sc.scalar_range()).all()
