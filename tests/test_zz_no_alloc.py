"""gvr_render_uniform_noalloc: the entry point for callers that may not
allocate device memory (a simulation whose pool allocator owns the GPU's
memory, where cudaMalloc could fail against the pool's budget and would
synchronise the device under the simulation's streams).

It is called here through the C ABI with caller-owned device buffers, twice
in a row, and each result is checked against gvr_render_volume on a scene
holding the same single domain and against the FP64 oracle (set up by its
own functions), with the parity bar the other GPU tests use. The device's
free memory after the second call must equal its free memory after the
first (the first call on a device may load the library's kernels). This
file is named to be collected last.
"""
import ctypes as C

import numpy as np
import pytest

from ascent_gb300 import _native as N
from ascent_gb300 import scene as S
from ascent_gb300 import volume as V
from ascent_gb300 import workloads as W
from oracle import oracle as O

from conftest import assert_parity

pytestmark = pytest.mark.gpu


def noalloc_fn():
    fn = N.lib().gvr_render_uniform_noalloc
    fn.restype = C.c_int
    fn.argtypes = [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_double), C.POINTER(C.c_double),
                   C.POINTER(N.Camera), C.POINTER(N.RenderParams), C.c_void_p, C.c_void_p,
                   C.c_void_p, C.POINTER(C.c_uint64)]
    return fn


def test_noalloc_matches_scene_render_on_two_calls_in_a_row():
    import torch
    wl = W.plain_small(n=48, width=160, height=120)
    d = wl.domains[0]
    cam = V.workload_camera(wl)
    p = V.workload_params(wl)
    with S.Scene(0) as sc:
        V.load_workload(sc, wl)
        ref, ref_depth, ref_n = sc.render(cam, p, count_samples=True)

    field = torch.from_numpy(d.field).cuda()
    rgba = torch.empty((wl.height, wl.width, 4), dtype=torch.float32, device="cuda")
    depth = torch.empty((wl.height, wl.width), dtype=torch.float32, device="cuda")
    dims = (C.c_int * 3)(*d.dims)
    origin = (C.c_double * 3)(*d.origin)
    spacing = (C.c_double * 3)(*d.spacing)
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    osc = O.OracleScene(64)
    osc.add_uniform(d.dims, d.origin, d.spacing, d.field)
    oracle_img, _, _ = osc.render(O.workload_camera(wl), O.workload_params(wl))
    fn = noalloc_fn()
    outs = []
    free_after = []
    for _ in range(2):
        rgba.fill_(-1.0)
        torch.cuda.synchronize()
        n = C.c_uint64(0)
        rc = fn(C.c_void_p(field.data_ptr()), dims, origin, spacing, C.byref(cam), C.byref(p),
                C.c_void_p(rgba.data_ptr()), C.c_void_p(depth.data_ptr()), stream, C.byref(n))
        assert rc == 0, N.lib().gvr_last_error()
        torch.cuda.synchronize()
        free_after.append(torch.cuda.mem_get_info()[0])
        g = rgba.cpu().numpy()
        gd = depth.cpu().numpy()
        assert_parity(g, ref)
        assert_parity(g, oracle_img)
        np.testing.assert_allclose(gd, ref_depth, rtol=0, atol=1e-5)
        assert n.value == ref_n
        outs.append(g)
    np.testing.assert_array_equal(outs[0], outs[1])
    assert free_after[1] == free_after[0], free_after
    assert ref[..., 3].max() > 0.2


def test_noalloc_rejects_lut_beyond_its_scratch():
    import torch
    wl = W.plain_small(n=16, width=16, height=16)
    d = wl.domains[0]
    cam = V.workload_camera(wl)
    lut = np.zeros((4097, 4), np.float32)
    p = N.make_params(16, 16, 0.01, wl.scalar_range, lut)
    field = torch.from_numpy(d.field).cuda()
    out = torch.empty((16, 16, 4), dtype=torch.float32, device="cuda")
    dep = torch.empty((16, 16), dtype=torch.float32, device="cuda")
    rc = noalloc_fn()(C.c_void_p(field.data_ptr()), (C.c_int * 3)(*d.dims),
                      (C.c_double * 3)(*d.origin), (C.c_double * 3)(*d.spacing), C.byref(cam),
                      C.byref(p), C.c_void_p(out.data_ptr()), C.c_void_p(dep.data_ptr()), None, None)
    assert rc == N.GVR_ERR_INVALID_ARGUMENT
    assert "exceeds the 4096 entries" in N.lib().gvr_last_error().decode()
