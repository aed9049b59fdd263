"""Python handle over a device-resident gvr_scene (C ABI in include/gvr.h)."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as N


def _field_args(field):
    """(pointer, dtype code, keepalive, location, count) for numpy or torch input."""
    try:
        import torch
    except ImportError:  # pragma: no cover - torch is always present here
        torch = None
    if torch is not None and isinstance(field, torch.Tensor):
        if field.dtype not in (torch.float32, torch.float64):
            raise N.GvrError(N.GVR_ERR_UNSUPPORTED, "field must be float32 or float64")
        t = field.contiguous()
        loc = N.MEM_DEVICE if t.is_cuda else N.MEM_HOST
        code = N.DTYPE_FLOAT64 if t.dtype == torch.float64 else N.DTYPE_FLOAT32
        return C.c_void_p(t.data_ptr()), code, t, loc, t.numel()
    a = np.asarray(field)
    if a.dtype not in (np.float32, np.float64):
        a = a.astype(np.float32)
    a = np.ascontiguousarray(a)
    code = N.DTYPE_FLOAT64 if a.dtype == np.float64 else N.DTYPE_FLOAT32
    return C.c_void_p(a.ctypes.data), code, a, N.MEM_HOST, a.size


class Scene:
    """Domains resident on one CUDA device, rendered by the fused march kernel."""

    def __init__(self, device: int = 0, brick_cells: int = 8):
        """brick_cells: cells per brick axis (4, 8 or 16) of the vertex fields
        this scene bricks (gvr_scene_set_brick_cells)."""
        h = C.c_void_p()
        N.call("gvr_scene_create", int(device), C.byref(h))
        self.handle = h
        self.device = int(device)
        self._hex_cells = {}
        if brick_cells != 8:
            self.set_brick_cells(brick_cells)
        self.brick_cells = int(brick_cells)

    def set_brick_cells(self, cells: int) -> None:
        """Brick size of vertex fields added from now on (before any is added)."""
        N.call("gvr_scene_set_brick_cells", self.handle, int(cells))
        self.brick_cells = int(cells)

    def add_uniform(self, field, origin, spacing, association: int = N.ASSOC_VERTEX) -> int:
        """field shaped (nz, ny, nx) nodes (or cells for element association)."""
        shape = tuple(field.shape)
        if len(shape) != 3:
            raise N.GvrError(N.GVR_ERR_INVALID_ARGUMENT, "field must be 3D (nz, ny, nx)")
        extra = 1 if association == N.ASSOC_ELEMENT else 0
        dims = (C.c_int * 3)(shape[2] + extra, shape[1] + extra, shape[0] + extra)
        o = (C.c_double * 3)(*map(float, origin))
        s = (C.c_double * 3)(*map(float, spacing))
        ptr, code, keep, loc, _ = _field_args(field)
        did = C.c_int(-1)
        N.call("gvr_scene_add_uniform", self.handle, dims, o, s, ptr, code, 1, int(association),
               loc, C.byref(did))
        del keep
        return did.value

    def add_rectilinear(self, field, x, y, z, association: int = N.ASSOC_VERTEX) -> int:
        xs = [np.ascontiguousarray(c, dtype=np.float64) for c in (x, y, z)]
        dims = (C.c_int * 3)(*[len(c) for c in xs])
        ptr, code, keep, loc, _ = _field_args(field)
        did = C.c_int(-1)
        N.call("gvr_scene_add_rectilinear", self.handle, dims, N.dptr(xs[0]), N.dptr(xs[1]),
               N.dptr(xs[2]), ptr, code, 1, int(association), loc, C.byref(did))
        del keep
        return did.value

    def add_hex(self, x, y, z, conn, field, association: int = N.ASSOC_VERTEX) -> int:
        """Unstructured hexahedra: node coordinates x, y, z (float32/float64), conn
        (n_cells, 8) int32/int64 in VTK hexahedron order, a vertex or element field.
        Arrays are all numpy (host) or all torch CUDA tensors (device)."""
        cx, ctype, k1, loc, nn = _field_args(x)
        cy, _, k2, _, _ = _field_args(y)
        cz, _, k3, _, _ = _field_args(z)
        fp, ftype, k4, _, _ = _field_args(field)
        try:
            import torch
            is_t = isinstance(conn, torch.Tensor)
        except ImportError:  # pragma: no cover
            is_t = False
        if is_t:
            cc = conn.contiguous()
            c64 = int(cc.dtype == torch.int64)
            cptr, ncells = C.c_void_p(cc.data_ptr()), cc.numel() // 8
        else:
            cc = np.ascontiguousarray(conn)
            if cc.dtype not in (np.int32, np.int64):
                cc = cc.astype(np.int32)
            c64 = int(cc.dtype == np.int64)
            cptr, ncells = C.c_void_p(cc.ctypes.data), cc.size // 8
        did = C.c_int(-1)
        N.call("gvr_scene_add_hex", self.handle, int(nn), cx, cy, cz, ctype, int(ncells), cptr, c64,
               fp, ftype, int(association), loc, C.byref(did))
        del k1, k2, k3, k4, cc
        self._hex_cells[did.value] = int(ncells)
        return did.value

    def hex_bvh(self, domain_id: int) -> dict:
        """The domain's LBVH as host arrays (for checking against a CPU rebuild)."""
        n = self.hex_cells(domain_id)
        out = {"codes": np.zeros(n, np.uint32), "ids": np.zeros(n, np.uint32),
               "left": np.zeros(max(n - 1, 1), np.int32), "right": np.zeros(max(n - 1, 1), np.int32),
               "parent": np.zeros(max(2 * n - 1, 1), np.int32),
               "inner_box": np.zeros((max(n - 1, 1), 6), np.float32)}
        ms = C.c_float(0)
        N.call("gvr_scene_hex_bvh", self.handle, int(domain_id), *[C.c_void_p(out[k].ctypes.data) for k in
               ("codes", "ids", "left", "right", "parent", "inner_box")], C.byref(ms))
        out["build_ms"] = ms.value
        return out

    def hex_build_ms(self, domain_id: int) -> float:
        """Wall time of the domain's on-device LBVH build (upload included)."""
        ms = C.c_float(0)
        N.call("gvr_scene_hex_bvh", self.handle, int(domain_id), None, None, None, None, None, None,
               C.byref(ms))
        return ms.value

    def hex_neighbors(self, domain_id: int, table: bool = True):
        """The domain's face-neighbour table, (n_cells, 6) int32 (None when
        table is False), and its build time in ms."""
        nbr = np.zeros((self.hex_cells(domain_id), 6), np.int32) if table else None
        ms = C.c_float(0)
        N.call("gvr_scene_hex_neighbors", self.handle, int(domain_id),
               C.c_void_p(nbr.ctypes.data) if table else None, C.byref(ms))
        return nbr, ms.value

    def hex_cells(self, domain_id: int) -> int:
        return int(self._hex_cells[domain_id])

    def hex_locate(self, domain_id: int, points):
        p = np.ascontiguousarray(points, dtype=np.float32).reshape(-1, 3)
        cells = np.zeros(len(p), np.int32)
        rst = np.zeros((len(p), 3), np.float32)
        N.call("gvr_scene_hex_locate", self.handle, int(domain_id), C.c_void_p(p.ctypes.data), len(p),
               C.c_void_p(cells.ctypes.data), C.c_void_p(rst.ctypes.data))
        return cells, rst

    def update_field(self, domain_id: int, field) -> None:
        ptr, code, keep, loc, _ = _field_args(field)
        N.call("gvr_scene_update_field", self.handle, int(domain_id), ptr, code, 1, loc)
        del keep

    def update_fields(self, domain_ids, fields, stream=None) -> None:
        """Replace several domains' fields in one pipelined upload (all numpy
        on the host, or all torch tensors on one side, same dtype)."""
        args = [_field_args(f) for f in fields]
        if len({a[1] for a in args}) > 1 or len({a[3] for a in args}) > 1:
            raise N.GvrError(N.GVR_ERR_INVALID_ARGUMENT, "fields must share dtype and location")
        ids = (C.c_int * len(args))(*[int(i) for i in domain_ids])
        ptrs = (C.c_void_p * len(args))(*[a[0].value for a in args])
        code = args[0][1] if args else N.DTYPE_FLOAT32
        loc = args[0][3] if args else N.MEM_HOST
        st = None if stream is None else C.c_void_p(int(getattr(stream, "cuda_stream", stream)))
        N.call("gvr_scene_update_fields", self.handle, len(args), ids, ptrs, code, 1, loc, st)
        del args

    def set_tuning(self, packet_w: int = 8, unroll: int = 2, min_blocks: int = 4, staged: int = 0,
                   tile_order: int = 0) -> None:
        """Launch shape of the march kernel, whether the plain path stages
        bricks in shared memory (0 no, 1 per slab of ray distance, 2 per
        brick layer, double-buffered) and how it orders its tiles (0 centre
        first, 1 longest first for each view); images depend on none."""
        N.call("gvr_scene_set_tuning", self.handle, int(packet_w), int(unroll), int(min_blocks))
        N.call("gvr_scene_set_staging", self.handle, int(staged))
        N.call("gvr_scene_set_tile_order", self.handle, int(tile_order))
        self.tuning = (int(packet_w), int(unroll), int(min_blocks), int(staged), int(tile_order))

    def staging_failures(self) -> int:
        """Tiles whose bounded wait for staged bricks gave up (0 normally)."""
        n = C.c_uint64(0)
        N.call("gvr_scene_staging_failures", self.handle, C.byref(n))
        return int(n.value)

    @property
    def num_domains(self) -> int:
        n = C.c_int()
        N.call("gvr_scene_num_domains", self.handle, C.byref(n))
        return n.value

    def bounds(self, domain_id: int = -1) -> np.ndarray:
        b = np.zeros(6, dtype=np.float64)
        N.call("gvr_scene_bounds", self.handle, int(domain_id), N.dptr(b))
        return b

    def scalar_range(self) -> np.ndarray:
        r = np.zeros(2, dtype=np.float64)
        N.call("gvr_scene_range", self.handle, N.dptr(r))
        return r

    def render(self, camera: N.Camera, params: N.RenderParams, *, device_out=False, stream=None,
               count_samples=False):
        """Render one view. Host numpy (H, W, 4)/(H, W) unless device_out, then torch CUDA tensors."""
        w, h = params.width, params.height
        n = C.c_uint64(0)
        nptr = C.byref(n) if count_samples else None
        st = C.c_void_p(stream) if stream is not None else None
        if device_out:
            import torch
            rgba = torch.empty((h, w, 4), dtype=torch.float32, device=f"cuda:{self.device}")
            depth = torch.empty((h, w), dtype=torch.float32, device=f"cuda:{self.device}")
            if stream is None:
                st = C.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)
            N.call("gvr_render_volume", self.handle, C.byref(camera), C.byref(params),
                   C.c_void_p(rgba.data_ptr()), C.c_void_p(depth.data_ptr()), N.MEM_DEVICE, st, nptr)
        else:
            rgba = np.empty((h, w, 4), dtype=np.float32)
            depth = np.empty((h, w), dtype=np.float32)
            N.call("gvr_render_volume", self.handle, C.byref(camera), C.byref(params),
                   C.c_void_p(rgba.ctypes.data), C.c_void_p(depth.ctypes.data), N.MEM_HOST, st, nptr)
        if count_samples:
            return rgba, depth, int(n.value)
        return rgba, depth

    def render_over(self, camera: N.Camera, params: N.RenderParams, canvas_rgba, canvas_depth, *,
                    count_samples=False):
        """Render the volume over an opaque canvas: canvas_rgba (H, W, 4) and
        canvas_depth (H, W, image depth, 1 = empty) as numpy arrays (host) or
        torch CUDA tensors (updated in place). Returns (rgba, depth)."""
        n = C.c_uint64(0)
        nptr = C.byref(n) if count_samples else None
        try:
            import torch
            on_device = isinstance(canvas_rgba, torch.Tensor) and canvas_rgba.is_cuda
        except ImportError:  # pragma: no cover
            on_device = False
        if on_device:
            rgba, depth = canvas_rgba, canvas_depth
            if not (rgba.is_contiguous() and depth.is_contiguous()):
                raise N.GvrError(N.GVR_ERR_INVALID_ARGUMENT, "canvas tensors must be contiguous")
            st = C.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)
            N.call("gvr_render_volume_over", self.handle, C.byref(camera), C.byref(params),
                   C.c_void_p(rgba.data_ptr()), C.c_void_p(depth.data_ptr()), N.MEM_DEVICE, st, nptr)
        else:
            rgba = np.array(canvas_rgba, dtype=np.float32, copy=True, order="C")
            depth = np.array(canvas_depth, dtype=np.float32, copy=True, order="C")
            N.call("gvr_render_volume_over", self.handle, C.byref(camera), C.byref(params),
                   C.c_void_p(rgba.ctypes.data), C.c_void_p(depth.ctypes.data), N.MEM_HOST, None, nptr)
        if count_samples:
            return rgba, depth, int(n.value)
        return rgba, depth

    def render_batch(self, cameras, params: N.RenderParams, *, device_out=False, stream=None,
                     count_samples=False, out=None):
        """Render many views in one persistent, graph-replayed launch. Returns
        (rgba (V, H, W, 4), depth (V, H, W)) as numpy, or torch CUDA tensors when
        device_out (then `out` may pass preallocated (rgba, depth) tensors)."""
        cams = (N.Camera * len(cameras))(*cameras)
        w, h, v = params.width, params.height, len(cameras)
        n = C.c_uint64(0)
        nptr = C.byref(n) if count_samples else None
        st = C.c_void_p(stream) if stream is not None else None
        if device_out:
            import torch
            if out is None:
                out = (torch.empty((v, h, w, 4), dtype=torch.float32, device=f"cuda:{self.device}"),
                       torch.empty((v, h, w), dtype=torch.float32, device=f"cuda:{self.device}"))
            rgba, depth = out
            if stream is None:
                st = C.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)
            N.call("gvr_render_volume_batch", self.handle, cams, v, C.byref(params),
                   C.c_void_p(rgba.data_ptr()), C.c_void_p(depth.data_ptr()), N.MEM_DEVICE, st, nptr)
        else:
            rgba = np.empty((v, h, w, 4), dtype=np.float32)
            depth = np.empty((v, h, w), dtype=np.float32)
            N.call("gvr_render_volume_batch", self.handle, cams, v, C.byref(params),
                   C.c_void_p(rgba.ctypes.data), C.c_void_p(depth.ctypes.data), N.MEM_HOST, st, nptr)
        if count_samples:
            return rgba, depth, int(n.value)
        return rgba, depth

    def set_batch_granularity(self, tiles_per_item: int) -> None:
        N.call("gvr_scene_set_batch_granularity", self.handle, int(tiles_per_item))

    @property
    def batch_graph_builds(self) -> int:
        n = C.c_int()
        N.call("gvr_scene_batch_graph_builds", self.handle, C.byref(n))
        return n.value

    def close(self) -> None:
        if self.handle:
            N.lib().gvr_scene_destroy(self.handle)
            self.handle = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---------------------------------------------------------------------------
# host-logic helpers (thin wrappers over the C ABI)
# ---------------------------------------------------------------------------

def correct_opacity(alpha, num_samples: int) -> np.ndarray:
    a = np.ascontiguousarray(alpha, dtype=np.float64)
    out = np.empty_like(a)
    N.call("gvr_correct_opacity", N.dptr(a), a.size, int(num_samples), N.dptr(out))
    return out


def sample_distance(bounds, num_samples: int) -> float:
    b = np.ascontiguousarray(bounds, dtype=np.float64)
    d = C.c_float()
    N.call("gvr_sample_distance", N.dptr(b), int(num_samples), C.byref(d))
    return d.value


def color_table_sample(rgb_pos, rgb, alpha_pos, alpha, n: int = 1024, uint8_mode: int = N.UINT8_NONE):
    rp = np.ascontiguousarray(rgb_pos, dtype=np.float64)
    rc = np.ascontiguousarray(rgb, dtype=np.float64).reshape(-1)
    ap = np.ascontiguousarray(alpha_pos, dtype=np.float64)
    av = np.ascontiguousarray(alpha, dtype=np.float64)
    t = N.ColorTable(len(rp), N.dptr(rp), N.dptr(rc), len(ap), N.dptr(ap), N.dptr(av))
    out = np.empty((n, 4), dtype=np.float32)
    N.call("gvr_color_table_sample", C.byref(t), int(n), int(uint8_mode), N.fptr(out))
    return out


def camera_reset_to_bounds(bounds) -> N.Camera:
    b = np.ascontiguousarray(bounds, dtype=np.float64)
    c = N.Camera()
    N.call("gvr_camera_reset_to_bounds", C.byref(c), N.dptr(b))
    return c


def camera_azimuth(cam: N.Camera, deg: float) -> None:
    N.call("gvr_camera_azimuth", C.byref(cam), float(deg))


def camera_elevation(cam: N.Camera, deg: float) -> None:
    N.call("gvr_camera_elevation", C.byref(cam), float(deg))


def cinema_cameras(bounds, phi_theta) -> list:
    b = np.ascontiguousarray(bounds, dtype=np.float64)
    pt = np.ascontiguousarray(phi_theta, dtype=np.float32).reshape(-1, 2)
    out = (N.Camera * max(len(pt), 1))()
    N.call("gvr_cinema_cameras", N.dptr(b), N.fptr(pt), len(pt), out)
    return [out[i].copy() for i in range(len(pt))]


def visibility_order(cam: N.Camera, domain_bounds) -> np.ndarray:
    b = np.ascontiguousarray(domain_bounds, dtype=np.float64).reshape(-1, 6)
    order = np.zeros(len(b), dtype=np.int32)
    N.call("gvr_visibility_order", C.byref(cam), N.dptr(b), len(b),
           order.ctypes.data_as(C.POINTER(C.c_int)))
    return order
