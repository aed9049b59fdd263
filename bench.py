#!/usr/bin/env python
"""Benchmark of Ascent's volume plot on GB300: samples/s of the fused march.

Workload (default): a 513^3-node float32 field (Gaussian blobs + 3-octave
sinusoidal turbulence, seed 2) split into 8 domains of 256^3 cells that share
face nodes, rendered at 1024x1024 with visibility-ordered compositing,
1774 samples over the bounds diagonal (0.5 cell), 256-point linear transfer
function (opacity 0 -> 0.3), camera reset to the bounds then azimuth 30,
elevation 20.

A step is one render of that view. Reported:
  value   Gsamples/s with the bricked field resident in HBM and the image
          written to device memory (CUDA events on the launching stream).
  e2e     the same metric through the C ABI with HOST buffers: every step
          uploads the 8 fields from pinned host memory (re-bricking them)
          and reads the RGBA + depth image back. Two scenes alternate so
          that step s+1's upload overlaps step s's render; the serial
          schedule (publish, render, read back, then the next step) is
          reported beside it.
  roofline  algorithmic bytes (32 B per sample + 20 B per pixel) per launch
          over the march kernel's event-timed duration, against the measured
          HBM copy bandwidth.
  cpu_baseline  the FP32 OpenMP port of the oracle on this host's cores,
          timed on a band of image rows of the same view.

--impl reference runs that CPU implementation alone (rank 0), each step a
bounded band of rows, and prints the same JSON keys.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

import numpy as np  # noqa: E402

BYTES_PER_SAMPLE = 32     # 8 float32 trilinear corners
BYTES_PER_PIXEL = 20      # RGBA float32 + depth float32
METRIC = "volume render Gsamples/s (512^3 in 8 domains, 1024^2)"
UNIT = "Gsamples/s"


def parse_args():
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--cells", type=int, default=512, help="cells per axis of the whole grid")
    ap.add_argument("--size", type=int, default=1024, help="image width = height")
    ap.add_argument("--cpu-seconds", type=float, default=12.0,
                    help="target CPU time of the cpu_baseline sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-configs", action="store_true",
                    help="skip the ingest, plain-64, hex, batched, differentiable and compositing configurations")
    ap.add_argument("--configs", default="",
                    help="comma-separated subset of ingest,plain_64,hex,batched,differentiable,composite,"
                         "zbuffer,noalloc (default: all)")
    ap.add_argument("--staging", choices=["auto", "off", "on"], default="auto",
                    help="plain path: let the tuner choose between L1 gathers and shared-memory brick "
                         "staging (auto), or time only one of them")
    return ap.parse_args()


def tile_order_ms(tuning: dict) -> dict:
    """The tuner's back-to-back timings of its winning shape with the
    centre-first (o0) and longest-first (o1) tile orders."""
    return {k: v for k, v in tuning.get("ms", {}).items() if k.endswith(("o0", "o1"))}


def peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return {"hbm_gbs": float(d["hbm_gbs"]), "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


def ncu_traffic(samples: int, pixels: int):
    """DRAM bytes per launch of the march kernel from the committed ncu summary."""
    f = ROOT / "profiles" / "march_kernel_ncu.md"
    if not f.exists():
        return None, None
    kv = {}
    for line in f.read_text().splitlines():
        if line.startswith("traffic_bytes_per_launch:"):
            kv["t"] = float(line.split(":", 1)[1])
        if line.startswith("traffic_workload:"):
            kv["w"] = line.split(":", 1)[1].strip()
    return kv.get("t"), kv.get("w")


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.file = None

    def start(self):
        try:
            self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.file, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.file.flush()
        rows = []
        for line in Path(self.file.name).read_text().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        os.unlink(self.file.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({n for r in rows for n, v in zip(names, r[5:9]) if v.lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def bricked_bytes(wl, cells: int = 8) -> int:
    """Device bytes of the bricked fields: (cells + 1)^3 nodes per brick of
    cells^3 cells, padded to a multiple of 32 floats (736 floats at 8)."""
    floats = ((cells + 1) ** 3 + 31) // 32 * 32
    total = 0
    for d in wl.domains:
        nb = 1
        for n in d.dims:
            nb *= (n - 1 + cells - 1) // cells
        total += nb * floats * 4
    return total


def workloads_module():
    """The seeded input generator (ascent_gb300/workloads.py, numpy only),
    loaded from its file so that the CPU arm never imports the product
    package or maps its library."""
    import importlib.util
    name = "gvr_bench_workloads"
    if name in sys.modules:
        return sys.modules[name]
    spec = importlib.util.spec_from_file_location(name, ROOT / "ascent_gb300" / "workloads.py")
    mod = importlib.util.module_from_spec(spec)
    sys.modules[name] = mod
    spec.loader.exec_module(mod)
    return mod


def setup_workload(args):
    W = workloads_module()
    t = time.time()
    wl = W.plain_large(n_cells=args.cells, width=args.size, height=args.size)
    return wl, time.time() - t


def bench_config(wl, args) -> dict:
    """The workload description both arms print, key for key."""
    return {"workload": wl.name, "grid_nodes": args.cells + 1, "domains": len(wl.domains),
            "image": [wl.width, wl.height], "samples_param": wl.samples,
            "sample_dist_cells": 0.5, "early_term": 0.99,
            "lut": "1024-entry float LUT for both arms; the reference's multi-domain "
                   "uint8 LUT would round opacity to 0 below s=0.98 at 1774 samples",
            "l2": f"field {sum(d.field.nbytes for d in wl.domains) / 2**20:.0f} MiB (more once "
                  "bricked) against a 129 MB L2; not flushed"}


def oracle_setup(wl, *, float_lut=False, camera=None):
    """Camera and render parameters built by the oracle's own functions
    (never the product library's): opacity correction, LUT sampling, sample
    distance and camera. float_lut: the benchmark's 1024-entry float LUT on
    the multi-domain path; camera: (phi, theta) of a Cinema view instead of
    the workload's reset + azimuth + elevation camera."""
    from oracle import oracle as O
    if camera is None:
        cam = O.workload_camera(wl)
    else:
        cam = O.cinema_cameras(wl.bounds, [camera])[0]
    if float_lut:
        params = O.workload_params(wl, lut=O.workload_lut(wl, single_domain=True), single_domain=False)
    else:
        params = O.workload_params(wl)
    return cam, params


def oracle_scene_of(wl, precision):
    from oracle import oracle as O
    osc = O.OracleScene(precision)
    for d in wl.domains:
        if hasattr(d, "conn"):
            osc.add_hex(d.x, d.y, d.z, d.conn, d.field)
        else:
            osc.add_uniform(d.dims, d.origin, d.spacing, d.field)
    return osc


def bench_params(wl):
    """Float 1024-entry LUT (see config["lut"]), no uint8 canvas round trip."""
    from ascent_gb300 import _native as N
    from ascent_gb300 import volume as V
    vr = V.workload_renderer(wl)
    lut = vr.lut(single_domain=True)          # float LUT
    return vr.params(wl.width, wl.height, wl.bounds, wl.scalar_range, single_domain=False, lut=lut), N


def cpu_sample(wl, seconds: float, *, float_lut=False, camera=None):
    """Time the FP32 OpenMP port of the oracle on this host's cores for about
    `seconds`: whole frames when one frame fits in a third of that, else
    bands of image rows (at least four rows per thread, walking outwards from
    the centre row) so that every thread has rows to render. Camera and
    parameters are built by the oracle (oracle_setup)."""
    from oracle import oracle as O
    cam, params = oracle_setup(wl, float_lut=float_lut, camera=camera)
    osc = oracle_scene_of(wl, 32)
    threads = O.num_threads(32)
    h, w = params.height, params.width
    rgba = np.zeros((h, w, 4), np.float32)
    depth = np.zeros((h, w), np.float32)
    # probe: a band of 4 rows per thread around the centre
    band = min(h, 4 * threads)
    r0 = max(0, h // 2 - band // 2)
    t0 = time.perf_counter()
    osc.render_rows(cam, params, r0, r0 + band, rgba, depth)
    per_row = max((time.perf_counter() - t0) / band, 1e-6)
    whole = per_row * h <= seconds / 3
    samples = rows = frames = 0
    t0 = time.perf_counter()
    if whole:
        while True:
            samples += osc.render_rows(cam, params, 0, h, rgba, depth)
            rows += h
            frames += 1
            if time.perf_counter() - t0 >= seconds:
                break
        what = f"{frames} whole {w}x{h} frames"
    else:
        row = r0
        while True:
            a = row % h
            b = min(a + band, h)
            samples += osc.render_rows(cam, params, a, b, rgba, depth)
            rows += b - a
            row = b if b < h else 0
            if time.perf_counter() - t0 >= seconds:
                break
        what = f"{rows} of {h} image rows in bands of {band} from the centre row"
    dt = time.perf_counter() - t0
    return {"value": samples / dt / 1e9, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{what} of the same view, {samples} samples in {dt:.1f} s; FP32 OpenMP "
                      "port of the oracle (camera, LUT and sample distance set up by the oracle)"}


def _timed(fn, stream, reps):
    """Median ms of `reps` calls of fn, CUDA events on `stream`."""
    import torch
    times = []
    for _ in range(reps):
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        fn()
        b.record(stream)
        b.synchronize()
        times.append(a.elapsed_time(b))
    return statistics.median(times)


def bench_hex(dev, n_cells=200, size=1024, reps=5):
    """Unstructured hexahedra: jittered n_cells^3 grid, device LBVH + Newton march."""
    import ctypes as C
    import torch
    from ascent_gb300 import _native as N
    from ascent_gb300 import scene as S
    from ascent_gb300 import volume as V
    from ascent_gb300 import workloads as W
    t0 = time.time()
    wl = W.hex_mesh(n_cells=n_cells, width=size, height=size)
    gen_s = time.time() - t0
    cam = V.workload_camera(wl)
    p = V.workload_params(wl)
    sc = S.Scene(dev)
    t0 = time.time()
    V.load_workload(sc, wl)
    load_s = time.time() - t0
    build_ms = sc.hex_build_ms(0)
    _, nbr_ms = sc.hex_neighbors(0, table=False)
    stream = torch.cuda.current_stream(dev)
    rgba = torch.empty((size, size, 4), dtype=torch.float32, device=f"cuda:{dev}")
    depth = torch.empty((size, size), dtype=torch.float32, device=f"cuda:{dev}")
    from ascent_gb300 import tune
    tuning = tune.autotune(sc, cam, p, reps=2, use_cache=False, staged=False)
    _, _, n = sc.render(cam, p, device_out=True, count_samples=True)
    args = (sc.handle, C.byref(cam), C.byref(p), C.c_void_p(rgba.data_ptr()), C.c_void_p(depth.data_ptr()),
            N.MEM_DEVICE, C.c_void_p(stream.cuda_stream), None)
    for _ in range(2):
        N.call("gvr_render_volume", *args)
    ms = _timed(lambda: N.call("gvr_render_volume", *args), stream, reps)
    pk = peaks()
    alg = n * 160 + size * size * BYTES_PER_PIXEL
    sc.close()
    ocam, op = oracle_setup(wl)
    acc = accuracy(dev, wl, [cam], p, [ocam], op)
    acc["pixels_fraction"] = acc["pixels_checked"] / (size * size)
    cpu = cpu_sample(wl, 5.0)
    return {"workload": wl.name, "cells": n_cells ** 3, "samples_per_frame": n,
            "error_vs_fp64_oracle": acc,
            "gsamples_per_s": n / ms / 1e6, "fps": 1e3 / ms, "ms_per_frame": ms,
            "cpu_port_gsamples_per_s": cpu["value"], "cpu_cores": cpu["cores"],
            "speedup_vs_cpu_port": n / ms / 1e6 / cpu["value"],
            "bvh_build_ms": build_ms, "face_neighbour_build_ms": nbr_ms, "load_s": round(load_s, 2), "generate_s": round(gen_s, 2),
            "tuning": tuning["best"], "tile_order_ms": tile_order_ms(tuning),
            "roofline": {"bound": "hbm", "achieved": alg / ms / 1e6, "peak": pk["hbm_gbs"],
                         "unit": "GB/s", "frac": alg / ms / 1e6 / pk["hbm_gbs"],
                         "bytes_per_sample": 160}}


def bench_batch(dev, reps=5):
    """37 uneven uniform domains, 64 Cinema views at 512^2: one persistent
    graph-replayed batch launch vs the plain per-view loop (device images)."""
    import ctypes as C
    import torch
    from ascent_gb300 import _native as N
    from ascent_gb300 import scene as S
    from ascent_gb300 import tune
    from ascent_gb300 import volume as V
    from ascent_gb300 import workloads as W
    from oracle import oracle as O
    wl = W.cinema_batch()
    cams = S.cinema_cameras(wl.bounds, wl.phi_theta)
    p = V.workload_params(wl)
    sc = S.Scene(dev)
    V.load_workload(sc, wl)
    stream = torch.cuda.current_stream(dev)
    v, h, w = len(cams), p.height, p.width
    out = (torch.empty((v, h, w, 4), dtype=torch.float32, device=f"cuda:{dev}"),
           torch.empty((v, h, w), dtype=torch.float32, device=f"cuda:{dev}"))
    # plain per-view loop, tuned for a single view
    single = tune.autotune(sc, cams[0], p, reps=2, use_cache=False)["best"]
    sptr = C.c_void_p(stream.cuda_stream)
    stride4, stride1 = h * w * 4 * 4, h * w * 4
    base4, base1 = out[0].data_ptr(), out[1].data_ptr()
    calls = [(sc.handle, C.byref(cams[i]), C.byref(p), C.c_void_p(base4 + i * stride4),
              C.c_void_p(base1 + i * stride1), N.MEM_DEVICE, sptr, None) for i in range(v)]

    def loop():
        for a in calls:
            N.call("gvr_render_volume", *a)

    loop()
    loop_ms = _timed(loop, stream, reps)
    ref = out[0].clone()
    # batched: tuned launch shape and queue granularity
    best = tune.autotune_batch(sc, cams, p, reps=2)
    _, _, n = sc.render_batch(cams, p, device_out=True, out=out, count_samples=True)
    batch_ms = _timed(lambda: sc.render_batch(cams, p, device_out=True, out=out), stream, reps)
    same = bool(torch.equal(ref, out[0]))
    builds = sc.batch_graph_builds
    sc.close()
    # every fourth view, whole images: a quarter of the batch's pixels
    picks = list(range(0, v, 4))
    _, op = oracle_setup(wl)
    ocams = O.cinema_cameras(wl.bounds, [wl.phi_theta[i] for i in picks])
    acc = accuracy(dev, wl, [cams[i] for i in picks], p, ocams, op)
    acc["pixels_fraction"] = acc["pixels_checked"] / (v * h * w)
    cpu = cpu_sample(wl, 5.0, camera=wl.phi_theta[0])
    cpu_images = cpu["value"] * 1e9 / (n / v)
    return {"workload": wl.name, "domains": len(wl.domains), "views": v, "image": [w, h],
            "cpu_port_images_per_s": cpu_images, "cpu_cores": cpu["cores"],
            "speedup_vs_cpu_port": v * 1e3 / batch_ms / cpu_images,
            "samples_per_batch": n, "per_view_loop_ms": loop_ms, "batched_ms": batch_ms,
            "per_view_loop_images_per_s": v * 1e3 / loop_ms, "batched_images_per_s": v * 1e3 / batch_ms,
            "speedup": loop_ms / batch_ms, "batched_gsamples_per_s": n / batch_ms / 1e6,
            "images_identical_to_loop": same, "loop_tuning": single, "batch_tuning": best["best"],
            "error_vs_fp64_oracle": acc,
            "graph_captures": builds}


def bench_diff(dev, n=128, views=16, size=256, reps=5):
    """Differentiable render: n^3 field, 256-entry LUT, `views` Cinema views at
    size^2; L2 loss against images of the field + N(0, 0.05) (seed 5)."""
    import torch
    from ascent_gb300 import diff as D
    from ascent_gb300 import scene as S
    from ascent_gb300 import workloads as W
    wl = W.plain_small(n=n, width=size, height=size, seed=5)
    d = wl.domains[0]
    side = int(round(views ** 0.5))
    cams = S.cinema_cameras(wl.bounds, W.cinema_angles(side, views // side))
    x = np.linspace(0, 1, 256)
    lut = torch.from_numpy(np.stack([x, np.full_like(x, 0.5), 1 - x, 0.3 * x], 1).astype(np.float32)).cuda(dev)
    sd = S.sample_distance(wl.bounds, int(np.ceil(np.sqrt(3) * (n - 1) / 0.5)))
    rng = np.random.default_rng(5)
    gt = torch.from_numpy(d.field).cuda(dev)
    with torch.no_grad():
        pert = gt + torch.from_numpy(rng.normal(0, 0.05, d.field.shape).astype(np.float32)).cuda(dev)
        target = D.render(pert, lut, cams, d.origin, d.spacing, size, size, sd, wl.scalar_range)
    f = gt.clone().requires_grad_(True)
    lt = lut.clone().requires_grad_(True)
    stream = torch.cuda.current_stream(dev)

    def fwd():
        with torch.no_grad():
            return D.render(f, lt, cams, d.origin, d.spacing, size, size, sd, wl.scalar_range)

    def fwd_bwd():
        f.grad = None
        lt.grad = None
        img = D.render(f, lt, cams, d.origin, d.spacing, size, size, sd, wl.scalar_range)
        ((img - target) ** 2).sum().backward()

    def fwd_train():
        return D.render(f, lt, cams, d.origin, d.spacing, size, size, sd, wl.scalar_range)

    for _ in range(2):
        fwd_bwd()
    fwd_ms = _timed(fwd, stream, reps)
    train_ms = _timed(fwd_train, stream, reps)
    fb_ms = _timed(fwd_bwd, stream, reps)
    from oracle import oracle as O
    # a quarter of the views, whole images, against the FP64 oracle with its
    # own cameras and sample distance
    picks = list(range(0, views, 4))
    p = O.make_params(size, size, O.sample_distance(wl.bounds, int(np.ceil(np.sqrt(3) * (n - 1) / 0.5))),
                      wl.scalar_range, lut.cpu().numpy(), lut_filter=O.LUT_LINEAR, alpha_cull=0.0,
                      early_term=1.0)
    ocams = O.cinema_cameras(wl.bounds, W.cinema_angles(side, views // side)[picks])
    osc = O.OracleScene(64)
    osc.add_uniform(d.dims, d.origin, d.spacing, d.field)
    with torch.no_grad():
        img = D.render(gt, lut, [cams[i] for i in picks], d.origin, d.spacing, size, size, sd,
                       wl.scalar_range).cpu().numpy()
    errs = [_err(img[k], osc.render(ocams[k], p)[0]) for k in range(len(picks))]
    acc = {k: max(e[k] for e in errs) if k != "frac_within_2_255" else min(e[k] for e in errs)
           for k in errs[0]}
    acc.update({"views": len(picks), "pixels_fraction": len(picks) / views,
                "oracle": "FP64 CPU oracle (oracle/gvr_oracle.c), linear LUT, no cull, set up by the oracle"})
    return {"workload": f"diff{n}^3x{views}views@{size}x{size}", "lut": 256, "checkpoint_every": 64,
            "error_vs_fp64_oracle": acc,
            "fwd_ms": fwd_ms, "fwd_train_ms": train_ms, "fwd_bwd_ms": fb_ms,
            "fwd_bwd_over_fwd": fb_ms / fwd_ms,
            "note": "fwd = inference forward (no workspace); fwd_bwd = training forward "
                    "(checkpoints + per-sample scalars) + L2 loss + adjoint",
            "grad_field_norm": float(f.grad.norm()), "grad_lut_norm": float(lt.grad.norm())}


def _err(g, o) -> dict:
    d = np.abs(g.astype(np.float64) - o.astype(np.float64))
    return {"max": float(d.max()), "mae": float(d.mean()),
            "frac_within_2_255": float((d <= 2 / 255 + 1e-7).all(axis=-1).mean()),
            "frac_over_4_255": float((d > 4 / 255).any(axis=-1).mean())}


def accuracy(dev, wl, cams, params, oracle_cams, oracle_params, rows=None, precision=64) -> dict:
    """Error of the GPU images against the FP64 oracle on the same inputs,
    over image rows [rows[0], rows[1]) (the whole image when None). The GPU
    renders with the product's cameras and parameters, the oracle with its
    own (oracle_setup), so the set-up is compared too."""
    from ascent_gb300 import scene as S
    from ascent_gb300 import volume as V
    osc = oracle_scene_of(wl, precision)
    h, w = params.height, params.width
    r0, r1 = rows if rows else (0, h)
    out = []
    with S.Scene(dev) as sc:
        V.load_workload(sc, wl)
        for cam, ocam in zip(cams, oracle_cams):
            g, _ = sc.render(cam, params)
            o = np.zeros((h, w, 4), np.float32)
            dep = np.zeros((h, w), np.float32)
            t0 = time.perf_counter()
            osc.render_rows(ocam, oracle_params, r0, r1, o, dep)
            e = _err(g[r0:r1], o[r0:r1])
            e["oracle_s"] = round(time.perf_counter() - t0, 2)
            out.append(e)
    worst = {k: (max if k in ("max", "mae", "frac_over_4_255") else min)(e[k] for e in out)
             for k in ("max", "mae", "frac_within_2_255", "frac_over_4_255")}
    worst["rows"] = [r0, r1]
    worst["views"] = len(cams)
    worst["pixels_checked"] = len(cams) * (r1 - r0) * w
    worst["oracle_s"] = round(sum(e["oracle_s"] for e in out), 1)
    worst["oracle"] = "FP64 CPU oracle (oracle/gvr_oracle.c), set up by the oracle"
    return worst


def bench_composite(dev, n_images=8, size=1024, cover=0.8, reps=10) -> dict:
    """Standalone partial compositing (PartialCompositor::composite): n_images
    partial images of size^2 pixels, each covering a seeded `cover` fraction
    of the pixels with random depths and premultiplied colours (seed 6);
    records resident on the device. Checked byte for byte against the FP32
    restatement of the reference compositor."""
    import torch
    from ascent_gb300 import compositing as CP
    from oracle import oracle as O
    rng = np.random.default_rng(6)
    ims = []
    for _ in range(n_images):
        ids = np.nonzero(rng.uniform(size=size * size) < cover)[0]
        p = np.zeros(len(ids), CP.PARTIAL_DTYPE)
        p["pixel_id"] = ids
        p["depth"] = rng.uniform(0, 10, len(ids)).astype(np.float32)
        a = rng.uniform(0.001, 1.0, len(ids)).astype(np.float32)
        p["alpha"] = a
        p["rgb"] = (rng.uniform(0, 1, (len(ids), 3)) * a[:, None]).astype(np.float32)
        ims.append(p)
    flat = np.concatenate(ims)
    d = CP.to_device(flat, f"cuda:{dev}")
    stream = torch.cuda.current_stream(dev)
    for _ in range(3):
        out = CP.composite_partials_device(d)
    ms = _timed(lambda: CP.composite_partials_device(d), stream, reps)
    out = CP.from_device(CP.composite_partials_device(d))
    ref = O.composite_partials_f32(ims)
    exact = out.tobytes() == ref.tobytes()
    # the caller-range path: ids known to lie in [0, size^2), count left on
    # the device, no host synchronisation inside the call
    aout, an = CP.composite_partials_device_async(d, 0, size * size - 1)
    for _ in range(3):
        CP.composite_partials_device_async(d, 0, size * size - 1, out=aout, n_out=an)
    async_ms = _timed(lambda: CP.composite_partials_device_async(d, 0, size * size - 1, out=aout, n_out=an),
                      stream, reps)
    async_exact = CP.from_device(aout[: int(an.item())]).tobytes() == ref.tobytes()
    # the same call through the C ABI with its arguments built once
    import ctypes as C
    from ascent_gb300 import _native as N
    cargs = (d.data_ptr(), d.shape[0], 0, size * size - 1, aout.data_ptr(), an.data_ptr(),
             C.c_void_p(stream.cuda_stream))
    for _ in range(3):
        N.call("gvr_composite_partials_async", *cargs)
    cabi_ms = _timed(lambda: N.call("gvr_composite_partials_async", *cargs), stream, reps)
    t0 = time.perf_counter()
    O.composite_partials(ims, precision=32)
    cpu_s = time.perf_counter() - t0
    alg = 24 * (len(flat) + len(out))
    pk = peaks()
    return {"workload": f"composite{n_images}x{size}^2@{cover}", "records": len(flat),
            "pixels_out": len(out), "ms": ms, "grecords_per_s": len(flat) / ms / 1e6,
            "bit_identical_to_reference_order_f32": exact,
            "caller_range_ms": async_ms, "caller_range_bit_identical": async_exact,
            "caller_range_roofline_frac": alg / (async_ms / 1e3) / 1e9 / peaks()["hbm_gbs"],
            "caller_range_c_abi_ms": cabi_ms,
            "cpu_oracle_ms": cpu_s * 1e3, "cpu_oracle_kind": "oracle C compositor (qsort, 1 thread)",
            "roofline": {"bound": "hbm", "achieved": alg / (ms / 1e3) / 1e9, "peak": pk["hbm_gbs"],
                         "unit": "GB/s", "frac": alg / (ms / 1e3) / 1e9 / pk["hbm_gbs"],
                         "bytes_per_record": "24 read + 24 per output record"}}


def bench_noalloc(dev, n_cells=512, size=1024, reps=10) -> dict:
    """gvr_render_uniform_noalloc (no device allocation; the caller's field
    read in its plain node layout) on the benchmark's 513^3 field as one
    domain at 1024^2, beside gvr_render_volume on a scene holding the same
    domain in bricks; both through the C ABI with prebuilt arguments. The
    two images are compared with each other over the whole frame."""
    import ctypes as C
    import torch
    from ascent_gb300 import _native as N
    from ascent_gb300 import scene as S
    from ascent_gb300 import volume as V
    W = workloads_module()
    wl = W.plain_large(n_cells=n_cells, width=size, height=size, parts=(1, 1, 1))
    d = wl.domains[0]
    cam = V.workload_camera(wl)
    p = V.workload_params(wl)
    stream = torch.cuda.current_stream(dev)
    field = torch.from_numpy(d.field).cuda(dev)
    rgba = torch.empty((size, size, 4), dtype=torch.float32, device=f"cuda:{dev}")
    depth = torch.empty((size, size), dtype=torch.float32, device=f"cuda:{dev}")
    fn = N.lib().gvr_render_uniform_noalloc
    fn.restype = C.c_int
    fn.argtypes = [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_double), C.POINTER(C.c_double),
                   C.POINTER(N.Camera), C.POINTER(N.RenderParams), C.c_void_p, C.c_void_p,
                   C.c_void_p, C.POINTER(C.c_uint64)]
    dims = (C.c_int * 3)(*d.dims)
    origin = (C.c_double * 3)(*d.origin)
    spacing = (C.c_double * 3)(*d.spacing)
    args = (C.c_void_p(field.data_ptr()), dims, origin, spacing, C.byref(cam), C.byref(p),
            C.c_void_p(rgba.data_ptr()), C.c_void_p(depth.data_ptr()), C.c_void_p(stream.cuda_stream))
    n = C.c_uint64(0)
    if fn(*args, C.byref(n)) != 0:
        raise RuntimeError(N.lib().gvr_last_error())
    samples = int(n.value)

    def call():
        if fn(*args, None) != 0:
            raise RuntimeError(N.lib().gvr_last_error())
    for _ in range(3):
        call()
    ms = _timed(call, stream, reps)
    na_img = rgba.cpu().numpy()
    with S.Scene(dev) as sc:
        sc.add_uniform(d.field, d.origin, d.spacing)
        sargs = (sc.handle, C.byref(cam), C.byref(p), C.c_void_p(rgba.data_ptr()),
                 C.c_void_p(depth.data_ptr()), N.MEM_DEVICE, C.c_void_p(stream.cuda_stream), None)
        for _ in range(3):
            N.call("gvr_render_volume", *sargs)
        scene_ms = _timed(lambda: N.call("gvr_render_volume", *sargs), stream, reps)
        sc_img = rgba.cpu().numpy()
    err = np.abs(na_img.astype(np.float64) - sc_img)
    del field
    return {"workload": f"noalloc uniform{n_cells}^3x1dom@{size}x{size}", "samples_per_frame": samples,
            "ms_per_frame": ms, "gsamples_per_s": samples / ms / 1e6,
            "scene_path_ms_per_frame": scene_ms, "scene_path_gsamples_per_s": samples / scene_ms / 1e6,
            "vs_scene_path": {"max": float(err.max()),
                              "frac_within_2_255": float((err <= 2 / 255 + 1e-7).all(axis=-1).mean())}}


def bench_zbuffer(dev, n_images=4, size=1024, reps=20) -> dict:
    """Z-buffer compositing of n_images opaque 1024^2 canvases (RGBA float +
    depth, device memory; seeded colours, depths uniform in [0, 1.2] so that
    some pixels hold nothing), checked bit for bit against the oracle's
    restatement of ImageCompositor::ZBufferComposite. Algorithmic bytes:
    each image's depth (4 B per pixel), the winning image's colour (16 B)
    and the result (20 B) per pixel."""
    import torch
    from ascent_gb300 import compositing as CP
    from oracle import oracle as O
    rng = np.random.default_rng(7)
    cols = [rng.uniform(0, 1, (size, size, 4)).astype(np.float32) for _ in range(n_images)]
    deps = [rng.uniform(0, 1.2, (size, size)).astype(np.float32) for _ in range(n_images)]
    dc = [torch.from_numpy(c).cuda(dev) for c in cols]
    dd = [torch.from_numpy(d).cuda(dev) for d in deps]
    import ctypes as C
    from ascent_gb300 import _native as N
    stream = torch.cuda.current_stream(dev)
    for _ in range(3):
        out = CP.zbuffer_composite(dc, dd)
    py_ms = _timed(lambda: CP.zbuffer_composite(dc, dd), stream, reps)
    # the C ABI call with its arguments built once, as the march is timed
    cp = (C.c_void_p * n_images)(*[c.data_ptr() for c in dc])
    dp = (C.c_void_p * n_images)(*[d.data_ptr() for d in dd])
    args = (n_images, cp, dp, size, size, C.c_void_p(out[0].data_ptr()), C.c_void_p(out[1].data_ptr()),
            N.MEM_DEVICE, C.c_void_p(stream.cuda_stream))
    for _ in range(3):
        N.call("gvr_zbuffer_composite", *args)
    ms = _timed(lambda: N.call("gvr_zbuffer_composite", *args), stream, reps)
    o, od = O.zbuffer_composite(cols, deps)
    exact = bool(np.array_equal(out[0].cpu().numpy(), o) and np.array_equal(out[1].cpu().numpy(), od))
    alg = (4 * n_images + 16 + 20) * size * size
    pk = peaks()
    return {"workload": f"zbuffer{n_images}x{size}^2", "ms": ms, "python_call_ms": py_ms,
            "bit_identical_to_oracle": exact,
            "roofline": {"bound": "hbm", "achieved": alg / ms / 1e6, "peak": pk["hbm_gbs"], "unit": "GB/s",
                         "frac": alg / ms / 1e6 / pk["hbm_gbs"],
                         "bytes": "4 B depth per pixel per canvas + 16 B of the winner's colour + 20 B written"}}


def bench_ingest(dev, wl, reps=20) -> dict:
    """Device-resident publish: the workload's fields already in device
    memory (a simulation's arrays) re-bricked by one gvr_scene_update_fields
    call; algorithmic bytes = field read + bricks written."""
    import torch
    from ascent_gb300 import scene as S
    from ascent_gb300 import volume as V
    fields = [torch.from_numpy(d.field).cuda(dev) for d in wl.domains]
    ids = list(range(len(fields)))
    stream = torch.cuda.current_stream(dev)
    with S.Scene(dev) as sc:
        V.load_workload(sc, wl)
        for _ in range(3):
            sc.update_fields(ids, fields)
        ms = _timed(lambda: sc.update_fields(ids, fields), stream, reps)
    alg = sum(d.field.nbytes for d in wl.domains) + bricked_bytes(wl)
    pk = peaks()
    return {"workload": f"publish {len(fields)} x {wl.domains[0].dims[0]}^3 float32 from device memory",
            "ms": ms, "gb_per_s": alg / ms / 1e6,
            "roofline": {"bound": "hbm", "achieved": alg / ms / 1e6, "peak": pk["hbm_gbs"], "unit": "GB/s",
                         "frac": alg / ms / 1e6 / pk["hbm_gbs"],
                         "bytes": "field read + bricks written (736 floats per 8^3-cell brick)"}}


def bench_plain_small(dev, reps=20) -> dict:
    """The CPU-runnable plain case: one 64^3 field, 512^2, 218 samples,
    single-domain path (float LUT, uint8 canvas round trip)."""
    import ctypes as C
    import torch
    from ascent_gb300 import _native as N
    from ascent_gb300 import scene as S
    from ascent_gb300 import volume as V
    from ascent_gb300 import workloads as W
    wl = W.plain_small()
    cam = V.workload_camera(wl)
    p = V.workload_params(wl)
    stream = torch.cuda.current_stream(dev)
    with S.Scene(dev) as sc:
        V.load_workload(sc, wl)
        rgba = torch.empty((512, 512, 4), dtype=torch.float32, device=f"cuda:{dev}")
        depth = torch.empty((512, 512), dtype=torch.float32, device=f"cuda:{dev}")
        from ascent_gb300 import tune
        tuning = tune.autotune(sc, cam, p, reps=3, use_cache=False)
        _, _, n = sc.render(cam, p, device_out=True, count_samples=True)
        args = (sc.handle, C.byref(cam), C.byref(p), C.c_void_p(rgba.data_ptr()),
                C.c_void_p(depth.data_ptr()), N.MEM_DEVICE, C.c_void_p(stream.cuda_stream), None)
        for _ in range(3):
            N.call("gvr_render_volume", *args)
        ms = _timed(lambda: N.call("gvr_render_volume", *args), stream, reps)
    cpu = cpu_sample(wl, 3.0)
    ocam, op = oracle_setup(wl)
    return {"workload": wl.name, "samples_per_frame": n, "gsamples_per_s": n / ms / 1e6,
            "fps": 1e3 / ms, "ms_per_frame": ms, "tuning": tuning["best"],
            "tile_order_ms": tile_order_ms(tuning),
            "cpu_port_gsamples_per_s": cpu["value"],
            "speedup_vs_cpu_port": n / ms / 1e6 / cpu["value"],
            "error_vs_fp64_oracle": accuracy(dev, wl, [cam], p, [ocam], op)}


def run_reference(args):
    """The CPU implementation of the path on this host (rank 0 only): the
    oracle's FP32 OpenMP port, set up by the oracle's own functions, on all
    host threads. A step is one whole frame of the workload; when the run
    would take over three minutes that way, a step is a band of rows (at
    least four per thread) sized to fit. Neither the product package nor its
    library is loaded."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    from oracle import oracle as O
    wl, _ = setup_workload(args)
    cam, params = oracle_setup(wl, float_lut=True)
    osc = oracle_scene_of(wl, 32)
    cores = O.num_threads(32)
    h, w = params.height, params.width
    rgba = np.zeros((h, w, 4), np.float32)
    depth = np.zeros((h, w), np.float32)
    # the first warm-up frame doubles as the estimate of a frame's time
    t0 = time.perf_counter()
    osc.render_rows(cam, params, 0, h, rgba, depth)
    frame_s = time.perf_counter() - t0
    budget = 180.0
    runs = args.steps + max(args.warmup - 1, 0)
    if frame_s * runs <= budget:
        r0, r1 = 0, h
    else:
        band = int(min(h, max(4 * cores, h * budget / (frame_s * runs))))
        r0 = max(0, h // 2 - band // 2)
        r1 = r0 + band
    for _ in range(max(args.warmup - 1, 0)):
        osc.render_rows(cam, params, r0, r1, rgba, depth)
    total = 0
    t0 = time.perf_counter()
    for _ in range(args.steps):
        total += osc.render_rows(cam, params, r0, r1, rgba, depth)
    dt = time.perf_counter() - t0
    value = total / dt / 1e9
    sample = (f"whole {w}x{h} frames, one per step" if (r0, r1) == (0, h) else
              f"rows {r0}..{r1} of {h} per step (whole frames would exceed {budget:.0f} s)")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "config": bench_config(wl, args),
            "samples_per_step": total // max(args.steps, 1),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": sample + "; the reference's VTK-m renderer cannot be built "
                                       "here, this is the oracle's FP32 OpenMP port of the same "
                                       "algorithm, set up by the oracle"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def max_over_ranks(x: float, dist=None, device=None) -> float:
    """Largest x over the ranks of the process group (x itself on one rank):
    the job's time is its slowest rank's."""
    if dist is None:
        return float(x)
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_rate(world: int, units_per_step: float, steps: int, seconds: float) -> float:
    """Whole-job rate (G units/s) of `world` replicas each doing
    units_per_step per step, the job taking `seconds` for `steps` steps."""
    return world * units_per_step * steps / seconds / 1e9


def run_ours(args):
    import torch
    from ascent_gb300 import _native as N
    from ascent_gb300 import scene as S
    from ascent_gb300 import volume as V

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    dev = local

    wl, gen_s = setup_workload(args)
    cam = V.workload_camera(wl)
    params, _ = bench_params(wl)
    pixels = wl.width * wl.height
    stream = torch.cuda.current_stream(dev)
    sptr = stream.cuda_stream

    # brick size and launch shape for this scene and view (untimed): one
    # scene per brick size, the fastest kept; then the sample count of the
    # view (deterministic) and the warm-up
    from ascent_gb300 import tune

    def build_scene(cells):
        sc = S.Scene(dev, brick_cells=cells)
        V.load_workload(sc, wl)
        return sc

    if args.staging == "on":
        scene = build_scene(8)
        tuning = tune.autotune(scene, cam, params, use_cache=False, only_staged=True)
        tuning["best"] = dict(tuning["best"], brick_cells=8)
    else:
        tuning = tune.autotune_bricks(build_scene, cam, params, staged=args.staging != "off")
        scene = tuning.pop("scene")
    _, _, n_samples = scene.render(cam, params, device_out=True, stream=sptr, count_samples=True)
    for _ in range(max(args.warmup, 3)):
        scene.render(cam, params, device_out=True, stream=sptr)
    torch.cuda.synchronize()

    rgba = torch.empty((wl.height, wl.width, 4), dtype=torch.float32, device=f"cuda:{dev}")
    depth = torch.empty((wl.height, wl.width), dtype=torch.float32, device=f"cuda:{dev}")
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    import ctypes as C
    clocks = ClockSampler(dev)
    clocks.start()
    time.sleep(0.3)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    launches0 = N.launch_count()
    for i in range(args.steps):
        starts[i].record(stream)
        N.call("gvr_render_volume", scene.handle, C.byref(cam), C.byref(params),
               C.c_void_p(rgba.data_ptr()), C.c_void_p(depth.data_ptr()), N.MEM_DEVICE,
               C.c_void_p(sptr), None)
        ends[i].record(stream)
    torch.cuda.synchronize()
    launches = N.launch_count() - launches0
    if dist:
        dist.barrier()
    per = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    total_ms = starts[0].elapsed_time(ends[-1])
    total_ms = max_over_ranks(total_ms, dist, f"cuda:{dev}")

    # end to end: host fields -> C ABI (upload + re-brick) -> render -> host image
    host_fields = [torch.from_numpy(d.field).pin_memory() for d in wl.domains]
    h_rgba = torch.empty((wl.height, wl.width, 4), dtype=torch.float32).pin_memory()
    h_depth = torch.empty((wl.height, wl.width), dtype=torch.float32).pin_memory()
    e2e_steps = max(3, min(args.steps, 20))

    ids = (C.c_int * len(host_fields))(*range(len(host_fields)))
    ptrs = (C.c_void_p * len(host_fields))(*[f.data_ptr() for f in host_fields])

    def e2e_step():
        # one publish of the 8 domains: pipelined H2D copies + bricking
        N.call("gvr_scene_update_fields", scene.handle, len(host_fields), ids, ptrs,
               N.DTYPE_FLOAT32, 1, N.MEM_HOST, None)
        N.call("gvr_render_volume", scene.handle, C.byref(cam), C.byref(params),
               C.c_void_p(h_rgba.data_ptr()), C.c_void_p(h_depth.data_ptr()), N.MEM_HOST, None, None)

    # serial: each step publishes, renders and reads its image back before
    # the next starts
    e2e_step()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        e2e_step()
    torch.cuda.synchronize()
    serial_s = max_over_ranks(time.perf_counter() - t0, dist, f"cuda:{dev}")

    # overlapped: two scenes, each driven by its own host thread (one thread
    # per scene, as the C ABI requires) on its own stream, take the steps in
    # turn; one scene's host-to-device copies (copy engine) and bricking run
    # while the other renders, and neither waits for the other's blocking
    # publish. Every step still uploads its fields and reads its image back.
    import threading
    scene2 = S.Scene(dev, brick_cells=scene.brick_cells)
    V.load_workload(scene2, wl)
    scene2.set_tuning(*scene.tuning)
    pair = [scene, scene2]
    streams = [torch.cuda.Stream(dev), torch.cuda.Stream(dev)]
    d_img = [(torch.empty_like(rgba), torch.empty_like(depth)) for _ in range(2)]
    h_img = [(torch.empty_like(h_rgba).pin_memory(), torch.empty_like(h_depth).pin_memory())
             for _ in range(2)]

    def e2e_worker(j, n_steps, errors):
        try:
            torch.cuda.set_device(dev)
            sp = C.c_void_p(streams[j].cuda_stream)
            for _ in range(n_steps):
                N.call("gvr_scene_update_fields", pair[j].handle, len(host_fields), ids, ptrs,
                       N.DTYPE_FLOAT32, 1, N.MEM_HOST, sp)
                N.call("gvr_render_volume", pair[j].handle, C.byref(cam), C.byref(params),
                       C.c_void_p(d_img[j][0].data_ptr()), C.c_void_p(d_img[j][1].data_ptr()),
                       N.MEM_DEVICE, sp, None)
                with torch.cuda.stream(streams[j]):
                    h_img[j][0].copy_(d_img[j][0], non_blocking=True)
                    h_img[j][1].copy_(d_img[j][1], non_blocking=True)
        except Exception as exc:  # re-raised by the caller after the join
            errors.append(exc)

    def e2e_overlapped(n_steps):
        errors = []
        threads = [threading.Thread(target=e2e_worker, args=(j, (n_steps + 1 - j) // 2, errors))
                   for j in range(2)]
        for t in threads:
            t.start()
        for t in threads:
            t.join()
        if errors:
            raise errors[0]

    e2e_overlapped(2)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    t0 = time.perf_counter()
    e2e_overlapped(e2e_steps)
    torch.cuda.synchronize()
    e2e_s = max_over_ranks(time.perf_counter() - t0, dist, f"cuda:{dev}")
    same_image = all(bool(torch.equal(h_img[j][0], h_rgba)) for j in range(2))
    scene2.close()
    clk = clocks.stop()

    if rank != 0:
        return 0
    pk = peaks()
    avg_launch_s = statistics.mean(per) / 1e3
    alg_bytes = n_samples * BYTES_PER_SAMPLE + pixels * BYTES_PER_PIXEL
    achieved = alg_bytes / avg_launch_s / 1e9
    # informational: the bytes a launch cannot avoid (the bricked field read
    # once, the image written once) over the same time
    compulsory = bricked_bytes(wl, scene.brick_cells) + pixels * BYTES_PER_PIXEL
    traffic, traffic_wl = ncu_traffic(n_samples, pixels)
    value = replica_rate(world, n_samples, args.steps, total_ms / 1e3)
    e2e_value = replica_rate(world, n_samples, e2e_steps, e2e_s)
    field_bytes = sum(d.field.nbytes for d in wl.domains)
    cpu = None
    if world == 1 and not args.no_cpu_baseline:
        cpu = cpu_sample(wl, args.cpu_seconds, float_lut=True)
    scene.close()
    others = {}
    main_acc = None
    if world == 1 and not args.no_configs:
        torch.cuda.synchronize()
        ocam, oparams = oracle_setup(wl, float_lut=True)
        main_acc = accuracy(dev, wl, [cam], params, [ocam], oparams)
        runs = {"ingest": lambda: bench_ingest(dev, wl), "plain_64": lambda: bench_plain_small(dev),
                "hex": lambda: bench_hex(dev), "batched": lambda: bench_batch(dev),
                "differentiable": lambda: bench_diff(dev), "composite": lambda: bench_composite(dev),
                "zbuffer": lambda: bench_zbuffer(dev), "noalloc": lambda: bench_noalloc(dev)}
        for name in (args.configs.split(",") if args.configs else runs):
            others[name] = runs[name]()
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "fps": 1e3 * args.steps / total_ms,
        "config": bench_config(wl, args),
        "samples_per_step": n_samples, "sample_dist": params.sample_dist,
        "parallelism": "replicas" if world > 1 else "single GPU",
        "tuning": {"best": tuning["best"], "ms": tuning["ms"]}, "generate_s": round(gen_s, 2),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": pk["hbm_gbs"], "unit": "GB/s",
                     "frac": achieved / pk["hbm_gbs"], "traffic": traffic,
                     "peak_source": pk["source"], "traffic_workload": traffic_wl,
                     "avg_launch_ms": avg_launch_s * 1e3,
                     "avg_launch_covers": "each step's render call: the march launch, plus the tile-cost "
                                          "and tile-sort launches when the tuner picked the longest-first "
                                          "order (so the march's own rate is a little higher)",
                     "algorithmic_bytes_per_launch": alg_bytes,
                     "compulsory_bytes_per_launch": compulsory,
                     "compulsory_gbs": compulsory / avg_launch_s / 1e9},
        "cpu_baseline": cpu,
        "error_vs_fp64_oracle": main_acc,
        "e2e": {"value": e2e_value, "unit": UNIT,
                "h2d_bytes_per_step": field_bytes,
                "d2h_bytes_per_step": pixels * BYTES_PER_PIXEL,
                "steps": e2e_steps, "ms_per_step": e2e_s / e2e_steps * 1e3,
                "schedule": "two scenes on two host threads take the steps in turn: one "
                            "scene's upload overlaps the other's render",
                "image_equals_serial": same_image,
                "serial_value": replica_rate(world, n_samples, e2e_steps, serial_s),
                "serial_ms_per_step": serial_s / e2e_steps * 1e3},
        "clocks": clk,
        "gpu_launches": launches,
        "configs": others,
    }
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()
    return 0


def main():
    args = parse_args()
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
