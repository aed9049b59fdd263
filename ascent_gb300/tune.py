"""Autotuner for the march kernel's launch shape.

Candidates are the shapes gvr_scene_set_tuning accepts: pixel packet width
per warp (4x8, 8x4, 16x2 rays), samples located per loop iteration (1 to
4; 16-wide packets up to 3) and the CTAs per SM the register budget
targets (3 or 4), plus the shared-memory brick staging of gvr_scene_set_staging at
each packet width; the winner is then timed with each tile launch order of
gvr_scene_set_tile_order (centre first, or longest first per view); autotune_bricks also sweeps the brick size (4^3, 8^3 or
16^3 cells, gvr_scene_set_brick_cells), building one scene per size. Every
candidate
renders the caller's own view on the caller's scene; the fastest median of
a few CUDA-event-timed launches wins. Images do not depend on the shape, so
tuning never changes results. Winners are cached per (GPU, workload key) in
a JSON file so later runs skip the search.
"""
from __future__ import annotations

import ctypes as C
import itertools
import json
import os
import statistics
from pathlib import Path

from . import _native as N

CANDIDATES = ([dict(packet_w=p, unroll=u, min_blocks=m)
               for p, u, m in itertools.product((8, 4, 16), (2, 1), (3, 4))] +
              [dict(packet_w=p, unroll=3, min_blocks=4) for p in (8, 4, 16)] +
              [dict(packet_w=p, unroll=u, min_blocks=m)
               for p, u, m in itertools.product((8, 4), (3, 4), (3, 4)) if (u, m) != (3, 4)])
# shared-memory brick staging (plain path, uniform vertex scenes; elsewhere
# the scene runs the gather kernel of the same packet shape)
STAGED_CANDIDATES = ([dict(packet_w=p, unroll=1, min_blocks=3, staged=1) for p in (8, 4, 16)] +
                     [dict(packet_w=p, unroll=1, min_blocks=m, staged=2) for p in (8, 4) for m in (3, 4)])
# the batch kernel has no 3- or 4-sample variant (it would run as 2) and no staging
BATCH_CANDIDATES = [c for c in CANDIDATES if c["unroll"] <= 2]
CACHE = Path(os.environ.get("GVR_TUNE_CACHE", Path.home() / ".cache" / "gvr_tune.json"))


def _key(scene, params) -> str:
    import torch
    name = torch.cuda.get_device_name(scene.device).replace(" ", "_")
    cells = getattr(scene, "brick_cells", 8)
    return f"{name}|dom{scene.num_domains}|{params.width}x{params.height}|lut{params.lut_size}|brick{cells}"


def _time(scene, camera, params, rgba, depth, stream, reps: int) -> float:
    import torch
    sptr = C.c_void_p(stream.cuda_stream)
    args = (scene.handle, C.byref(camera), C.byref(params), C.c_void_p(rgba.data_ptr()),
            C.c_void_p(depth.data_ptr()), N.MEM_DEVICE, sptr, None)
    N.call("gvr_render_volume", *args)  # warm
    times = []
    for _ in range(reps):
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        N.call("gvr_render_volume", *args)
        b.record(stream)
        b.synchronize()
        times.append(a.elapsed_time(b))
    return statistics.median(times)


GRANULARITY = (1, 2, 4, 8)


def autotune_batch(scene, cameras, params, reps: int = 2) -> dict:
    """Pick launch shape and work-queue granularity (16x16 tiles per item) for
    the persistent batch path on these views; returns {"best", "ms"}."""
    import torch
    v = len(cameras)
    dev = f"cuda:{scene.device}"
    out = (torch.empty((v, params.height, params.width, 4), dtype=torch.float32, device=dev),
           torch.empty((v, params.height, params.width), dtype=torch.float32, device=dev))
    stream = torch.cuda.current_stream(scene.device)
    results = {}
    for cand in BATCH_CANDIDATES:
        for g in GRANULARITY:
            scene.set_tuning(**cand)
            scene.set_batch_granularity(g)
            scene.render_batch(cameras, params, device_out=True, out=out)  # capture + warm
            times = []
            for _ in range(reps):
                a = torch.cuda.Event(enable_timing=True)
                b = torch.cuda.Event(enable_timing=True)
                a.record(stream)
                scene.render_batch(cameras, params, device_out=True, out=out)
                b.record(stream)
                b.synchronize()
                times.append(a.elapsed_time(b))
            results[f"p{cand['packet_w']}u{cand['unroll']}m{cand['min_blocks']}g{g}"] = (
                statistics.median(times), cand, g)
    name, (ms, best, g) = min(results.items(), key=lambda kv: kv[1][0])
    scene.set_tuning(**best)
    scene.set_batch_granularity(g)
    return {"best": dict(best, tiles_per_item=g), "ms": {k: round(r[0], 4) for k, r in results.items()}}


def autotune(scene, camera, params, reps: int = 3, use_cache: bool = True, staged: bool = True,
             only_staged: bool = False) -> dict:
    """Pick and set the fastest launch shape for this scene and view (with
    staged=True also the shared-memory staging variant); returns {"best":
    shape, "ms": {shape-string: median ms}, "cached": bool}."""
    import torch
    key = _key(scene, params)
    cache = {}
    if use_cache and CACHE.exists():
        try:
            cache = json.loads(CACHE.read_text())
        except Exception:
            cache = {}
    key += "|staged" if only_staged else ("" if staged else "|gather")
    if use_cache and key in cache:
        best = cache[key]["best"]
        scene.set_tuning(**best)
        return {"best": best, "ms": cache[key].get("ms", {}), "cached": True}
    dev = f"cuda:{scene.device}"
    rgba = torch.empty((params.height, params.width, 4), dtype=torch.float32, device=dev)
    depth = torch.empty((params.height, params.width), dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream(scene.device)
    results = {}
    cands = STAGED_CANDIDATES if only_staged else CANDIDATES + (STAGED_CANDIDATES if staged else [])
    for cand in cands:
        scene.set_tuning(**cand)
        name = (f"p{cand['packet_w']}u{cand['unroll']}m{cand['min_blocks']}"
                + {0: "", 1: "s", 2: "L"}[cand.get("staged", 0)])
        results[name] = (_time(scene, camera, params, rgba, depth, stream, reps), cand)
    name, (ms, best) = min(results.items(), key=lambda kv: kv[1][0])
    # the winner again with each tile order, timed back to back
    for order in (0, 1):
        cand = dict(best, tile_order=order)
        scene.set_tuning(**cand)
        results[name + f"o{order}"] = (_time(scene, camera, params, rgba, depth, stream, 2 * reps), cand)
    best = min((results[name + "o0"], results[name + "o1"]), key=lambda r: r[0])[1]
    scene.set_tuning(**best)
    out = {"best": best, "ms": {k: round(v[0], 4) for k, v in results.items()}, "cached": False}
    if use_cache:
        try:
            CACHE.parent.mkdir(parents=True, exist_ok=True)
            cache[key] = {"best": best, "ms": out["ms"]}
            CACHE.write_text(json.dumps(cache, indent=1))
        except OSError:
            pass
    return out


BRICK_CELLS = (4, 8, 16)


def autotune_bricks(build_scene, camera, params, reps: int = 3, staged: bool = True) -> dict:
    """Pick the brick size as well as the launch shape: build_scene(cells)
    returns a Scene holding the workload bricked with `cells` cells per
    brick axis; each is tuned with autotune() on this view. Returns {"best":
    shape with "brick_cells", "ms": {brick size: {shape: ms}}, "scene": the
    winning Scene (the others are closed)}. Images do not depend on the
    brick size."""
    results = {}
    scenes = {}
    for cells in BRICK_CELLS:
        sc = build_scene(cells)
        out = autotune(sc, camera, params, reps=reps, use_cache=False, staged=staged and cells == 8)
        results[cells] = out
        scenes[cells] = sc
    best_cells = min(results, key=lambda c: min(results[c]["ms"].values()))
    for c, sc in scenes.items():
        if c != best_cells:
            sc.close()
    best = dict(results[best_cells]["best"], brick_cells=best_cells)
    scenes[best_cells].set_tuning(**results[best_cells]["best"])
    return {"best": best, "ms": {str(c): r["ms"] for c, r in results.items()}, "scene": scenes[best_cells]}
