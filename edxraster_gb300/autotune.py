"""Autotuner of the launch tunables (edxr_set_tuning).

For one workload — a callable that renders a frame or a batched pass on a
renderer — it times every candidate of a small grid with CUDA events on the
renderer's stream (L2 flushed before each timed call), keeps the fastest, and
sizes the bin buffer from the entries the workload needs, so steady-state
frames never re-render after an overflow.  Results are stored as JSON keyed
by workload and GPU name (``tuning.json`` beside this file) and read back by
``load``.  Tunables change speed only: every candidate renders identical
images.
"""
from __future__ import annotations

import itertools
import json
import math
import os

DEFAULT_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "tuning.json")

GRID = {
    "small_region": [0, 4, 16, 64],
    "raster_variant": [0, 1, 2],
    "bin_blocks_per_sm": [4, 8, 16],
    "item_entries": [128, 224],
}


def _gpu_name():
    import torch
    return torch.cuda.get_device_name()


def time_calls(r, stream, render, steps, warmup, flush=None):
    import torch
    for _ in range(warmup):
        if flush:
            flush()
        render()
    r.Synchronize()
    total = 0.0
    for _ in range(steps):
        if flush:
            flush()
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record(stream)
        render()
        e.record(stream)
        r.Synchronize()
        e.synchronize()
        total += s.elapsed_time(e)
    return total / steps


def tune(r, stream, render, triangles: int, steps: int = 5, warmup: int = 2, flush=None, grid=None, finalists=6,
         rounds=3):
    """Return (best tuning dict, [(candidate, ms), ...]).  Every candidate of
    the grid is timed once; the `finalists` fastest are timed again `rounds`
    times, interleaved, and the one with the lowest median wins (a single
    timing of a sub-millisecond frame is too noisy to rank close candidates)."""
    import statistics
    grid = grid or GRID
    keys = list(grid)
    table = []
    for values in itertools.product(*[grid[k] for k in keys]):
        cand = dict(zip(keys, values))
        r.SetTuning(cand)
        table.append((cand, time_calls(r, stream, render, steps, warmup, flush)))
    final = [c for c, _ in sorted(table, key=lambda x: x[1])[:finalists]]
    times = [[] for _ in final]
    for _ in range(rounds):
        for i, cand in enumerate(final):
            r.SetTuning(cand)
            times[i].append(time_calls(r, stream, render, 2 * steps, warmup, flush))
    medians = [statistics.median(t) for t in times]
    best = dict(final[min(range(len(final)), key=lambda i: medians[i])])
    table = [(c, medians[final.index(c)] if c in final else ms) for c, ms in table]
    r.SetTuning(best)
    render()
    r.Synchronize()
    entries = int(r.Stats().bin_entries)
    best["bin_entries_per_triangle"] = max(1, int(math.ceil(1.15 * entries / max(triangles, 1))))
    best["raster_blocks_per_sm"] = 0
    return best, table


def save(workload: str, best: dict, table, path: str = DEFAULT_PATH):
    data = {}
    if os.path.exists(path):
        with open(path) as fh:
            data = json.load(fh)
    data.setdefault(_gpu_name(), {})[workload] = {
        "tuning": best, "candidates": [{"tuning": c, "ms": round(ms, 5)} for c, ms in table]}
    with open(path, "w") as fh:
        json.dump(data, fh, indent=1, sort_keys=True)


def plain_workload(sc, device=0):
    """(renderer, stream, render callable, triangles) for one plain frame."""
    import torch
    from . import renderer as R
    stream = torch.cuda.Stream()
    r = R.Renderer(device=device, stream=stream)
    r.Initialize(sc.view.width, sc.view.height)
    R.configure(r, sc.view)
    dm = R.DeviceMesh.from_mesh(sc.mesh, device="cuda:%d" % device)
    return r, stream, (lambda: r.RenderMesh(dm, synchronize=False)), sc.mesh.nt, dm


def batched_workload(meshes, views, width, height, device=0):
    import torch
    from . import renderer as R
    stream = torch.cuda.Stream()
    r = R.Renderer(device=device, stream=stream)
    r.Initialize(width, height)
    dms = [R.DeviceMesh.from_mesh(m, device="cuda:%d" % device) for m in meshes]
    batch = r.PrepareBatch(dms, views)
    tris = sum(meshes[v.mesh].nt for v in views)
    return r, stream, (lambda: r.RenderBatched(batch, None, width, height, synchronize=False)), tris, dms


def main(path: str = DEFAULT_PATH):
    import torch
    from . import scenes
    flush_buf = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    work = {
        "terrain": lambda: plain_workload(scenes.terrain_scene(1024, 1920, 1080, seed=1)),
        "stress": lambda: plain_workload(scenes.stress_scene(1_000_000, 3840, 2160, seed=7)),
        "sphere": lambda: plain_workload(scenes.sphere_scene(1280, 720, seed=0)),
    }

    def batched():
        meshes = scenes.batched_meshes(256, 500, 200_000, seed=11)
        views = []
        for m in range(len(meshes)):
            for v in scenes.orbit_views(4, 512, 512, seed=1000 + m):
                v.mesh = m
                views.append(v)
        return batched_workload(meshes, views, 512, 512)

    work["batched"] = batched
    for name, make in work.items():
        r, stream, render, tris, keep = make()

        def flush():
            with torch.cuda.stream(stream):
                flush_buf.zero_()

        best, table = tune(r, stream, render, tris, flush=flush)
        save(name, best, table, path)
        print(name, best, "%.4f ms" % min(ms for _, ms in table))
        r.close()


def load(workload: str, path: str = DEFAULT_PATH):
    """The stored tuning for this workload on this GPU, or None."""
    try:
        with open(path) as fh:
            data = json.load(fh)
        return data[_gpu_name()][workload]["tuning"]
    except (OSError, KeyError, ValueError):
        return None


if __name__ == "__main__":
    import sys
    main(sys.argv[1] if len(sys.argv) > 1 else DEFAULT_PATH)
