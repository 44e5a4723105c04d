#!/usr/bin/env python3
"""Benchmark of the GB300 rasterization pipeline.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--workload terrain|sphere|stress]
    python bench.py --impl reference ...

A step is one frame of the workload: Renderer::RenderMesh semantics (clear,
vertex transform, clipping, setup, binning, rasterization, shading, depth
test) over one synthetic mesh.  The default workload is the heightfield
terrain (1024x1024 quads = 2,097,152 triangles at 1920x1080), the
configuration the throughput metric is quoted on.

Printed JSON (one line, rank 0):
  value       input triangles per second (Mtris/s), inputs resident in HBM,
              device time of K frames from CUDA events on the renderer's
              stream, L2 flushed (a 512 MiB write) before every frame;
  e2e         the same metric through the public API as the reference's
              viewer uses it: RenderMesh on a mesh in pinned host memory
              (uploaded by the call) and GetBackBuffer (the RGBA8 image read
              back to the host) every frame, wall clock, with a few
              renderers on their own streams keeping frames in flight;
  roofline    HBM roofline of the pixel back end (k_raster, stage
              events);
  cpu_baseline the CPU restatement of the reference pipeline (oracle port)
              on this host's cores, one full frame.
With --impl reference the CPU implementation of the reference pipeline is
timed instead (the reference's own sources compiled against the shim when
they are present here, else the oracle port).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

from edxraster_gb300 import scenes  # noqa: E402

WORKLOADS = {
    "terrain": ("heightfield 1024x1024 quads (2,097,152 tris) at 1920x1080, low camera, Blinn-Phong, depth LESS",
                lambda: scenes.terrain_scene(1024, 1920, 1080, seed=1)),
    "sphere": ("UV sphere 32x64 (4,032 tris) at 1280x720, Blinn-Phong ks 0.5 shininess 32, depth LESS",
               lambda: scenes.sphere_scene(1280, 720, seed=0)),
    "stress": ("binning stress: 1,000,000 clip-space tris, log-uniform areas 0.1-1e4 px, at 3840x2160, depth LESS",
               lambda: scenes.stress_scene(1_000_000, 3840, 2160, seed=7)),
}
PIXEL_BYTES = 24  # RGBA32F colour + D32F depth + u32 triangle id per pixel
E2E_RENDERERS = 6  # frames in flight in the end-to-end measurement
E2E_MIN_FRAMES = 64  # end-to-end frames timed at least (each renderer's thread start is in the timed region)


def mesh_bytes(mesh) -> int:
    # compulsory input: position, normal, albedo per vertex, 3 indices per triangle
    return mesh.nv * 36 + mesh.nt * 12


def algorithmic_bytes(sc) -> int:
    return mesh_bytes(sc.mesh) + sc.view.width * sc.view.height * PIXEL_BYTES


def load_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as fh:
            p = json.load(fh)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def traffic_from_profiles(workload):
    """DRAM bytes per k_raster launch from the committed ncu summary, if any."""
    path = os.path.join(ROOT, "profiles", "k_raster_%s.md" % workload)
    try:
        for line in open(path):
            if line.startswith("traffic_bytes_per_launch:"):
                return int(float(line.split(":", 1)[1].strip()))
    except OSError:
        pass
    return None


class ClockSampler:
    """nvidia-smi SM clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, ValueError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for name, flag in zip(names, parts[5:9]):
                if flag.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def max_over_ranks(x: float, world: int, device=None) -> float:
    """The largest x over all ranks: the job's time is its slowest rank's.
    Every rank renders its own replica of the workload (frames are
    independent; there is no exchange step), so this is the only collective."""
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_throughput(world: int, units_per_rank: int, steps: int, total_ms: float) -> float:
    """Whole-job throughput (millions of units per second) of `world` ranks
    that each processed units_per_rank x steps units in at most total_ms."""
    return world * units_per_rank * steps / (total_ms / 1e3) / 1e6


def workload_config(workload: str, sc, world: int) -> dict:
    """The `config` of both arms' JSON lines (the GPU arm and the reference arm)."""
    return {"workload": workload, "description": WORKLOADS[workload][0], "triangles": sc.mesh.nt,
            "width": sc.view.width, "height": sc.view.height, "l2": "512 MiB write between timed frames",
            "parallelism": "replicas" if world > 1 else "single GPU"}


def oracle_parity(mesh, view, color, depth, tid, threads=None, msaa_log2=0):
    """The GPU frame against the CPU oracle on the same inputs: winning
    triangle and depth bit for bit, colour as the largest absolute error
    against the oracle's FP64 shading over covered pixels (with several
    samples per pixel: the per-sample ids and depths)."""
    from oracle import pyoracle
    o = pyoracle.render_oracle(mesh, view, threads=threads or os.cpu_count(), with_color=msaa_log2 == 0,
                               msaa_log2=msaa_log2)
    out = {"id_exact": bool(np.array_equal(tid, o["id"])),
           "depth_exact": bool(np.array_equal(np.asarray(depth).view(np.uint32), o["depth"].view(np.uint32)))}
    if msaa_log2 == 0:
        cov = o["id"] != 0xFFFFFFFF
        out["color_err_max"] = float(np.abs(color[cov, :3] - o["color"][cov, :3]).max()) if cov.any() else 0.0
    out["covered_pixels"] = int((o["id"] != 0xFFFFFFFF).sum())
    return out


def cpu_oracle_time(sc, threads: int):
    from oracle import pyoracle
    t0 = time.perf_counter()
    pyoracle.render_oracle(sc.mesh, sc.view, threads=threads, with_color=True)
    return time.perf_counter() - t0


def cpu_baseline(sc, frames: int = 5):
    """The oracle port on this host: median of `frames` full frames after one warm-up frame."""
    threads = os.cpu_count() or 1
    cpu_oracle_time(sc, threads)
    times = [cpu_oracle_time(sc, threads) for _ in range(max(1, frames))]
    t = statistics.median(times)
    return {"value": sc.mesh.nt / t / 1e6, "unit": "Mtris/s", "cores": threads, "kind": "port",
            "sample": "full frames of the workload (%d tris, %dx%d), median of %d after one warm-up frame"
                      % (sc.mesh.nt, sc.view.width, sc.view.height, len(times))}


def run_reference(args, world, rank):
    if rank != 0:
        return 0
    name, make = WORKLOADS[args.workload]
    sc = make()
    kind = "port"
    t_frames = []
    cores = os.cpu_count() or 1
    from oracle import pyoracle
    use_ref = pyoracle.reference_lib() is not None
    if use_ref:
        kind = "reference"
        t, cores = pyoracle.time_reference(sc.mesh, sc.view, frames=args.steps, warmup=args.warmup)
        t_frames = [t]
    else:
        for i in range(args.warmup + args.steps):
            dt = cpu_oracle_time(sc, cores)
            if i >= args.warmup:
                t_frames.append(dt)
    t = statistics.median(t_frames)
    value = sc.mesh.nt / t / 1e6
    sample = ("Renderer::RenderMesh of the reference (its Core sources built against oracle/shim), "
              "median of %d frames" % args.steps) if use_ref else \
        ("CPU restatement of the reference pipeline (oracle/edxr_oracle.c), median of %d full frames" % args.steps)
    line = {
        "impl": "reference", "metric": "Mtris/s", "value": value, "unit": "Mtris/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": t * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "int32+f32", "data": "synthetic",
        "config": workload_config(args.workload, sc, world),
        "gpix_per_s": sc.view.width * sc.view.height / t / 1e9, "fps": 1.0 / t,
        "cpu_baseline": {"value": value, "unit": "Mtris/s", "cores": cores, "kind": kind, "sample": sample},
        "e2e": {"value": value, "unit": "Mtris/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


class DeviceArray:
    """A torch-visible view of a renderer-owned device buffer."""

    def __init__(self, ptr, shape, typestr="<f4"):
        self.__cuda_array_interface__ = {"shape": tuple(shape), "typestr": typestr, "data": (int(ptr), False),
                                         "version": 3, "strides": None}


def time_frames(r, stream, flush_l2, render, steps, warmup):
    """Summed CUDA-event time (ms) of `steps` calls of render(), L2 flushed before each."""
    import torch
    for _ in range(warmup):
        flush_l2()
        render()
    r.Synchronize()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    for i in range(steps):
        flush_l2()
        starts[i].record(stream)
        render()
        ends[i].record(stream)
    r.Synchronize()
    torch.cuda.synchronize()
    return sum(s.elapsed_time(e) for s, e in zip(starts, ends))


def apply_tuning(r, workload):
    """Launch tunables the autotuner stored for this workload on this GPU, if any."""
    from edxraster_gb300 import autotune
    t = autotune.load(workload)
    if t:
        r.SetTuning(t)
    return t


def measure_plain(sc, device, steps, warmup, flush_l2, workload=None, msaa_log2=0):
    import torch
    from edxraster_gb300 import renderer as R
    stream = torch.cuda.Stream()
    r = R.Renderer(device=device, stream=stream)
    r.Initialize(sc.view.width, sc.view.height)
    R.configure(r, sc.view)
    if workload:
        apply_tuning(r, workload)
    if msaa_log2:
        r.SetMSAAMode(msaa_log2)
    dm = R.DeviceMesh.from_mesh(sc.mesh, device="cuda:%d" % device)
    ms = time_frames(r, stream, lambda: flush_l2(stream), lambda: r.RenderMesh(dm, synchronize=False),
                     steps, warmup) / steps
    st = r.Stats()
    color, depth, tid = r.ReadOutputs()
    r.close()
    W, H = sc.view.width, sc.view.height
    return {"triangles": sc.mesh.nt, "width": W, "height": H, "ms_per_frame": ms,
            "mtris_per_s": sc.mesh.nt / ms / 1e3, "gpix_per_s": W * H / ms / 1e6, "fps": 1e3 / ms,
            "hbm_frac": algorithmic_bytes(sc) / (ms / 1e3) / 1e9 / load_peaks()[0],
            "raster_triangles": int(st.raster_triangles), "bin_entries": int(st.bin_entries),
            "parity": oracle_parity(sc.mesh, sc.view, color, depth, tid, msaa_log2=msaa_log2)}


def measure_batched(device, steps, warmup, flush_l2, oracle_views=16):
    """256 meshes x 4 orbit views at 512x512: one batched pass against one
    plain pass per view, and `oracle_views` batched views (spread from the
    smallest mesh to the largest) against the CPU oracle."""
    import ctypes
    import torch
    from edxraster_gb300 import _lib
    from edxraster_gb300 import renderer as R
    meshes = scenes.batched_meshes(256, 500, 200_000, seed=11)
    views = []
    for m in range(len(meshes)):
        for v in scenes.orbit_views(4, 512, 512, seed=1000 + m):
            v.mesh = m
            views.append(v)
    dms = [R.DeviceMesh.from_mesh(m, device="cuda:%d" % device) for m in meshes]
    stream = torch.cuda.Stream()
    r = R.Renderer(device=device, stream=stream)
    r.Initialize(512, 512)
    apply_tuning(r, "batched")
    batch = r.PrepareBatch(dms, views)
    ms_b = time_frames(r, stream, lambda: flush_l2(stream),
                       lambda: r.RenderBatched(batch, None, 512, 512, synchronize=False), steps, warmup) / steps
    by_size = sorted(range(len(views)), key=lambda i: (meshes[views[i].mesh].nt, i))
    sample = sorted({by_size[round(k * (len(by_size) - 1) / (oracle_views - 1))] for k in range(oracle_views)})
    cb, db, tb = [], [], []
    for i in sample:
        c, d, t = r.ReadBatchOutputs(i, 1, 512, 512)
        cb.append(c[0])
        db.append(d[0])
        tb.append(t[0])
    r.close()
    checks = [oracle_parity(meshes[views[i].mesh], views[i], cb[j], db[j], tb[j]) for j, i in enumerate(sample)]
    parity = {"views": len(sample), "triangles": [meshes[views[i].mesh].nt for i in sample],
              "id_exact": all(c["id_exact"] for c in checks), "depth_exact": all(c["depth_exact"] for c in checks),
              "color_err_max": max(c["color_err_max"] for c in checks)}

    # One plain pass per view, in submission order.  The per-view arguments
    # are built once (as PrepareBatch does for the batched pass), and each
    # view is three calls of the C ABI: edxr_set_transform, edxr_set_shader,
    # edxr_render.
    p = R.Renderer(device=device, stream=stream)
    p.Initialize(512, 512)
    apply_tuning(p, "batched")
    lib, h = p._lib, p._h
    args = []
    for v in views:
        mv, pr, ra = R._f16(v.mv), R._f16(v.proj), R._f16(v.raster)
        sp = _lib.ShaderParams((ctypes.c_float * 3)(*[float(x) for x in v.light]), v.ks, v.shininess)
        args.append((mv, pr, ra, ctypes.addressof(mv), ctypes.addressof(pr), ctypes.addressof(ra), v.shader,
                     ctypes.byref(sp), sp, ctypes.byref(batch[1][v.mesh])))
    assert len({v.depth_func for v in views}) == 1
    p.SetDepthFunc(views[0].depth_func)

    def per_view(on_view=None):
        for a in args:
            _lib.check(lib.edxr_set_transform(h, a[3], a[4], a[5]))
            _lib.check(lib.edxr_set_shader(h, 0, a[6], a[7]))
            _lib.check(lib.edxr_render(h, a[9]))
            if on_view:
                on_view()

    per_view()
    p.Synchronize()
    torch.cuda.synchronize()
    # (1) stream time: CUDA events around the whole loop on the renderer's
    # stream (device time, including any gaps while the host issues views)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t0 = time.perf_counter()
    e0.record(stream)
    per_view()
    e1.record(stream)
    p.Synchronize()
    torch.cuda.synchronize()
    ms_wall = (time.perf_counter() - t0) * 1e3
    ms_stream = e0.elapsed_time(e1)
    # (2) device time of each plain pass, from before its first kernel to
    # after its last (stage events), summed over the views.  A plain pass
    # waits for the previous frame's status word (its overflow check) before
    # it is issued, so the passes of different views cannot overlap.
    p.SetProfiling(True)
    acc = [0.0]
    per_view(lambda: acc.__setitem__(0, acc[0] + sum(p.StageTimes().values())))
    p.SetProfiling(False)
    ms_kernels = acc[0]
    exact = True
    for j, i in enumerate(sample[:4]):
        R.configure(p, views[i])
        p.RenderMesh(dms[views[i].mesh])
        c, d, t = p.ReadOutputs()
        exact = exact and np.array_equal(t, tb[j]) and np.array_equal(d.view(np.uint32), db[j].view(np.uint32)) \
            and np.array_equal(c, cb[j])
    p.close()
    tris = sum(meshes[v.mesh].nt for v in views)
    return {"views": len(views), "meshes": len(meshes), "triangles_per_pass": tris,
            "batched_ms": ms_b, "views_per_s": len(views) / ms_b * 1e3,
            "plain_kernel_ms": ms_kernels, "plain_stream_ms": ms_stream, "plain_wall_ms": ms_wall,
            "plain_views_per_s": len(views) / ms_kernels * 1e3,
            "speedup_vs_plain": ms_kernels / ms_b,
            "speedup_vs_plain_stream": ms_stream / ms_b, "speedup_vs_plain_wall": ms_wall / ms_b,
            "speedup_basis": "device time against device time: the batched pass's CUDA-event time against the "
                             "sum over views of each plain pass's CUDA-event time from its first kernel to its "
                             "last (stage events)",
            "bit_exact_vs_plain_views": exact, "parity": parity}


def measure_diff(device, steps, warmup):
    """Torus of 50,000 triangles, 64 views at 256x256: forward vs forward + adjoint."""
    import ctypes
    import torch
    from edxraster_gb300 import _lib
    from edxraster_gb300 import renderer as R
    mesh = scenes.diff_torus(seed=13)
    views = scenes.orbit_views(64, 256, 256, seed=31)
    rng = np.random.default_rng(17)
    tgt = scenes.Mesh(mesh.positions * (1 + 0.05 * rng.uniform(-1, 1, size=mesh.positions.shape)).astype(np.float32),
                      mesh.normals * (1 + 0.05 * rng.uniform(-1, 1, size=mesh.normals.shape)).astype(np.float32),
                      np.clip(mesh.albedo * (1 + 0.05 * rng.uniform(-1, 1, size=mesh.albedo.shape)), 0, 1)
                      .astype(np.float32), mesh.uvs, mesh.indices)
    tviews = []
    for v in views:
        tv = scenes.View(**{k: getattr(v, k) for k in v.__dataclass_fields__})
        tv.light = (v.light * (1 + 0.05 * rng.uniform(-1, 1, 3))).astype(np.float32)
        tv.ks, tv.shininess = v.ks * 1.05, v.shininess * 1.05
        tviews.append(tv)
    stream = torch.cuda.Stream()
    r = R.Renderer(device=device, stream=stream)
    r.Initialize(256, 256)
    dev = "cuda:%d" % device
    r.RenderBatched([R.DeviceMesh.from_mesh(tgt, device=dev)], tviews, 256, 256)
    o = r.BatchOutputs()
    n = len(views)
    target = torch.as_tensor(DeviceArray(o.color, (n, 256, 256, 4)), device=dev).clone()
    dm = R.DeviceMesh.from_mesh(mesh, device=dev)
    g_pos = torch.zeros_like(dm.positions)
    g_nrm = torch.zeros_like(dm.normals)
    g_alb = torch.zeros_like(dm.albedo)
    g_glob = torch.zeros(5, device=dev)
    grads = _lib.Grads(g_alb.data_ptr(), g_nrm.data_ptr(), g_pos.data_ptr(), g_glob.data_ptr(),
                       g_glob.data_ptr() + 12, g_glob.data_ptr() + 16)
    abi = dm.abi()
    loss = torch.zeros((), device=dev)
    batch = r.PrepareBatch([dm], views)  # the views' ABI records, built once

    def forward():
        r.RenderBatched(batch, None, 256, 256, synchronize=False)
        out = r.BatchOutputs()
        c = torch.as_tensor(DeviceArray(out.color, (n, 256, 256, 4)), device=dev)
        with torch.cuda.stream(stream):
            loss.copy_(((c - target) ** 2).sum())
        return c

    def forward_backward():
        c = forward()
        with torch.cuda.stream(stream):
            grad = 2.0 * (c - target)
            for t in (g_pos, g_nrm, g_alb, g_glob):
                t.zero_()
        _lib.check(r._lib.edxr_backward(r._h, ctypes.byref(abi), None, grad.data_ptr(), ctypes.byref(grads)))

    def timed(fn):
        for _ in range(warmup):
            fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / steps

    ms_f = timed(forward)
    ms_fb = timed(forward_backward)
    r.RenderBatched(batch, None, 256, 256)
    checks = []
    for i in (0, n // 2, n - 1):
        c, d, t = r.ReadBatchOutputs(i, 1, 256, 256)
        checks.append(oracle_parity(mesh, views[i], c[0], d[0], t[0]))
    r.close()
    parity = {"views": len(checks), "id_exact": all(c["id_exact"] for c in checks),
              "depth_exact": all(c["depth_exact"] for c in checks),
              "color_err_max": max(c["color_err_max"] for c in checks)}
    return {"triangles": mesh.nt, "views": n, "width": 256, "height": 256, "fwd_ms": ms_f,
            "fwd_iters_per_s": 1e3 / ms_f, "fwd_bwd_ms": ms_fb, "fwd_bwd_iters_per_s": 1e3 / ms_fb,
            "fwd_bwd_over_fwd": ms_fb / ms_f, "parity": parity}


def measure_e2e(sc, device, steps, warmup, workload, world=1, renderers=E2E_RENDERERS):
    """End to end through the public interface, as the reference's viewer
    drives it: every frame is RenderMesh on a mesh in pinned host memory
    (positions and indices uploaded by the call, normals and albedo read in
    place by the shading) followed by GetBackBuffer (the RGBA8 image read
    back to the host).  `renderers` renderers, each with its own stream and
    host thread, keep frames in flight so uploads, kernels and read-backs of
    different frames overlap; every frame still reads all of its own input."""
    import threading
    import torch
    from edxraster_gb300 import renderer as R

    W, H = sc.view.width, sc.view.height
    hmesh = R.HostMesh(sc.mesh, pinned=True)
    rs = []
    for _ in range(renderers):
        r = R.Renderer(device=device, stream=torch.cuda.Stream(device=device))
        r.Initialize(W, H)
        R.configure(r, sc.view)
        apply_tuning(r, workload)
        rs.append(r)

    def frames(r, n):
        for _ in range(n):
            r.RenderMesh(hmesh, synchronize=False)
            r.GetBackBuffer(copy=False)

    def run(total):
        share = [total // renderers + (1 if k < total % renderers else 0) for k in range(renderers)]
        ts = [threading.Thread(target=frames, args=(r, n)) for r, n in zip(rs, share)]
        for t in ts:
            t.start()
        for t in ts:
            t.join()

    run(max(warmup, renderers))
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    t0 = time.perf_counter()
    run(steps)
    torch.cuda.synchronize()
    elapsed = max_over_ranks(time.perf_counter() - t0, world, "cuda:%d" % device)
    for r in rs:
        r.close()
    return {"value": job_throughput(world, sc.mesh.nt, steps, elapsed * 1e3), "unit": "Mtris/s",
            "h2d_bytes_per_step": hmesh.nbytes(), "d2h_bytes_per_step": W * H * 4,
            "h2d_copied_bytes_per_step": hmesh.copied_nbytes(),
            "h2d_read_in_place": "normals and albedo (pinned) are read by the shading over NVLink-C2C: "
                                 "only the winning triangles' vertex lines cross the link",
            "ms_per_step": elapsed * 1e3 / steps, "frames": steps, "renderers_in_flight": renderers,
            "step": "RenderMesh(pinned host mesh) + GetBackBuffer (RGBA8 to host)"}


def run_gpu(args, world, rank, local):
    import torch
    from edxraster_gb300 import renderer as R

    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    name, make = WORKLOADS[args.workload]
    sc = make()
    W, H = sc.view.width, sc.view.height
    stream = torch.cuda.Stream()
    r = R.Renderer(device=local, stream=stream)
    r.Initialize(W, H)
    R.configure(r, sc.view)
    tuning = apply_tuning(r, args.workload)
    dmesh = R.DeviceMesh.from_mesh(sc.mesh, device="cuda:%d" % local)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda:%d" % local)

    def flush_l2():
        with torch.cuda.stream(stream):
            flush.zero_()

    # ---- device-resident throughput ------------------------------------
    for _ in range(args.warmup):
        flush_l2()
        r.RenderMesh(dmesh, synchronize=False)
    r.Synchronize()
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    clocks = ClockSampler(local)
    clocks.start()
    for i in range(args.steps):
        flush_l2()
        starts[i].record(stream)
        r.RenderMesh(dmesh, synchronize=False)
        ends[i].record(stream)
    r.Synchronize()
    torch.cuda.synchronize()
    clock_info = clocks.stop()
    per = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    total_ms = max_over_ranks(sum(per), world, "cuda:%d" % local)
    stats = r.Stats()
    r_tuning = r.GetTuning()
    ms_per_step = total_ms / args.steps
    value = job_throughput(world, sc.mesh.nt, args.steps, total_ms)

    # ---- stage times (dominant kernel) ---------------------------------
    r.SetProfiling(True)
    stage_sum = {}
    for i in range(args.warmup + args.steps):
        flush_l2()
        r.RenderMesh(dmesh, synchronize=True)
        if i >= args.warmup:
            for k, v in r.StageTimes().items():
                stage_sum[k] = stage_sum.get(k, 0.0) + v
    r.SetProfiling(False)
    stage_ms = {k: v / args.steps for k, v in stage_sum.items()}
    # the pixel back end, k_raster: coverage, depth test, winner, its shading
    # and the one write of colour, depth and id
    raster_ms = stage_ms.get("raster+shade", float("nan"))
    peak, peak_kind = load_peaks()
    raster_bytes = W * H * PIXEL_BYTES
    achieved = raster_bytes / (raster_ms / 1e3) / 1e9
    frame_achieved = algorithmic_bytes(sc) / (ms_per_step / 1e3) / 1e9

    frame_out = r.ReadOutputs()
    r.close()
    e2e = measure_e2e(sc, local, max(args.steps, E2E_MIN_FRAMES), args.warmup, args.workload, world)

    # ---- the other configurations (same GPU, shorter runs) ----------------
    per_config = {}
    if not args.no_configs and rank == 0:
        def flush_on(s):
            with torch.cuda.stream(s):
                flush.zero_()
        for wname in ("sphere", "stress"):
            if wname != args.workload:
                per_config[wname] = measure_plain(WORKLOADS[wname][1](), local, max(3, args.steps // 4), 3, flush_on,
                                                  workload=wname)
        # Renderer::SetMSAAMode: 4 and 8 samples per pixel
        for wname, lg in (("sphere", 2), ("terrain", 2), ("terrain", 3)):
            per_config["%s_msaa%d" % (wname, 1 << lg)] = measure_plain(
                WORKLOADS[wname][1](), local, max(3, args.steps // 4), 3, flush_on, workload=wname, msaa_log2=lg)
        per_config["batched"] = measure_batched(local, 3, 3, flush_on)
        per_config["differentiable"] = measure_diff(local, 5, 3)

    if rank != 0:
        return 0
    cpu = None
    if not args.no_cpu_baseline:
        cpu = cpu_baseline(sc)
    traffic = traffic_from_profiles(args.workload)
    parity = oracle_parity(sc.mesh, sc.view, *frame_out)
    line = {
        "metric": "Mtris/s", "value": value, "unit": "Mtris/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step, "ms_per_step_median": statistics.median(per),
        "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "int32+f32", "data": "synthetic (seeded scene generators)",
        "config": workload_config(args.workload, sc, world),
        "gpix_per_s": world * W * H / (ms_per_step / 1e3) / 1e9,
        "fps": world * 1e3 / ms_per_step,
        "stage_ms": stage_ms,
        "frame_roofline": {"algorithmic_bytes": algorithmic_bytes(sc), "achieved_gbs": frame_achieved,
                           "frac": frame_achieved / peak},
        "roofline": {"kernel": "k_raster", "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_kind": peak_kind, "traffic": traffic,
                     "algorithmic_bytes_per_launch": raster_bytes, "launch_ms": raster_ms},
        "e2e": e2e,
        "gpu_launches": int(stats.kernels_per_pass) * args.steps,
        "tuning": r_tuning,
        "clocks": clock_info,
        "raster_triangles": int(stats.raster_triangles), "bin_entries": int(stats.bin_entries),
        "cpu_baseline": cpu,
        "parity": parity,
        "color_err_max": parity["color_err_max"],
        "per_config": per_config,
    }
    print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


def profile_frames(args):
    """Frames of the workload for a profiler (ncu): device-resident mesh, one
    synchronised RenderMesh per frame, no timing and no JSON line."""
    import torch
    from edxraster_gb300 import renderer as R
    sc = WORKLOADS[args.workload][1]()
    r = R.Renderer(device=0)
    r.Initialize(sc.view.width, sc.view.height)
    R.configure(r, sc.view)
    apply_tuning(r, args.workload)
    if args.msaa:
        r.SetMSAAMode(args.msaa)
    dm = R.DeviceMesh.from_mesh(sc.mesh, device="cuda:0")
    for _ in range(args.profile_frames):
        r.RenderMesh(dm)
    torch.cuda.synchronize()
    r.close()
    print("rendered %d frames of %s (%d samples per pixel)" % (args.profile_frames, args.workload, 1 << args.msaa))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="terrain", choices=sorted(WORKLOADS))
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-configs", action="store_true", help="skip the per-configuration measurements")
    ap.add_argument("--profile-frames", type=int, default=0,
                    help="render this many frames of the workload and exit (a target for a profiler; no timing)")
    ap.add_argument("--msaa", type=int, default=0, choices=range(0, 6),
                    help="with --profile-frames: 2^MSAA samples per pixel")
    args = ap.parse_args()
    if args.profile_frames:
        return profile_frames(args)
    if args.warmup < 3:
        args.warmup = 3
    world, rank, local = dist_setup()
    if args.impl == "reference":
        return run_reference(args, world, rank)
    return run_gpu(args, world, rank, local)


if __name__ == "__main__":
    sys.exit(main())
