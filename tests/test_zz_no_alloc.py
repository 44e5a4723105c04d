"""edxr_render_noalloc: the entry point for callers that cannot allocate
device memory (a host that owns the whole device-memory budget, or a render
loop that must not call cudaMalloc / cudaFree and their device-wide
synchronisation).  Its intermediates live in a fixed device array inside the
library; the test provides only the inputs and outputs.

Two frames in a row through the C ABI, each compared with edxr_render of the
same scene: triangle id and depth bit-identical, colour within COLOR_TOL.  The
second frame reuses the array the first one left behind.  Kept in its own
file, collected last.
"""
import ctypes

import numpy as np
import pytest

from edxraster_gb300 import _lib
from edxraster_gb300 import renderer as R
from edxraster_gb300 import scenes

pytestmark = pytest.mark.gpu
COLOR_TOL = 1e-5


def _f16(m):
    return (ctypes.c_float * 16)(*np.ascontiguousarray(np.asarray(m, np.float32).reshape(16)))


def render_regular(sc):
    r = R.Renderer()
    r.Initialize(sc.view.width, sc.view.height)
    R.configure(r, sc.view)
    r.RenderMesh(sc.mesh)
    out = r.ReadOutputs()
    r.close()
    return out


def call_noalloc(lib, sc, stream):
    """One edxr_render_noalloc call; returns its status and the three images."""
    import torch
    v = sc.view
    dm = R.DeviceMesh.from_mesh(sc.mesh)
    W, H = v.width, v.height
    color = torch.empty((H, W, 4), dtype=torch.float32, device="cuda")
    depth = torch.empty((H, W), dtype=torch.float32, device="cuda")
    tid = torch.empty((H, W), dtype=torch.int32, device="cuda")
    state = _lib.State(v.depth_func, 1, 0, 0)
    params = _lib.ShaderParams((ctypes.c_float * 3)(*[float(x) for x in v.light]), v.ks, v.shininess)
    mesh = dm.abi()
    mv, proj, raster = _f16(v.mv), _f16(v.proj), _f16(v.raster)
    rc = lib.edxr_render_noalloc(ctypes.byref(mesh), ctypes.addressof(mv), ctypes.addressof(proj),
                                 ctypes.addressof(raster), ctypes.byref(state), v.shader, ctypes.byref(params),
                                 W, H, color.data_ptr(), depth.data_ptr(), tid.data_ptr(), stream.cuda_stream)
    torch.cuda.synchronize()
    return rc, (color.cpu().numpy(), depth.cpu().numpy(), tid.cpu().numpy().view(np.uint32))


def render_noalloc(lib, sc, stream):
    rc, out = call_noalloc(lib, sc, stream)
    _lib.check(rc)
    return out


def left_edge_scene(n=12000, width=256, height=256, seed=5):
    """n triangles that each straddle the left clip plane (x = -w): every one
    is queued for clipping, more than the 8192 clipped polygons the fixed
    array holds."""
    rng = np.random.default_rng(seed)
    y = rng.uniform(-0.8, 0.8, size=n)
    w = rng.uniform(1.0, 2.0, size=n)
    ndc = np.stack([np.stack([np.full(n, -1.4), y], -1), np.stack([np.full(n, -0.9), y + 0.05], -1),
                    np.stack([np.full(n, -0.9), y - 0.05], -1)], 1)  # (n, 3, 2)
    pos = np.concatenate([ndc * w[:, None, None], np.repeat(w[:, None, None], 3, 1)], -1).reshape(-1, 3)
    nrm = np.tile(np.array([0.0, 0.0, -1.0], np.float32), (3 * n, 1))
    mesh = scenes.Mesh(pos.astype(np.float32), nrm, np.full((3 * n, 3), 0.5, np.float32),
                       np.zeros((3 * n, 2), np.float32), np.arange(3 * n, dtype=np.uint32).reshape(n, 3))
    proj = np.array([[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, scenes.STRESS_A, scenes.STRESS_B], [0, 0, 1, 0]],
                    np.float32)
    view = scenes.View(width, height, np.eye(4, dtype=np.float32), proj, scenes.raster_matrix(width, height),
                       np.array([0.3, 0.5, -1.0], np.float32))
    return scenes.Scene("left_edge", mesh, view)


def test_noalloc_matches_render_twice(cuda_lib):
    import torch
    stream = torch.cuda.Stream()
    cases = [scenes.stress_scene(20000, 640, 360, seed=7, max_area=3e3),
             scenes.terrain_scene(96, 512, 288, seed=3)]
    for sc in cases:
        c0, d0, t0 = render_regular(sc)
        c1, d1, t1 = render_noalloc(cuda_lib, sc, stream)
        assert np.array_equal(t1, t0)
        assert np.array_equal(d1.view(np.uint32), d0.view(np.uint32))
        cov = t0 != 0xFFFFFFFF
        assert cov.any()
        assert float(np.abs(c1 - c0).max()) <= COLOR_TOL


def test_noalloc_rejects_sizes_over_its_limits(cuda_lib):
    import torch
    sc = scenes.stress_scene(70000, 64, 64, seed=1)  # 70,000 triangles > 65,536
    v = sc.view
    dm = R.DeviceMesh.from_mesh(sc.mesh)
    out = torch.empty((64, 64, 4), dtype=torch.float32, device="cuda")
    state = _lib.State(0, 1, 0, 0)
    params = _lib.ShaderParams((ctypes.c_float * 3)(1.0, 1.0, -1.0), 0.5, 32.0)
    mesh = dm.abi()
    mv, proj, raster = _f16(v.mv), _f16(v.proj), _f16(v.raster)
    rc = cuda_lib.edxr_render_noalloc(ctypes.byref(mesh), ctypes.addressof(mv), ctypes.addressof(proj),
                                      ctypes.addressof(raster), ctypes.byref(state), 0, ctypes.byref(params),
                                      64, 64, out.data_ptr(), out.data_ptr(), out.data_ptr(), None)
    assert rc == 1  # EDXR_ERR_INVALID_ARG
    assert b"limit" in cuda_lib.edxr_last_error_string()


def test_noalloc_overflow_then_next_frame_exact(cuda_lib):
    """A frame that does not fit the fixed array fails with EDXR_ERR_OVERFLOW
    (it cannot grow and render again, as edxr_render does); the next call on
    the same array, which the failed frame left behind, renders exactly."""
    import torch
    stream = torch.cuda.Stream()
    rc, _ = call_noalloc(cuda_lib, left_edge_scene(), stream)
    assert rc == 2  # EDXR_ERR_OVERFLOW
    assert b"scratch" in cuda_lib.edxr_last_error_string()
    sc = scenes.stress_scene(20000, 640, 360, seed=9, max_area=3e3)
    c0, d0, t0 = render_regular(sc)
    c1, d1, t1 = render_noalloc(cuda_lib, sc, stream)
    assert np.array_equal(t1, t0)
    assert np.array_equal(d1.view(np.uint32), d0.view(np.uint32))
    assert (t0 != 0xFFFFFFFF).any()
    assert float(np.abs(c1 - c0).max()) <= COLOR_TOL
