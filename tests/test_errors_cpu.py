"""Error behaviour of the C ABI that needs no GPU.

The reference ignores bad input; this library returns a status and a message
(edxr_last_error_string) instead.  Every call below is rejected by the host-side
argument checks before any CUDA call, so it runs on a machine without a GPU.
"""
import ctypes

import numpy as np
import pytest

from edxraster_gb300 import _lib

INVALID, UNSUPPORTED = 1, 6


def last_error(lib):
    return lib.edxr_last_error_string().decode()


def test_create_rejects_bad_arguments(cuda_lib):
    out = ctypes.c_void_p(1)
    assert cuda_lib.edxr_create(None, None) == INVALID
    assert last_error(cuda_lib) == "NULL argument"
    for w, h in [(0, 64), (64, 0), (32769, 64), (64, 40000)]:
        init = _lib.Init(w, h, None, 0)
        assert cuda_lib.edxr_create(ctypes.byref(out), ctypes.byref(init)) == INVALID
        assert "framebuffer size" in last_error(cuda_lib)
        assert out.value is None  # the handle is cleared on failure


def test_create_without_a_device_fails_cleanly(cuda_lib):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    out = ctypes.c_void_p(1)
    init = _lib.Init(64, 64, None, 0)
    assert cuda_lib.edxr_create(ctypes.byref(out), ctypes.byref(init)) != 0
    assert out.value is None and last_error(cuda_lib)


def test_null_renderer_is_rejected(cuda_lib):
    m = _lib.Mesh()
    st = _lib.State(0, 1, 0, 2)
    assert cuda_lib.edxr_destroy(None) == 0
    assert cuda_lib.edxr_render(None, ctypes.byref(m)) == INVALID
    assert last_error(cuda_lib) == "NULL renderer"
    assert cuda_lib.edxr_set_state(None, ctypes.byref(st)) == INVALID
    assert cuda_lib.edxr_resize(None, 64, 64) == INVALID
    assert cuda_lib.edxr_synchronize(None) == INVALID
    assert cuda_lib.edxr_set_shader(None, 0, 0, None) == INVALID
    assert cuda_lib.edxr_debug_scan_stall(None, 0, 16) == INVALID


def _noalloc_case(**change):
    """Arguments of one edxr_render_noalloc call; the buffers are host arrays
    that the rejected calls never touch."""
    keep = []

    def buf(n):
        a = np.zeros(n, np.float32)
        keep.append(a)
        return a.ctypes.data

    m = _lib.Mesh(buf(12), 12, buf(12), 12, None, 0, buf(12), 12, buf(3), 4, 1, _lib.MEMORY_DEVICE, None)
    args = dict(mesh=m, state=_lib.State(0, 1, 0, 2), ps=0, params=_lib.ShaderParams((0.0, 0.0, -1.0), 0.5, 32.0),
                width=64, height=64)
    for k, v in change.items():
        if k in ("memory", "num_vertices", "num_triangles", "position_stride", "albedo_stride", "positions"):
            setattr(m, k, v)
        elif k in ("depth_func", "msaa_log2"):
            setattr(args["state"], k, v)
        elif k == "light":
            args["params"].light[:] = v
        else:
            args[k] = v
    mat = (ctypes.c_float * 16)()
    return keep, (ctypes.byref(args["mesh"]), mat, mat, mat, ctypes.byref(args["state"]), args["ps"],
                  ctypes.byref(args["params"]), args["width"], args["height"], buf(1), buf(1), buf(1), None)


@pytest.mark.parametrize("change,status,words", [
    (dict(memory=_lib.MEMORY_HOST), INVALID, "device memory"),
    (dict(positions=None), INVALID, "positions and indices"),
    (dict(position_stride=8), INVALID, "position stride"),
    (dict(albedo_stride=4), INVALID, "attribute stride"),
    (dict(num_vertices=65537), INVALID, "65536 vertices"),
    (dict(num_triangles=65537), INVALID, "65536 triangles"),
    (dict(width=0), INVALID, "framebuffer"),
    (dict(width=4097), INVALID, "framebuffer"),
    (dict(width=2048, height=1024), INVALID, "2^20 pixels"),
    (dict(depth_func=7), INVALID, "depth function"),
    (dict(msaa_log2=2), UNSUPPORTED, "one sample per pixel"),
    (dict(ps=4), UNSUPPORTED, "texture"),
    (dict(ps=9), INVALID, "pixel shader"),
    (dict(light=(0.0, 0.0, 0.0)), INVALID, "light direction"),
    (dict(light=(float("nan"), 0.0, 1.0)), INVALID, "light direction"),
])
def test_noalloc_rejects_before_any_gpu_work(cuda_lib, change, status, words):
    keep, args = _noalloc_case(**change)
    assert cuda_lib.edxr_render_noalloc(*args) == status
    assert words in last_error(cuda_lib)


def test_noalloc_null_arguments(cuda_lib):
    keep, args = _noalloc_case()
    for i in (0, 1, 4, 6, 9):
        a = list(args)
        a[i] = None
        assert cuda_lib.edxr_render_noalloc(*a) == INVALID
        assert last_error(cuda_lib) == "NULL argument"
