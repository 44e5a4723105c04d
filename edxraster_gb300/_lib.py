"""ctypes binding of the C ABI in include/edxr.h (libedxr.so).

The library is the CUDA build in ``edxraster_gb300/_build``.  There is no
fallback: if it has not been built, loading raises.
"""
from __future__ import annotations

import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libedxr.so")

EDXR_OK = 0
STATUS_NAMES = {0: "EDXR_OK", 1: "EDXR_ERR_INVALID_ARG", 2: "EDXR_ERR_OVERFLOW", 3: "EDXR_ERR_TIMEOUT",
                4: "EDXR_ERR_CUDA", 5: "EDXR_ERR_OUT_OF_MEMORY", 6: "EDXR_ERR_UNSUPPORTED"}
MEMORY_HOST, MEMORY_DEVICE = 0, 1

_f16 = ctypes.c_float * 16


class EdxrError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__("%s: %s" % (STATUS_NAMES.get(status, str(status)), message))
        self.status = status


class Init(ctypes.Structure):
    _fields_ = [("width", ctypes.c_uint32), ("height", ctypes.c_uint32), ("stream", ctypes.c_void_p),
                ("device", ctypes.c_int)]


class State(ctypes.Structure):
    _fields_ = [("depth_func", ctypes.c_int), ("hierarchical", ctypes.c_int), ("msaa_log2", ctypes.c_int),
                ("texture_filter", ctypes.c_int)]


class ShaderParams(ctypes.Structure):
    _fields_ = [("light", ctypes.c_float * 3), ("ks", ctypes.c_float), ("shininess", ctypes.c_float)]


class Mesh(ctypes.Structure):
    _fields_ = [("positions", ctypes.c_void_p), ("position_stride", ctypes.c_uint32),
                ("normals", ctypes.c_void_p), ("normal_stride", ctypes.c_uint32),
                ("uvs", ctypes.c_void_p), ("uv_stride", ctypes.c_uint32),
                ("albedo", ctypes.c_void_p), ("albedo_stride", ctypes.c_uint32),
                ("indices", ctypes.c_void_p), ("num_vertices", ctypes.c_uint32),
                ("num_triangles", ctypes.c_uint32), ("memory", ctypes.c_int),
                ("texture_ids", ctypes.c_void_p)]


class Texture(ctypes.Structure):
    _fields_ = [("width", ctypes.c_uint32), ("height", ctypes.c_uint32), ("format", ctypes.c_int),
                ("texels", ctypes.c_void_p)]


class ObjMesh(ctypes.Structure):
    _fields_ = [("num_vertices", ctypes.c_uint32), ("num_triangles", ctypes.c_uint32),
                ("num_textures", ctypes.c_uint32),
                ("positions", ctypes.POINTER(ctypes.c_float)), ("normals", ctypes.POINTER(ctypes.c_float)),
                ("uvs", ctypes.POINTER(ctypes.c_float)), ("indices", ctypes.POINTER(ctypes.c_uint32)),
                ("texture_ids", ctypes.POINTER(ctypes.c_uint32)), ("textures", ctypes.POINTER(Texture))]


class Outputs(ctypes.Structure):
    _fields_ = [("color", ctypes.c_void_p), ("depth", ctypes.c_void_p), ("triangle_id", ctypes.c_void_p),
                ("width", ctypes.c_uint32), ("height", ctypes.c_uint32), ("samples", ctypes.c_uint32)]


class Stats(ctypes.Structure):
    _fields_ = [("raster_triangles", ctypes.c_uint64), ("bin_entries", ctypes.c_uint64),
                ("bin_capacity", ctypes.c_uint64), ("rerenders", ctypes.c_uint32), ("tile_size", ctypes.c_uint32),
                ("kernels_per_pass", ctypes.c_uint32), ("clipped_polygons", ctypes.c_uint32)]


class Tuning(ctypes.Structure):
    _fields_ = [("small_region", ctypes.c_int), ("raster_variant", ctypes.c_int),
                ("bin_blocks_per_sm", ctypes.c_int), ("raster_blocks_per_sm", ctypes.c_int),
                ("bin_entries_per_triangle", ctypes.c_uint32), ("item_entries", ctypes.c_int)]


class View(ctypes.Structure):
    _fields_ = [("mesh", ctypes.c_uint32), ("mv", _f16), ("proj", _f16), ("raster", _f16),
                ("shading", ShaderParams), ("ps_kind", ctypes.c_int), ("depth_func", ctypes.c_int)]


class BatchOutputs(ctypes.Structure):
    _fields_ = [("color", ctypes.c_void_p), ("depth", ctypes.c_void_p), ("triangle_id", ctypes.c_void_p),
                ("num_views", ctypes.c_uint32), ("width", ctypes.c_uint32), ("height", ctypes.c_uint32)]


class Grads(ctypes.Structure):
    _fields_ = [("albedo", ctypes.c_void_p), ("normals", ctypes.c_void_p), ("positions", ctypes.c_void_p),
                ("light", ctypes.c_void_p), ("ks", ctypes.c_void_p), ("shininess", ctypes.c_void_p)]


# Every entry point declared in include/edxr.h, with its ctypes signature.
_P = ctypes.c_void_p
SIGNATURES = {
    "edxr_create": ([ctypes.POINTER(_P), ctypes.POINTER(Init)], ctypes.c_int),
    "edxr_destroy": ([_P], ctypes.c_int),
    "edxr_resize": ([_P, ctypes.c_uint32, ctypes.c_uint32], ctypes.c_int),
    "edxr_set_transform": ([_P, _P, _P, _P], ctypes.c_int),
    "edxr_set_state": ([_P, ctypes.POINTER(State)], ctypes.c_int),
    "edxr_set_shader": ([_P, ctypes.c_int, ctypes.c_int, ctypes.POINTER(ShaderParams)], ctypes.c_int),
    "edxr_render": ([_P, ctypes.POINTER(Mesh)], ctypes.c_int),
    "edxr_set_textures": ([_P, ctypes.POINTER(Texture), ctypes.c_uint32], ctypes.c_int),
    "edxr_load_obj": ([ctypes.c_char_p, _P, _P, _P, ctypes.POINTER(ctypes.POINTER(ObjMesh))], ctypes.c_int),
    "edxr_free_obj": ([ctypes.POINTER(ObjMesh)], None),
    "edxr_synchronize": ([_P], ctypes.c_int),
    "edxr_get_outputs": ([_P, ctypes.POINTER(Outputs)], ctypes.c_int),
    "edxr_read_outputs": ([_P, _P, _P, _P], ctypes.c_int),
    "edxr_get_back_buffer": ([_P, ctypes.POINTER(_P)], ctypes.c_int),
    "edxr_get_stats": ([_P, ctypes.POINTER(Stats)], ctypes.c_int),
    "edxr_set_profiling": ([_P, ctypes.c_int], ctypes.c_int),
    "edxr_set_tuning": ([_P, ctypes.POINTER(Tuning)], ctypes.c_int),
    "edxr_get_tuning": ([_P, ctypes.POINTER(Tuning)], ctypes.c_int),
    "edxr_debug_scan_stall": ([_P, ctypes.c_int, ctypes.c_int], ctypes.c_int),
    "edxr_get_stage_times": ([_P, _P, ctypes.POINTER(ctypes.c_uint32)], ctypes.c_int),
    "edxr_last_error_string": ([], ctypes.c_char_p),
    "edxr_render_batched": ([_P, ctypes.POINTER(Mesh), ctypes.c_uint32, ctypes.POINTER(View), ctypes.c_uint32,
                             ctypes.c_uint32, ctypes.c_uint32], ctypes.c_int),
    "edxr_get_batch_outputs": ([_P, ctypes.POINTER(BatchOutputs)], ctypes.c_int),
    "edxr_read_batch_outputs": ([_P, ctypes.c_uint32, ctypes.c_uint32, _P, _P, _P], ctypes.c_int),
    "edxr_shade_visible": ([_P, ctypes.POINTER(Mesh), ctypes.POINTER(ShaderParams), _P], ctypes.c_int),
    "edxr_backward": ([_P, ctypes.POINTER(Mesh), ctypes.POINTER(ShaderParams), _P, ctypes.POINTER(Grads)],
                      ctypes.c_int),
    "edxr_render_noalloc": ([ctypes.POINTER(Mesh), _P, _P, _P, ctypes.POINTER(State), ctypes.c_int,
                             ctypes.POINTER(ShaderParams), ctypes.c_uint32, ctypes.c_uint32, _P, _P, _P, _P],
                            ctypes.c_int),
}

_lib = None


def load(path: str = LIB_PATH):
    """Load libedxr.so (raises when it is missing: there is no CPU path)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise ImportError("libedxr.so is not built (%s); run `python -m edxraster_gb300.build` "
                          "or __graft_entry__.build()" % path)
    lib = ctypes.CDLL(path)
    for name, (args, res) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    _lib = lib
    return lib


def check(status: int):
    if status != EDXR_OK:
        msg = load().edxr_last_error_string()
        raise EdxrError(status, msg.decode() if msg else "")
