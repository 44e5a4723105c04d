"""ctypes front end of the CPU oracle (test infrastructure).

``render_oracle`` calls the C restatement (``oracle/edxr_oracle.c``);
``render_reference`` / ``time_reference`` call the reference's own pipeline
compiled against the shim (``oracle/ref_harness.cpp``).  Only tests, the smoke
check and the benchmark's CPU-baseline leg import this module.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import build as _build

_f16 = ctypes.c_float * 16


class _Params(ctypes.Structure):
    _fields_ = [("width", ctypes.c_int), ("height", ctypes.c_int),
                ("mv", _f16), ("proj", _f16), ("raster", _f16),
                ("depth_func", ctypes.c_int), ("hierarchical", ctypes.c_int),
                ("shader", ctypes.c_int), ("light", ctypes.c_float * 3),
                ("ks", ctypes.c_float), ("shininess", ctypes.c_float),
                ("threads", ctypes.c_int), ("msaa_log2", ctypes.c_int),
                ("textures", ctypes.c_void_p), ("num_textures", ctypes.c_int), ("texture_filter", ctypes.c_int)]


class _Texture(ctypes.Structure):
    _fields_ = [("width", ctypes.c_int), ("height", ctypes.c_int), ("format", ctypes.c_int),
                ("texels", ctypes.c_void_p)]


class _Mesh(ctypes.Structure):
    _fields_ = [("positions", ctypes.c_void_p), ("position_stride", ctypes.c_int),
                ("normals", ctypes.c_void_p), ("normal_stride", ctypes.c_int),
                ("uvs", ctypes.c_void_p), ("uv_stride", ctypes.c_int),
                ("albedo", ctypes.c_void_p), ("albedo_stride", ctypes.c_int),
                ("indices", ctypes.c_void_p), ("nv", ctypes.c_int), ("nt", ctypes.c_int),
                ("texture_ids", ctypes.c_void_p)]


class _Out(ctypes.Structure):
    _fields_ = [("id", ctypes.c_void_p), ("depth", ctypes.c_void_p),
                ("lambda0", ctypes.c_void_p), ("lambda1", ctypes.c_void_p),
                ("color", ctypes.c_void_p),
                ("fragments", ctypes.c_longlong), ("raster_tris", ctypes.c_longlong),
                ("clipped_input_tris", ctypes.c_longlong), ("bin_refs", ctypes.c_longlong)]


_lib = None
_ref = None


def _oracle_lib():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(_build.build_oracle())
        _lib.edxr_oracle_render.argtypes = [ctypes.POINTER(_Params), ctypes.POINTER(_Mesh), ctypes.POINTER(_Out)]
        _lib.edxr_oracle_render.restype = ctypes.c_int
        _lib.edxr_oracle_shade.argtypes = [ctypes.POINTER(_Params)] + [ctypes.c_void_p] * 6
        _lib.edxr_oracle_shade.restype = None
    return _lib


def reference_lib():
    """The reference pipeline library, or None when it cannot be built here."""
    global _ref
    if _ref is None:
        path = _build.REF_SO if os.path.exists(_build.REF_SO) else _build.build_ref()
        if path is None:
            return None
        _ref = ctypes.CDLL(path)
        fp, up, i = ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int
        _ref.edxr_ref_parity.argtypes = [i, i, fp, fp, fp, fp, i, up, i, i, up, fp, fp, fp]
        _ref.edxr_ref_parity.restype = ctypes.c_longlong
        _ref.edxr_ref_parity_ms.argtypes = [i, i, fp, fp, fp, fp, i, up, i, i, i, up, fp]
        _ref.edxr_ref_parity_ms.restype = ctypes.c_longlong
        _ref.edxr_ref_time.argtypes = [i, i, fp, fp, fp, fp, i, up, i, i, i, ctypes.POINTER(ctypes.c_int)]
        _ref.edxr_ref_time.restype = ctypes.c_double
    return _ref


def _ptr(a):
    return None if a is None else a.ctypes.data


def make_params(view, threads=None, hierarchical=True, shader=None, depth_func=None, msaa_log2=0):
    p = _Params()
    p.width, p.height = view.width, view.height
    p.mv = _f16(*np.asarray(view.mv, np.float32).ravel())
    p.proj = _f16(*np.asarray(view.proj, np.float32).ravel())
    p.raster = _f16(*np.asarray(view.raster, np.float32).ravel())
    p.depth_func = view.depth_func if depth_func is None else depth_func
    p.hierarchical = 1 if hierarchical else 0
    p.shader = view.shader if shader is None else shader
    p.light = (ctypes.c_float * 3)(*np.asarray(view.light, np.float32))
    p.ks, p.shininess = view.ks, view.shininess
    p.threads = threads or os.cpu_count() or 1
    p.msaa_log2 = msaa_log2
    return p


def render_oracle(mesh, view, threads=None, hierarchical=True, depth_func=None, shader=None,
                  with_color=True, msaa_log2=0, textures=None, texture_filter=2):
    """Run the C restatement.  Returns a dict of numpy arrays and statistics;
    with msaa_log2 > 0, id and depth are (samples, H, W).  `textures`: the
    texture slots of the textured shader, (H, W, 4) uint8 or float32 arrays."""
    lib = _oracle_lib()
    W, H = view.width, view.height
    pos = np.ascontiguousarray(mesh.positions, np.float32)
    nrm = np.ascontiguousarray(mesh.normals, np.float32)
    alb = np.ascontiguousarray(mesh.albedo, np.float32)
    uv = np.ascontiguousarray(mesh.uvs, np.float32)
    idx = np.ascontiguousarray(mesh.indices, np.uint32)
    tid = getattr(mesh, "texture_ids", None)
    tid = None if tid is None else np.ascontiguousarray(tid, np.uint32)
    m = _Mesh(pos.ctypes.data, 3, nrm.ctypes.data, 3, uv.ctypes.data, 2, alb.ctypes.data, 3,
              idx.ctypes.data, mesh.nv, mesh.nt, _ptr(tid))
    S = 1 << msaa_log2
    shape = (H, W) if S == 1 else (S, H, W)
    out_id = np.empty(shape, np.uint32)
    out_depth = np.empty(shape, np.float32)
    l0 = np.empty((H, W), np.float32)
    l1 = np.empty((H, W), np.float32)
    color = np.empty((H, W, 4), np.float64) if with_color else None
    o = _Out(out_id.ctypes.data, out_depth.ctypes.data, l0.ctypes.data, l1.ctypes.data, _ptr(color))
    p = make_params(view, threads, hierarchical, shader, depth_func, msaa_log2)
    keep = []
    if textures:
        descs = []
        for t in textures:
            a = np.ascontiguousarray(t)
            keep.append(a)
            descs.append(_Texture(a.shape[1], a.shape[0], 0 if a.dtype == np.uint8 else 1, a.ctypes.data))
        arr = (_Texture * len(descs))(*descs)
        keep.append(arr)
        p.textures = ctypes.cast(arr, ctypes.c_void_p)
        p.num_textures = len(descs)
    p.texture_filter = texture_filter
    rc = lib.edxr_oracle_render(ctypes.byref(p), ctypes.byref(m), ctypes.byref(o))
    if rc != 0:
        raise RuntimeError("oracle failed with code %d" % rc)
    if S > 1:
        l0 = l1 = None
    return {"id": out_id, "depth": out_depth, "lambda0": l0, "lambda1": l1, "color": color,
            "fragments": o.fragments, "raster_tris": o.raster_tris,
            "clipped_input_tris": o.clipped_input_tris, "bin_refs": o.bin_refs}


def shade_fp64(view, b, pos, nrm, alb, eye, shader=None):
    """FP64 shading model at one point (see edxr_oracle_shade)."""
    lib = _oracle_lib()
    p = make_params(view, 1, True, shader)
    b = np.ascontiguousarray(b, np.float64)
    arrs = [np.ascontiguousarray(a, np.float64) for a in (pos, nrm, alb, eye)]
    rgb = np.empty(3, np.float64)
    lib.edxr_oracle_shade(ctypes.byref(p), b.ctypes.data, *[a.ctypes.data for a in arrs], rgb.ctypes.data)
    return rgb


def render_reference(mesh, view, hierarchical=True):
    """Run the reference's own pipeline (LEQUAL, its only depth function)."""
    lib = reference_lib()
    if lib is None:
        return None
    W, H = view.width, view.height
    verts = mesh.interleaved_pnt()
    idx = np.ascontiguousarray(mesh.indices, np.uint32)
    mv = np.ascontiguousarray(view.mv, np.float32)
    pr = np.ascontiguousarray(view.proj, np.float32)
    ra = np.ascontiguousarray(view.raster, np.float32)
    out_id = np.empty((H, W), np.uint32)
    out_depth = np.empty((H, W), np.float32)
    l0 = np.empty((H, W), np.float32)
    l1 = np.empty((H, W), np.float32)
    frags = lib.edxr_ref_parity(W, H, mv.ctypes.data, pr.ctypes.data, ra.ctypes.data,
                                verts.ctypes.data, mesh.nv, idx.ctypes.data, mesh.nt,
                                1 if hierarchical else 0, out_id.ctypes.data, out_depth.ctypes.data,
                                l0.ctypes.data, l1.ctypes.data)
    if frags < 0:
        raise RuntimeError("reference harness rejected the arguments")
    return {"id": out_id, "depth": out_depth, "lambda0": l0, "lambda1": l1, "fragments": frags}


def render_reference_ms(mesh, view, msaa_log2, hierarchical=True):
    """The reference's own pipeline with 2^msaa_log2 samples per pixel
    (Renderer::SetMSAAMode): per-sample winners and depths, (S, H, W)."""
    lib = reference_lib()
    if lib is None:
        return None
    W, H, S = view.width, view.height, 1 << msaa_log2
    verts = mesh.interleaved_pnt()
    idx = np.ascontiguousarray(mesh.indices, np.uint32)
    mv = np.ascontiguousarray(view.mv, np.float32)
    pr = np.ascontiguousarray(view.proj, np.float32)
    ra = np.ascontiguousarray(view.raster, np.float32)
    out_id = np.empty((S, H, W), np.uint32)
    out_depth = np.empty((S, H, W), np.float32)
    frags = lib.edxr_ref_parity_ms(W, H, mv.ctypes.data, pr.ctypes.data, ra.ctypes.data,
                                   verts.ctypes.data, mesh.nv, idx.ctypes.data, mesh.nt,
                                   1 if hierarchical else 0, msaa_log2, out_id.ctypes.data,
                                   out_depth.ctypes.data)
    if frags < 0:
        raise RuntimeError("reference harness rejected the arguments")
    return {"id": out_id, "depth": out_depth, "fragments": frags}


def time_reference(mesh, view, frames=5, warmup=1):
    """Median seconds per Renderer::RenderMesh of the reference, and its core count."""
    lib = reference_lib()
    if lib is None:
        return None
    verts = mesh.interleaved_pnt()
    idx = np.ascontiguousarray(mesh.indices, np.uint32)
    mv = np.ascontiguousarray(view.mv, np.float32)
    pr = np.ascontiguousarray(view.proj, np.float32)
    ra = np.ascontiguousarray(view.raster, np.float32)
    cores = ctypes.c_int(0)
    t = lib.edxr_ref_time(view.width, view.height, mv.ctypes.data, pr.ctypes.data, ra.ctypes.data,
                          verts.ctypes.data, mesh.nv, idx.ctypes.data, mesh.nt, frames, warmup,
                          ctypes.byref(cores))
    return t, cores.value
