"""Python mirror of EDXRaster's Renderer (EDXRaster/Core/Renderer.h:15-59) over
the C ABI of include/edxr.h.

Method names and meaning follow the reference: Initialize, Resize,
SetTransform, RenderMesh, WriteFrameToFile, GetBackBuffer, SetMSAAMode,
SetTextureFilter, SetHierarchicalRasterize, SetWriteFrames.  Where the
reference returns nothing and ignores errors, these raise ``EdxrError``.
Extra methods expose what the GPU build adds: the depth function, pixel-shader
selection, float outputs, the batched form and the adjoint.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import _lib
from ._lib import EdxrError  # noqa: F401  (re-exported)

DEPTH_LEQUAL, DEPTH_LESS = 0, 1
PS_BLINN_PHONG, PS_BLINN_PHONG_REFERENCE, PS_LAMBERTIAN_ALBEDO, PS_LAMBERTIAN = 0, 1, 2, 3
PS_LAMBERTIAN_TEXTURED = 4
# TextureFilter (RenderStates.h:23)
FILTER_NEAREST, FILTER_LINEAR, FILTER_TRILINEAR = 0, 1, 2
FILTER_ANISOTROPIC_4X, FILTER_ANISOTROPIC_8X, FILTER_ANISOTROPIC_16X = 3, 4, 5


def _f16(m):
    m = np.ascontiguousarray(np.asarray(m, np.float32).reshape(16))
    return (ctypes.c_float * 16)(*m)


class DeviceMesh:
    """A mesh resident in device memory (torch CUDA tensors), passed by pointer."""

    def __init__(self, positions, indices, normals=None, albedo=None, uvs=None, texture_ids=None):
        import torch
        dev = positions.device

        def prep(t, dtype, cols):
            if t is None:
                return None
            if not isinstance(t, torch.Tensor):
                t = torch.from_numpy(np.ascontiguousarray(t))
            t = t.to(device=dev, dtype=dtype).contiguous()
            assert t.dim() == 2 and t.shape[1] == cols
            return t

        self.positions = prep(positions, torch.float32, 3)
        self.indices = prep(indices, torch.int32, 3)
        self.normals = prep(normals, torch.float32, 3)
        self.albedo = prep(albedo, torch.float32, 3)
        self.uvs = prep(uvs, torch.float32, 2)
        self.texture_ids = None
        if texture_ids is not None:
            ids = texture_ids if isinstance(texture_ids, torch.Tensor) else torch.from_numpy(
                np.ascontiguousarray(texture_ids).astype(np.int32))
            self.texture_ids = ids.to(device=dev, dtype=torch.int32).contiguous().view(-1)

    @classmethod
    def from_mesh(cls, mesh, device="cuda"):
        import torch
        t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(device)  # noqa: E731
        tid = getattr(mesh, "texture_ids", None)
        return cls(t(mesh.positions), t(mesh.indices.astype(np.int32)), t(mesh.normals), t(mesh.albedo), t(mesh.uvs),
                   None if tid is None else t(tid.astype(np.int32)))

    @property
    def nv(self):
        return int(self.positions.shape[0])

    @property
    def nt(self):
        return int(self.indices.shape[0])

    def abi(self) -> _lib.Mesh:
        p = lambda t: None if t is None else t.data_ptr()  # noqa: E731
        return _lib.Mesh(p(self.positions), 12, p(self.normals), 12, p(self.uvs), 8, p(self.albedo), 12,
                         p(self.indices), self.nv, self.nt, _lib.MEMORY_DEVICE, p(self.texture_ids))


class HostMesh:
    """A mesh in host memory (numpy) read by every render call: positions and
    indices are copied to the device; with pinned=True (page-locked arrays)
    the shading reads normals and albedo in place, otherwise they are copied
    as well."""

    def __init__(self, mesh, pinned=False):
        self._keep = []
        self.pinned = pinned

        def prep(a, dtype):
            a = np.ascontiguousarray(a, dtype)
            if pinned:
                import torch
                t = torch.from_numpy(a).pin_memory()
                self._keep.append(t)
                return t.numpy()
            return a

        self.positions = prep(mesh.positions, np.float32)
        self.normals = prep(mesh.normals, np.float32)
        self.albedo = prep(mesh.albedo, np.float32)
        self.uvs = prep(mesh.uvs, np.float32)
        self.indices = prep(mesh.indices, np.uint32)
        tid = getattr(mesh, "texture_ids", None)
        self.texture_ids = None if tid is None else prep(tid, np.uint32)
        self.nv, self.nt = int(self.positions.shape[0]), int(self.indices.shape[0])

    def nbytes(self) -> int:
        """Bytes of host input one render call reads (texture coordinates are
        not read: no shader samples them)."""
        return sum(a.nbytes for a in (self.positions, self.normals, self.albedo, self.indices))

    def copied_nbytes(self) -> int:
        """Bytes one render call copies to the device: positions and indices,
        plus normals and albedo unless they are pinned (read in place)."""
        n = self.positions.nbytes + self.indices.nbytes
        return n if self.pinned else n + self.normals.nbytes + self.albedo.nbytes

    def abi(self) -> _lib.Mesh:
        tid = None if self.texture_ids is None else self.texture_ids.ctypes.data
        return _lib.Mesh(self.positions.ctypes.data, 12, self.normals.ctypes.data, 12, self.uvs.ctypes.data, 8,
                         self.albedo.ctypes.data, 12, self.indices.ctypes.data, self.nv, self.nt, _lib.MEMORY_HOST,
                         tid)


def _as_abi_mesh(mesh):
    if isinstance(mesh, (DeviceMesh, HostMesh)):
        return mesh, mesh.abi()
    hm = HostMesh(mesh)
    return hm, hm.abi()


class Renderer:
    """GPU renderer with the reference's public interface."""

    def __init__(self, device: int = 0, stream=None):
        self._lib = _lib.load()
        self._h = ctypes.c_void_p()
        self._device = device
        self._stream = stream
        self._width = self._height = 0
        self._state = _lib.State(DEPTH_LEQUAL, 1, 0, FILTER_TRILINEAR)  # RenderStates::DefaultSettings
        self._write_frames = False
        self._frame = 0
        self._keep = None

    # -- lifetime -----------------------------------------------------------
    def Initialize(self, width: int, height: int):
        """Renderer::Initialize (Renderer.cpp:22-62)."""
        if self._h:
            self.Resize(width, height)
            return
        stream = self._stream
        if stream is None:
            import torch
            stream = torch.cuda.Stream(device=self._device)
            self._stream = stream
        handle = getattr(stream, "cuda_stream", stream)
        init = _lib.Init(width, height, handle, self._device)
        _lib.check(self._lib.edxr_create(ctypes.byref(self._h), ctypes.byref(init)))
        self._width, self._height = width, height
        _lib.check(self._lib.edxr_set_state(self._h, ctypes.byref(self._state)))

    def close(self):
        if self._h:
            self._lib.edxr_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def stream(self):
        return self._stream

    # -- reference interface ---------------------------------------------------
    def Resize(self, width: int, height: int):
        """Renderer::Resize (Renderer.cpp:64-83)."""
        _lib.check(self._lib.edxr_resize(self._h, width, height))
        self._width, self._height = width, height

    def SetTransform(self, model_view, proj, to_raster):
        """Renderer::SetTransform (Renderer.cpp:85-92)."""
        self._mv, self._proj, self._raster = _f16(model_view), _f16(proj), _f16(to_raster)
        _lib.check(self._lib.edxr_set_transform(self._h, ctypes.addressof(self._mv), ctypes.addressof(self._proj),
                                                ctypes.addressof(self._raster)))

    def SetMSAAMode(self, msaa_count_log2: int):
        """Renderer::SetMSAAMode (Renderer.cpp:94-98): 2^msaa_count_log2 samples
        per pixel, 0..5 (1 to 32 samples)."""
        old = self._state.msaa_log2
        self._state.msaa_log2 = msaa_count_log2
        try:
            _lib.check(self._lib.edxr_set_state(self._h, ctypes.byref(self._state)))
        except Exception:
            self._state.msaa_log2 = old
            raise

    @property
    def samples(self) -> int:
        return 1 << self._state.msaa_log2

    def SetTextureFilter(self, texture_filter: int):
        """Renderer::SetTextureFilter (Renderer.h:48): FILTER_* (trilinear is the reference default)."""
        old = self._state.texture_filter
        self._state.texture_filter = int(texture_filter)
        try:
            _lib.check(self._lib.edxr_set_state(self._h, ctypes.byref(self._state)))
        except Exception:
            self._state.texture_filter = old
            raise

    def SetTextures(self, textures):
        """The texture slots (Mesh::GetTextures / RenderStates::TextureSlots): a list of
        (H, W, 4) arrays, uint8 (RGBA8) or float32 (RGBA32F); row 0 at v = 0."""
        arrs, descs = [], []
        for t in textures:
            a = np.ascontiguousarray(t)
            if a.ndim != 3 or a.shape[2] != 4 or a.dtype not in (np.uint8, np.float32):
                raise ValueError("a texture is an (H, W, 4) uint8 or float32 array")
            arrs.append(a)
            descs.append(_lib.Texture(a.shape[1], a.shape[0], 0 if a.dtype == np.uint8 else 1, a.ctypes.data))
        arr = (_lib.Texture * max(1, len(descs)))(*descs)
        _lib.check(self._lib.edxr_set_textures(self._h, arr, len(descs)))

    def SetHierarchicalRasterize(self, h: bool):
        """Renderer::SetHierarchicalRasterize (Renderer.h:49)."""
        self._state.hierarchical = 1 if h else 0
        _lib.check(self._lib.edxr_set_state(self._h, ctypes.byref(self._state)))

    def SetWriteFrames(self, wf: bool):
        """Renderer::SetWriteFrames (Renderer.h:50)."""
        self._write_frames = bool(wf)

    def SetDepthFunc(self, func: int):
        self._state.depth_func = int(func)
        _lib.check(self._lib.edxr_set_state(self._h, ctypes.byref(self._state)))

    def SetPixelShader(self, kind: int, light=(1.0, 1.0, -1.0), ks: float = 0.5, shininess: float = 32.0):
        p = _lib.ShaderParams((ctypes.c_float * 3)(*[float(x) for x in light]), float(ks), float(shininess))
        _lib.check(self._lib.edxr_set_shader(self._h, 0, int(kind), ctypes.byref(p)))

    def RenderMesh(self, mesh, synchronize: bool = True):
        """Renderer::RenderMesh (Renderer.cpp:100-118): clear and render one mesh."""
        keep, m = _as_abi_mesh(mesh)
        self._keep = (keep, m)
        _lib.check(self._lib.edxr_render(self._h, ctypes.byref(m)))
        if synchronize:
            self.Synchronize()
        self._frame += 1
        if self._write_frames:
            self.WriteFrameToFile()

    def Synchronize(self):
        _lib.check(self._lib.edxr_synchronize(self._h))

    def GetBackBuffer(self, copy: bool = True) -> np.ndarray:
        """Renderer::GetBackBuffer (Renderer.cpp:360-363): RGBA8, bottom-up rows.

        With copy=False the array is a view of the renderer's pinned host
        buffer, borrowed like the reference's pointer: valid until the next
        GetBackBuffer, Resize or close of this renderer.
        """
        p = ctypes.c_void_p()
        _lib.check(self._lib.edxr_get_back_buffer(self._h, ctypes.byref(p)))
        buf = (ctypes.c_uint8 * (4 * self._width * self._height)).from_address(p.value)
        img = np.frombuffer(buf, np.uint8).reshape(self._height, self._width, 4)
        return img.copy() if copy else img

    def WriteFrameToFile(self, directory: str = "Frames"):
        """Renderer::WriteFrameToFile (Renderer.cpp:352-358): a BMP of the back buffer."""
        os.makedirs(directory, exist_ok=True)
        img = self.GetBackBuffer()  # bottom-up rows, which is BMP's native row order
        h, w = img.shape[:2]
        bgra = img[..., [2, 1, 0, 3]].tobytes()
        hdr = b"BM" + (54 + len(bgra)).to_bytes(4, "little") + b"\0\0\0\0" + (54).to_bytes(4, "little")
        dib = (40).to_bytes(4, "little") + w.to_bytes(4, "little") + h.to_bytes(4, "little", signed=True) + \
            (1).to_bytes(2, "little") + (32).to_bytes(2, "little") + b"\0" * 24
        path = os.path.join(directory, "Frame%05d.bmp" % self._frame)
        with open(path, "wb") as fh:
            fh.write(hdr + dib + bgra)
        return path

    # -- outputs -------------------------------------------------------------
    def ReadOutputs(self):
        """Host copies of the last frame: colour (H,W,4) f32, depth (H,W) f32, triangle id (H,W) u32;
        with several samples per pixel depth and id are (S,H,W) and colour is the resolve."""
        W, H = self._width, self._height
        o = self.DeviceOutputs()
        shape = (H, W) if o.samples <= 1 else (o.samples, H, W)
        color = np.empty((H, W, 4), np.float32)
        depth = np.empty(shape, np.float32)
        tid = np.empty(shape, np.uint32)
        _lib.check(self._lib.edxr_read_outputs(self._h, color.ctypes.data, depth.ctypes.data, tid.ctypes.data))
        return color, depth, tid

    def DeviceOutputs(self) -> _lib.Outputs:
        o = _lib.Outputs()
        _lib.check(self._lib.edxr_get_outputs(self._h, ctypes.byref(o)))
        return o

    def Stats(self) -> _lib.Stats:
        s = _lib.Stats()
        _lib.check(self._lib.edxr_get_stats(self._h, ctypes.byref(s)))
        return s

    TUNING_FIELDS = ("small_region", "raster_variant", "bin_blocks_per_sm", "raster_blocks_per_sm",
                     "bin_entries_per_triangle", "item_entries")

    def SetTuning(self, tuning: dict):
        cur = self.GetTuning()
        cur.update({k: int(v) for k, v in tuning.items() if k in self.TUNING_FIELDS})
        t = _lib.Tuning(*[cur[k] for k in self.TUNING_FIELDS])
        _lib.check(self._lib.edxr_set_tuning(self._h, ctypes.byref(t)))

    def GetTuning(self) -> dict:
        t = _lib.Tuning()
        _lib.check(self._lib.edxr_get_tuning(self._h, ctypes.byref(t)))
        return {k: int(getattr(t, k)) for k in self.TUNING_FIELDS}

    STAGES = ("clear", "setup+bin count", "bin scan", "bin scatter", "raster+shade")

    def SetProfiling(self, enable: bool):
        _lib.check(self._lib.edxr_set_profiling(self._h, 1 if enable else 0))

    def StageTimes(self) -> dict:
        """Milliseconds per stage of the last pass (profiling must be on)."""
        ms = (ctypes.c_float * 8)()
        n = ctypes.c_uint32(8)
        _lib.check(self._lib.edxr_get_stage_times(self._h, ms, ctypes.byref(n)))
        return {self.STAGES[i]: float(ms[i]) for i in range(n.value)}

    # -- batched form ----------------------------------------------------------
    @staticmethod
    def PrepareBatch(meshes, views):
        """ABI arrays for a batched pass, built once and reusable across calls."""
        keeps, abis = [], []
        for m in meshes:
            k, a = _as_abi_mesh(m)
            keeps.append(k)
            abis.append(a)
        marr = (_lib.Mesh * len(abis))(*abis)
        varr = (_lib.View * len(views))()
        for i, v in enumerate(views):
            varr[i].mesh = v.mesh
            varr[i].mv = _f16(v.mv)
            varr[i].proj = _f16(v.proj)
            varr[i].raster = _f16(v.raster)
            varr[i].shading = _lib.ShaderParams((ctypes.c_float * 3)(*[float(x) for x in v.light]), v.ks, v.shininess)
            varr[i].ps_kind = v.shader
            varr[i].depth_func = v.depth_func
        return (keeps, marr, len(abis), varr, len(views))

    def RenderBatched(self, meshes, views, width: int, height: int, synchronize: bool = True):
        """Render every (mesh, view) pair in one pass; views are scenes.View with a .mesh index.
        `meshes` may instead be the result of PrepareBatch (then `views` is ignored)."""
        batch = meshes if isinstance(meshes, tuple) else self.PrepareBatch(meshes, views)
        self._keep = batch
        _, marr, nm, varr, nv = batch
        _lib.check(self._lib.edxr_render_batched(self._h, marr, nm, varr, nv, width, height))
        if synchronize:
            self.Synchronize()

    def BatchOutputs(self) -> _lib.BatchOutputs:
        o = _lib.BatchOutputs()
        _lib.check(self._lib.edxr_get_batch_outputs(self._h, ctypes.byref(o)))
        return o

    def ReadBatchOutputs(self, first: int, count: int, width: int, height: int):
        color = np.empty((count, height, width, 4), np.float32)
        depth = np.empty((count, height, width), np.float32)
        tid = np.empty((count, height, width), np.uint32)
        _lib.check(self._lib.edxr_read_batch_outputs(self._h, first, count, color.ctypes.data, depth.ctypes.data,
                                                     tid.ctypes.data))
        return color, depth, tid


def load_obj(path: str, pos=(0.0, 0.0, 0.0), scale=(1.0, 1.0, 1.0), rot=(0.0, 0.0, 0.0)):
    """Mesh::LoadMesh (Mesh.cpp:11-34) through edxr_load_obj: a Wavefront OBJ
    file with its MTL materials.  Returns (scenes.Mesh with texture_ids, list of
    (H, W, 4) float32 textures, one per material slot, slot 0 = white default)."""
    from . import scenes
    lib = _lib.load()
    f3 = ctypes.c_float * 3
    p, s, r = f3(*pos), f3(*scale), f3(*rot)
    m = ctypes.POINTER(_lib.ObjMesh)()
    _lib.check(lib.edxr_load_obj(os.fsencode(path), ctypes.addressof(p), ctypes.addressof(s), ctypes.addressof(r),
                                 ctypes.byref(m)))
    try:
        o = m.contents
        nv, nt = o.num_vertices, o.num_triangles
        arr = lambda ptr, n, dt: np.ctypeslib.as_array(ptr, shape=(n,)).astype(dt).copy() if n else np.zeros(0, dt)  # noqa: E731
        pos_ = arr(o.positions, 3 * nv, np.float32).reshape(-1, 3)
        nrm = arr(o.normals, 3 * nv, np.float32).reshape(-1, 3)
        uvs = arr(o.uvs, 2 * nv, np.float32).reshape(-1, 2)
        idx = arr(o.indices, 3 * nt, np.uint32).reshape(-1, 3)
        tid = arr(o.texture_ids, nt, np.uint32)
        textures = []
        for k in range(o.num_textures):
            t = o.textures[k]
            buf = ctypes.cast(t.texels, ctypes.POINTER(ctypes.c_float))
            textures.append(np.ctypeslib.as_array(buf, shape=(t.height * t.width * 4,)).reshape(
                t.height, t.width, 4).copy())
    finally:
        lib.edxr_free_obj(m)
    mesh = scenes.Mesh(pos_, nrm, np.ones_like(pos_), uvs, idx)
    mesh.texture_ids = tid
    return mesh, textures


def configure(r: Renderer, view, hierarchical: bool = True):
    """Apply a scenes.View (camera, shader, depth function) to a renderer."""
    r.SetTransform(view.mv, view.proj, view.raster)
    r.SetPixelShader(view.shader, view.light, view.ks, view.shininess)
    r.SetDepthFunc(view.depth_func)
    r.SetHierarchicalRasterize(hierarchical)
