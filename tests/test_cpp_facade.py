"""The C++ facade (include/edxr/Renderer.h): compiles against the C ABI on the
CPU side; on the GPU it renders a scene with the reference's method sequence
and must agree bit for bit with the C oracle."""
import os
import subprocess

import numpy as np
import pytest

from edxraster_gb300 import build as lib_build
from edxraster_gb300 import scenes

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "facade_render.cpp")


def compile_facade(tmp_path):
    lib_build.build()
    exe = str(tmp_path / "facade_render")
    subprocess.run(["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"), SRC, "-o", exe,
                    "-L", lib_build.BUILD_DIR, "-ledxr", "-Wl,-rpath," + lib_build.BUILD_DIR],
                   check=True, capture_output=True, text=True)
    return exe


def test_facade_compiles_and_links(tmp_path):
    assert os.path.exists(compile_facade(tmp_path))


def run_facade(tmp_path, sc, mode="arrays", write=False):
    """Writes the scene for facade_render, runs it (in tmp_path) and returns
    the triangle ids, depth, colour and back buffer it read back."""
    exe = compile_facade(tmp_path)
    v, m = sc.view, sc.mesh
    scene_bin = tmp_path / "scene.bin"
    with open(scene_bin, "wb") as fh:
        fh.write(np.array([v.width, v.height, m.nv, m.nt], np.uint32).tobytes())
        fh.write(np.concatenate([v.mv.ravel(), v.proj.ravel(), v.raster.ravel()]).astype(np.float32).tobytes())
        fh.write(np.array([*v.light, v.ks, v.shininess], np.float32).tobytes())
        for a in (m.positions, m.normals, m.albedo):
            fh.write(np.ascontiguousarray(a, np.float32).tobytes())
        fh.write(np.ascontiguousarray(m.indices, np.uint32).tobytes())
    out = tmp_path / "out.bin"
    args = [exe, str(scene_bin), str(out), mode] + (["write"] if write else [])
    r = subprocess.run(args, capture_output=True, text=True, cwd=str(tmp_path))
    assert r.returncode == 0, r.stderr
    n = v.width * v.height
    raw = open(out, "rb").read()
    ids = np.frombuffer(raw[:4 * n], np.uint32).reshape(v.height, v.width)
    depth = np.frombuffer(raw[4 * n:8 * n], np.float32).reshape(v.height, v.width)
    color = np.frombuffer(raw[8 * n:24 * n], np.float32).reshape(v.height, v.width, 4)
    bb = np.frombuffer(raw[24 * n:], np.uint8).reshape(v.height, v.width, 4)
    return ids, depth, color, bb


def read_bmp(path):
    """A 32-bit BMP as written by WriteFrameToFile: (height, width, 4) BGRA rows
    in file order (bottom-up for a positive height) and the header fields."""
    raw = open(path, "rb").read()
    assert raw[:2] == b"BM"
    size, off = int.from_bytes(raw[2:6], "little"), int.from_bytes(raw[10:14], "little")
    w, h = int.from_bytes(raw[18:22], "little"), int.from_bytes(raw[22:26], "little", signed=True)
    planes, bpp = int.from_bytes(raw[26:28], "little"), int.from_bytes(raw[28:30], "little")
    assert size == len(raw) and planes == 1 and bpp == 32 and h > 0
    return np.frombuffer(raw[off:], np.uint8).reshape(h, w, 4), (w, h)


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["arrays", "interleaved"])
def test_facade_renders_like_the_oracle(tmp_path, mode):
    """The viewer's call sequence through the C++ facade, with the mesh as
    separate arrays or in the reference's Vertex_PositionNormalTex layout
    (InputBuffer.h:16-28, 32-byte stride): triangle ids and depth bit for bit,
    colour within 1e-5 of the oracle's FP64 shading, the back buffer's alpha
    marking covered pixels (bottom-up rows)."""
    from oracle import pyoracle
    sc = scenes.sphere_scene(320, 180)
    ids, depth, color, bb = run_facade(tmp_path, sc, mode)
    o = pyoracle.render_oracle(sc.mesh, sc.view, depth_func=scenes.DEPTH_LESS)
    assert np.array_equal(ids, o["id"])
    assert np.array_equal(depth.view(np.uint32), o["depth"].view(np.uint32))
    cov = o["id"] != 0xFFFFFFFF
    assert cov.any() and float(np.abs(color[cov, :3] - o["color"][cov, :3]).max()) <= 1e-5
    assert np.array_equal(bb[::-1, :, 3] == 255, cov)


@pytest.mark.gpu
def test_facade_writes_frame_bmp(tmp_path):
    """SetWriteFrames + RenderMesh write Frames/FrameNNNNN.bmp
    (Renderer::WriteFrameToFile, Renderer.cpp:352-358): a 54-byte header,
    32-bit BGRA pixels in the back buffer's bottom-up row order."""
    sc = scenes.sphere_scene(160, 96)
    (tmp_path / "Frames").mkdir()
    ids, depth, color, bb = run_facade(tmp_path, sc, "arrays", write=True)
    files = sorted((tmp_path / "Frames").glob("Frame*.bmp"))
    assert len(files) == 1
    px, (w, h) = read_bmp(files[0])
    assert (w, h) == (sc.view.width, sc.view.height)
    assert np.array_equal(px[..., [2, 1, 0, 3]], bb)
    assert (bb[..., 3] == 255).any()


@pytest.mark.gpu
def test_python_writes_frame_bmp(tmp_path):
    """The Python Renderer's WriteFrameToFile: the same BMP of GetBackBuffer."""
    from edxraster_gb300 import renderer as R
    sc = scenes.sphere_scene(160, 96)
    r = R.Renderer()
    r.Initialize(sc.view.width, sc.view.height)
    R.configure(r, sc.view)
    r.RenderMesh(sc.mesh)
    path = r.WriteFrameToFile(str(tmp_path / "Frames"))
    bb = r.GetBackBuffer()
    r.close()
    px, (w, h) = read_bmp(path)
    assert (w, h) == (sc.view.width, sc.view.height)
    assert np.array_equal(px[..., [2, 1, 0, 3]], bb)
    assert (bb[..., 3] == 255).any()
