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


@pytest.mark.gpu
def test_facade_renders_like_the_oracle(tmp_path):
    from oracle import pyoracle
    exe = compile_facade(tmp_path)
    sc = scenes.sphere_scene(320, 180)
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
    r = subprocess.run([exe, str(scene_bin), str(out)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    n = v.width * v.height
    raw = open(out, "rb").read()
    ids = np.frombuffer(raw[:4 * n], np.uint32).reshape(v.height, v.width)
    depth = np.frombuffer(raw[4 * n:8 * n], np.float32).reshape(v.height, v.width)
    bb = np.frombuffer(raw[8 * n:], np.uint8).reshape(v.height, v.width, 4)
    o = pyoracle.render_oracle(m, v, depth_func=scenes.DEPTH_LESS)
    assert np.array_equal(ids, o["id"])
    assert np.array_equal(depth.view(np.uint32), o["depth"].view(np.uint32))
    assert np.array_equal(bb[::-1, :, 3] == 255, o["id"] != 0xFFFFFFFF)
