"""Mesh input (Mesh::LoadMesh over an OBJ file, Mesh.cpp:11-34) through
edxr_load_obj: host code, no GPU needed."""
import os
import struct

import numpy as np
import pytest

from edxraster_gb300 import renderer as R


def write_bmp(path, rgb_rows_bottom_up, bpp=24):
    h, w = len(rgb_rows_bottom_up), len(rgb_rows_bottom_up[0])
    bypp = bpp // 8
    row = (w * bypp + 3) & ~3
    data = b""
    for r in rgb_rows_bottom_up:
        line = b"".join(bytes([b, g, rr] + ([255] if bpp == 32 else [])) for rr, g, b in r)
        data += line + b"\0" * (row - len(line))
    hdr = b"BM" + struct.pack("<IHHI", 54 + len(data), 0, 0, 54)
    dib = struct.pack("<IiiHHIIiiII", 40, w, h, 1, bpp, 0, len(data), 2835, 2835, 0, 0)
    open(path, "wb").write(hdr + dib + data)


@pytest.fixture
def obj_dir(tmp_path):
    (tmp_path / "m.mtl").write_text(
        "newmtl red\nKd 1 0 0\n"
        "newmtl ppm\nKd 0.5 0.5 0.5\nmap_Kd tex.ppm\n"
        "newmtl bmp\nmap_Kd -bm 1 sub/tex.bmp\n")
    (tmp_path / "tex.ppm").write_bytes(b"P6\n# comment\n2 2\n255\n" + bytes([255, 0, 0, 0, 255, 0, 0, 0, 255, 255, 255, 255]))
    os.makedirs(tmp_path / "sub")
    write_bmp(str(tmp_path / "sub" / "tex.bmp"), [[(10, 20, 30), (40, 50, 60), (70, 80, 90)], [(1, 2, 3), (4, 5, 6), (7, 8, 9)]])
    (tmp_path / "scene.obj").write_text(
        "mtllib m.mtl\n"
        "v 0 0 0\nv 1 0 0\nv 1 1 0\nv 0 1 0\nv 0 0 1\n"
        "vt 0 0\nvt 1 0\nvt 1 1\nvt 0 1\n"
        "vn 0 0 -1\n"
        "f 1 2 3\n"                      # before usemtl: slot 0
        "usemtl red\nf 1/1/1 2/2/1 3/3/1 4/4/1\n"  # a quad: two triangles
        "usemtl ppm\nf -5//1 -4//1 -1//1\n"       # negative indices, no texture coordinate
        "usemtl bmp\nf 1/1 3/3 5/2\n"
        "usemtl nosuch\nf 2 3 5\n")
    return tmp_path


def test_obj_loads_topology_materials_and_textures(obj_dir, cuda_lib):
    mesh, tex = R.load_obj(str(obj_dir / "scene.obj"))
    assert mesh.nt == 6
    assert list(mesh.texture_ids) == [0, 1, 1, 2, 3, 0]
    # one vertex per distinct (v, vt, vn) corner: 3 + 4 + 3 + 3 + 1
    assert mesh.nv == 14
    assert len(tex) == 4
    assert tex[0].shape == (1, 1, 4) and np.allclose(tex[0], 1.0)
    assert np.allclose(tex[1][0, 0], [1, 0, 0, 1])
    ppm = tex[2]
    assert ppm.shape == (2, 2, 4)
    assert np.allclose(ppm[1, 0, :3], [1, 0, 0]) and np.allclose(ppm[0, 0, :3], [0, 0, 1])  # row 0 = image bottom
    bmp = tex[3]
    assert bmp.shape == (2, 3, 4)
    assert np.allclose(bmp[0, 0, :3] * 255, [10, 20, 30]) and np.allclose(bmp[1, 2, :3] * 255, [7, 8, 9])
    # a face without normals gets its face normal
    tri = mesh.indices[4]
    n = mesh.normals[tri[0]]
    assert abs(np.linalg.norm(n) - 1) < 1e-6


def test_obj_transform(obj_dir, cuda_lib):
    base, _ = R.load_obj(str(obj_dir / "scene.obj"))
    moved, _ = R.load_obj(str(obj_dir / "scene.obj"), pos=(1, 2, 3), scale=(2, 3, 4), rot=(0, 0, 90))
    p = base.positions.astype(np.float64) * [2, 3, 4]
    rz = np.array([[0, -1, 0], [1, 0, 0], [0, 0, 1]], np.float64)
    expect = p @ rz.T + [1, 2, 3]
    assert np.allclose(moved.positions, expect, atol=1e-5)
    assert np.allclose(np.linalg.norm(moved.normals, axis=1), 1.0, atol=1e-6)


def test_obj_errors(tmp_path, cuda_lib):
    with pytest.raises(R.EdxrError):
        R.load_obj(str(tmp_path / "missing.obj"))
    (tmp_path / "bad.obj").write_text("v 0 0 0\nf 1 2 3\n")
    with pytest.raises(R.EdxrError):
        R.load_obj(str(tmp_path / "bad.obj"))
