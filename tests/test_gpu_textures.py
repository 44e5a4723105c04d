"""The textured Lambertian shader (LambertianAlbedoPixelShader, Shader.h:209-244)
through the C ABI: texture slots, per-triangle texture ids and every filter.

Coverage, winners and depth are bit-exact with the oracle.  The texture
sample is the build's own sampler (EDXUtil's is absent), restated in the
oracle with the same FP32 operations, so colour agrees to 1e-5 (the FP64
diffuse term of the oracle) except where the level of detail of trilinear or
anisotropic filtering sits on an integer and the two sides' log2 round to
different levels: a handful of pixels.
"""
import numpy as np
import pytest

from edxraster_gb300 import renderer as R
from edxraster_gb300 import scenes
from oracle import pyoracle

pytestmark = pytest.mark.gpu


def render(sc, textures, texture_filter, msaa_log2=0, device_mesh=False):
    r = R.Renderer()
    r.Initialize(sc.view.width, sc.view.height)
    R.configure(r, sc.view)
    r.SetTextures(textures)
    r.SetTextureFilter(texture_filter)
    if msaa_log2:
        r.SetMSAAMode(msaa_log2)
    r.RenderMesh(R.DeviceMesh.from_mesh(sc.mesh) if device_mesh == True else  # noqa: E712
                 R.HostMesh(sc.mesh, pinned=True) if device_mesh == "pinned" else sc.mesh)
    out = r.ReadOutputs()
    r.close()
    return out


def check(sc, textures, flt, msaa_log2=0, device_mesh=False):
    color, depth, tid = render(sc, textures, flt, msaa_log2, device_mesh)
    o = pyoracle.render_oracle(sc.mesh, sc.view, textures=textures, texture_filter=flt, msaa_log2=msaa_log2)
    assert np.array_equal(tid, o["id"])
    assert np.array_equal(depth.view(np.uint32), o["depth"].view(np.uint32))
    cov = (tid != 0xFFFFFFFF) if msaa_log2 == 0 else (tid != 0xFFFFFFFF).any(axis=0)
    err = np.abs(color[cov, :3].astype(np.float64) - o["color"][cov, :3]).max(axis=-1)
    tol = 1e-5 if msaa_log2 == 0 else 1.0 / 255.0 + 1e-6
    assert (err > tol).mean() < 0.002, "%d of %d pixels beyond %.g" % ((err > tol).sum(), err.size, tol)
    return err


@pytest.mark.parametrize("flt", [R.FILTER_NEAREST, R.FILTER_LINEAR, R.FILTER_TRILINEAR, R.FILTER_ANISOTROPIC_4X,
                                 R.FILTER_ANISOTROPIC_8X, R.FILTER_ANISOTROPIC_16X])
def test_textured_filters(cuda_lib, flt):
    err = check(scenes.textured_scene(), scenes.test_textures(), flt)
    if flt <= R.FILTER_LINEAR:  # no level of detail involved: same operations on both sides
        assert err.max() <= 1e-5


def test_textured_device_mesh_and_msaa(cuda_lib):
    sc = scenes.textured_scene(160, 96, seed=1)
    check(sc, scenes.test_textures(1), R.FILTER_TRILINEAR, device_mesh=True)
    # page-locked uvs and texture ids are read in place
    check(sc, scenes.test_textures(1), R.FILTER_TRILINEAR, device_mesh="pinned")
    check(sc, scenes.test_textures(1), R.FILTER_LINEAR, msaa_log2=2)


def test_filters_differ_and_slots_matter(cuda_lib):
    sc = scenes.textured_scene(160, 96)
    tex = scenes.test_textures()
    near, _, _ = render(sc, tex, R.FILTER_NEAREST)
    tri, _, _ = render(sc, tex, R.FILTER_TRILINEAR)
    assert np.abs(near - tri).max() > 0.05
    flat = [np.full((1, 1, 4), 0.5, np.float32)] * 3
    c, _, tid = render(sc, flat, R.FILTER_TRILINEAR)
    o = pyoracle.render_oracle(sc.mesh, sc.view, textures=flat, texture_filter=R.FILTER_TRILINEAR)
    cov = tid != 0xFFFFFFFF
    assert np.abs(c[cov, :3] - o["color"][cov, :3]).max() <= 1e-5


def test_texture_errors(cuda_lib):
    r = R.Renderer()
    r.Initialize(16, 16)
    with pytest.raises(R.EdxrError):
        r.SetTextures([np.zeros((0, 4, 4), np.uint8)])
    with pytest.raises(R.EdxrError):
        r.SetTextureFilter(9)
    r.SetTextures([])  # clearing is allowed
    r.close()


def test_obj_file_renders_like_the_oracle(cuda_lib, tmp_path):
    """Mesh::LoadMesh's path: an OBJ file with MTL materials (an image texture
    and a constant colour) loaded by edxr_load_obj and rendered textured."""
    sc = scenes.textured_scene(160, 96)
    m = sc.mesh
    checker = scenes.test_textures()[0]
    ppm = checker[::-1, :, :3]  # PPM rows run top-down; the texture's row 0 is its bottom
    (tmp_path / "check.ppm").write_bytes(b"P6\n64 64\n255\n" + np.ascontiguousarray(ppm).tobytes())
    (tmp_path / "scene.mtl").write_text("newmtl check\nmap_Kd check.ppm\nnewmtl warm\nKd 0.9 0.6 0.3\n")
    lines = ["mtllib scene.mtl"]
    lines += ["v %.9g %.9g %.9g" % tuple(p) for p in m.positions]
    lines += ["vt %.9g %.9g" % tuple(t) for t in m.uvs]
    lines += ["vn %.9g %.9g %.9g" % tuple(n) for n in m.normals]
    cur = None
    for tri, slot in zip(m.indices, m.texture_ids):
        name = "check" if slot == 0 else "warm"
        if name != cur:
            lines.append("usemtl " + name)
            cur = name
        lines.append("f " + " ".join("%d/%d/%d" % (i + 1, i + 1, i + 1) for i in tri))
    (tmp_path / "scene.obj").write_text("\n".join(lines) + "\n")
    mesh, tex = R.load_obj(str(tmp_path / "scene.obj"))
    assert mesh.nt == m.nt and len(tex) == 3
    assert np.allclose(tex[1][..., :3], checker[..., :3] / 255.0)
    loaded = scenes.Scene("obj", mesh, sc.view)
    check(loaded, tex, R.FILTER_TRILINEAR)
