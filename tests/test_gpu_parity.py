"""Parity of the CUDA pipeline (through the C ABI) with the reference.

Coverage, the winning triangle and the depth buffer must be bit-identical to
the reference's Renderer (golden fixtures) and to the C oracle; colour must be
within 1e-5 absolute of the oracle's FP64 shading (COLOR_TOL).
"""
import numpy as np
import pytest

from edxraster_gb300 import renderer as R
from edxraster_gb300 import scenes
from oracle import pyoracle
from _scenes import deep_clip_scene, golden_names, load_golden, mismatch_report

pytestmark = pytest.mark.gpu
COLOR_TOL = 1e-5


def render_gpu(sc, hierarchical=True, device_mesh=False, depth_func=None, shader=None):
    r = R.Renderer()
    r.Initialize(sc.view.width, sc.view.height)
    v = sc.view
    R.configure(r, v, hierarchical)
    if depth_func is not None:
        r.SetDepthFunc(depth_func)
    if shader is not None:
        r.SetPixelShader(shader, v.light, v.ks, v.shininess)
    mesh = R.DeviceMesh.from_mesh(sc.mesh) if device_mesh else sc.mesh
    r.RenderMesh(mesh)
    out = r.ReadOutputs()
    stats = r.Stats()
    r.close()
    return out, stats


def check_against_oracle(sc, hierarchical=True, depth_func=None, shader=None, device_mesh=False):
    (color, depth, tid), _ = render_gpu(sc, hierarchical, device_mesh, depth_func, shader)
    o = pyoracle.render_oracle(sc.mesh, sc.view, hierarchical=hierarchical,
                               depth_func=sc.view.depth_func if depth_func is None else depth_func,
                               shader=shader)
    assert not mismatch_report("triangle id", tid, o["id"])
    assert not mismatch_report("depth", depth.view(np.uint32), o["depth"].view(np.uint32))
    cov = tid != 0xFFFFFFFF
    err = np.abs(color[cov, :3].astype(np.float64) - o["color"][cov, :3])
    max_err = float(err.max()) if err.size else 0.0
    assert max_err <= COLOR_TOL, "max colour error %.3g" % max_err
    assert np.all(color[~cov] == 0.0)
    assert np.all(color[cov, 3] == 1.0)
    return max_err, cov.mean()


@pytest.mark.parametrize("name", golden_names())
def test_golden_bit_exact(cuda_lib, name):
    sc, hier, exp = load_golden(name)
    (color, depth, tid), _ = render_gpu(sc, hier)
    assert not mismatch_report("triangle id", tid, exp["id"])
    assert not mismatch_report("depth", depth.view(np.uint32), exp["depth_bits"])


@pytest.mark.parametrize("name", golden_names())
def test_golden_color(cuda_lib, name):
    sc, hier, _ = load_golden(name)
    check_against_oracle(sc, hier, depth_func=scenes.DEPTH_LEQUAL)


@pytest.mark.parametrize("depth_func", [scenes.DEPTH_LEQUAL, scenes.DEPTH_LESS])
def test_depth_ties_follow_submission_order(cuda_lib, depth_func):
    sc = scenes.stress_scene(6000, 320, 200, seed=7, max_area=3e3, dup_fraction=0.25)
    check_against_oracle(sc, depth_func=depth_func)


@pytest.mark.parametrize("shader", [0, 1, 2, 3])
def test_pixel_shaders(cuda_lib, shader):
    sc = scenes.sphere_scene(256, 160)
    if shader == 1:
        sc.view.ks, sc.view.shininess = 3.0, 200.0
    check_against_oracle(sc, shader=shader)


def test_sphere_full_size(cuda_lib):
    check_against_oracle(scenes.sphere_scene())


def test_terrain_clipping(cuda_lib):
    check_against_oracle(scenes.terrain_scene(192, 640, 360, seed=1))


def test_stress_medium(cuda_lib):
    check_against_oracle(scenes.stress_scene(40000, 960, 540, seed=7))


@pytest.mark.parametrize("workload", ["terrain", "stress"])
def test_benchmark_workloads_full_size(cuda_lib, workload):
    """The benchmark's own scenes at full size (the heightfield's 2,097,152
    triangles at 1920x1080 with its vertex stage and clipping; the stress
    scene's 1,000,000 triangles at 3840x2160 with split tiles and occluder
    bounds): every pixel's winner and depth bit-exact, colour within 1e-5."""
    sc = {"terrain": lambda: scenes.terrain_scene(1024, 1920, 1080, seed=1),
          "stress": lambda: scenes.stress_scene(1_000_000, 3840, 2160, seed=7)}[workload]()
    _, coverage = check_against_oracle(sc)
    assert coverage > 0.3


@pytest.mark.parametrize("n,width,height", [(400, 160, 120), (16000, 48, 32)])
def test_deep_clipping(cuda_lib, n, width, height):
    """Short clip queues are clipped by 16-lane groups (one polygon vertex per
    lane), long ones (more triangles than one round of the grid's groups,
    64 per SM) by one lane per triangle: both against the oracle."""
    import torch
    sc = deep_clip_scene(n, width, height, seed=n)
    check_against_oracle(sc)
    _, stats = render_gpu(sc)
    groups = torch.cuda.get_device_properties(0).multi_processor_count * 64
    if n > 1000:
        assert stats.clipped_polygons > groups
    else:
        assert 0 < stats.clipped_polygons <= groups


def test_non_hierarchical(cuda_lib):
    check_against_oracle(scenes.stress_scene(3000, 400, 240, seed=5), hierarchical=False)


@pytest.mark.parametrize("size", [(97, 61), (33, 17), (1, 1), (250, 130)])
def test_odd_framebuffer_sizes(cuda_lib, size):
    sc = scenes.small_random_scene(21, size[0], size[1], ntris=150)
    check_against_oracle(sc)


def test_device_mesh_equals_host_mesh(cuda_lib):
    sc = scenes.small_random_scene(5, 128, 96, ntris=300)
    (c0, d0, t0), _ = render_gpu(sc, device_mesh=False)
    (c1, d1, t1), _ = render_gpu(sc, device_mesh=True)
    assert np.array_equal(t0, t1) and np.array_equal(d0.view(np.uint32), d1.view(np.uint32))
    assert np.array_equal(c0, c1)


def test_pinned_host_mesh_reads_attributes_in_place(cuda_lib):
    """Page-locked normals and albedo are read in place by the shading; the
    frame is identical to the one rendered from device memory."""
    sc = scenes.small_random_scene(6, 128, 96, ntris=300)
    outs = []
    for mesh in (R.DeviceMesh.from_mesh(sc.mesh), R.HostMesh(sc.mesh, pinned=True), R.HostMesh(sc.mesh)):
        r = R.Renderer()
        r.Initialize(sc.view.width, sc.view.height)
        R.configure(r, sc.view)
        r.RenderMesh(mesh)
        outs.append([a.copy() for a in r.ReadOutputs()])
        r.close()
    for other in outs[1:]:
        for a, b in zip(outs[0], other):
            assert np.array_equal(a.view(np.uint32), b.view(np.uint32))


def test_empty_mesh(cuda_lib):
    sc = scenes.small_random_scene(1, 40, 30, ntris=4)
    sc.mesh.indices = sc.mesh.indices[:0]
    (color, depth, tid), stats = render_gpu(sc)
    assert np.all(tid == 0xFFFFFFFF) and np.all(depth == 1.0) and np.all(color == 0.0)


def test_repeated_frames_are_identical(cuda_lib):
    sc = scenes.stress_scene(5000, 320, 240, seed=2)
    r = R.Renderer()
    r.Initialize(320, 240)
    R.configure(r, sc.view)
    outs = []
    for _ in range(3):
        r.RenderMesh(sc.mesh)
        outs.append(r.ReadOutputs())
    r.close()
    for o in outs[1:]:
        assert all(np.array_equal(a, b) for a, b in zip(outs[0], o))


def test_back_buffer_is_bottom_up_rgba8(cuda_lib):
    sc = scenes.sphere_scene(64, 48)
    r = R.Renderer()
    r.Initialize(64, 48)
    R.configure(r, sc.view)
    r.RenderMesh(sc.mesh)
    color, _, tid = r.ReadOutputs()
    bb = r.GetBackBuffer()
    r.close()
    expect = (np.clip(color[::-1, :, :3], 0, 1) * 255 + 0.5).astype(np.uint8)
    assert np.array_equal(bb[..., :3], expect)
    assert np.array_equal(bb[..., 3] == 255, (tid != 0xFFFFFFFF)[::-1])


def test_invalid_arguments_raise(cuda_lib):
    r = R.Renderer()
    r.Initialize(32, 32)
    with pytest.raises(R.EdxrError):
        r.RenderMesh(scenes.small_random_scene(0).mesh)  # no transform yet
    sc = scenes.small_random_scene(0, 32, 32)
    R.configure(r, sc.view)
    bad = scenes.Mesh(sc.mesh.positions, sc.mesh.normals, sc.mesh.albedo, sc.mesh.uvs, sc.mesh.indices.copy())
    bad.indices[0, 0] = 10 ** 6
    with pytest.raises(R.EdxrError):
        r.RenderMesh(bad)
    with pytest.raises(R.EdxrError):
        r.SetMSAAMode(6)  # at most 32 samples
    r.RenderMesh(sc.mesh)  # the renderer is still usable
    r.close()
