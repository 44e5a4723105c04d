"""Multisampling (Renderer::SetMSAAMode, 2 to 32 samples per pixel) through the C ABI.

Per sample, the winning triangle and its depth must be bit-identical to the
reference's multisample path (golden fixtures made from it) and to the C
oracle.  The colour is the reference's resolve of 8-bit sample colours; each
sample colour comes from FP32 shading here and FP64 shading in the oracle,
so a sample may round to the neighbouring byte: the resolved colour is
allowed one byte of difference in a few pixels and must otherwise agree to
1e-6.
"""
import numpy as np
import pytest

from edxraster_gb300 import renderer as R
from edxraster_gb300 import scenes
from oracle import pyoracle
from _scenes import golden_names, load_golden_ms, mismatch_report

pytestmark = pytest.mark.gpu


def render_ms(sc, msaa_log2, hierarchical=True, depth_func=None):
    r = R.Renderer()
    r.Initialize(sc.view.width, sc.view.height)
    R.configure(r, sc.view, hierarchical)
    if depth_func is not None:
        r.SetDepthFunc(depth_func)
    r.SetMSAAMode(msaa_log2)
    r.RenderMesh(sc.mesh)
    color, depth, tid = r.ReadOutputs()
    back = r.GetBackBuffer()
    r.close()
    return color, depth, tid, back


def check_color(color, expect, samples):
    diff = np.abs(color.astype(np.float64) - expect)
    assert diff.max() <= 1.0 / 255.0 + 1e-6, "max resolved colour difference %.3g" % diff.max()
    assert (diff > 1e-6).any(axis=-1).mean() < 0.01


@pytest.mark.parametrize("name", golden_names(msaa=True))
def test_msaa_golden_bit_exact(cuda_lib, name):
    sc, hier, lg, exp = load_golden_ms(name)
    color, depth, tid, _ = render_ms(sc, lg, hier, depth_func=scenes.DEPTH_LEQUAL)
    assert tid.shape == (1 << lg, sc.view.height, sc.view.width)
    for s in range(1 << lg):
        assert not mismatch_report("triangle id[%d]" % s, tid[s], exp["id"][s])
        assert not mismatch_report("depth[%d]" % s, depth[s].view(np.uint32), exp["depth_bits"][s])
    o = pyoracle.render_oracle(sc.mesh, sc.view, hierarchical=hier, depth_func=scenes.DEPTH_LEQUAL, msaa_log2=lg)
    check_color(color, o["color"], 1 << lg)


@pytest.mark.parametrize("lg,depth_func", [(1, scenes.DEPTH_LESS), (2, scenes.DEPTH_LEQUAL), (3, scenes.DEPTH_LESS),
                                           (4, scenes.DEPTH_LEQUAL), (5, scenes.DEPTH_LEQUAL)])
def test_msaa_matches_oracle(cuda_lib, lg, depth_func):
    sc = scenes.stress_scene(4000, 160, 120, seed=30 + lg, max_area=3e3, dup_fraction=0.1)
    color, depth, tid, _ = render_ms(sc, lg, depth_func=depth_func)
    o = pyoracle.render_oracle(sc.mesh, sc.view, depth_func=depth_func, msaa_log2=lg)
    assert np.array_equal(tid, o["id"])
    assert np.array_equal(depth.view(np.uint32), o["depth"].view(np.uint32))
    check_color(color, o["color"], 1 << lg)


def test_msaa_clipping_and_split_tiles(cuda_lib):
    """The terrain clips at the frustum and packs hundreds of bin entries into
    horizon tiles, so tiles are split over several work items."""
    sc = scenes.terrain_scene(96, 320, 180, seed=4)
    color, depth, tid, _ = render_ms(sc, 2)
    o = pyoracle.render_oracle(sc.mesh, sc.view, depth_func=sc.view.depth_func, msaa_log2=2)
    assert np.array_equal(tid, o["id"])
    assert np.array_equal(depth.view(np.uint32), o["depth"].view(np.uint32))
    check_color(color, o["color"], 4)


@pytest.mark.parametrize("workload,lg", [("terrain", 2), ("stress", 1)])
def test_msaa_benchmark_workloads_full_size(cuda_lib, workload, lg):
    """The benchmark's full-size scenes with samples: per-sample winners and
    depths bit-exact (wrap-free triangles binned and rasterized over the
    pixels their box overlaps, tile occluder bounds over samples)."""
    sc = {"terrain": lambda: scenes.terrain_scene(1024, 1920, 1080, seed=1),
          "stress": lambda: scenes.stress_scene(1_000_000, 3840, 2160, seed=7)}[workload]()
    color, depth, tid, _ = render_ms(sc, lg)
    o = pyoracle.render_oracle(sc.mesh, sc.view, depth_func=sc.view.depth_func, msaa_log2=lg)
    assert not mismatch_report("triangle id", tid, o["id"])
    assert not mismatch_report("depth", depth.view(np.uint32), o["depth"].view(np.uint32))
    check_color(color, o["color"], 1 << lg)


def test_msaa_back_buffer_is_the_resolve(cuda_lib):
    sc = scenes.sphere_scene(160, 96)
    color, depth, tid, back = render_ms(sc, 3)
    expect = (np.clip(color[::-1], 0, 1) * np.float32(255) + np.float32(0.5)).astype(np.uint8)
    assert np.array_equal(back, expect)
    # edges are partly covered: some alpha strictly between 0 and 1
    assert ((color[..., 3] > 0) & (color[..., 3] < 1)).any()


def test_msaa_mode_switch(cuda_lib):
    """Switching the sample count re-renders with the new layout; one sample
    is the plain path again."""
    sc = scenes.small_random_scene(4)
    r = R.Renderer()
    r.Initialize(sc.view.width, sc.view.height)
    R.configure(r, sc.view)
    r.SetMSAAMode(2)
    r.RenderMesh(sc.mesh)
    _, d4, t4 = r.ReadOutputs()
    r.SetMSAAMode(0)
    r.RenderMesh(sc.mesh)
    c1, d1, t1 = r.ReadOutputs()
    r.close()
    assert t4.shape[0] == 4 and t1.ndim == 2
    o = pyoracle.render_oracle(sc.mesh, sc.view, depth_func=sc.view.depth_func)
    assert np.array_equal(t1, o["id"])
    r = R.Renderer()
    r.Initialize(8, 8)
    with pytest.raises(R.EdxrError):
        r.SetMSAAMode(6)  # at most 32 samples
    assert r.samples == 1
    r.close()


def test_msaa_unsupported_forms(cuda_lib):
    sc = scenes.small_random_scene(2)
    r = R.Renderer()
    r.Initialize(sc.view.width, sc.view.height)
    R.configure(r, sc.view)
    r.SetMSAAMode(1)
    views = [scenes.View(sc.view.width, sc.view.height, sc.view.mv, sc.view.proj, sc.view.raster, sc.view.light)]
    with pytest.raises(R.EdxrError):
        r.RenderBatched([sc.mesh], views, sc.view.width, sc.view.height)
    r.close()
