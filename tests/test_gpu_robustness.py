"""Targeted GPU parity cases: capacity overflow and recovery, int32 edge
wraparound at 4K, every clip plane, degenerate and non-finite vertices,
empty views.  Each is checked bit for bit against the C oracle."""
import numpy as np
import pytest

from edxraster_gb300 import renderer as R
from edxraster_gb300 import scenes
from oracle import pyoracle
from _scenes import (coplanar_scene, degenerate_scene, every_clip_plane_scene, far_and_behind_scene,
                     mismatch_report, occluder_scene, wraparound_4k_scene)

pytestmark = pytest.mark.gpu


def gpu(sc, hierarchical=True):
    r = R.Renderer()
    r.Initialize(sc.view.width, sc.view.height)
    R.configure(r, sc.view, hierarchical)
    r.RenderMesh(sc.mesh)
    out = r.ReadOutputs()
    st = r.Stats()
    r.close()
    return out, st


def assert_parity(sc, hierarchical=True, color=True):
    (c, d, t), st = gpu(sc, hierarchical)
    o = pyoracle.render_oracle(sc.mesh, sc.view, hierarchical=hierarchical)
    assert not mismatch_report("triangle id", t, o["id"])
    assert not mismatch_report("depth", d.view(np.uint32), o["depth"].view(np.uint32))
    if color:
        cov = t != 0xFFFFFFFF
        if cov.any():
            assert float(np.nanmax(np.abs(c[cov, :3] - o["color"][cov, :3]))) <= 1e-5
    return st


def test_overflow_recovery(cuda_lib, monkeypatch):
    monkeypatch.setenv("EDXR_DEBUG_CAPACITY", "16")
    sc = scenes.stress_scene(3000, 320, 240, seed=4, max_area=4e3)
    st = assert_parity(sc)
    assert st.rerenders >= 1


def test_overflow_recovery_with_clipping(cuda_lib, monkeypatch):
    monkeypatch.setenv("EDXR_DEBUG_CAPACITY", "8")
    st = assert_parity(scenes.small_random_scene(31, 128, 96, ntris=400))
    assert st.rerenders >= 1


@pytest.mark.parametrize("seed", [31, 32, 33])
def test_overflow_recovery_dense_tiles(cuda_lib, monkeypatch, seed):
    """Tiny capacities on a scene with over 256 entries per tile (tiles
    rasterized as several work items): the passes that overflow drop bin
    entries and triangles, and must leave nothing behind (no bin read with
    missing entries, no partial merge state) for the pass that renders the
    frame in full."""
    monkeypatch.setenv("EDXR_DEBUG_CAPACITY", "8")
    st = assert_parity(scenes.small_random_scene(seed, 128, 96, ntris=1600))
    assert st.rerenders >= 1


@pytest.mark.parametrize("depth_func", [R.DEPTH_LEQUAL, R.DEPTH_LESS])
def test_occluders_cull_only_hidden_entries(cuda_lib, depth_func):
    """Tiles covered whole by a triangle skip the entries beyond its far
    depth.  Planes at equal and nearly equal depths (ties decided by
    submission order), triangles that straddle the occluder's depth, small
    ones in front of and just behind it: all winners as the oracle's."""
    sc = occluder_scene()
    sc.view.depth_func = depth_func
    (c, d, t), _ = gpu(sc)
    o = pyoracle.render_oracle(sc.mesh, sc.view, depth_func=depth_func)
    assert not mismatch_report("triangle id", t, o["id"])
    assert not mismatch_report("depth", d.view(np.uint32), o["depth"].view(np.uint32))


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_int32_wraparound_at_4k(cuda_lib, seed):
    """Screen-sized triangles at 3840x2160: edge functions of the coarse and
    binning corner tests exceed int32 and wrap, as in the reference."""
    sc = wraparound_4k_scene(seed)
    assert_parity(sc)
    assert_parity(sc, hierarchical=False, color=False)


def test_every_clip_plane(cuda_lib):
    sc = every_clip_plane_scene()
    assert_parity(sc)


def test_far_plane_and_behind_camera(cuda_lib):
    sc = far_and_behind_scene()
    assert_parity(sc)


def test_degenerate_and_non_finite_vertices(cuda_lib):
    sc = degenerate_scene()
    assert_parity(sc, color=False)


def test_depth_funcs_on_coplanar_layers(cuda_lib):
    """Many triangles on the same plane: every covered pixel is an exact depth
    tie, decided by submission order alone."""
    sc = coplanar_scene()
    for f in (scenes.DEPTH_LEQUAL, scenes.DEPTH_LESS):
        sc.view.depth_func = f
        assert_parity(sc)


def test_scan_wait_runs_out_and_renderer_recovers(cuda_lib):
    """The tile-count scan's bounded wait: a scan block that never publishes
    its sum (edxr_debug_scan_stall) makes the next block give up after a short
    spin limit.  The frame fails with EDXR_ERR_TIMEOUT instead of hanging, the
    kernels after the scan do nothing, and the next frame on the same renderer
    is exact.  (The reference's binning has neither a wait nor a check,
    Tile.h:34.)"""
    from edxraster_gb300 import _lib
    sc = scenes.terrain_scene(96, 640, 480, seed=3)  # 40 x 30 = 1,200 tiles: two scan blocks
    r = R.Renderer()
    r.Initialize(sc.view.width, sc.view.height)
    R.configure(r, sc.view)
    dm = R.DeviceMesh.from_mesh(sc.mesh)
    _lib.check(r._lib.edxr_debug_scan_stall(r._h, 0, 4096))
    with pytest.raises(_lib.EdxrError) as err:
        r.RenderMesh(dm)
    assert err.value.status == 3  # EDXR_ERR_TIMEOUT
    _lib.check(r._lib.edxr_debug_scan_stall(r._h, -1, 0))
    r.RenderMesh(dm)
    c, d, t = r.ReadOutputs()
    r.close()
    o = pyoracle.render_oracle(sc.mesh, sc.view)
    assert not mismatch_report("triangle id", t, o["id"])
    assert not mismatch_report("depth", d.view(np.uint32), o["depth"].view(np.uint32))
    cov = t != 0xFFFFFFFF
    assert cov.any() and float(np.abs(c[cov, :3] - o["color"][cov, :3]).max()) <= 1e-5
