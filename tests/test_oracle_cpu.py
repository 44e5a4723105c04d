"""The CPU oracle (C restatement) against the reference's own pipeline.

The golden fixtures hold what the reference's Renderer (its Core sources
compiled unmodified against oracle/shim) produced; the oracle must match them
bit for bit: winning triangle, depth buffer, barycentrics.  When the
reference sources are present, further seeded scenes are compared live.
"""
import numpy as np
import pytest

from edxraster_gb300 import scenes
from oracle import pyoracle
import _scenes
from _scenes import deep_clip_scene, golden_names, load_golden, load_golden_ms, mismatch_report


@pytest.mark.parametrize("name", golden_names())
def test_oracle_matches_golden(name):
    sc, hier, exp = load_golden(name)
    o = pyoracle.render_oracle(sc.mesh, sc.view, hierarchical=hier, depth_func=scenes.DEPTH_LEQUAL, threads=2)
    assert not mismatch_report("id", o["id"], exp["id"])
    assert not mismatch_report("depth", o["depth"].view(np.uint32), exp["depth_bits"])
    covered = exp["id"] != 0xFFFFFFFF
    assert np.array_equal(o["lambda0"].view(np.uint32)[covered], exp["lambda0_bits"][covered])
    assert np.array_equal(o["lambda1"].view(np.uint32)[covered], exp["lambda1_bits"][covered])
    assert o["fragments"] == exp["fragments"]


@pytest.mark.parametrize("name", golden_names(msaa=True))
def test_oracle_matches_golden_msaa(name):
    sc, hier, lg, exp = load_golden_ms(name)
    o = pyoracle.render_oracle(sc.mesh, sc.view, hierarchical=hier, depth_func=scenes.DEPTH_LEQUAL, threads=2,
                               msaa_log2=lg)
    for s in range(1 << lg):
        assert not mismatch_report("id[%d]" % s, o["id"][s], exp["id"][s])
        assert not mismatch_report("depth[%d]" % s, o["depth"][s].view(np.uint32), exp["depth_bits"][s])
    assert o["fragments"] == exp["fragments"]


@pytest.mark.parametrize("lg", [1, 2, 3, 4, 5])
def test_oracle_matches_reference_live_msaa(lg):
    if pyoracle.reference_lib() is None:
        pytest.skip("reference sources not available here")
    sc = scenes.stress_scene(1500, 96, 72, seed=20 + lg, max_area=2e3)
    r = pyoracle.render_reference_ms(sc.mesh, sc.view, lg)
    o = pyoracle.render_oracle(sc.mesh, sc.view, depth_func=scenes.DEPTH_LEQUAL, threads=2, with_color=False,
                               msaa_log2=lg)
    assert np.array_equal(o["id"], r["id"])
    assert np.array_equal(o["depth"].view(np.uint32), r["depth"].view(np.uint32))
    assert o["fragments"] == r["fragments"]


@pytest.mark.parametrize("lg,hier", [(2, True), (3, False)])
def test_oracle_matches_reference_live_msaa_clipping(lg, hier):
    if pyoracle.reference_lib() is None:
        pytest.skip("reference sources not available here")
    sc = deep_clip_scene(120, 64, 48, seed=30 + lg)
    r = pyoracle.render_reference_ms(sc.mesh, sc.view, lg, hierarchical=hier)
    o = pyoracle.render_oracle(sc.mesh, sc.view, hierarchical=hier, depth_func=scenes.DEPTH_LEQUAL, threads=2,
                               with_color=False, msaa_log2=lg)
    assert (r["id"] != 0xFFFFFFFF).any()
    assert np.array_equal(o["id"], r["id"])
    assert np.array_equal(o["depth"].view(np.uint32), r["depth"].view(np.uint32))
    assert o["fragments"] == r["fragments"]


@pytest.mark.parametrize("scene,lg", [("stress", 2), ("stress", 4), ("stress", 5), ("terrain", 2)])
def test_oracle_matches_reference_on_msaa_test_scenes(scene, lg):
    """The LEQUAL scenes of the GPU multisample tests (duplicated triangles,
    clipping and split horizon tiles) against the reference's own code."""
    if pyoracle.reference_lib() is None:
        pytest.skip("reference sources not available here")
    if scene == "stress":
        sc = scenes.stress_scene(4000, 160, 120, seed=30 + lg, max_area=3e3, dup_fraction=0.1)
    else:
        sc = scenes.terrain_scene(96, 320, 180, seed=4)
    r = pyoracle.render_reference_ms(sc.mesh, sc.view, lg)
    o = pyoracle.render_oracle(sc.mesh, sc.view, depth_func=scenes.DEPTH_LEQUAL, threads=2, with_color=False,
                               msaa_log2=lg)
    assert np.array_equal(o["id"], r["id"])
    assert np.array_equal(o["depth"].view(np.uint32), r["depth"].view(np.uint32))
    assert o["fragments"] == r["fragments"]


BENCH_SCENES = {
    "terrain": lambda: scenes.terrain_scene(1024, 1920, 1080, seed=1),
    "stress": lambda: scenes.stress_scene(1_000_000, 3840, 2160, seed=7),
}


@pytest.mark.parametrize("workload,lg", [("terrain", 0), ("stress", 0), ("terrain", 2), ("stress", 1)])
def test_oracle_matches_reference_on_benchmark_workloads(workload, lg):
    """The benchmark's workloads at full size (terrain: 2,097,152 triangles at
    1920x1080; stress: 1,000,000 at 3840x2160), single-sample and with the
    sample counts of the GPU full-size multisample test."""
    if pyoracle.reference_lib() is None:
        pytest.skip("reference sources not available here")
    sc = BENCH_SCENES[workload]()
    if lg:
        r = pyoracle.render_reference_ms(sc.mesh, sc.view, lg)
    else:
        r = pyoracle.render_reference(sc.mesh, sc.view)
    o = pyoracle.render_oracle(sc.mesh, sc.view, depth_func=scenes.DEPTH_LEQUAL, with_color=False, msaa_log2=lg)
    assert not mismatch_report("id", o["id"].reshape(-1, sc.view.width), r["id"].reshape(-1, sc.view.width))
    assert np.array_equal(o["depth"].view(np.uint32), r["depth"].view(np.uint32))
    assert o["fragments"] == r["fragments"]


def test_msaa_resolve_arithmetic():
    """The resolved colour of a pixel is the float average of its samples'
    8-bit colours; a pixel whose samples all see one triangle resolves to
    that triangle's 8-bit colour, and its alpha to 1."""
    sc = scenes.sphere_scene(160, 96, slices=12, stacks=9)
    one = pyoracle.render_oracle(sc.mesh, sc.view, threads=2)
    four = pyoracle.render_oracle(sc.mesh, sc.view, threads=2, msaa_log2=2)
    full = (four["id"] == one["id"][None]).all(axis=0) & (one["id"] != 0xFFFFFFFF)
    assert full.sum() > 1000
    q = np.floor(np.clip(one["color"][..., :3].astype(np.float32), 0, 1) * np.float32(255) + np.float32(0.5))
    expect = (q / np.float32(255)).astype(np.float32)
    # the float sum of four equal samples may round in its last bit
    assert np.allclose(four["color"][..., :3][full], expect[full], rtol=0, atol=1e-6)
    assert np.all(four["color"][..., 3][full] == 1.0)
    empty = (four["id"] == 0xFFFFFFFF).all(axis=0)
    assert np.all(four["color"][empty] == 0.0)


def _live_cases():
    yield scenes.small_random_scene(11, 80, 64, ntris=120), True
    yield scenes.small_random_scene(12, 80, 64, ntris=120), False
    yield scenes.small_random_scene(13, 64, 48, ntris=200, clip_heavy=False), True
    yield scenes.stress_scene(3000, 320, 240, seed=3, max_area=5e3), True
    yield scenes.terrain_scene(40, 160, 96, seed=5), True
    yield scenes.sphere_scene(200, 120, slices=12, stacks=9), True
    # triangles crossing several clip planes at once, w < 0 included
    yield deep_clip_scene(300, 96, 72, seed=21), True
    yield deep_clip_scene(40, 96, 72, seed=22), False


@pytest.mark.parametrize("case", range(8))
def test_oracle_matches_reference_live(case):
    if pyoracle.reference_lib() is None:
        pytest.skip("reference sources not available here")
    sc, hier = list(_live_cases())[case]
    r = pyoracle.render_reference(sc.mesh, sc.view, hierarchical=hier)
    o = pyoracle.render_oracle(sc.mesh, sc.view, hierarchical=hier, depth_func=scenes.DEPTH_LEQUAL, threads=2)
    assert not mismatch_report("id", o["id"], r["id"])
    assert not mismatch_report("depth", o["depth"].view(np.uint32), r["depth"].view(np.uint32))
    assert o["fragments"] == r["fragments"]


EDGE_SCENES = {
    "int32_wraparound_4k": lambda: _scenes.wraparound_4k_scene(0),
    "every_clip_plane": _scenes.every_clip_plane_scene,
    "far_plane_and_behind": _scenes.far_and_behind_scene,
    "degenerate_and_non_finite": _scenes.degenerate_scene,
    "coplanar_ties": _scenes.coplanar_scene,
    "occluders": _scenes.occluder_scene,
    "duplicate_triangles": lambda: scenes.stress_scene(6000, 320, 200, seed=7, max_area=3e3, dup_fraction=0.25),
}


@pytest.mark.parametrize("hier", [True, False])
@pytest.mark.parametrize("name", sorted(EDGE_SCENES))
def test_oracle_matches_reference_on_edge_scenes(name, hier):
    """The scenes of the GPU robustness tests, so that the GPU's agreement
    with the oracle there is agreement with the reference's own code."""
    if pyoracle.reference_lib() is None:
        pytest.skip("reference sources not available here")
    sc = EDGE_SCENES[name]()
    r = pyoracle.render_reference(sc.mesh, sc.view, hierarchical=hier)
    o = pyoracle.render_oracle(sc.mesh, sc.view, hierarchical=hier, depth_func=scenes.DEPTH_LEQUAL, threads=2,
                               with_color=False)
    assert (r["id"] != 0xFFFFFFFF).any()
    assert not mismatch_report("id", o["id"], r["id"])
    assert not mismatch_report("depth", o["depth"].view(np.uint32), r["depth"].view(np.uint32))
    assert o["fragments"] == r["fragments"]


def test_less_differs_only_on_ties():
    """LESS keeps the first of equal-depth fragments, LEQUAL the last; the
    stress scene has exact duplicates, so some pixels must differ and every
    differing pixel must carry the same depth."""
    sc = scenes.stress_scene(4000, 200, 160, seed=7, max_area=3e3, dup_fraction=0.2)
    a = pyoracle.render_oracle(sc.mesh, sc.view, depth_func=scenes.DEPTH_LEQUAL, threads=2, with_color=False)
    b = pyoracle.render_oracle(sc.mesh, sc.view, depth_func=scenes.DEPTH_LESS, threads=2, with_color=False)
    diff = a["id"] != b["id"]
    assert diff.any()
    assert np.array_equal(a["depth"][diff], b["depth"][diff])


def test_hierarchical_flag_does_not_change_coverage():
    sc = scenes.stress_scene(2000, 256, 160, seed=9, max_area=1e4)
    a = pyoracle.render_oracle(sc.mesh, sc.view, hierarchical=True, threads=2, with_color=False)
    b = pyoracle.render_oracle(sc.mesh, sc.view, hierarchical=False, threads=2, with_color=False)
    assert np.array_equal(a["id"], b["id"])
    assert np.array_equal(a["depth"].view(np.uint32), b["depth"].view(np.uint32))


def test_oracle_rejects_bad_indices():
    sc = scenes.small_random_scene(1)
    sc.mesh.indices = sc.mesh.indices.copy()
    sc.mesh.indices[3, 1] = sc.mesh.nv + 5
    with pytest.raises(RuntimeError):
        pyoracle.render_oracle(sc.mesh, sc.view, threads=1)


def test_shading_model_fp64_known_values():
    """Head-on Blinn-Phong at one point: N = L = E = +z-facing."""
    v = scenes.View(4, 4, np.eye(4, dtype=np.float32), np.eye(4, dtype=np.float32), np.eye(4, dtype=np.float32),
                    np.array([0, 0, -1], np.float32), 0.5, 32.0)
    b = np.array([1.0, 0.0, 0.0])
    pos = np.zeros((3, 3))
    nrm = np.tile([0.0, 0.0, -1.0], (3, 1))
    alb = np.tile([0.25, 0.5, 1.0], (3, 1))
    eye = np.array([0.0, 0.0, -5.0])
    rgb = pyoracle.shade_fp64(v, b, pos, nrm, alb, eye)
    diffuse = (1.0 + 0.2) * 3.0 / np.pi
    assert np.allclose(rgb, alb[0] * diffuse + 0.5, rtol=0, atol=1e-12)
