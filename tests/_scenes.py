"""Shared helpers of the test suite: fixtures as scenes, and comparisons."""
import glob
import os

import numpy as np

from edxraster_gb300 import scenes

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def golden_names(msaa=False):
    """Single-sample fixtures, or the MSAA ones (names starting with msaa)."""
    names = sorted(os.path.splitext(os.path.basename(p))[0] for p in glob.glob(os.path.join(GOLDEN, "*.npz")))
    return [n for n in names if n.startswith("msaa") == msaa]


def load_golden_ms(name):
    """An MSAA fixture: scene, hierarchical flag, log2 of the sample count and
    the per-sample expectations, (samples, H, W)."""
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    mesh = scenes.Mesh(z["positions"], z["normals"], z["albedo"], z["uvs"], z["indices"])
    view = scenes.View(int(z["width"]), int(z["height"]), z["mv"], z["proj"], z["raster"], z["light"],
                       float(z["ks"]), float(z["shininess"]), scenes.SHADER_BLINN_PHONG, scenes.DEPTH_LEQUAL)
    expect = {"id": z["id"], "depth_bits": z["depth_bits"], "fragments": int(z["fragments"])}
    return scenes.Scene(name, mesh, view), bool(z["hierarchical"]), int(z["msaa_log2"]), expect


def load_golden(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    mesh = scenes.Mesh(z["positions"], z["normals"], z["albedo"], z["uvs"], z["indices"])
    view = scenes.View(int(z["width"]), int(z["height"]), z["mv"], z["proj"], z["raster"], z["light"],
                       float(z["ks"]), float(z["shininess"]), scenes.SHADER_BLINN_PHONG, scenes.DEPTH_LEQUAL)
    expect = {"id": z["id"], "depth_bits": z["depth_bits"], "lambda0_bits": z["lambda0_bits"],
              "lambda1_bits": z["lambda1_bits"], "fragments": int(z["fragments"])}
    return scenes.Scene(name, mesh, view), bool(z["hierarchical"]), expect


def mismatch_report(name, a, b):
    bad = np.argwhere(a != b)
    if len(bad) == 0:
        return ""
    y, x = bad[0][:2]
    return "%s: %d mismatching pixels, first at (x=%d, y=%d): %r vs %r" % (name, len(bad), x, y, a[y, x], b[y, x])


def deep_clip_scene(n, width, height, seed):
    """Large clip-space triangles that cross several clip planes at once
    (sides, near, far, w < 0): clipped polygons of up to nine vertices."""
    rng = np.random.default_rng(seed)
    xy = rng.uniform(-8.0, 8.0, size=(n, 3, 2))
    w = rng.uniform(-1.0, 6.0, size=(n, 3, 1))
    pos = np.concatenate([xy, w], -1).reshape(-1, 3).astype(np.float32)  # object = (x_clip, y_clip, w)
    nrm = rng.normal(size=(3 * n, 3))
    nrm /= np.linalg.norm(nrm, axis=-1, keepdims=True)
    alb = rng.uniform(0.0, 1.0, size=(3 * n, 3))
    mesh = scenes.Mesh(pos, nrm.astype(np.float32), alb.astype(np.float32), np.zeros((3 * n, 2), np.float32),
                       np.arange(3 * n, dtype=np.uint32).reshape(n, 3))
    proj = np.array([[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, scenes.STRESS_A, scenes.STRESS_B], [0, 0, 1, 0]],
                    np.float32)
    view = scenes.View(width, height, np.eye(4, dtype=np.float32), proj, scenes.raster_matrix(width, height),
                       np.array([0.3, 0.5, -0.81], np.float32) / np.linalg.norm([0.3, 0.5, -0.81]))
    return scenes.Scene("deep_clip", mesh, view)
