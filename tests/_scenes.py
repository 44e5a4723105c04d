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
