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


def clip_space_scene(tris_clip, width, height, seed=0):
    """Triangles given directly in clip space (MVP = identity)."""
    n = len(tris_clip)
    rng = np.random.default_rng(seed)
    pos4 = np.asarray(tris_clip, np.float64).reshape(n * 3, 4)
    # object position (x, y, w) with proj mapping (x, y, w) -> (x, y, z(w), w) is not general enough for
    # arbitrary z, so carry z through the model-view: object (x, y, z) and w fixed by the proj row
    pos = pos4[:, :3].astype(np.float32)
    nrm = rng.normal(size=(n * 3, 3)).astype(np.float32)
    alb = rng.uniform(size=(n * 3, 3)).astype(np.float32)
    mesh = scenes.Mesh(pos, nrm, alb, np.zeros((n * 3, 2), np.float32), np.arange(n * 3, dtype=np.uint32).reshape(n, 3))
    view = scenes.View(width, height, np.eye(4, dtype=np.float32), np.eye(4, dtype=np.float32),
                       scenes.raster_matrix(width, height), np.array([0.3, 0.5, -0.8], np.float32))
    return scenes.Scene("clip", mesh, view)


def wraparound_4k_scene(seed):
    """Screen-sized triangles at 3840x2160: edge functions of the coarse and
    binning corner tests exceed int32 and wrap."""
    rng = np.random.default_rng(seed)
    tris = []
    for _ in range(24):
        xy = rng.uniform(-1.0, 1.0, size=(3, 2))
        z = rng.uniform(0.05, 0.95)
        t = [(x, y, z + rng.uniform(-0.04, 0.04), 1.0) for x, y in xy]
        a = np.cross(np.r_[xy[1] - xy[0], 0], np.r_[xy[2] - xy[0], 0])[2]
        if a > 0:  # clockwise on screen (raster y points down)
            t = [t[0], t[2], t[1]]
        tris.append(t)
    return clip_space_scene(tris, 3840, 2160, seed)


def every_clip_plane_scene():
    """Triangles crossing the side, near (z < 0) and far (z > w) planes."""
    rng = np.random.default_rng(9)
    tris = []
    for _ in range(300):
        c = rng.uniform(-1.6, 1.6, size=2)
        w = rng.uniform(0.2, 3.0)
        pts = []
        for _ in range(3):
            x, y = c + rng.normal(scale=0.5, size=2)
            z = rng.uniform(-0.4, 1.4)  # crosses the near (z < 0) and far (z > w) planes
            pts.append((x * w, y * w, z * w, w))
        tris.append(pts)
    # clip-space input: carry w through the position's z and let the projection
    # produce it: (x, y, z) -> (x, y, z, w) needs w per vertex, so render each
    # triangle's vertices through MVP = identity with w = 1 after scaling
    return clip_space_scene([[(x / w, y / w, z / w, 1.0) for x, y, z, w in t] for t in tris], 200, 160, 9)


def far_and_behind_scene():
    sc = scenes.small_random_scene(41, 120, 90, ntris=250)
    sc.mesh.positions[:, 2] *= 2.5  # beyond the far plane (8) and behind the eye
    return sc


def degenerate_scene():
    sc = scenes.small_random_scene(17, 96, 64, ntris=120, clip_heavy=False)
    p = sc.mesh.positions
    p[3:6] = p[3]            # zero-area triangle
    p[6:9, 0] = p[6, 0]      # collinear in x
    p[12] = np.nan           # NaN vertex
    p[15] = [np.inf, 0, 2]   # infinite vertex
    p[18:21] = [0, 0, 0]     # at the eye
    return sc


def coplanar_scene():
    """Many triangles on one plane: every covered pixel is an exact depth tie."""
    rng = np.random.default_rng(2)
    tris = []
    for _ in range(200):
        c = rng.uniform(-0.9, 0.9, size=2)
        pts = [(c[0] + 0.3 * np.cos(a), c[1] + 0.3 * np.sin(a), 0.5, 1.0) for a in (0.0, -2.1, -4.2)]
        tris.append(pts)
    return clip_space_scene(tris, 256, 192, 2)


def occluder_scene():
    """Screen-covering planes at equal and nearly equal depths, triangles that
    straddle their depth, small ones just in front and just behind."""
    rng = np.random.default_rng(5)
    tris = []
    for k in range(300):
        z = float(rng.choice([0.3, 0.3, 0.5, np.nextafter(np.float32(0.3), np.float32(1.0))]))
        if k % 3 == 0:  # screen-covering quad halves (accepted over whole tiles)
            quad = [(-1.2, -1.2), (1.2, -1.2), (1.2, 1.2), (-1.2, 1.2)]
            t1 = [(x, y, z, 1.0) for x, y in (quad[0], quad[2], quad[1])]
            t2 = [(x, y, z, 1.0) for x, y in (quad[0], quad[3], quad[2])]
            tris += [t1, t2]
        else:
            c = rng.uniform(-0.9, 0.9, size=2)
            xy = c + rng.uniform(-0.3, 0.3, size=(3, 2))
            zs = z + rng.uniform(-0.05, 0.05, size=3) * (k % 2)
            t = [(x, y, float(zz), 1.0) for (x, y), zz in zip(xy, zs)]
            a = np.cross(np.r_[xy[1] - xy[0], 0], np.r_[xy[2] - xy[0], 0])[2]
            if a > 0:  # clockwise on screen (raster y points down)
                t = [t[0], t[2], t[1]]
            tris.append(t)
    return clip_space_scene(tris, 160, 128)
