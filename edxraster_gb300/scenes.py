"""Seeded synthetic scenes for the rasterization pipeline.

Every scene is plain numpy data: float32 positions / normals / albedo / uv,
uint32 triangle indices, and the three row-major 4x4 float32 matrices the
renderer takes (model-view, projection, raster), plus the shading parameters.
Generation is deterministic for a given seed.

Conventions (the ones EDXRaster's viewer camera uses, RealtimeViewer/Main.cpp:39,71):
left-handed view space looking down +z, a D3D-style projection with clip
z in [0, w], and a raster matrix mapping NDC x in [-1, 1] to [0, W] and y in
[-1, 1] to [H, 0].  Front faces are clockwise on screen, which in object space
means cross(v1 - v0, v2 - v0) points towards the viewer; generators orient
closed meshes so that outward normals satisfy this.
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

SHADER_BLINN_PHONG = 0
SHADER_BLINN_PHONG_REFERENCE = 1
SHADER_LAMBERTIAN_ALBEDO = 2
SHADER_LAMBERTIAN = 3
SHADER_LAMBERTIAN_TEXTURED = 4

DEPTH_LEQUAL = 0
DEPTH_LESS = 1


@dataclasses.dataclass
class View:
    width: int
    height: int
    mv: np.ndarray       # (4,4) float32
    proj: np.ndarray     # (4,4) float32
    raster: np.ndarray   # (4,4) float32
    light: np.ndarray    # (3,) float32, direction towards the light
    ks: float = 0.5
    shininess: float = 32.0
    shader: int = SHADER_BLINN_PHONG
    depth_func: int = DEPTH_LESS
    mesh: int = 0        # mesh index, for batched rendering


@dataclasses.dataclass
class Mesh:
    positions: np.ndarray  # (nv,3) float32
    normals: np.ndarray    # (nv,3) float32
    albedo: np.ndarray     # (nv,3) float32
    uvs: np.ndarray        # (nv,2) float32
    indices: np.ndarray    # (nt,3) uint32
    texture_ids: np.ndarray = None  # (nt,) uint32 texture slot per triangle, None = slot 0

    @property
    def nv(self) -> int:
        return int(self.positions.shape[0])

    @property
    def nt(self) -> int:
        return int(self.indices.shape[0])

    def interleaved_pnt(self) -> np.ndarray:
        """Vertex_PositionNormalTex layout (InputBuffer.h:16-28): 8 floats per vertex."""
        return np.ascontiguousarray(
            np.concatenate([self.positions, self.normals, self.uvs], axis=1), dtype=np.float32)


@dataclasses.dataclass
class Scene:
    name: str
    mesh: Mesh
    view: View


# --------------------------------------------------------------------------
# matrices

def look_at_lh(eye, target, up) -> np.ndarray:
    eye = np.asarray(eye, np.float64)
    z = np.asarray(target, np.float64) - eye
    z /= np.linalg.norm(z)
    x = np.cross(np.asarray(up, np.float64), z)
    x /= np.linalg.norm(x)
    y = np.cross(z, x)
    m = np.eye(4)
    m[0, :3], m[1, :3], m[2, :3] = x, y, z
    m[0, 3], m[1, 3], m[2, 3] = -x @ eye, -y @ eye, -z @ eye
    return m.astype(np.float32)


def perspective_lh(fovy_deg: float, aspect: float, near: float, far: float) -> np.ndarray:
    ys = 1.0 / math.tan(math.radians(fovy_deg) * 0.5)
    xs = ys / aspect
    m = np.zeros((4, 4))
    m[0, 0], m[1, 1] = xs, ys
    m[2, 2] = far / (far - near)
    m[2, 3] = -near * far / (far - near)
    m[3, 2] = 1.0
    return m.astype(np.float32)


def raster_matrix(width: int, height: int) -> np.ndarray:
    m = np.eye(4)
    m[0, 0], m[0, 3] = width * 0.5, width * 0.5
    m[1, 1], m[1, 3] = -height * 0.5, height * 0.5
    return m.astype(np.float32)


def _unit(v) -> np.ndarray:
    v = np.asarray(v, np.float64)
    return (v / np.linalg.norm(v)).astype(np.float32)


def _seeded_light(rng: np.random.Generator) -> np.ndarray:
    # a direction on the viewer's side of the scene (z < 0 in view space for
    # the default cameras), so lit surfaces face the camera
    while True:
        v = rng.normal(size=3)
        n = np.linalg.norm(v)
        if n > 1e-3:
            v = v / n
            v[2] = -abs(v[2])
            return v.astype(np.float32)


def _orient_outward(pos: np.ndarray, idx: np.ndarray, outward: np.ndarray) -> np.ndarray:
    """Swap v1/v2 where cross(v1-v0, v2-v0) points against `outward`."""
    p = pos.astype(np.float64)
    a, b, c = p[idx[:, 0]], p[idx[:, 1]], p[idx[:, 2]]
    n = np.cross(b - a, c - a)
    flip = np.einsum("ij,ij->i", n, outward) < 0
    idx = idx.copy()
    idx[flip, 1], idx[flip, 2] = idx[flip, 2].copy(), idx[flip, 1].copy()
    return idx


# --------------------------------------------------------------------------
# meshes

def uv_sphere(slices: int, stacks: int, radius: float = 1.0, center=(0, 0, 0)) -> Mesh:
    """Sphere with `slices` longitude segments and `stacks` latitude bands, fan caps.

    Triangles: 2*slices*(stacks-1); vertices: slices*(stacks-1) + 2.
    """
    center = np.asarray(center, np.float64)
    J, I = np.meshgrid(np.arange(1, stacks), np.arange(slices), indexing="ij")
    th = np.pi * J / stacks
    ph = 2.0 * np.pi * I / slices
    ring_n = np.stack([np.sin(th) * np.cos(ph), np.cos(th), np.sin(th) * np.sin(ph)], -1).reshape(-1, 3)
    ring_uv = np.stack([I / slices, J / stacks], -1).reshape(-1, 2)
    nrm = np.concatenate([[[0.0, 1.0, 0.0]], ring_n, [[0.0, -1.0, 0.0]]], 0)
    uvs = np.concatenate([[[0.5, 0.0]], ring_uv, [[0.5, 1.0]]], 0)
    pos = center + radius * nrm
    north, south = 0, len(nrm) - 1

    def ring(j, i):
        return 1 + (j - 1) * slices + (i % slices)

    i = np.arange(slices)
    cap_n = np.stack([np.full(slices, north), ring(1, i), ring(1, i + 1)], -1)
    jj, ii = np.meshgrid(np.arange(1, stacks - 1), np.arange(slices), indexing="ij")
    a, b = ring(jj, ii), ring(jj, ii + 1)
    c, d = ring(jj + 1, ii), ring(jj + 1, ii + 1)
    band = np.stack([np.stack([a, c, b], -1), np.stack([b, c, d], -1)], 2).reshape(-1, 3)
    cap_s = np.stack([np.full(slices, south), ring(stacks - 1, i + 1), ring(stacks - 1, i)], -1)
    idx = np.concatenate([cap_n, band, cap_s], 0).astype(np.int64)
    cent = pos[idx].mean(axis=1) - center
    idx = _orient_outward(pos, idx, cent).astype(np.uint32)
    return Mesh(pos.astype(np.float32), nrm.astype(np.float32),
                np.ones((len(pos), 3), np.float32), np.asarray(uvs, np.float32), idx)


def torus(nu: int, nv: int, R: float = 1.0, r: float = 0.35, center=(0, 0, 0)) -> Mesh:
    """Torus around the y axis: nu segments around the ring, nv around the tube; 2*nu*nv triangles."""
    center = np.asarray(center, np.float64)
    u = 2.0 * np.pi * np.arange(nu) / nu
    v = 2.0 * np.pi * np.arange(nv) / nv
    U, V = np.meshgrid(u, v, indexing="ij")
    cx, cz = np.cos(U), np.sin(U)
    nrm = np.stack([cx * np.cos(V), np.sin(V), cz * np.cos(V)], axis=-1).reshape(-1, 3)
    ring = np.stack([cx * R, np.zeros_like(U), cz * R], axis=-1).reshape(-1, 3)
    pos = center + ring + r * nrm
    uv = np.stack([U / (2 * np.pi), V / (2 * np.pi)], axis=-1).reshape(-1, 2)
    ii, jj = np.meshgrid(np.arange(nu), np.arange(nv), indexing="ij")
    a = ii * nv + jj
    b = ((ii + 1) % nu) * nv + jj
    c = ii * nv + (jj + 1) % nv
    d = ((ii + 1) % nu) * nv + (jj + 1) % nv
    idx = np.concatenate([np.stack([a, b, c], -1).reshape(-1, 3),
                          np.stack([b, d, c], -1).reshape(-1, 3)], axis=0)
    p = pos
    cent = p[idx].mean(axis=1)
    out = cent - (center + np.stack([cent[:, 0] - center[0], np.zeros(len(cent)), cent[:, 2] - center[2]], -1)
                  / np.maximum(np.linalg.norm(np.stack([cent[:, 0] - center[0], cent[:, 2] - center[2]], -1),
                                              axis=1, keepdims=True), 1e-12) * R)
    out[:, 1] = cent[:, 1] - center[1]
    idx = _orient_outward(pos, idx, out).astype(np.uint32)
    return Mesh(pos.astype(np.float32), nrm.astype(np.float32),
                np.ones((len(pos), 3), np.float32), uv.astype(np.float32), idx)


def test_textures(seed: int = 0):
    """Three texture slots: an 8-bit 64x64 checkerboard with noise, a float
    48x20 gradient (non-square, odd mip chain) and a 1x1 constant colour (the
    reference's ConstantTexture2D)."""
    rng = np.random.default_rng(seed)
    y, x = np.mgrid[0:64, 0:64]
    check = (((x // 8) + (y // 8)) % 2).astype(np.float64)
    rgba8 = np.stack([200 * check + 40, 120 + 80 * (1 - check), rng.integers(0, 256, (64, 64)),
                      np.full((64, 64), 255)], -1).astype(np.uint8)
    gy, gx = np.mgrid[0:20, 0:48]
    grad = np.stack([gx / 47.0, gy / 19.0, 0.5 + 0.5 * np.sin(gx * 0.7), np.ones_like(gx, dtype=np.float64)],
                    -1).astype(np.float32)
    const = np.array([[[0.9, 0.6, 0.3, 1.0]]], np.float32)
    return [rgba8, grad, const]


def textured_scene(width=320, height=180, seed=0) -> Scene:
    """A textured sphere and a ground plane seen at a grazing angle (strongly
    anisotropic texture footprints), texture coordinates repeating several
    times; triangles cycle through the slots of test_textures()."""
    sph = uv_sphere(24, 16, 1.0, center=(0.0, 0.2, 0.0))
    sph.uvs = (sph.uvs * np.array([4.0, 2.0], np.float32)).astype(np.float32)
    n = 24
    gx, gz = np.meshgrid(np.linspace(-6.0, 6.0, n + 1), np.linspace(-2.0, 14.0, n + 1), indexing="xy")
    gpos = np.stack([gx, np.full_like(gx, -1.0), gz], -1).reshape(-1, 3)
    guv = np.stack([gx * 0.75, gz * 0.75], -1).reshape(-1, 2)
    a = (np.arange(n)[None, :] + (n + 1) * np.arange(n)[:, None]).ravel()
    quads = np.stack([a, a + n + 1, a + 1, a + 1, a + n + 1, a + n + 2], -1).reshape(-1, 3)
    g = Mesh(gpos.astype(np.float32), np.tile([[0.0, 1.0, 0.0]], (len(gpos), 1)).astype(np.float32),
             np.ones((len(gpos), 3), np.float32), guv.astype(np.float32), quads.astype(np.uint32))
    cent = g.positions[g.indices].mean(axis=1)
    g.indices = _orient_outward(g.positions, g.indices.astype(np.int64), np.tile([0.0, 1.0, 0.0], (len(cent), 1))
                                ).astype(np.uint32)
    off = sph.nv
    mesh = Mesh(np.concatenate([sph.positions, g.positions]), np.concatenate([sph.normals, g.normals]),
                np.ones((sph.nv + g.nv, 3), np.float32), np.concatenate([sph.uvs, g.uvs]),
                np.concatenate([sph.indices, g.indices + off]).astype(np.uint32))
    mesh.texture_ids = (np.arange(mesh.nt) % 3).astype(np.uint32)
    mesh.texture_ids[sph.nt:] = 0
    view = View(width, height,
                look_at_lh((0.0, 0.6, -3.2), (0.0, -0.2, 2.0), (0, 1, 0)),
                perspective_lh(60.0, width / height, 0.1, 100.0),
                raster_matrix(width, height),
                np.array([0.3, 1.0, -0.4], np.float32), 0.0, 1.0, SHADER_LAMBERTIAN_TEXTURED, DEPTH_LEQUAL)
    return Scene("textured", mesh, view)


# --------------------------------------------------------------------------
# the benchmark scenes

def sphere_scene(width=1280, height=720, seed=0, slices=32, stacks=64) -> Scene:
    """UV sphere, 32x64 segments (4,032 triangles), camera at distance 3, FOV 60."""
    rng = np.random.default_rng(seed)
    mesh = uv_sphere(slices, stacks, 1.0)
    mesh.albedo = rng.uniform(0.0, 1.0, size=(mesh.nv, 3)).astype(np.float32)
    view = View(width, height,
                look_at_lh((0.0, 0.0, -3.0), (0, 0, 0), (0, 1, 0)),
                perspective_lh(60.0, width / height, 0.1, 100.0),
                raster_matrix(width, height), _seeded_light(rng))
    return Scene("sphere", mesh, view)


def _height(x, z, octaves):
    h = np.zeros_like(x)
    dhx = np.zeros_like(x)
    dhz = np.zeros_like(x)
    for (amp, kx, kz, ph) in octaves:
        arg = kx * x + kz * z + ph
        h += amp * np.sin(arg)
        dhx += amp * kx * np.cos(arg)
        dhz += amp * kz * np.cos(arg)
    return h, dhx, dhz


def terrain_scene(quads=1024, width=1920, height=1080, seed=1, extent=40.0) -> Scene:
    """Heightfield of quads x quads cells (2*quads^2 triangles), low camera."""
    rng = np.random.default_rng(seed)
    octaves = []
    for o in range(4):
        ang = rng.uniform(0, 2 * np.pi)
        freq = 0.25 * (2.1 ** o)
        octaves.append((1.6 / (2.0 ** o), freq * math.cos(ang), freq * math.sin(ang), rng.uniform(0, 2 * np.pi)))
    n = quads + 1
    g = np.linspace(-extent / 2, extent / 2, n)
    X, Z = np.meshgrid(g, g, indexing="xy")
    H, dx, dz = _height(X, Z, octaves)
    H = H + rng.uniform(-0.02, 0.02, size=H.shape)
    pos = np.stack([X, H, Z], -1).reshape(-1, 3)
    nrm = np.stack([-dx, np.ones_like(dx), -dz], -1).reshape(-1, 3)
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    ii, jj = np.meshgrid(np.arange(quads), np.arange(quads), indexing="ij")
    a = ii * n + jj
    b = a + 1
    c = a + n
    d = c + 1
    idx = np.concatenate([np.stack([a, c, b], -1).reshape(-1, 3),
                          np.stack([b, c, d], -1).reshape(-1, 3)], 0)
    up = np.zeros((len(idx), 3)); up[:, 1] = 1.0
    idx = _orient_outward(pos, idx, up).astype(np.uint32)
    uv = np.stack([(X + extent / 2) / extent, (Z + extent / 2) / extent], -1).reshape(-1, 2)
    albedo = rng.uniform(0.2, 1.0, size=(len(pos), 3))
    mesh = Mesh(pos.astype(np.float32), nrm.astype(np.float32), albedo.astype(np.float32),
                uv.astype(np.float32), idx)
    # camera low over the terrain near one edge, looking across it
    ex, ez = -extent * 0.30, -extent * 0.30
    eh, _, _ = _height(np.array(ex), np.array(ez), octaves)
    eye = (ex, float(eh) + 0.35, ez)
    target = (extent * 0.25, float(eh) - 0.6, extent * 0.25)
    view = View(width, height, look_at_lh(eye, target, (0, 1, 0)),
                perspective_lh(60.0, width / height, 0.1, 100.0),
                raster_matrix(width, height), _seeded_light(rng))
    view.light[1] = abs(view.light[1]) + 0.3
    view.light = _unit(view.light)
    return Scene("terrain", mesh, view)


# clip-space mapping used by the binning-stress scene: object (x, y, w) ->
# clip (x, y, A*w + B, w), so NDC depth = A + B/w runs from -0.05 at w=0.5
# (slightly in front of the near plane) to 1.0 at w=4.
STRESS_A = 1.15
STRESS_B = -0.6


def stress_scene(ntris=1_000_000, width=3840, height=2160, seed=7, dup_fraction=0.02,
                 backface_fraction=0.05, min_area=0.1, max_area=1e4) -> Scene:
    """Independent triangles in clip space; log-uniform screen areas; exact duplicates."""
    rng = np.random.default_rng(seed)
    n = ntris
    area = np.exp(rng.uniform(math.log(min_area), math.log(max_area), size=n))
    rad = np.sqrt(4.0 * area / (3.0 * math.sqrt(3.0)))
    cx = rng.uniform(-1.5, 1.5, size=n)
    cy = rng.uniform(-1.5, 1.5, size=n)
    w = rng.uniform(0.5, 4.0, size=n)
    th0 = rng.uniform(0, 2 * np.pi, size=n)
    jit = rng.uniform(-0.3, 0.3, size=(n, 3))
    ang = th0[:, None] + np.array([0.0, 2 * np.pi / 3, 4 * np.pi / 3])[None, :] + jit
    # raster-space vertices (y down); increasing angle is clockwise on screen
    rx = (cx[:, None] + 1.0) * 0.5 * width + rad[:, None] * np.cos(ang)
    ry = (1.0 - cy[:, None]) * 0.5 * height + rad[:, None] * np.sin(ang)
    back = rng.uniform(size=n) < backface_fraction
    rx[back] = rx[back][:, ::-1]
    ry[back] = ry[back][:, ::-1]
    ndx = rx / width * 2.0 - 1.0
    ndy = 1.0 - ry / height * 2.0
    wv = w[:, None] * (1.0 + rng.uniform(-0.02, 0.02, size=(n, 3)))
    pos = np.stack([ndx * wv, ndy * wv, wv], -1)  # (n,3,3) object = (x_clip, y_clip, w)
    nrm = rng.normal(size=(n, 3, 3))
    nrm /= np.linalg.norm(nrm, axis=-1, keepdims=True)
    nrm[..., 2] = -np.abs(nrm[..., 2])
    alb = rng.uniform(0.0, 1.0, size=(n, 3, 3))
    # exact duplicates of a recent earlier triangle: identical depth at every
    # shared pixel, so only submission order decides the winner
    dup = np.nonzero(rng.uniform(size=n) < dup_fraction)[0]
    dup = dup[dup > 8]
    src = dup - 1 - rng.integers(0, 8, size=len(dup))
    pos[dup] = pos[src]
    nrm[dup] = nrm[src]
    mesh = Mesh(pos.reshape(-1, 3).astype(np.float32), nrm.reshape(-1, 3).astype(np.float32),
                alb.reshape(-1, 3).astype(np.float32), np.zeros((3 * n, 2), np.float32),
                np.arange(3 * n, dtype=np.uint32).reshape(n, 3))
    proj = np.array([[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, STRESS_A, STRESS_B], [0, 0, 1, 0]], np.float32)
    view = View(width, height, np.eye(4, dtype=np.float32), proj, raster_matrix(width, height),
                _seeded_light(rng))
    return Scene("stress", mesh, view)


def orbit_views(n_views: int, width: int, height: int, seed: int, distance=3.2, fov=55.0,
                ks=0.5, shininess=32.0):
    rng = np.random.default_rng(seed)
    views = []
    for _ in range(n_views):
        az = rng.uniform(0, 2 * np.pi)
        el = rng.uniform(-0.6, 0.9)
        eye = (distance * math.cos(el) * math.sin(az), distance * math.sin(el), -distance * math.cos(el) * math.cos(az))
        mv = look_at_lh(eye, (0, 0, 0), (0, 1, 0))
        light_view = _seeded_light(rng)
        # express the light in object space so it faces the camera side
        R = mv[:3, :3].astype(np.float64)
        light = _unit(R.T @ light_view.astype(np.float64))
        views.append(View(width, height, mv, perspective_lh(fov, width / height, 0.1, 100.0),
                          raster_matrix(width, height), light, ks, shininess))
    return views


def batched_meshes(n_meshes=256, min_tris=500, max_tris=200_000, seed=11):
    """Spheres and tori with log-uniform triangle counts."""
    rng = np.random.default_rng(seed)
    meshes = []
    for m in range(n_meshes):
        target = math.exp(rng.uniform(math.log(min_tris), math.log(max_tris)))
        if m % 2 == 0:
            slices = max(3, int(round(math.sqrt(target / 4.0))))
            stacks = max(2, int(round(target / (2 * slices))) + 1)
            mesh = uv_sphere(slices, stacks, 1.0)
        else:
            nu = max(3, int(round(math.sqrt(target / 2.0 * 2.5))))
            nv = max(3, int(round(target / (2 * nu))))
            mesh = torus(nu, nv, 1.0, 0.35)
        mesh.albedo = rng.uniform(0.0, 1.0, size=(mesh.nv, 3)).astype(np.float32)
        meshes.append(mesh)
    return meshes


def diff_torus(seed=13) -> Mesh:
    """Torus of 250 x 100 x 2 = 50,000 triangles with seeded albedo."""
    rng = np.random.default_rng(seed)
    mesh = torus(250, 100, 1.0, 0.35)
    mesh.albedo = rng.uniform(0.1, 0.9, size=(mesh.nv, 3)).astype(np.float32)
    return mesh


def small_random_scene(seed: int, width=64, height=64, ntris=48, clip_heavy=True) -> Scene:
    """Tiny scene for debugging-sized parity cases: random triangles around the
    frustum, some crossing every clip plane, some back-facing, some huge."""
    rng = np.random.default_rng(seed)
    n = ntris
    pos = rng.uniform(-2.5 if clip_heavy else -1.0, 2.5 if clip_heavy else 1.0, size=(n, 3, 3))
    pos[..., 2] = rng.uniform(-1.5 if clip_heavy else 1.0, 6.0, size=(n, 3))
    nrm = rng.normal(size=(n, 3, 3))
    nrm /= np.linalg.norm(nrm, axis=-1, keepdims=True)
    alb = rng.uniform(size=(n, 3, 3))
    mesh = Mesh(pos.reshape(-1, 3).astype(np.float32), nrm.reshape(-1, 3).astype(np.float32),
                alb.reshape(-1, 3).astype(np.float32), rng.uniform(size=(3 * n, 2)).astype(np.float32),
                np.arange(3 * n, dtype=np.uint32).reshape(n, 3))
    view = View(width, height, look_at_lh((0, 0, -1.0), (0, 0, 1.0), (0, 1, 0)),
                perspective_lh(70.0, width / height, 0.5, 8.0), raster_matrix(width, height),
                _seeded_light(rng))
    return Scene(f"random{seed}", mesh, view)
