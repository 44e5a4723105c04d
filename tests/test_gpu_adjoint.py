"""Differentiable form: the hand-written adjoint (edxr_backward) against an
FP64 CPU autograd reference and against central finite differences of the GPU
forward (edxr_shade_visible), visibility held fixed.  The GPU pair is wrapped
in a torch.autograd.Function here, in the test harness only."""
import ctypes

import numpy as np
import pytest

from edxraster_gb300 import _lib
from edxraster_gb300 import renderer as R
from edxraster_gb300 import scenes

pytestmark = pytest.mark.gpu
REL_TOL = 1e-4          # gradient vs the FP64 reference, relative L2 error per parameter group
FD_H = 1e-3


def setup(nviews=4, size=96, shader=0):
    import torch
    mesh = scenes.torus(40, 16, 1.0, 0.35)
    rng = np.random.default_rng(3)
    mesh.albedo = rng.uniform(0.1, 0.9, size=(mesh.nv, 3)).astype(np.float32)
    views = scenes.orbit_views(nviews, size, size, seed=21)
    for v in views:
        v.shader = shader
        v.ks, v.shininess = 0.5, 32.0
    light = views[0].light.copy()
    r = R.Renderer()
    r.Initialize(size, size)
    dm = R.DeviceMesh.from_mesh(mesh)
    r.RenderBatched([dm], views, size, size)
    _, _, ids = r.ReadBatchOutputs(0, nviews, size, size)
    gen = torch.Generator(device="cuda").manual_seed(5)
    grad = torch.randn((nviews, size, size, 4), dtype=torch.float32, device="cuda", generator=gen)
    return mesh, views, light, r, dm, ids, grad


def params(light, ks, shin):
    return _lib.ShaderParams((ctypes.c_float * 3)(*[float(x) for x in light]), float(ks), float(shin))


class ShadeVisible:
    """torch.autograd.Function over edxr_shade_visible / edxr_backward."""

    @staticmethod
    def make(r, nviews, size):
        import torch

        class Fn(torch.autograd.Function):
            @staticmethod
            def forward(ctx, positions, normals, albedo, light, ks, shininess, indices):
                ctx.save_for_backward(positions, normals, albedo, light, ks, shininess, indices)
                dm = R.DeviceMesh(positions, indices, normals, albedo)
                out = torch.empty((nviews, size, size, 4), dtype=torch.float32, device="cuda")
                p = params(light.tolist(), ks.item(), shininess.item())
                _lib.check(r._lib.edxr_shade_visible(r._h, ctypes.byref(dm.abi()), ctypes.byref(p), out.data_ptr()))
                return out

            @staticmethod
            def backward(ctx, gout):
                positions, normals, albedo, light, ks, shininess, indices = ctx.saved_tensors
                dm = R.DeviceMesh(positions, indices, normals, albedo)
                g = [torch.zeros_like(positions), torch.zeros_like(normals), torch.zeros_like(albedo),
                     torch.zeros(3, device="cuda"), torch.zeros(1, device="cuda"), torch.zeros(1, device="cuda")]
                grads = _lib.Grads(g[2].data_ptr(), g[1].data_ptr(), g[0].data_ptr(), g[3].data_ptr(),
                                   g[4].data_ptr(), g[5].data_ptr())
                p = params(light.tolist(), ks.item(), shininess.item())
                gc = gout.contiguous()
                _lib.check(r._lib.edxr_backward(r._h, ctypes.byref(dm.abi()), ctypes.byref(p), gc.data_ptr(),
                                                ctypes.byref(grads)))
                torch.cuda.synchronize()
                return g[0], g[1], g[2], g[3].cpu(), g[4].reshape(()).cpu(), g[5].reshape(()).cpu(), None

        return Fn


def gpu_grads(mesh, views, light, r, dm, grad):
    import torch
    size, nviews = views[0].width, len(views)
    Fn = ShadeVisible.make(r, nviews, size)
    pos = dm.positions.clone().requires_grad_(True)
    nrm = dm.normals.clone().requires_grad_(True)
    alb = dm.albedo.clone().requires_grad_(True)
    lt = torch.tensor(light, dtype=torch.float32, requires_grad=True)
    ks = torch.tensor(views[0].ks, requires_grad=True)
    sh = torch.tensor(views[0].shininess, requires_grad=True)
    col = Fn.apply(pos, nrm, alb, lt, ks, sh, dm.indices)
    (col * grad).sum().backward()
    return {"positions": pos.grad.cpu().numpy(), "normals": nrm.grad.cpu().numpy(),
            "albedo": alb.grad.cpu().numpy(), "light": lt.grad.numpy(), "ks": float(ks.grad),
            "shininess": float(sh.grad), "color": col.detach().cpu().numpy()}


def rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


@pytest.mark.parametrize("shader", [0, 2])
def test_adjoint_matches_fp64_reference(cuda_lib, shader):
    from oracle import adjoint_fp64
    mesh, views, light, r, dm, ids, grad = setup(shader=shader)
    g = gpu_grads(mesh, views, light, r, dm, grad)
    ref = adjoint_fp64.reference_gradients(mesh, light, views[0].ks, views[0].shininess, views, ids,
                                           grad.cpu().numpy(), shader=shader)
    covered = ids != 0xFFFFFFFF
    assert covered.mean() > 0.1
    assert float(np.abs(g["color"][..., :3] - ref["color"]).max()) <= 1e-5
    groups = ["albedo", "normals", "positions", "light"] + (["ks", "shininess"] if shader == 0 else [])
    errs = {k: rel(g[k], ref[k]) for k in groups}
    r.close()
    assert all(e <= REL_TOL for e in errs.values()), errs


def test_adjoint_matches_finite_differences(cuda_lib):
    import torch
    mesh, views, light, r, dm, ids, grad = setup(nviews=2, size=64)
    g = gpu_grads(mesh, views, light, r, dm, grad)
    size, nviews = 64, 2
    gd = grad.double()

    def loss(pos, nrm, alb, lt, ks, sh):
        out = torch.empty((nviews, size, size, 4), dtype=torch.float32, device="cuda")
        m = R.DeviceMesh(pos, dm.indices, nrm, alb)
        p = params(lt, ks, sh)
        _lib.check(r._lib.edxr_shade_visible(r._h, ctypes.byref(m.abi()), ctypes.byref(p), out.data_ptr()))
        return float((out.double() * gd).sum())

    base = [dm.positions, dm.normals, dm.albedo]
    rng = np.random.default_rng(0)
    checks = []
    visible = np.unique(mesh.indices[np.unique(ids[ids != 0xFFFFFFFF])].ravel())
    for gi, name in enumerate(["positions", "normals", "albedo"]):
        for _ in range(4):
            vtx = int(rng.choice(visible))
            c = int(rng.integers(0, 3))
            args = []
            for sgn in (1, -1):
                t = [b.clone() for b in base]
                t[gi][vtx, c] += sgn * FD_H
                args.append(loss(*t, light, views[0].ks, views[0].shininess))
            checks.append((name, (args[0] - args[1]) / (2 * FD_H), g[name][vtx, c]))
    for c in range(3):
        lp, lm = light.copy(), light.copy()
        lp[c] += FD_H
        lm[c] -= FD_H
        fd = (loss(*base, lp, views[0].ks, views[0].shininess) - loss(*base, lm, views[0].ks, views[0].shininess)) / (2 * FD_H)
        checks.append(("light", fd, g["light"][c]))
    ks, sh = views[0].ks, views[0].shininess
    checks.append(("ks", (loss(*base, light, ks + FD_H, sh) - loss(*base, light, ks - FD_H, sh)) / (2 * FD_H), g["ks"]))
    checks.append(("shininess", (loss(*base, light, ks, sh + FD_H) - loss(*base, light, ks, sh - FD_H)) / (2 * FD_H),
                   g["shininess"]))
    r.close()
    scale = max(abs(c[2]) for c in checks)
    bad = [c for c in checks if abs(c[1] - c[2]) > 2e-2 * max(abs(c[2]), 0.05 * scale)]
    assert not bad, bad


def diff_config(nviews=8, size=256):
    """The differentiable configuration: the 50,000-triangle torus, orbit views
    at 256x256 (every eighth of the 64 views of the benchmark), and targets
    rendered with seeded perturbations of 5% on every parameter (positions,
    normals, albedo, light, ks, shininess)."""
    import torch
    mesh = scenes.diff_torus(seed=13)
    views = scenes.orbit_views(64, size, size, seed=31)[::64 // nviews]
    light = views[0].light.astype(np.float32).copy()
    ks, shin = views[0].ks, views[0].shininess
    rng = np.random.default_rng(17)
    tgt = scenes.Mesh(mesh.positions * (1 + 0.05 * rng.uniform(-1, 1, size=mesh.positions.shape)).astype(np.float32),
                      mesh.normals * (1 + 0.05 * rng.uniform(-1, 1, size=mesh.normals.shape)).astype(np.float32),
                      np.clip(mesh.albedo * (1 + 0.05 * rng.uniform(-1, 1, size=mesh.albedo.shape)), 0, 1)
                      .astype(np.float32), mesh.uvs, mesh.indices)
    t_light = (light * (1 + 0.05 * rng.uniform(-1, 1, 3))).astype(np.float32)
    r = R.Renderer()
    r.Initialize(size, size)
    tdm = R.DeviceMesh.from_mesh(tgt)
    r.RenderBatched([tdm], views, size, size)
    target = torch.empty((len(views), size, size, 4), dtype=torch.float32, device="cuda")
    p = params(t_light, ks * 1.05, shin * 1.05)
    _lib.check(r._lib.edxr_shade_visible(r._h, ctypes.byref(tdm.abi()), ctypes.byref(p), target.data_ptr()))
    dm = R.DeviceMesh.from_mesh(mesh)
    r.RenderBatched([dm], views, size, size)   # visibility of the parameters being optimised
    _, _, ids = r.ReadBatchOutputs(0, len(views), size, size)
    return mesh, views, light, ks, shin, r, dm, ids, target


def test_adjoint_at_diff_config_matches_fp64(cuda_lib):
    """Gradients of the L2 image loss at the differentiable configuration,
    summed by the adjoint's atomics over 8 x 65,536 pixels, within REL_TOL
    (relative L2 per parameter group) of the FP64 reference."""
    import torch
    from oracle import adjoint_fp64
    mesh, views, light, ks, shin, r, dm, ids, target = diff_config()
    n, size = len(views), views[0].width
    Fn = ShadeVisible.make(r, n, size)
    pos = dm.positions.clone().requires_grad_(True)
    nrm = dm.normals.clone().requires_grad_(True)
    alb = dm.albedo.clone().requires_grad_(True)
    lt = torch.tensor(light, dtype=torch.float32, requires_grad=True)
    k = torch.tensor(ks, requires_grad=True)
    s = torch.tensor(shin, requires_grad=True)
    col = Fn.apply(pos, nrm, alb, lt, k, s, dm.indices)
    gcol = (2.0 * (col - target)).detach()
    ((col - target) ** 2).sum().backward()
    r.close()
    ref = adjoint_fp64.reference_gradients(mesh, light, ks, shin, views, ids, gcol.cpu().numpy())
    covered = ids != 0xFFFFFFFF
    assert covered.mean() > 0.1
    assert float(np.abs(col.detach().cpu().numpy()[..., :3] - ref["color"]).max()) <= 1e-5
    got = {"positions": pos.grad.cpu().numpy(), "normals": nrm.grad.cpu().numpy(), "albedo": alb.grad.cpu().numpy(),
           "light": lt.grad.numpy(), "ks": float(k.grad), "shininess": float(s.grad)}
    errs = {g: rel(got[g], ref[g]) for g in got}
    assert all(e <= REL_TOL for e in errs.values()), errs


def test_adjoint_at_diff_config_matches_finite_differences(cuda_lib):
    """Central differences of the same L2 loss on the GPU forward, visibility
    fixed: a few visible vertices' positions, normals and albedo, the light,
    ks and shininess.  The step is h = FD_H; the torus's triangles are about
    two pixels across at 256x256, so moving a vertex by h shifts the
    barycentrics of its pixels by several percent and the h^2 truncation term
    of one central difference is visible.  Each check therefore takes the
    differences at h and h/2 and compares the Richardson extrapolation
    (4 D(h/2) - D(h)) / 3, whose error is O(h^4), with the adjoint."""
    import torch
    mesh, views, light, ks, shin, r, dm, ids, target = diff_config(nviews=8)
    n, size = len(views), views[0].width
    tgt = target.double()

    def loss(pos, nrm, alb, lt, k, s):
        out = torch.empty((n, size, size, 4), dtype=torch.float32, device="cuda")
        m = R.DeviceMesh(pos, dm.indices, nrm, alb)
        _lib.check(r._lib.edxr_shade_visible(r._h, ctypes.byref(m.abi()), ctypes.byref(params(lt, k, s)),
                                             out.data_ptr()))
        return float(((out.double() - tgt)[..., :3] ** 2).sum())

    Fn = ShadeVisible.make(r, n, size)
    pos = dm.positions.clone().requires_grad_(True)
    nrm = dm.normals.clone().requires_grad_(True)
    alb = dm.albedo.clone().requires_grad_(True)
    lt = torch.tensor(light, dtype=torch.float32, requires_grad=True)
    k = torch.tensor(ks, requires_grad=True)
    s = torch.tensor(shin, requires_grad=True)
    col = Fn.apply(pos, nrm, alb, lt, k, s, dm.indices)
    ((col - target)[..., :3] ** 2).sum().backward()
    g = {"positions": pos.grad.cpu().numpy(), "normals": nrm.grad.cpu().numpy(), "albedo": alb.grad.cpu().numpy(),
         "light": lt.grad.numpy(), "ks": float(k.grad), "shininess": float(s.grad)}
    base = [dm.positions, dm.normals, dm.albedo]

    def richardson(f):
        """f(step) -> loss; returns (central difference at FD_H, extrapolated derivative)."""
        d1 = (f(FD_H) - f(-FD_H)) / (2 * FD_H)
        d2 = (f(FD_H / 2) - f(-FD_H / 2)) / FD_H
        return d1, (4 * d2 - d1) / 3

    def moved(gi, vtx, c, step):
        t = [b.clone() for b in base]
        t[gi][vtx, c] += step
        return loss(*t, light, ks, shin)

    def lit(c, step):
        l2 = light.copy()
        l2[c] += step
        return loss(*base, l2, ks, shin)

    rng = np.random.default_rng(1)
    visible = np.unique(mesh.indices[np.unique(ids[ids != 0xFFFFFFFF])].ravel())
    checks = []
    for gi, name in enumerate(["positions", "normals", "albedo"]):
        for _ in range(3):
            vtx, c = int(rng.choice(visible)), int(rng.integers(0, 3))
            checks.append((name, *richardson(lambda st: moved(gi, vtx, c, st)), g[name][vtx, c]))
    for c in range(3):
        checks.append(("light", *richardson(lambda st: lit(c, st)), g["light"][c]))
    checks.append(("ks", *richardson(lambda st: loss(*base, light, ks + st, shin)), g["ks"]))
    checks.append(("shininess", *richardson(lambda st: loss(*base, light, ks, shin + st)), g["shininess"]))
    r.close()
    scale = max(abs(c[3]) for c in checks)
    bad = [c for c in checks if abs(c[2] - c[3]) > 2e-2 * max(abs(c[3]), 0.05 * scale)]
    assert not bad, bad  # (group, D(h), extrapolated, adjoint)
