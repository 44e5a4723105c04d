"""FP64 CPU reference of the differentiable form (test infrastructure).

Restates, in double precision with torch's CPU autograd, the forward that
edxr_shade_visible evaluates on the GPU: for every pixel whose winning
triangle is fixed by the triangle-id buffer, the perspective-correct
barycentrics of the pixel centre from the un-snapped clip-space vertices,
interpolation of position, normal and albedo (Fragment::Interpolate,
EDXRaster/Core/Shader.h:142-170) and the Blinn-Phong model
(Shader.h:249-281, with per-vertex albedo, ks and shininess as parameters).
The gradient of sum(colour * grad_colour) is the reference the hand-written
adjoint kernel is checked against.  Only tests import this module.
"""
from __future__ import annotations

import numpy as np
import torch

NO_TRIANGLE = 0xFFFFFFFF


def _ndc_from_raster(raster):
    R = np.asarray(raster, np.float64).reshape(4, 4)
    A = R[:2, :2]
    t = R[:2, 3]
    Ai = np.linalg.inv(A)
    return Ai, -Ai @ t


def mvp_float32(proj, mv):
    """P * MV as the pipeline forms it (Renderer.cpp:90): float32, each entry
    summed left to right.  The differentiable forward takes this float matrix
    as the given transform."""
    P = np.asarray(proj, np.float32).reshape(4, 4)
    M = np.asarray(mv, np.float32).reshape(4, 4)
    C = np.zeros((4, 4), np.float32)
    for i in range(4):
        for j in range(4):
            s = np.float32(P[i, 0] * M[0, j])
            for k in range(1, 4):
                s = np.float32(s + np.float32(P[i, k] * M[k, j]))
            C[i, j] = s
    return C


def _eye(mv):
    inv = np.linalg.inv(np.asarray(mv, np.float64).reshape(4, 4))
    return inv[:3, 3] / inv[3, 3]


def shade_visible(positions, normals, albedo, indices, light, ks, shininess, views, ids, shader=0):
    """Colour (frames, H, W, 3) as double tensors; parameters are double tensors
    (positions/normals/albedo (nv,3), light (3,), ks, shininess scalars)."""
    out = []
    idx = torch.as_tensor(np.asarray(indices, np.int64))
    L = light / torch.linalg.norm(light)
    for v, view in enumerate(views):
        H, W = view.height, view.width
        idv = np.asarray(ids[v]).reshape(H, W)
        mask = idv != NO_TRIANGLE
        py, px = np.nonzero(mask)
        tri = torch.as_tensor(idv[mask].astype(np.int64))
        vi = idx[tri]                                  # (n,3)
        p = positions[vi]                              # (n,3,3)
        n = normals[vi]
        a = albedo[vi]
        mvp = torch.as_tensor(mvp_float32(view.proj, view.mv).astype(np.float64))
        ph = torch.cat([p, torch.ones_like(p[..., :1])], -1)
        clip = ph @ mvp.T                              # (n,3,4)
        X, Y, Wc = clip[..., 0], clip[..., 1], clip[..., 3]
        Ai, t = _ndc_from_raster(view.raster)
        rx, ry = px + 0.5, py + 0.5
        u = torch.as_tensor(Ai[0, 0] * rx + Ai[0, 1] * ry + t[0])[:, None]
        vv = torch.as_tensor(Ai[1, 0] * rx + Ai[1, 1] * ry + t[1])[:, None]
        ac = X - u * Wc
        cc = Y - vv * Wc
        bt = torch.stack([ac[:, 1] * cc[:, 2] - ac[:, 2] * cc[:, 1],
                          ac[:, 2] * cc[:, 0] - ac[:, 0] * cc[:, 2],
                          ac[:, 0] * cc[:, 1] - ac[:, 1] * cc[:, 0]], -1)
        b = bt / bt.sum(-1, keepdim=True)
        P = (b[..., None] * p).sum(1)
        N = (b[..., None] * n).sum(1)
        A = (b[..., None] * a).sum(1)
        Nn = N / torch.linalg.norm(N, dim=-1, keepdim=True)
        nl = (Nn * L).sum(-1)
        diffuse = (torch.clamp(nl, min=0.0) + 0.2) * 3.0 / np.pi
        E = torch.as_tensor(_eye(view.mv)) - P
        E = E / torch.linalg.norm(E, dim=-1, keepdim=True)
        Hv = L + E
        Hv = Hv / torch.linalg.norm(Hv, dim=-1, keepdim=True)
        nh = (Nn * Hv).sum(-1)
        if shader == 0:
            nh = torch.clamp(nh, min=0.0)
        spec = ks * torch.pow(nh, shininess)
        if shader == 0:
            col = A * diffuse[:, None] + spec[:, None]
        elif shader == 1:
            col = (diffuse + spec)[:, None].expand(-1, 3)
        elif shader == 2:
            col = A * diffuse[:, None]
        else:
            col = diffuse[:, None].expand(-1, 3)
        img = torch.zeros((H * W, 3), dtype=torch.float64)
        img = img.index_put((torch.as_tensor(py * W + px),), col)
        out.append(img.reshape(H, W, 3))
    return torch.stack(out)


def reference_gradients(mesh, light, ks, shininess, views, ids, grad_color, shader=0):
    """d/d{albedo, normals, positions, light, ks, shininess} of sum(colour * grad_colour), in FP64."""
    pos = torch.tensor(np.asarray(mesh.positions, np.float64), requires_grad=True)
    nrm = torch.tensor(np.asarray(mesh.normals, np.float64), requires_grad=True)
    alb = torch.tensor(np.asarray(mesh.albedo, np.float64), requires_grad=True)
    lt = torch.tensor(np.asarray(light, np.float64), requires_grad=True)
    k = torch.tensor(float(ks), dtype=torch.float64, requires_grad=True)
    s = torch.tensor(float(shininess), dtype=torch.float64, requires_grad=True)
    col = shade_visible(pos, nrm, alb, mesh.indices, lt, k, s, views, ids, shader)
    g = torch.as_tensor(np.asarray(grad_color, np.float64)[..., :3])
    (col * g).sum().backward()
    def scalar(t):  # shaders without a specular term leave ks/shininess unused
        return 0.0 if t.grad is None else float(t.grad)

    return {"albedo": alb.grad.numpy(), "normals": nrm.grad.numpy(), "positions": pos.grad.numpy(),
            "light": lt.grad.numpy(), "ks": scalar(k), "shininess": scalar(s),
            "color": col.detach().numpy()}
