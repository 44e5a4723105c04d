"""Generate the golden parity fixtures from the reference's own pipeline.

Each fixture holds a small seeded scene (inputs) and what the reference's
Renderer produces for it (EDXRaster/Core sources compiled unmodified against
the shim in oracle/shim, see oracle/ref_harness.cpp): per pixel the winning
input-triangle id, the depth buffer and the winner's two barycentrics, all
bit patterns.  Run in a checkout that has the reference sources:

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from edxraster_gb300 import scenes  # noqa: E402
from oracle import pyoracle  # noqa: E402


def cases():
    yield "sphere_320x180", scenes.sphere_scene(320, 180), True
    yield "sphere_320x180_flat", scenes.sphere_scene(320, 180), False
    for s in range(4):
        yield "random%d_64x64" % s, scenes.small_random_scene(s), True
    yield "random7_96x80", scenes.small_random_scene(7, 96, 80, ntris=160), True
    yield "stress_5k_256x144", scenes.stress_scene(5000, 256, 144, seed=7, max_area=2e3), True
    yield "terrain_48_192x108", scenes.terrain_scene(48, 192, 108, seed=1), True


def save(name, sc, hier):
    ref = pyoracle.render_reference(sc.mesh, sc.view, hierarchical=hier)
    v = sc.view
    np.savez_compressed(
        os.path.join(HERE, name + ".npz"),
        positions=sc.mesh.positions, normals=sc.mesh.normals, albedo=sc.mesh.albedo, uvs=sc.mesh.uvs,
        indices=sc.mesh.indices, width=v.width, height=v.height, mv=v.mv, proj=v.proj, raster=v.raster,
        light=v.light, ks=v.ks, shininess=v.shininess, hierarchical=int(hier),
        id=ref["id"], depth_bits=ref["depth"].view(np.uint32), lambda0_bits=ref["lambda0"].view(np.uint32),
        lambda1_bits=ref["lambda1"].view(np.uint32), fragments=ref["fragments"])
    return ref


if __name__ == "__main__":
    if pyoracle.reference_lib() is None:
        sys.exit("reference sources not available: cannot generate golden fixtures")
    for name, sc, hier in cases():
        ref = save(name, sc, hier)
        print(name, "covered", int((ref["id"] != 0xFFFFFFFF).sum()), "fragments", ref["fragments"])
