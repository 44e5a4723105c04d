"""Generate the golden parity fixtures from the reference's own pipeline.

Each fixture holds a small seeded scene (inputs) and what the reference's
Renderer produces for it (EDXRaster/Core sources compiled unmodified against
the shim in oracle/shim, see oracle/ref_harness.cpp): per pixel the winning
input-triangle id, the depth buffer and the winner's two barycentrics, all
bit patterns.  The msaa* fixtures hold, per sample, the winning id and the
depth with 2^msaa_log2 samples per pixel.  Run in a checkout that has the
reference sources:

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


def ms_cases():
    """MSAA fixtures (Renderer::SetMSAAMode): name, scene, hierarchical, log2 of the sample count."""
    yield "msaa2_sphere_160x96", scenes.sphere_scene(160, 96), True, 1
    yield "msaa4_random5_64x64", scenes.small_random_scene(5), True, 2
    yield "msaa8_stress_2k_128x96", scenes.stress_scene(2000, 128, 96, seed=5, max_area=1.5e3), True, 3
    yield "msaa8_terrain_24_96x64_flat", scenes.terrain_scene(24, 96, 64, seed=2), False, 3
    yield "msaa16_random6_48x40", scenes.small_random_scene(6, 48, 40, ntris=90), True, 4
    yield "msaa32_random8_40x32", scenes.small_random_scene(8, 40, 32, ntris=70), True, 5


def save_ms(name, sc, hier, msaa_log2):
    ref = pyoracle.render_reference_ms(sc.mesh, sc.view, msaa_log2, hierarchical=hier)
    v = sc.view
    np.savez_compressed(
        os.path.join(HERE, name + ".npz"),
        positions=sc.mesh.positions, normals=sc.mesh.normals, albedo=sc.mesh.albedo, uvs=sc.mesh.uvs,
        indices=sc.mesh.indices, width=v.width, height=v.height, mv=v.mv, proj=v.proj, raster=v.raster,
        light=v.light, ks=v.ks, shininess=v.shininess, hierarchical=int(hier), msaa_log2=msaa_log2,
        id=ref["id"], depth_bits=ref["depth"].view(np.uint32), fragments=ref["fragments"])
    return ref


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
    for name, sc, hier, lg in ms_cases():
        ref = save_ms(name, sc, hier, lg)
        print(name, "covered samples", int((ref["id"] != 0xFFFFFFFF).sum()), "fragments", ref["fragments"])
