"""Host-side logic that needs no GPU: the byte accounting of host meshes
(what a render call reads and what it copies) and the scene generators'
determinism (the benchmark's inputs are seeded)."""
import numpy as np

from edxraster_gb300 import renderer as R
from edxraster_gb300 import scenes


def test_host_mesh_bytes():
    sc = scenes.sphere_scene(320, 180)
    hm = R.HostMesh(sc.mesh)
    nv, nt = sc.mesh.positions.shape[0], sc.mesh.indices.shape[0]
    assert hm.nbytes() == 36 * nv + 12 * nt  # positions, normals, albedo; indices (uvs are not read)
    # pageable arrays are copied whole; page-locked normals and albedo would be read in place
    assert hm.copied_nbytes() == hm.nbytes()
    abi = hm.abi()
    assert abi.num_vertices == nv and abi.num_triangles == nt


def test_scenes_are_seeded():
    a = scenes.stress_scene(2000, 160, 120, seed=3)
    b = scenes.stress_scene(2000, 160, 120, seed=3)
    c = scenes.stress_scene(2000, 160, 120, seed=4)
    assert np.array_equal(a.mesh.positions, b.mesh.positions)
    assert not np.array_equal(a.mesh.positions, c.mesh.positions)
    t = scenes.terrain_scene(16, 64, 36, seed=1)
    assert t.mesh.indices.shape == (2 * 16 * 16, 3) and t.mesh.positions.shape == (17 * 17, 3)
