"""Launch tunables change speed, never results: every candidate of the
autotuner's grid renders bit-identical images."""
import itertools

import numpy as np
import pytest

from edxraster_gb300 import autotune
from edxraster_gb300 import renderer as R
from edxraster_gb300 import scenes

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("scene", ["stress", "terrain"])
def test_tuning_grid_is_result_invariant(cuda_lib, scene):
    sc = scenes.stress_scene(20000, 480, 320, seed=3, max_area=3e3) if scene == "stress" \
        else scenes.terrain_scene(128, 480, 270, seed=2)
    r = R.Renderer()
    r.Initialize(sc.view.width, sc.view.height)
    R.configure(r, sc.view)
    ref = None
    keys = list(autotune.GRID)
    for values in itertools.product(*[autotune.GRID[k] for k in keys]):
        t = dict(zip(keys, values))
        t["raster_blocks_per_sm"] = 1 if t["bin_blocks_per_sm"] == 4 else 0
        t["bin_entries_per_triangle"] = 1
        r.SetTuning(t)
        r.RenderMesh(sc.mesh)
        out = r.ReadOutputs()
        if ref is None:
            ref = out
        else:
            assert all(np.array_equal(a, b) for a, b in zip(ref, out)), t
    r.close()


def test_tuning_rejects_bad_values(cuda_lib):
    r = R.Renderer()
    r.Initialize(16, 16)
    with pytest.raises(R.EdxrError):
        r.SetTuning({"raster_variant": 7})
    r.close()
