"""GPU solid voxelisation against the reference's own voxeliser (golden
vectors, bit for bit), and a design problem built from the resulting domain
bit mask."""
import numpy as np
import pytest

from tests.golden import vox
from topoptspline3d_gb300 import capi

pytestmark = pytest.mark.gpu

G = vox.load()


@pytest.mark.parametrize("i", range(int(G["n"])))
def test_voxelize_matches_reference(i):
    reso, box, words = capi.voxelize_mesh(G[f"c{i}_verts"], G[f"c{i}_tris"], int(G[f"c{i}_prefer"]))
    assert reso == int(G[f"c{i}_reso"])
    assert np.array_equal(box, G[f"c{i}_box"])
    assert np.array_equal(words, G[f"c{i}_words"]), (
        str(G[f"c{i}_name"]), int(np.unpackbits(words.view(np.uint8)).sum()),
        int(np.unpackbits(G[f"c{i}_words"].view(np.uint8)).sum()))


def test_problem_from_mesh_domain():
    i = 1  # torus, 64^3 frame
    reso, box, words = capi.voxelize_mesh(G[f"c{i}_verts"], G[f"c{i}_tris"], int(G[f"c{i}_prefer"]))
    ea = capi.bitmask_to_eactive((reso,) * 3, words, reso, reso, reso)
    p = capi.Problem(reso, reso, reso, bitmask=((reso,) * 3, words))
    assert np.array_equal(p.get("eactive"), ea)
    assert int(ea.sum()) == int(np.unpackbits(words.view(np.uint8)).sum())
    p.close()
