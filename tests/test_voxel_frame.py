"""Host side of the mesh voxeliser against the reference's own code (golden
vectors from tests/golden/make_vox_golden.py): the cube frame of
voxelize_mesh (voxelizer/voxelize_main.cpp:292-341) bit for bit, and the OBJ
reader."""
import numpy as np
import pytest

from tests.golden import vox
from topoptspline3d_gb300 import capi, meshio

G = vox.load()


@pytest.mark.parametrize("i", range(int(G["n"])))
def test_frame_matches_reference(i):
    reso, box = capi.voxel_frame(G[f"c{i}_verts"], int(G[f"c{i}_prefer"]))
    assert reso == int(G[f"c{i}_reso"])
    assert np.array_equal(box, G[f"c{i}_box"])


def test_obj_round_trip(tmp_path):
    v, t = meshio.torus(nu=12, nv=6)
    p = str(tmp_path / "t.obj")
    meshio.write_obj(p, v, t)
    v2, t2 = meshio.read_obj(p)
    assert np.array_equal(t2, t)
    assert np.abs(v2 - v).max() <= 1e-6
    # polygons become fans, 'v/vt/vn' and relative indices are accepted
    with open(p, "a") as f:
        f.write("f -1/1/1 -2/2/2 -3 -4\n")
    v3, t3 = meshio.read_obj(p)
    n = len(v3)
    assert t3[-2].tolist() == [n - 1, n - 2, n - 3] and t3[-1].tolist() == [n - 1, n - 3, n - 4]


def test_test_meshes_are_closed():
    """Every edge of the generated surfaces is shared by exactly two triangles."""
    for v, t in (meshio.uv_sphere(), meshio.torus(), meshio.box((0, 0, 0), (1, 2, 3), meshio.rotation(1))):
        e = np.sort(np.concatenate([t[:, [0, 1]], t[:, [1, 2]], t[:, [2, 0]]]), axis=1)
        _, cnt = np.unique(e, axis=0, return_counts=True)
        assert (cnt == 2).all()
