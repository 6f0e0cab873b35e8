"""Writes vox_solid.npz: the reference's own solid voxeliser run on seeded
test meshes.

oracle/ref_build.py cuts voxelize_triangle_solid (voxelizer/voxelize_solid.cu)
and the cube frame of voxelize_mesh (voxelizer/voxelize_main.cpp) out of the
reference sources and compiles them as host code; this script runs them and
stores each mesh with its resolution, frame and LSB-first words.  Committed,
so the tests need neither the reference nor this script.

  python tests/golden/make_vox_golden.py
"""
from __future__ import annotations

import ctypes as C
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import ref_build  # noqa: E402
from topoptspline3d_gb300 import meshio  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "vox_solid.npz")


def cases():
    return [
        ("sphere", meshio.uv_sphere((0.1, 0.2, -0.3), 0.8, 24, 12), 30),
        ("torus", meshio.torus((0.0, 0.5, 0.0), 1.0, 0.35, 32, 16), 40),
        ("box_rotated", meshio.box((-0.5, -0.3, -0.2), (0.6, 0.4, 0.25), meshio.rotation(11)), 20),
        ("union", meshio.merge(meshio.uv_sphere((1.2, 0.0, 0.0), 0.5, 16, 8),
                               meshio.box((-1.0, -0.4, -0.4), (0.2, 0.4, 0.4), meshio.rotation(5))), 12),
    ]


def main():
    lib = C.CDLL(ref_build.build()[2])
    fp, ip, up = C.POINTER(C.c_float), C.POINTER(C.c_int), C.POINTER(C.c_uint)
    lib.ref_voxelize.argtypes = [fp, C.c_int, ip, C.c_int, C.c_int, ip, fp, up, C.c_size_t]
    g = {}
    for i, (name, (v, t), prefer) in enumerate(cases()):
        cap = (2 * prefer) ** 3 // 32 + 1
        words = np.zeros(cap, dtype=np.uint32)
        reso, box = C.c_int(), np.zeros(6, dtype=np.float32)
        rc = lib.ref_voxelize(v.ctypes.data_as(fp), len(v), t.ctypes.data_as(ip), len(t), prefer, C.byref(reso),
                              box.ctypes.data_as(fp), words.ctypes.data_as(up), cap)
        assert rc == 0
        n = reso.value ** 3 // 32
        g[f"c{i}_name"] = np.array(name)
        g[f"c{i}_verts"], g[f"c{i}_tris"] = v, t
        g[f"c{i}_prefer"] = np.int32(prefer)
        g[f"c{i}_reso"] = np.int32(reso.value)
        g[f"c{i}_box"] = box
        g[f"c{i}_words"] = words[:n]
        print(name, reso.value, int(sum(bin(int(x)).count("1") for x in words[:n])), "solid voxels")
    g["n"] = np.int32(len(cases()))
    np.savez_compressed(OUT, **g)
    print("wrote", OUT, os.path.getsize(OUT), "bytes")


if __name__ == "__main__":
    main()
