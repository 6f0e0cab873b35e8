"""Golden vectors of the reference's solid voxeliser (see make_vox_golden.py)."""
from __future__ import annotations

import os

import numpy as np

PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "vox_solid.npz")


def load():
    return np.load(PATH)
