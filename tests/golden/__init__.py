"""Golden vectors produced by the reference's own code (see make_ref_golden.py)."""
from __future__ import annotations

import os

import numpy as np

PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "ref_spline_filter.npz")


def load():
    return np.load(PATH)


def words_to_mask(words, n):
    """LSB-first uint32 bit words (x fastest) -> uint8 mask [n^3]."""
    w = np.asarray(words, dtype=np.uint32)
    bits = ((w[:, None] >> np.arange(32, dtype=np.uint32)[None, :]) & 1).astype(np.uint8)
    return bits.ravel()[: n ** 3]
