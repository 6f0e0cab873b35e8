"""The reference's domain input (an LSB-first uint32 bit mask over a
power-of-two frame, HierarchyGrid::genFromMesh(const std::vector<unsigned>&,
int[3]), grid/Grid.cpp:977) converted on the host: bit masks of the golden
vectors (the reference's own gBitSAT reads them) round-trip to the same
element masks, and set bits outside the box are refused."""
import numpy as np
import pytest

from tests import golden
from topoptspline3d_gb300 import capi, workloads


def test_golden_words_round_trip():
    G = golden.load()
    n = int(G["cube"])
    for key in ("dens_1_words", "filt_0_words"):
        w = G[key]
        ea = capi.bitmask_to_eactive((n, n, n), w, n, n, n)
        assert np.array_equal(ea, golden.words_to_mask(w, n))
        assert np.array_equal(capi.eactive_to_bitmask(n, n, n, ea, (n, n, n)), w)


@pytest.mark.parametrize("dims,reso", [((48, 24, 24), (64, 64, 64)), ((37, 21, 13), (64, 32, 16)),
                                       ((40, 24, 20), (64, 64, 64))])
def test_box_inside_power_of_two_frame(dims, reso):
    nx, ny, nz = dims
    ea = workloads.perforated(nx, ny, nz, holes=5, radius=(2.0, 4.0), seed=3).astype(np.uint8)
    w = capi.eactive_to_bitmask(nx, ny, nz, ea, reso)
    # the bits sit where the frame's own indexing puts them
    bits = ((w[:, None] >> np.arange(32, dtype=np.uint32)) & 1).ravel()[: int(np.prod(reso))]
    frame = bits.reshape(reso[2], reso[1], reso[0])
    assert np.array_equal(frame[:nz, :ny, :nx].ravel(), ea)
    assert frame.sum() == ea.sum()
    assert np.array_equal(capi.bitmask_to_eactive(reso, w, nx, ny, nz), ea)


def test_bits_outside_the_box_are_refused():
    reso = (16, 16, 16)
    w = capi.eactive_to_bitmask(16, 16, 16, None, reso)
    with pytest.raises(capi.TopoError):
        capi.bitmask_to_eactive(reso, w, 15, 16, 16)
