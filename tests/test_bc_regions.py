"""Region-predicate boundary conditions (topo_plan_bc_regions / topo_set_bc_regions)
against the numpy restatement in oracle/bc_oracle.py.  Integer masks must match
bit for bit and loads to rounding.  The specs use the reference's JSON schema
with values written for these tests."""
import json

import numpy as np
import pytest

from oracle import bc_oracle
from topoptspline3d_gb300 import bc_regions, workloads

NX, NY, NZ = 20, 10, 12

SPECS = {
    "halfspace_support_sphere_loads": {
        "fixedarea": [{"type": "halfspace", "p1": [0.5, 0, 0], "p2": [0.5, 0, 1], "p3": [0.5, 1, 0]}],
        "loadarea": [{"type": "sphere", "center": [20, 5, 12], "radius": 2.5},
                     {"type": "sphere", "center": [20, 0, 0], "radius": 1.0, "closed": True}],
        "force": [{"type": "const", "norm": 2.0, "direction": [0, 0, -3],
                   "region": {"type": "sphere", "center": [20, 5, 12], "radius": 2.5}},
                  {"type": "const", "norm": 1.0, "direction": [1, 1, 0],
                   "region": {"type": "box", "p": [19, -1, -1], "q": [21, 11, 13]}}],
    },
    "boxes_closed_open_complement": {
        "fixedarea": [{"type": "box", "p": [0, 0, 0], "q": [1, 10, 12], "closed": True},
                      {"type": "box", "p": [18, 0, 0], "q": [20, 10, 1]}],
        "loadarea": [{"type": "box", "p": [5, 3, 3], "q": [15, 7, 9], "complement": True}],
        "force": [{"type": "ConstNormRadialDir", "norm": 0.5, "center": [10, 5, 6],
                   "region": {"type": "sphere", "center": [10, 5, 6], "radius": 100}},
                  {"type": "RadialNormConstDir", "center": [20, 5, 6], "amplifier": 3.0, "dampRatio": 0.5,
                   "direction": [0, -1, 0], "region": {"type": "halfspace", "p1": [10, 0, 0], "p2": [10, 1, 0],
                                                       "p3": [10, 0, 1], "closed": True}}],
    },
    "cylinder_and_twist": {
        "fixedarea": [{"type": "cylinder", "bottomCenter": [0, 5, 6], "heightVector": [2, 0, 0], "radius": 3.5}],
        "loadarea": [{"type": "cylinder", "bottomCenter": [20, 5, 6], "heightVector": [-1, 0, 0], "radius": 6}],
        "force": [{"type": "Twist", "AxisStart": [0, 5, 6], "AxisEnd": [20, 5, 6], "amplifier": 0.25,
                   "region": {"type": "box", "p": [19.5, -1, -1], "q": [21, 11, 13]}},
                  {"type": "RadialNormRadialDir", "NormCenter": [20, 0, 0], "DirCenter": [10, 5, 6],
                   "amplifier": 2.0, "dampRatio": 0.3,
                   "region": {"type": "sphere", "center": [20, 0, 0], "radius": 4, "complement": True}}],
    },
}


@pytest.mark.parametrize("name", sorted(SPECS))
@pytest.mark.parametrize("masked", [False, True])
def test_plan_matches_oracle(name, masked):
    doc = SPECS[name]
    ea = workloads.perforated(NX, NY, NZ, holes=4, radius=(1.5, 3.0), seed=3) if masked else None
    origin, spacing = (0.0, 0.0, 0.0), 1.0
    spec = bc_regions.parse(json.dumps(doc), origin, spacing)
    fx, ld, nf, nl = bc_regions.plan(NX, NY, NZ, spec, ea)
    fo, lo, nfo, nlo = bc_oracle.plan(NX, NY, NZ, doc, origin, spacing, ea)
    assert np.array_equal(fx, fo)
    assert (nf, nl) == (nfo, nlo)
    assert nf > 0 and nl > 0
    assert np.allclose(ld, lo, rtol=1e-13, atol=1e-15)


def test_only_surface_vertices_and_support_wins():
    doc = SPECS["halfspace_support_sphere_loads"]
    spec = bc_regions.parse(doc)
    fx, ld, _, _ = bc_regions.plan(NX, NY, NZ, spec)
    _, surf = bc_oracle.surface_vertices(NX, NY, NZ)
    nv = (NX + 1) * (NY + 1) * (NZ + 1)
    loaded = np.abs(ld.reshape(3, nv)).sum(axis=0) > 0
    assert not (fx[~surf] != 0).any() and not loaded[~surf].any()
    assert not (loaded & (fx != 0)).any()
    # halfspace x < 0.5 fixes exactly the x = 0 face
    x = np.arange(nv) % (NX + 1)
    assert np.array_equal(fx != 0, x == 0)


def test_origin_and_spacing_scale_positions():
    doc = {"fixedarea": [{"type": "box", "p": [-1, -1, -1], "q": [0.01, 100, 100]}],
           "loadarea": [{"type": "box", "p": [0.99, -1, -1], "q": [2, 100, 100]}],
           "force": [{"type": "const", "norm": 1, "direction": [0, 0, 1],
                      "region": {"type": "box", "p": [0.99, -1, -1], "q": [2, 100, 100]}}]}
    spec = bc_regions.parse(doc, origin=(0.0, 0.0, 0.0), spacing=1.0 / NX)
    fx, ld, nf, nl = bc_regions.plan(NX, NY, NZ, spec)
    fo, lo, nfo, nlo = bc_oracle.plan(NX, NY, NZ, doc, (0.0, 0.0, 0.0), 1.0 / NX)
    assert np.array_equal(fx, fo) and np.allclose(ld, lo)
    assert nf == (NY + 1) * (NZ + 1) and nl == (NY + 1) * (NZ + 1)


def test_bad_specs_rejected():
    with pytest.raises(ValueError):
        bc_regions.parse({"fixedarea": [{"type": "torus"}]})
    with pytest.raises(ValueError):
        bc_regions.parse({"force": [{"type": "const", "norm": 1, "direction": [0, 0, 1]}]})
    with pytest.raises(ValueError):
        bc_regions.parse({"fixedarea": [{"type": "box", "p": [0, 0, 0, 0], "q": [1, 1, 1]}]})


@pytest.mark.gpu
def test_set_bc_regions_equals_set_bc():
    from tests.helpers import rel
    from topoptspline3d_gb300 import capi
    doc = SPECS["boxes_closed_open_complement"]
    spec = bc_regions.parse(doc)
    fx, ld, nf, nl = bc_regions.plan(NX, NY, NZ, spec)
    a = capi.Problem(NX, NY, NZ)
    assert a.set_bc_regions(spec) == (nf, nl)
    b = capi.Problem(NX, NY, NZ)
    b.set_bc(fx, ld)
    assert np.array_equal(a.get("vmask"), b.get("vmask"))
    assert rel(a.get("f"), b.get("f")) == 0.0
