"""Region-predicate boundary conditions in the reference's JSON schema.

The reference reads a JSON file with three sections (config_parser.cpp:389-455):
``"fixedarea"`` and ``"loadarea"`` are lists of regions (``{"type": "box", "p": [...],
"q": [...]}``, ``"sphere"`` with ``center``/``radius``, ``"halfspace"`` with
``p1``/``p2``/``p3``, ``"cylinder"`` with ``bottomCenter``/``heightVector``/``radius``;
optional ``"closed"`` and ``"complement"`` flags); ``"force"`` is a list of fields
(``"const"`` with ``norm``/``direction``, ``"RadialNormConstDir"``,
``"ConstNormRadialDir"``, ``"RadialNormRadialDir"``, ``"Twist"``), each with its own
``"region"``.  ``parse`` turns such a document into the C structs of
``topo_set_bc_regions``; ``plan`` evaluates it on the host.
"""
from __future__ import annotations

import ctypes as C
import json

import numpy as np

REGION_BOX, REGION_SPHERE, REGION_HALFSPACE, REGION_CYLINDER = range(4)
FIELD_CONST, FIELD_RADIAL_NORM_CONST_DIR, FIELD_CONST_NORM_RADIAL_DIR, FIELD_RADIAL_NORM_RADIAL_DIR, \
    FIELD_TWIST = range(5)

_FIELD_TYPES = {"const": FIELD_CONST, "RadialNormConstDir": FIELD_RADIAL_NORM_CONST_DIR,
                "ConstNormRadialDir": FIELD_CONST_NORM_RADIAL_DIR,
                "RadialNormRadialDir": FIELD_RADIAL_NORM_RADIAL_DIR, "Twist": FIELD_TWIST}

V3 = C.c_double * 3


class Region(C.Structure):
    _fields_ = [("type", C.c_int), ("closed", C.c_int), ("complement", C.c_int), ("a", V3), ("b", V3),
                ("c", V3), ("r", C.c_double)]


class ForceField(C.Structure):
    _fields_ = [("type", C.c_int), ("region", Region), ("norm", C.c_double), ("amplifier", C.c_double),
                ("damp_ratio", C.c_double), ("direction", V3), ("center", V3), ("center2", V3)]


class BcRegions(C.Structure):
    _fields_ = [("origin", V3), ("spacing", C.c_double), ("fixed", C.POINTER(Region)), ("nfixed", C.c_int),
                ("load", C.POINTER(Region)), ("nload", C.c_int), ("force", C.POINTER(ForceField)),
                ("nforce", C.c_int)]


def _v3(d, key, default=(0.0, 0.0, 0.0)):
    v = d.get(key, default)
    if len(v) > 3:
        raise ValueError(f"{key}: at most 3 components")
    out = [0.0, 0.0, 0.0]
    for i, x in enumerate(v):
        out[i] = float(x)
    return V3(*out)


def _region(d) -> Region:
    t = d.get("type")
    r = Region()
    r.closed = int(bool(d.get("closed", False)))
    r.complement = int(bool(d.get("complement", False)))
    if t == "box":
        r.type, r.a, r.b = REGION_BOX, _v3(d, "p"), _v3(d, "q")
    elif t == "sphere":
        r.type, r.a, r.r = REGION_SPHERE, _v3(d, "center"), float(d.get("radius", 0.0))
    elif t == "halfspace":
        r.type, r.a, r.b, r.c = REGION_HALFSPACE, _v3(d, "p1"), _v3(d, "p2"), _v3(d, "p3")
    elif t == "cylinder":
        r.type, r.a, r.b, r.r = REGION_CYLINDER, _v3(d, "bottomCenter"), _v3(d, "heightVector"), \
            float(d["radius"])
    else:
        raise ValueError(f"unknown region type {t!r}")
    return r


def _field(d) -> ForceField:
    f = ForceField()
    if "region" not in d:
        raise ValueError("a force field needs a region")
    f.region = _region(d["region"])
    t = d.get("type")
    if t not in _FIELD_TYPES:
        raise ValueError(f"unknown force field type {t!r}")
    f.type = _FIELD_TYPES[t]
    f.norm = float(d.get("norm", 0.0))
    f.amplifier = float(d.get("amplifier", 1.0))
    f.damp_ratio = float(d.get("dampRatio", 1.0))
    f.direction = _v3(d, "direction")
    if t in ("RadialNormConstDir", "ConstNormRadialDir"):
        f.center = _v3(d, "center")
    elif t == "RadialNormRadialDir":
        f.center, f.center2 = _v3(d, "NormCenter"), _v3(d, "DirCenter")
    elif t == "Twist":
        f.center, f.center2 = _v3(d, "AxisStart"), _v3(d, "AxisEnd")
    return f


class Spec:
    """Parsed region spec; keeps the ctypes arrays alive."""

    def __init__(self, doc, origin=(0.0, 0.0, 0.0), spacing=1.0):
        if isinstance(doc, str):
            doc = json.loads(doc)
        self.doc = doc
        fx = [_region(r) for r in doc.get("fixedarea", [])]
        ld = [_region(r) for r in doc.get("loadarea", [])]
        ff = [_field(f) for f in doc.get("force", [])]
        self._fx = (Region * max(len(fx), 1))(*fx)
        self._ld = (Region * max(len(ld), 1))(*ld)
        self._ff = (ForceField * max(len(ff), 1))(*ff)
        self.c = BcRegions(V3(*[float(x) for x in origin]), float(spacing), self._fx, len(fx), self._ld, len(ld),
                           self._ff, len(ff))


def parse(doc, origin=(0.0, 0.0, 0.0), spacing=1.0) -> Spec:
    return Spec(doc, origin, spacing)


def plan(nx, ny, nz, spec: Spec, eactive=None):
    """Host evaluation (topo_plan_bc_regions): (fixed uint8[nv], loads [3*nv], nfixed, nloaded)."""
    from . import capi
    lib = capi.load()
    nv = (nx + 1) * (ny + 1) * (nz + 1)
    fixed = np.zeros(nv, dtype=np.uint8)
    loads = np.zeros(3 * nv)
    ea = None
    if eactive is not None:
        ea = np.ascontiguousarray(eactive, dtype=np.uint8).ravel()
    nf, nl = C.c_int(), C.c_int()
    rc = lib.topo_plan_bc_regions(nx, ny, nz, ea.ctypes.data if ea is not None else None, C.byref(spec.c),
                                  fixed.ctypes.data, loads.ctypes.data, C.byref(nf), C.byref(nl))
    if rc != capi.TOPO_OK:
        raise capi.TopoError(rc, "topo_plan_bc_regions")
    return fixed, loads, nf.value, nl.value
