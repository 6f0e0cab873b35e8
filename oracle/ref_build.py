"""Builds pieces of the reference's own spline and filter code as host code.

Test infrastructure only: it produces the golden vectors that pin the oracle
(tests/golden/make_ref_golden.py).  The reference as a whole cannot be built
here (Eigen, gflags, CGAL, OpenVDB, MATLAB and a CUDA 11 toolchain are
missing), but these routines are self-contained arithmetic:

  grid/Grid.cpp   grid::Grid::set_spline_knot_series   (knots, up to the device upload)
  grid/Grid.cu    SplineBasisX / SplineBasisY / SplineBasisZ (Cox-de Boor, float)
  grid/Grid.cu    coeff2density_kernel + the calc_node lambda of Grid::coeff2density
  grid/Grid.cu    ddensity2dcoeff_kernel + the node_diff lambda of Grid::ddensity2dcoeff_update
  grid/Grid.cu    filterSensitivity_kernel + the fr weight lambda of Grid::filterSensitivity
  grid/Grid.h     BitCount;  culib/lib.cuh  gBitSAT, read_gbit(word), clamp
  voxelizer/voxelize_solid.cu   voxelize_triangle_solid and its helpers (solid
                                voxelisation by x-ray parity, Schwarz-Seidel)
  voxelizer/voxelize_main.cpp   get_point_bb, padd2SatifyResolution (the cube frame)
  voxelizer/util.h              AABox, voxinfo
  grid/Grid.cu    applyK_OTFA_kernel, update_residual_OTFA_WS_kernel,
                  gs_relax_OTFA_WS_kernel and the helpers they call (isValidNode,
                  loadTemplateMatrix, loadNeighborNodesAndFlags)
  grid/Grid.h     the Bitmask enum of grid::Grid;  culib/lib.cuh  devArray_t

The recipe cuts those blocks out of the reference sources where they lie (by
their opening lines, brace-matched) into oracle/_ref/, never into the
repository, and compiles them with oracle/ref_harness.cpp, which supplies the
CUDA keywords, thread indices and __constant__ symbols as host globals and runs
each kernel as a serial loop over its threads.  Two libraries are built: the
reference's tap count m_iM = 3 (grid/Grid.h:35) and m_iM = 4 (the same code at
cubic order, which the reference's hard-wired constant does not allow).  The
voxeliser pieces go into a third (oracle/ref_vox_harness.cpp), which supplies
the few glm vector operations they use, written from glm's documented
definitions (normalize = v * inversesqrt(dot(v, v)), the usual cross product).
The fine-level elasticity kernels go into a fourth (oracle/ref_ops_harness.cpp),
which runs every thread of a block as a host thread so their __syncthreads and
shared-memory block sums behave as on the GPU.

  python -m oracle.ref_build [--reference DIR]
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
DEFAULT_REF = os.environ.get("TOPO_REFERENCE_DIR", "/root/reference")


def _block(lines, start, template_prev=False, stop_marker=None):
    """Lines of the block that opens at index `start`: through the brace that
    closes its first '{' (and a trailing ';' of a lambda statement), or up to
    the line holding `stop_marker`, closed with '}'."""
    first = start - 1 if template_prev and lines[start - 1].lstrip().startswith("template") else start
    out, depth, opened = [], 0, False
    for i in range(first, len(lines)):
        ln = lines[i]
        if stop_marker is not None and stop_marker in ln:
            out.append("}")
            return out
        out.append(ln)
        if i < start:
            continue
        code = ln.split("//", 1)[0]
        for ch in code:
            if ch == "{":
                depth += 1
                opened = True
            elif ch == "}":
                depth -= 1
        if opened and depth == 0:
            return out
    raise RuntimeError("unterminated block")


def _find(lines, needle, after=0):
    for i in range(after, len(lines)):
        if needle in lines[i]:
            return i
    raise RuntimeError(f"not found in reference source: {needle!r}")


def extract(ref: str) -> dict:
    def read(rel):
        with open(os.path.join(ref, rel), encoding="utf-8", errors="replace") as f:
            return f.read().split("\n")

    gcu, gcpp, gh, lib = read("grid/Grid.cu"), read("grid/Grid.cpp"), read("grid/Grid.h"), read("culib/lib.cuh")
    parts = {}
    parts["ref_lib_grid.inc"] = _block(gh, _find(gh, "struct BitCount {"), template_prev=True)
    parts["ref_lib_cu.inc"] = (
        _block(lib, _find(lib, "__device__ bool read_gbit(T word, int id)"), template_prev=True)
        + _block(lib, _find(lib, "__device__ T clamp(T value, T low, T upp)"), template_prev=True)
        + _block(lib, _find(lib, "struct gBitSAT {"), template_prev=True))
    parts["ref_basis.inc"] = sum((_block(gcu, _find(gcu, f"__device__ void SplineBasis{a}(")) for a in "XYZ"), [])
    parts["ref_kernels.inc"] = (
        _block(gcu, _find(gcu, "__global__ void coeff2density_kernel("), template_prev=True)
        + _block(gcu, _find(gcu, "__global__ void ddensity2dcoeff_kernel("), template_prev=True)
        + _block(gcu, _find(gcu, "__global__ void filterSensitivity_kernel("), template_prev=True))
    c2d = _find(gcu, "void Grid::coeff2density(void)")
    parts["ref_calc_node.inc"] = _block(gcu, _find(gcu, "auto calc_node = [=] __device__(int id)", c2d))
    adj = _find(gcu, "void Grid::ddensity2dcoeff_update(void)")
    parts["ref_node_diff.inc"] = _block(gcu, _find(gcu, "auto node_diff = [=] __device__(int id, int eid)", adj))
    flt = _find(gcu, "void Grid::filterSensitivity(double radii)")
    parts["ref_fr.inc"] = _block(gcu, _find(gcu, "auto fr = [=] __device__(float r)", flt))
    parts["ref_knots.inc"] = _block(gcpp, _find(gcpp, "void grid::Grid::set_spline_knot_series(void)"),
                                    stop_marker="// upload to device")
    vs, vm, vu = read("voxelizer/voxelize_solid.cu"), read("voxelizer/voxelize_main.cpp"), read("voxelizer/util.h")
    parts["ref_vox.inc"] = (
        [vs[_find(vs, "#define float_error")]]
        + sum((_block(vs, _find(vs, sig)) for sig in (
            "__device__ __inline__ void setBitXor(", "__device__ inline int check_point_triangle(",
            "__device__ inline float get_x_coordinate(", "__device__ inline bool checkCCW(",
            "__device__ inline bool TopLeftEdge(", "__global__ void voxelize_triangle_solid(")), []))
    parts["ref_vox_frame.inc"] = (
        _block(vu, _find(vu, "struct AABox {"), template_prev=True)
        + _block(vu, _find(vu, "struct voxinfo {"))
        + _block(vm, _find(vm, "std::pair<glm::vec3, glm::vec3> get_point_bb("))
        + _block(vm, _find(vm, "int padd2SatifyResolution(")))
    parts["ref_bitmask.inc"] = _block(gh, _find(gh, "enum Bitmask {"))
    parts["ref_devarray.inc"] = _block(lib, _find(lib, "struct devArray_t {"), template_prev=True)
    parts["ref_ops.inc"] = (
        _block(gcu, _find(gcu, "__device__ bool isValidNode(int vid)"))
        + _block(gcu, _find(gcu, "__device__ void loadTemplateMatrix("))
        + _block(gcu, _find(gcu, "__device__ void loadNeighborNodesAndFlags("))
        + _block(gcu, _find(gcu, "__global__ void gs_relax_OTFA_WS_kernel("), template_prev=True)
        + _block(gcu, _find(gcu, "__global__ void update_residual_OTFA_WS_kernel(int nv, float* rholist)"))
        + _block(gcu, _find(gcu, "__global__ void applyK_OTFA_kernel(")))
    return {k: "\n".join(v) + "\n" for k, v in parts.items()}


def build(ref: str = DEFAULT_REF, force: bool = False) -> list:
    """Returns the paths of the libraries (spline pieces at m_iM = 3 and 4, the
    voxeliser, the fine-level elasticity kernels); builds them when the
    reference sources are present."""
    libs = ([os.path.join(OUT, f"libref_pieces_m{m}.so") for m in (3, 4)] + [os.path.join(OUT, "libref_vox.so")]
            + [os.path.join(OUT, "libref_ops.so")])
    if not force and all(os.path.exists(p) for p in libs):
        return libs
    if not os.path.isdir(os.path.join(ref, "grid")):
        raise FileNotFoundError(f"reference sources not found under {ref}")
    os.makedirs(OUT, exist_ok=True)
    for name, text in extract(ref).items():
        with open(os.path.join(OUT, name), "w") as f:
            f.write(text)
    harness = os.path.join(HERE, "ref_harness.cpp")
    for m, lib in zip((3, 4), libs):
        tmp = lib + f".tmp{os.getpid()}"
        subprocess.check_call(["g++", "-O1", "-fPIC", "-shared", "-std=c++17", "-ffp-contract=off",
                               "-w", f"-DREF_M_IM={m}", "-I" + OUT, harness, "-o", tmp])
        os.replace(tmp, lib)
    tmp = libs[2] + f".tmp{os.getpid()}"
    subprocess.check_call(["g++", "-O1", "-fPIC", "-shared", "-std=c++17", "-ffp-contract=off", "-w",
                           "-I" + OUT, os.path.join(HERE, "ref_vox_harness.cpp"), "-o", tmp])
    os.replace(tmp, libs[2])
    tmp = libs[3] + f".tmp{os.getpid()}"
    subprocess.check_call(["g++", "-O1", "-fPIC", "-shared", "-std=c++20", "-pthread", "-ffp-contract=off", "-w",
                           "-I" + OUT, os.path.join(HERE, "ref_ops_harness.cpp"), "-o", tmp])
    os.replace(tmp, libs[3])
    return libs


if __name__ == "__main__":
    ref = DEFAULT_REF
    if "--reference" in sys.argv:
        ref = sys.argv[sys.argv.index("--reference") + 1]
    for p in build(ref, force=True):
        print("built", p)
