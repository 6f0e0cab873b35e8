// Host harness for pieces of the reference's spline and filter code.
//
// Test infrastructure only (see ref_build.py): the reference's own routines are
// cut out of its sources into oracle/_ref/*.inc at build time and compiled
// here as host code.  This file supplies what they expect from CUDA and from
// the rest of the reference: the function-space keywords (empty), the thread
// coordinates of an emulated launch, the __constant__ symbols of the spline
// (grid/Grid.cu:42-50) as plain globals, the static members of grid::Grid that
// set_spline_knot_series reads and writes (grid/Grid.h:239-257, 425), and a
// serial launcher that runs every thread of a kernel in order.  None of the
// kernels used here synchronise within a block, so a serial run computes what
// one launch computes, with the racy `+=` of the adjoint (Q2) taken in thread
// order.
#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstring>
#include <type_traits>
#include <vector>

#define __global__
#define __device__
#define __host__
#define __constant__

struct RefDim3 { unsigned x = 0, y = 0, z = 0; };
static RefDim3 threadIdx, blockIdx, blockDim;

// names the extracted gBitSAT mentions in members these tests never call
static inline int __popc(unsigned v) { return __builtin_popcount(v); }
enum { cudaMemcpyHostToDevice = 1 };
template <typename P> static int cudaMalloc(P, size_t) { return 0; }
static int cudaMemcpy(void*, const void*, size_t, int) { return 0; }
static int cudaFree(void*) { return 0; }

#ifndef REF_M_IM
#define REF_M_IM 3
#endif
constexpr static int m_iM = REF_M_IM;

// spline symbols (grid/Grid.cu:42-50), set by ref_set_spline
static int gorder[1];
static int gnbasis[3];
static float gnstep[3];
static float gnBoundMin[3];
static float* gpu_KnotSer[3];

namespace grid {
#include "ref_lib_grid.inc"
struct Grid {
  enum { mask_shellelement = 0b1000000000000 };  // grid/Grid.h:389
  static int n_order;
  static size_t n_partitionx, n_partitiony, n_partitionz;
  static float m_sStep[3];
  static float m_3sBoundMin[3], m_3sBoundMax[3];
  std::vector<float> KnotSer[3];
  float m_sStepX, m_sStepY, m_sStepZ;
  float _box[2][3];
  void set_spline_knot_series(void);
};
int Grid::n_order;
size_t Grid::n_partitionx, Grid::n_partitiony, Grid::n_partitionz;
float Grid::m_sStep[3];
float Grid::m_3sBoundMin[3], Grid::m_3sBoundMax[3];
#include "ref_knots.inc"
}  // namespace grid
using grid::BitCount;

#include "ref_lib_cu.inc"
#include "ref_basis.inc"
#include "ref_kernels.inc"

// Runs fn once per thread of a 1-D launch of `block`-thread blocks covering n.
template <typename Fn>
static void launch_serial(int n, int block, Fn&& fn) {
  const int grid = (n + block - 1) / block;
  blockDim.x = block;
  for (int b = 0; b < grid; ++b)
    for (int t = 0; t < block; ++t) {
      blockIdx.x = b;
      threadIdx.x = t;
      fn();
    }
}

static grid::Grid g_grid;
static std::vector<float> g_knots[3];

extern "C" {

int ref_m_im(void) { return m_iM; }

// HierarchyGrid::set_spline_partition + Grid::set_spline_knot_series +
// set_spline_knot_infoSymbol (grid/Grid.cu:3134-3216): box[6] = min xyz, max xyz.
// Writes the knots (2*order + part[a] per axis, concatenated), the enlarged
// minimum and the step.
void ref_set_spline(int order, const int* part, const float* box, float* knots_out, float* bmin_out,
                    float* step_out) {
  grid::Grid::n_order = order;
  grid::Grid::n_partitionx = part[0];
  grid::Grid::n_partitiony = part[1];
  grid::Grid::n_partitionz = part[2];
  for (int a = 0; a < 3; ++a) {
    g_grid._box[0][a] = box[a];
    g_grid._box[1][a] = box[3 + a];
    g_grid.KnotSer[a].clear();
  }
  g_grid.set_spline_knot_series();
  gorder[0] = order;
  int off = 0;
  for (int a = 0; a < 3; ++a) {
    gnbasis[a] = order + part[a];
    g_knots[a] = g_grid.KnotSer[a];
    gpu_KnotSer[a] = g_knots[a].data();
    gnstep[a] = grid::Grid::m_sStep[a];
    gnBoundMin[a] = grid::Grid::m_3sBoundMin[a];
    bmin_out[a] = gnBoundMin[a];
    step_out[a] = gnstep[a];
    for (float k : g_knots[a]) knots_out[off++] = k;
  }
}

// SplineBasisX/Y/Z at x (grid/Grid.cu:384-466): out[m_iM + 1].
void ref_basis(int axis, float x, float* out) {
  if (axis == 0) SplineBasisX(x, out);
  else if (axis == 1) SplineBasisY(x, out);
  else SplineBasisZ(x, out);
}

// Grid::coeff2density on an ereso^3 cube given by its active-bit words and
// their prefix counts (gBitSAT), eidmap = nullptr: rho_out[active rank].
void ref_coeff2density(int ereso, int nword, const unsigned* bits, const int* sat, const float* box_origin, float eh,
                       float min_density, const float* coeffs, int nactive, float* rho_out) {
  float* cijk_value = const_cast<float*>(coeffs);
  float boxOrigin[3] = {box_origin[0], box_origin[1], box_origin[2]};
#include "ref_calc_node.inc"
  gBitSAT<unsigned int> esat(bits, sat);
  std::vector<int> eflag(std::max(nactive, 1), 0);
  std::fill(rho_out, rho_out + nactive, 0.f);
  launch_serial(nword, 512, [&] {
    coeff2density_kernel(nword, min_density, esat, ereso, rho_out, calc_node, nullptr, eflag.data());
  });
}

// Grid::ddensity2dcoeff_update's scatter: csens_out[n_cijk] from rho_diff[active rank].
void ref_spline_adjoint(int ereso, int nword, const unsigned* bits, const int* sat, const float* box_origin, float eh,
                        const float* rho_diff_in, int nactive, float* csens_out, int ncoeff) {
  std::vector<float> dcv(ncoeff, 0.f);
  float* dc_tmp = dcv.data();
  const float* rho_diff = rho_diff_in;
  std::vector<int> eflagv(std::max(nactive, 1), 0);
  const int* eflag = eflagv.data();
  float boxOrigin[3] = {box_origin[0], box_origin[1], box_origin[2]};
#include "ref_node_diff.inc"
  gBitSAT<unsigned int> esat(bits, sat);
  launch_serial(nword, 512, [&] { ddensity2dcoeff_kernel(nword, esat, ereso, node_diff, nullptr); });
  std::copy(dcv.begin(), dcv.end(), csens_out);
}

// Grid::filterSensitivity (grid/Grid.cu:4130-4246): dst[active rank].
void ref_filter(int ereso, int nword, const unsigned* bits, const int* sat, const float* sens, double radius,
                int nactive, float* dst) {
#include "ref_fr.inc"
  gBitSAT<unsigned int> esat(bits, sat);
  std::fill(dst, dst + nactive, 0.f);
  launch_serial(nword, 512, [&] {
    filterSensitivity_kernel(nword, esat, ereso, sens, dst, (float)radius, fr, nullptr);
  });
}

}  // extern "C"
