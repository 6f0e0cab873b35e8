// Host harness for the reference's fine-level elasticity kernels.
//
// Test infrastructure only (see ref_build.py): the reference's own kernels are
// cut out of grid/Grid.cu into oracle/_ref/ref_ops.inc at build time and
// compiled here as host code:
//
//   applyK_OTFA_kernel               K u on the finest level (grid/Grid.cu:4278-4356)
//   update_residual_OTFA_WS_kernel   r = f - K u with supports (grid/Grid.cu:2277-2333)
//   gs_relax_OTFA_WS_kernel          one colour of the point-block Gauss-Seidel sweep
//                                    with supports (grid/Grid.cu:1698-1842)
//   isValidNode, loadTemplateMatrix, loadNeighborNodesAndFlags (grid/Grid.cu:344-377)
//
// with the Bitmask enum of grid::Grid (grid/Grid.h:376-418) and devArray_t
// (culib/lib.cuh:93-110).  This file supplies what they expect from CUDA and
// from the rest of the reference: the function-space keywords, __shared__
// arrays as block-wide statics, the __constant__ symbols they read
// (grid/Grid.cu:19-38) as plain globals, and a launcher that runs every thread
// of a block as its own host thread, so __syncthreads is a real barrier and the
// kernels' block-wide shared-memory sums run as on the GPU (blocks one after
// another).
//
// The neighbour maps gV2E / gV2V are built here for a dense box with an
// element mask, in the convention the kernels read them: gV2E[e][v] is the
// element whose local node 7 - e is v, gV2V[l][v] the vertex at offset
// (l % 3 - 1, l / 3 % 3 - 1, l / 9 - 1) from v; inactive entries are -1, and
// gV2V[13][v] = -1 marks an inactive vertex.  The kernels' arithmetic (which
// element matrix blocks couple which vertices, the support rule, the
// Gauss-Seidel block update) is the reference's own.
#include <barrier>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <functional>
#include <thread>
#include <vector>

#define __global__
#define __device__
#define __host__
#define __constant__
#define __shared__ static

struct RefDim3 { unsigned x = 0, y = 0, z = 0; };
static thread_local RefDim3 threadIdx, blockIdx;
static RefDim3 blockDim;
static std::barrier<>* g_block_barrier = nullptr;
static void __syncthreads() { g_block_barrier->arrive_and_wait(); }

// symbols of grid/Grid.cu:19-38 that the kernels read
static double gTemplateMatrix[24][24];
static int* gV2E[8];
static int* gV2V[27];
static float power_penalty[1];
static double* gU[3];
static double* gF[3];
static double* gR[3];
static int* gVflag[1];

namespace grid {
struct Grid {
#include "ref_bitmask.inc"
};
}  // namespace grid
using namespace grid;

#include "ref_devarray.inc"
#include "ref_ops.inc"

// Runs fn once per thread of `blocks` blocks of `block` threads; the threads of
// a block run concurrently (one host thread each) and meet at __syncthreads.
static void launch_blocks(int blocks, int block, const std::function<void()>& fn) {
  blockDim.x = block;
  for (int b = 0; b < blocks; ++b) {
    std::barrier<> bar(block);
    g_block_barrier = &bar;
    std::vector<std::thread> ts;
    ts.reserve(block);
    for (int t = 0; t < block; ++t)
      ts.emplace_back([&, b, t] {
        blockIdx.x = b;
        threadIdx.x = t;
        fn();
      });
    for (auto& th : ts) th.join();
  }
  g_block_barrier = nullptr;
}

namespace {

// Vertex numbering and maps of one problem.  perm[k] = lexicographic vertex of
// slot k (-1 for padding), slots grouped by Gauss-Seidel colour when coloured.
struct Maps {
  int vx = 0, vy = 0, vz = 0;
  std::vector<int> perm, slot;     // slot -> box vertex, box vertex -> slot
  std::vector<int> v2e[8], v2v[27];
  std::vector<int> flag;
  int gs_num[8] = {0};
};

Maps build_maps(int ex, int ey, int ez, const uint8_t* eactive, const uint8_t* support, bool coloured) {
  Maps m;
  m.vx = ex + 1; m.vy = ey + 1; m.vz = ez + 1;
  const int64_t nvb = (int64_t)m.vx * m.vy * m.vz;
  auto eact = [&](int x, int y, int z) {
    return x >= 0 && y >= 0 && z >= 0 && x < ex && y < ey && z < ez && eactive[x + ex * (y + ey * z)];
  };
  auto vact = [&](int x, int y, int z) {
    for (int d = 0; d < 8; ++d)
      if (eact(x - 1 + (d & 1), y - 1 + ((d >> 1) & 1), z - 1 + (d >> 2))) return true;
    return false;
  };
  m.slot.assign(nvb, -1);
  if (!coloured) {
    for (int64_t v = 0; v < nvb; ++v) m.perm.push_back((int)v);
  } else {
    for (int c = 0; c < 8; ++c) {
      int n = 0;
      for (int z = 0; z < m.vz; ++z)
        for (int y = 0; y < m.vy; ++y)
          for (int x = 0; x < m.vx; ++x)
            if ((x & 1) + 2 * (y & 1) + 4 * (z & 1) == c && vact(x, y, z)) {
              m.perm.push_back(x + m.vx * (y + m.vy * z));
              ++n;
            }
      const int pad = (n + 31) / 32 * 32;
      for (int k = n; k < pad; ++k) m.perm.push_back(-1);
      m.gs_num[c] = pad;
    }
  }
  const int ns = (int)m.perm.size();
  for (int k = 0; k < ns; ++k)
    if (m.perm[k] >= 0) m.slot[m.perm[k]] = k;
  for (auto& a : m.v2e) a.assign(ns, -1);
  for (auto& a : m.v2v) a.assign(ns, -1);
  m.flag.assign(ns, 0);
  for (int k = 0; k < ns; ++k) {
    const int v = m.perm[k];
    if (v < 0) { m.flag[k] = Grid::mask_invalid; continue; }
    const int x = v % m.vx, y = v / m.vx % m.vy, z = v / (m.vx * m.vy);
    if (!vact(x, y, z)) continue;  // inactive: gV2V[13] stays -1
    if (support[v]) m.flag[k] |= Grid::mask_supportnodes;
    for (int e = 0; e < 8; ++e) {
      const int qx = x - 1 + (e & 1), qy = y - 1 + ((e >> 1) & 1), qz = z - 1 + (e >> 2);
      if (eact(qx, qy, qz)) m.v2e[e][k] = qx + ex * (qy + ey * qz);
    }
    for (int l = 0; l < 27; ++l) {
      const int qx = x + l % 3 - 1, qy = y + l / 3 % 3 - 1, qz = z + l / 9 - 1;
      if (qx < 0 || qy < 0 || qz < 0 || qx >= m.vx || qy >= m.vy || qz >= m.vz || !vact(qx, qy, qz)) continue;
      m.v2v[l][k] = m.slot[qx + m.vx * (qy + m.vy * qz)];
    }
  }
  return m;
}

struct Bound {  // vectors in slot order, bound to the kernels' symbols
  std::vector<double> u[3], f[3], r[3];
};

void bind(Maps& m, Bound& b, const double* ke, double penal, const double* u, const double* f) {
  const int ns = (int)m.perm.size();
  const int64_t nvb = (int64_t)m.vx * m.vy * m.vz;
  for (int i = 0; i < 576; ++i) gTemplateMatrix[i / 24][i % 24] = ke[i];
  power_penalty[0] = (float)penal;
  for (int c = 0; c < 3; ++c) {
    b.u[c].assign(ns, 0.0); b.f[c].assign(ns, 0.0); b.r[c].assign(ns, 0.0);
    for (int k = 0; k < ns; ++k)
      if (m.perm[k] >= 0) {
        b.u[c][k] = u[c * nvb + m.perm[k]];
        if (f) b.f[c][k] = f[c * nvb + m.perm[k]];
      }
    gU[c] = b.u[c].data(); gF[c] = b.f[c].data(); gR[c] = b.r[c].data();
  }
  for (int e = 0; e < 8; ++e) gV2E[e] = m.v2e[e].data();
  for (int l = 0; l < 27; ++l) gV2V[l] = m.v2v[l].data();
  gVflag[0] = m.flag.data();
}

void unbind(const Maps& m, const std::vector<double>* src, double* out) {
  const int64_t nvb = (int64_t)m.vx * m.vy * m.vz;
  for (int c = 0; c < 3; ++c)
    for (size_t k = 0; k < m.perm.size(); ++k)
      if (m.perm[k] >= 0) out[c * nvb + m.perm[k]] = src[c][k];
}

}  // namespace

extern "C" {

// Each call: the box (ex, ey, ez), the element mask, the per-vertex support
// flag (whole node fixed, the reference's rule), rho per element (FP32, as the
// reference stores it), the 24x24 element matrix (row-major), the penalty, and
// [3][nv] vectors in lexicographic vertex order.

// out = K u (applyK_OTFA_kernel, use_support = true).
void ref_apply_k(int ex, int ey, int ez, const uint8_t* eactive, const uint8_t* support, const float* rho,
                 const double* ke, double penal, const double* u, double* out) {
  Maps m = build_maps(ex, ey, ez, eactive, support, false);
  Bound b;
  bind(m, b, ke, penal, u, nullptr);
  const int nv = (int)m.perm.size();
  std::vector<double> fo[3];
  for (auto& a : fo) a.assign(nv, 0.0);
  devArray_t<double*, 3> du{{b.u[0].data(), b.u[1].data(), b.u[2].data()}};
  devArray_t<double*, 3> df{{fo[0].data(), fo[1].data(), fo[2].data()}};
  float* rl = const_cast<float*>(rho);
  launch_blocks((nv + 127) / 128, 128, [&] { applyK_OTFA_kernel(nv, du, df, rl, true); });
  unbind(m, fo, out);
}

// r = f - K u (update_residual_OTFA_WS_kernel).
void ref_residual(int ex, int ey, int ez, const uint8_t* eactive, const uint8_t* support, const float* rho,
                  const double* ke, double penal, const double* u, const double* f, double* r) {
  Maps m = build_maps(ex, ey, ez, eactive, support, false);
  Bound b;
  bind(m, b, ke, penal, u, f);
  const int nv = (int)m.perm.size();
  float* rl = const_cast<float*>(rho);
  launch_blocks((nv + 127) / 128, 128, [&] { update_residual_OTFA_WS_kernel(nv, rl); });
  unbind(m, b.r, r);
}

// `sweeps` forward Gauss-Seidel sweeps, colours 0..7 (Grid::gs_relax on the
// finest level with supports: gs_relax_OTFA_WS_kernel<256>); u updated in place.
void ref_gs_sweeps(int ex, int ey, int ez, const uint8_t* eactive, const uint8_t* support, const float* rho,
                   const double* ke, double penal, double* u, const double* f, int sweeps) {
  Maps m = build_maps(ex, ey, ez, eactive, support, true);
  Bound b;
  bind(m, b, ke, penal, u, f);
  float* rl = const_cast<float*>(rho);
  for (int s = 0; s < sweeps; ++s) {
    int off = 0;
    for (int c = 0; c < 8; ++c) {
      const int n = m.gs_num[c];
      if (n > 0) launch_blocks(n * 8 / 256, 256, [&] { gs_relax_OTFA_WS_kernel<256>(n, off, rl); });
      off += n;
    }
  }
  unbind(m, b.u, u);
}

}  // extern "C"
