/*
 * topo_oracle.cpp -- CPU FP64 restatement of the reference's topology-optimisation
 * hot path.  TEST INFRASTRUCTURE ONLY: the parity checker and the timed CPU
 * baseline; never linked or called by the product library.
 *
 * Each routine cites the reference (NanXYZH/TopOptSpline3D) file:line it restates.
 * Deliberate differences from the reference, applied identically in the CUDA
 * product (documented per routine):
 *  - FP64 throughout (the reference keeps rho, coefficients and sensitivities in FP32);
 *  - a dense element grid with an active mask instead of the bitmask/GS-ordered
 *    sparse storage; GS-order index maps are reproduced separately (orc_gs_maps);
 *  - fixed DOFs are per DOF (a whole-node fix is the reference special case);
 *  - loads on fixed DOFs are dropped (the reference leaves R = F there);
 *  - the coarsest level is solved by dense Cholesky instead of a BDCSVD
 *    pseudo-inverse (equal for the SPD systems used here).
 */
#include "topo_oracle.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

constexpr double kDirichletWeight = 1e6;  // grid/Grid.cu:14 DIRICHLET_DIAGONAL_WEIGHT

struct Level {
  int ex = 0, ey = 0, ez = 0;
  int vx = 0, vy = 0, vz = 0;
  int64_t ne = 0, nv = 0;
  int factor = 1;                 // coarsening factor from the previous used level
  std::vector<uint8_t> eactive;   // [ne]
  std::vector<uint8_t> vmask;     // [nv] bits 0-2: DOF free, bit 3: vertex active
  std::vector<double> U, F, R;    // [3][nv]
  std::vector<double> kel;        // coarse: [ne][576]
  std::vector<double> stencil;    // coarse: [243][nv]
  int64_t vid(int x, int y, int z) const { return x + (int64_t)vx * (y + (int64_t)vy * z); }
  int64_t eid(int x, int y, int z) const { return x + (int64_t)ex * (y + (int64_t)ey * z); }
};

}  // namespace

struct orc_problem {
  int nx, ny, nz;
  double h, E, nu, penal, rho_min;
  double Ke[576];
  std::vector<Level> lv;  // used levels only (dummy level 1 skipped)
  std::vector<double> rho, rhop, sens, coeff, csens;
  std::vector<double> loads;  // [3][nv0] as given (before masking)
  // spline
  int order = 3;
  int part[3] = {0, 0, 0};
  int nbasis[3] = {0, 0, 0};
  std::vector<double> knots[3];
  double kmin[3], kstep[3];
  // coarsest dense Cholesky factor (lower, row-major)
  std::vector<double> Lc;
  std::vector<uint8_t> dropped;
  int nc_dense = 0;
  // chebyshev
  int cheb_degree = 2;
  double cheb_lo = 0.3, cheb_hi = 1.1;
  std::vector<double> lmax;  // per level
};

// ----------------------------------------------------------------------------
// Element template: element/templateMatrix.cpp:15-99.
// B (6x24) with engineering shear rows (yz, xz, xy), D isotropic, 2x2x2 Gauss on
// the unit parameter cube, scaled by (h/2)^3.
// ----------------------------------------------------------------------------
extern "C" void orc_ke_template(double E, double nu, double h, double* Ke) {
  double D[6][6] = {{0}};
  double c = E / ((1 + nu) * (1 - 2 * nu));
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) D[i][j] = c * (i == j ? 1 - nu : nu);
  for (int i = 3; i < 6; ++i) D[i][i] = c * (1 - 2 * nu) / 2;
  std::memset(Ke, 0, sizeof(double) * 576);
  const double g = std::sqrt(3.0) / 3.0;
  for (int q = 0; q < 8; ++q) {
    double prm[3] = {((2 * (q % 2) - 1) * g + 1) / 2, ((2 * (q / 2 % 2) - 1) * g + 1) / 2,
                     ((2 * (q / 4) - 1) * g + 1) / 2};
    double dN[8][3];
    for (int a = 0; a < 8; ++a) {
      int id[3] = {a % 2, a / 2 % 2, a / 4};
      double r[3];
      for (int k = 0; k < 3; ++k) r[k] = id[k] ? prm[k] : 1 - prm[k];
      for (int k = 0; k < 3; ++k)
        dN[a][k] = (id[k] ? 1.0 / h : -1.0 / h) * r[(k + 1) % 3] * r[(k + 2) % 3];
    }
    double B[6][24] = {{0}};
    for (int a = 0; a < 8; ++a) {
      for (int k = 0; k < 3; ++k) B[k][3 * a + k] = dN[a][k];
      B[3][3 * a + 1] = dN[a][2]; B[3][3 * a + 2] = dN[a][1];
      B[4][3 * a + 0] = dN[a][2]; B[4][3 * a + 2] = dN[a][0];
      B[5][3 * a + 0] = dN[a][1]; B[5][3 * a + 1] = dN[a][0];
    }
    double DB[6][24];
    for (int i = 0; i < 6; ++i)
      for (int j = 0; j < 24; ++j) {
        double s = 0;
        for (int k = 0; k < 6; ++k) s += D[i][k] * B[k][j];
        DB[i][j] = s;
      }
    for (int i = 0; i < 24; ++i)
      for (int j = 0; j < 24; ++j) {
        double s = 0;
        for (int k = 0; k < 6; ++k) s += B[k][i] * DB[k][j];
        Ke[i * 24 + j] += s;
      }
  }
  double sc = std::pow(h / 2, 3);
  for (int i = 0; i < 576; ++i) Ke[i] *= sc;
}

// ----------------------------------------------------------------------------
// Hierarchy: coarsen by child-OR while the active element count exceeds 400
// (grid/Grid.cpp:747-769); level 1 is a dummy so level 0 restricts by 4 to
// level 2 (grid/Grid.cpp:909-911, optimization/optimization.cpp:20).
// ----------------------------------------------------------------------------
static void finish_level(Level& L) {
  L.vx = L.ex + 1; L.vy = L.ey + 1; L.vz = L.ez + 1;
  L.ne = (int64_t)L.ex * L.ey * L.ez;
  L.nv = (int64_t)L.vx * L.vy * L.vz;
  L.vmask.assign(L.nv, 0);
  for (int z = 0; z < L.ez; ++z)
    for (int y = 0; y < L.ey; ++y)
      for (int x = 0; x < L.ex; ++x) {
        if (!L.eactive[L.eid(x, y, z)]) continue;
        for (int a = 0; a < 8; ++a) L.vmask[L.vid(x + a % 2, y + a / 2 % 2, z + a / 4)] = 0xF;
      }
  L.U.assign(3 * L.nv, 0.0); L.F.assign(3 * L.nv, 0.0); L.R.assign(3 * L.nv, 0.0);
}

static Level coarsen(const Level& f, int factor) {
  Level c;
  c.ex = (f.ex + factor - 1) / factor; c.ey = (f.ey + factor - 1) / factor;
  c.ez = (f.ez + factor - 1) / factor;
  c.factor = factor;
  c.eactive.assign((int64_t)c.ex * c.ey * c.ez, 0);
  for (int z = 0; z < f.ez; ++z)
    for (int y = 0; y < f.ey; ++y)
      for (int x = 0; x < f.ex; ++x)
        if (f.eactive[f.eid(x, y, z)])
          c.eactive[(x / factor) + (int64_t)c.ex * ((y / factor) + (int64_t)c.ey * (z / factor))] = 1;
  finish_level(c);
  return c;
}

static int64_t count_active(const Level& L) {
  int64_t n = 0;
  for (auto a : L.eactive) n += a ? 1 : 0;
  return n;
}

extern "C" orc_problem* orc_create(int nx, int ny, int nz, double h, double E, double nu,
                                   double penal, double rho_min, const uint8_t* eactive) {
  orc_problem* p = new orc_problem();
  p->nx = nx; p->ny = ny; p->nz = nz; p->h = h; p->E = E; p->nu = nu; p->penal = penal;
  p->rho_min = rho_min;
  orc_ke_template(E, nu, h, p->Ke);
  Level L0;
  L0.ex = nx; L0.ey = ny; L0.ez = nz;
  L0.eactive.assign((int64_t)nx * ny * nz, 1);
  if (eactive)
    for (int64_t i = 0; i < (int64_t)nx * ny * nz; ++i) L0.eactive[i] = eactive[i] ? 1 : 0;
  finish_level(L0);
  // reference level list (including the dummy level 1)
  std::vector<Level> all;
  all.push_back(L0);
  while (count_active(all.back()) > 400) all.push_back(coarsen(all.back(), 2));
  p->lv.push_back(all[0]);
  if (all.size() >= 3) {
    Level c2 = coarsen(all[0], 4);
    p->lv.push_back(c2);
    for (size_t i = 3; i < all.size(); ++i) p->lv.push_back(coarsen(p->lv.back(), 2));
  } else if (all.size() == 2) {
    p->lv.push_back(coarsen(all[0], 2));
  }
  p->rho.assign(p->lv[0].ne, 1.0);
  p->rhop.assign(p->lv[0].ne, 1.0);
  p->sens.assign(p->lv[0].ne, 0.0);
  p->loads.assign(3 * p->lv[0].nv, 0.0);
  p->lmax.assign(p->lv.size(), 0.0);
  for (size_t l = 0; l < p->lv.size(); ++l)
    if (l > 0) p->lv[l].stencil.assign(243 * p->lv[l].nv, 0.0);
  return p;
}

extern "C" void orc_destroy(orc_problem* p) { delete p; }
extern "C" int orc_num_levels(const orc_problem* p) { return (int)p->lv.size(); }
extern "C" void orc_level_dims(const orc_problem* p, int l, int* d) {
  d[0] = p->lv[l].ex; d[1] = p->lv[l].ey; d[2] = p->lv[l].ez;
}
extern "C" int orc_level_factor(const orc_problem* p, int l) { return p->lv[l].factor; }

// ----------------------------------------------------------------------------
// Boundary conditions: support flags fix DOFs (grid/Grid.cpp:2681-2726 sets whole
// nodes; here per DOF), loads are the per-node field values
// (optimization/projection.cpp:271-282) scattered into F (projection.cu:344-368).
// ----------------------------------------------------------------------------
extern "C" void orc_set_bc(orc_problem* p, const uint8_t* fixed, const double* loads) {
  Level& L = p->lv[0];
  for (int64_t v = 0; v < L.nv; ++v) {
    uint8_t m = L.vmask[v] & 0x8;
    if (m) m |= (uint8_t)(~fixed[v] & 0x7);
    L.vmask[v] = m;
  }
  std::copy(loads, loads + 3 * L.nv, p->loads.begin());
  for (int c = 0; c < 3; ++c)
    for (int64_t v = 0; v < L.nv; ++v)
      L.F[c * L.nv + v] = ((L.vmask[v] >> c) & 1) ? loads[c * L.nv + v] : 0.0;
}

// ----------------------------------------------------------------------------
// Fine operator (WS mode): y_i = sum_{e ni v} rho_e^p Ke[a_v, :] u_e with fixed
// columns removed and fixed rows zero (grid/Grid.cu:2277-2333, 4278-4356).
// u is kept zero on fixed DOFs, so the column mask is applied by masking u.
// ----------------------------------------------------------------------------
static inline double masked_u(const Level& L, const double* u, int64_t v, int c) {
  return ((L.vmask[v] >> c) & 1) ? u[c * L.nv + v] : 0.0;
}

static void fine_row(const orc_problem* p, const double* u, int x, int y, int z, double out[3],
                     double S[9]) {
  const Level& L = p->lv[0];
  out[0] = out[1] = out[2] = 0;
  if (S) for (int i = 0; i < 9; ++i) S[i] = 0;
  for (int w = 0; w < 8; ++w) {
    int ex = x - 1 + w % 2, ey = y - 1 + w / 2 % 2, ez = z - 1 + w / 4;
    if (ex < 0 || ey < 0 || ez < 0 || ex >= L.ex || ey >= L.ey || ez >= L.ez) continue;
    int64_t e = L.eid(ex, ey, ez);
    if (!L.eactive[e]) continue;
    double pe = p->rhop[e];
    int a = 7 - w;
    for (int b = 0; b < 8; ++b) {
      int64_t vb = L.vid(ex + b % 2, ey + b / 2 % 2, ez + b / 4);
      double ub[3] = {masked_u(L, u, vb, 0), masked_u(L, u, vb, 1), masked_u(L, u, vb, 2)};
      for (int i = 0; i < 3; ++i) {
        const double* kr = &p->Ke[(3 * a + i) * 24 + 3 * b];
        out[i] += pe * (kr[0] * ub[0] + kr[1] * ub[1] + kr[2] * ub[2]);
      }
      if (S && b == a)
        for (int i = 0; i < 3; ++i)
          for (int j = 0; j < 3; ++j) S[3 * i + j] += pe * p->Ke[(3 * a + i) * 24 + 3 * a + j];
    }
  }
}

extern "C" void orc_apply_fine(orc_problem* p, const double* u, double* yv) {
  const Level& L = p->lv[0];
#pragma omp parallel for collapse(2) schedule(static)
  for (int z = 0; z < L.vz; ++z)
    for (int y = 0; y < L.vy; ++y)
      for (int x = 0; x < L.vx; ++x) {
        int64_t v = L.vid(x, y, z);
        double o[3];
        fine_row(p, u, x, y, z, o, nullptr);
        for (int c = 0; c < 3; ++c) yv[c * L.nv + v] = ((L.vmask[v] >> c) & 1) ? o[c] : 0.0;
      }
}

// ----------------------------------------------------------------------------
// Coarse stencil apply: sum over 27 neighbours of 3x3 blocks
// (grid/Grid.cu:2126-2224 residual, 1454-1566 GS).
// ----------------------------------------------------------------------------
static void stencil_row(const Level& L, const double* u, int x, int y, int z, double out[3],
                        bool skip_center) {
  out[0] = out[1] = out[2] = 0;
  int64_t v = L.vid(x, y, z);
  for (int d = 0; d < 27; ++d) {
    if (skip_center && d == 13) continue;
    int nx_ = x + d % 3 - 1, ny_ = y + d / 3 % 3 - 1, nz_ = z + d / 9 - 1;
    if (nx_ < 0 || ny_ < 0 || nz_ < 0 || nx_ >= L.vx || ny_ >= L.vy || nz_ >= L.vz) continue;
    int64_t n = L.vid(nx_, ny_, nz_);
    for (int i = 0; i < 3; ++i) {
      double s = 0;
      for (int j = 0; j < 3; ++j) s += L.stencil[(d * 9 + 3 * i + j) * L.nv + v] * u[j * L.nv + n];
      out[i] += s;
    }
  }
}

static void level_residual(orc_problem* p, int l) {
  Level& L = p->lv[l];
  if (l == 0) {
    orc_apply_fine(p, L.U.data(), L.R.data());
    for (int64_t i = 0; i < 3 * L.nv; ++i) L.R[i] = L.F[i] - L.R[i];
    for (int c = 0; c < 3; ++c)
      for (int64_t v = 0; v < L.nv; ++v)
        if (!((L.vmask[v] >> c) & 1)) L.R[c * L.nv + v] = 0.0;
    return;
  }
#pragma omp parallel for collapse(2) schedule(static)
  for (int z = 0; z < L.vz; ++z)
    for (int y = 0; y < L.vy; ++y)
      for (int x = 0; x < L.vx; ++x) {
        int64_t v = L.vid(x, y, z);
        double o[3];
        stencil_row(L, L.U.data(), x, y, z, o, false);
        for (int c = 0; c < 3; ++c) L.R[c * L.nv + v] = L.F[c * L.nv + v] - o[c];
      }
}

extern "C" void orc_residual(orc_problem* p, int l) { level_residual(p, l); }

// ----------------------------------------------------------------------------
// 8-colour point-block Gauss-Seidel (grid/Grid.cu:1699-1842 fine, 1454-1566 coarse,
// colour x%2 + 2(y%2) + 4(z%2), grid/Grid.cu:1286-1328).  Within a vertex the
// three DOFs are relaxed in order 0,1,2 (reverse: colours 7..0, DOFs 2,1,0, the
// adjoint sweep used by the symmetric V-cycle in PCG).
// ----------------------------------------------------------------------------
static void gs_vertex_update(double* U, int64_t nv, int64_t v, const double r[3], const double S[9],
                             uint8_t freebits, bool reverse) {
  double du[3] = {0, 0, 0};
  if (!reverse) {
    for (int i = 0; i < 3; ++i) {
      if (!((freebits >> i) & 1)) continue;
      double s = r[i];
      for (int j = 0; j < i; ++j) s -= S[3 * i + j] * du[j];
      du[i] = s / S[4 * i];
    }
  } else {
    for (int i = 2; i >= 0; --i) {
      if (!((freebits >> i) & 1)) continue;
      double s = r[i];
      for (int j = i + 1; j < 3; ++j) s -= S[3 * i + j] * du[j];
      du[i] = s / S[4 * i];
    }
  }
  for (int i = 0; i < 3; ++i) U[i * nv + v] += du[i];
}

static void smooth_level(orc_problem* p, int l, int sweeps, bool reverse) {
  Level& L = p->lv[l];
  for (int s = 0; s < sweeps; ++s) {
    for (int cc = 0; cc < 8; ++cc) {
      int col = reverse ? 7 - cc : cc;
      int cx = col % 2, cy = col / 2 % 2, cz = col / 4;
#pragma omp parallel for collapse(2) schedule(static)
      for (int z = cz; z < L.vz; z += 2)
        for (int y = cy; y < L.vy; y += 2)
          for (int x = cx; x < L.vx; x += 2) {
            int64_t v = L.vid(x, y, z);
            uint8_t fb = L.vmask[v] & 0x7;
            if (!(L.vmask[v] & 0x8) || !fb) continue;
            double o[3], S[9], r[3];
            if (l == 0) {
              fine_row(p, L.U.data(), x, y, z, o, S);
            } else {
              stencil_row(L, L.U.data(), x, y, z, o, false);
              for (int k = 0; k < 9; ++k) S[k] = L.stencil[(13 * 9 + k) * L.nv + v];
            }
            for (int c = 0; c < 3; ++c) r[c] = L.F[c * L.nv + v] - o[c];
            gs_vertex_update(L.U.data(), L.nv, v, r, S, fb, reverse);
          }
    }
  }
}

// ----------------------------------------------------------------------------
// Point-block Jacobi Chebyshev smoother (the fast-path alternative to GS; no
// reference counterpart).  Polynomial of degree k in D^{-1}A targeting
// [lo*lmax, hi*lmax], three-term recurrence (Saad, Iterative Methods, Alg. 12.1).
// ----------------------------------------------------------------------------
static void diag_blocks(const orc_problem* p, int l, std::vector<double>& Dinv) {
  const Level& L = p->lv[l];
  Dinv.assign(9 * L.nv, 0.0);
#pragma omp parallel for collapse(2) schedule(static)
  for (int z = 0; z < L.vz; ++z)
    for (int y = 0; y < L.vy; ++y)
      for (int x = 0; x < L.vx; ++x) {
        int64_t v = L.vid(x, y, z);
        double S[9] = {0};
        if (l == 0) {
          for (int w = 0; w < 8; ++w) {
            int ex = x - 1 + w % 2, ey = y - 1 + w / 2 % 2, ez = z - 1 + w / 4;
            if (ex < 0 || ey < 0 || ez < 0 || ex >= L.ex || ey >= L.ey || ez >= L.ez) continue;
            int64_t e = L.eid(ex, ey, ez);
            if (!L.eactive[e]) continue;
            int a = 7 - w;
            for (int i = 0; i < 3; ++i)
              for (int j = 0; j < 3; ++j) S[3 * i + j] += p->rhop[e] * p->Ke[(3 * a + i) * 24 + 3 * a + j];
          }
        } else {
          for (int k = 0; k < 9; ++k) S[k] = L.stencil[(13 * 9 + k) * L.nv + v];
        }
        uint8_t fb = L.vmask[v] & 0x7;
        if (!(L.vmask[v] & 0x8)) fb = 0;
        // restrict to free DOFs: fixed rows/cols -> identity
        for (int i = 0; i < 3; ++i)
          for (int j = 0; j < 3; ++j)
            if (!((fb >> i) & 1) || !((fb >> j) & 1)) S[3 * i + j] = (i == j) ? 1.0 : 0.0;
        // inverse of the symmetric 3x3 block (adjugate)
        double a = S[0], b = S[1], c = S[2], d = S[4], e = S[5], f = S[8];
        double A0 = d * f - e * e, A1 = c * e - b * f, A2 = b * e - c * d;
        double det = a * A0 + b * A1 + c * A2;
        double inv[9] = {A0, A1, A2, A1, a * f - c * c, b * c - a * e, A2, b * c - a * e, a * d - b * b};
        for (int k = 0; k < 9; ++k) {
          int i = k / 3, j = k % 3;
          bool keep = ((fb >> i) & 1) && ((fb >> j) & 1);
          Dinv[k * L.nv + v] = keep ? inv[k] / det : 0.0;
        }
      }
}

static void apply_level(orc_problem* p, int l, const double* u, double* y) {
  Level& L = p->lv[l];
  if (l == 0) { orc_apply_fine(p, u, y); return; }
#pragma omp parallel for collapse(2) schedule(static)
  for (int z = 0; z < L.vz; ++z)
    for (int yy = 0; yy < L.vy; ++yy)
      for (int x = 0; x < L.vx; ++x) {
        int64_t v = L.vid(x, yy, z);
        double o[3];
        stencil_row(L, u, x, yy, z, o, false);
        for (int c = 0; c < 3; ++c) y[c * L.nv + v] = o[c];
      }
}

static void dinv_apply(const Level& L, const std::vector<double>& Dinv, const double* r, double* z) {
#pragma omp parallel for schedule(static)
  for (int64_t v = 0; v < L.nv; ++v) {
    double rv[3] = {r[v], r[L.nv + v], r[2 * L.nv + v]};
    for (int i = 0; i < 3; ++i)
      z[i * L.nv + v] = Dinv[(3 * i) * L.nv + v] * rv[0] + Dinv[(3 * i + 1) * L.nv + v] * rv[1] +
                        Dinv[(3 * i + 2) * L.nv + v] * rv[2];
  }
}

static double level_lmax(orc_problem* p, int l) {
  // power iteration on D^{-1}A from a deterministic start vector
  Level& L = p->lv[l];
  std::vector<double> Dinv, x(3 * L.nv), y(3 * L.nv), t(3 * L.nv);
  diag_blocks(p, l, Dinv);
  for (int64_t i = 0; i < 3 * L.nv; ++i) {
    uint64_t hsh = (uint64_t)i * 0x9E3779B97F4A7C15ull;
    hsh ^= hsh >> 29;
    x[i] = 0.5 + (double)(hsh % 1000) / 1000.0;
    int64_t v = i % L.nv; int c = (int)(i / L.nv);
    if (!((L.vmask[v] >> c) & 1) || !(L.vmask[v] & 0x8)) x[i] = 0;
  }
  double lam = 0;
  for (int it = 0; it < 12; ++it) {
    double nx = 0;
    for (double a : x) nx += a * a;
    nx = std::sqrt(nx);
    for (double& a : x) a /= nx;
    apply_level(p, l, x.data(), t.data());
    dinv_apply(L, Dinv, t.data(), y.data());
    double num = 0;
    for (int64_t i = 0; i < 3 * L.nv; ++i) num += x[i] * y[i];
    lam = num;
    x.swap(y);
  }
  return lam;
}

static void cheb_level(orc_problem* p, int l, const std::vector<double>& Dinv) {
  Level& L = p->lv[l];
  double lmax = p->lmax[l] * p->cheb_hi, lmin = p->lmax[l] * p->cheb_lo;
  double theta = 0.5 * (lmax + lmin), delta = 0.5 * (lmax - lmin);
  double sigma = theta / delta, rho_old = 1.0 / sigma;
  int64_t n3 = 3 * L.nv;
  std::vector<double> r(n3), d(n3), z(n3);
  level_residual(p, l);
  dinv_apply(L, Dinv, L.R.data(), z.data());
  for (int64_t i = 0; i < n3; ++i) { d[i] = z[i] / theta; L.U[i] += d[i]; }
  for (int k = 1; k < p->cheb_degree; ++k) {
    level_residual(p, l);
    dinv_apply(L, Dinv, L.R.data(), z.data());
    double rho_new = 1.0 / (2.0 * sigma - rho_old);
    for (int64_t i = 0; i < n3; ++i) {
      d[i] = rho_new * rho_old * d[i] + 2.0 * rho_new / delta * z[i];
      L.U[i] += d[i];
    }
    rho_old = rho_new;
  }
}

extern "C" void orc_set_chebyshev(orc_problem* p, int degree, double lo, double hi) {
  p->cheb_degree = degree; p->cheb_lo = lo; p->cheb_hi = hi;
}

extern "C" void orc_smooth(orc_problem* p, int l, int sweeps, int reverse) {
  smooth_level(p, l, sweeps, reverse != 0);
}

// ----------------------------------------------------------------------------
// Transfers: trilinear prolongation and its exact transpose (no 1/8 scale):
// nondyadic factor 4 weights (4-i)(4-j)(4-k)/64 (grid/Grid.cu:2509-2570, 2635-2671),
// dyadic factor 2 weights 1, 1/2, 1/4, 1/8 (grid/Grid.cu:2456-2507, 2594-2632).
// The prolongated correction is masked on fixed DOFs (the reference resets it
// in the following GS sweep; identical results).
// ----------------------------------------------------------------------------
extern "C" void orc_restrict(orc_problem* p, int lc) {
  Level& C = p->lv[lc];
  const Level& Fl = p->lv[lc - 1];
  int fct = C.factor;
#pragma omp parallel for collapse(2) schedule(static)
  for (int z = 0; z < C.vz; ++z)
    for (int y = 0; y < C.vy; ++y)
      for (int x = 0; x < C.vx; ++x) {
        double s[3] = {0, 0, 0};
        for (int dz = -(fct - 1); dz <= fct - 1; ++dz) {
          int fz = z * fct + dz;
          if (fz < 0 || fz >= Fl.vz) continue;
          for (int dy = -(fct - 1); dy <= fct - 1; ++dy) {
            int fy = y * fct + dy;
            if (fy < 0 || fy >= Fl.vy) continue;
            for (int dx = -(fct - 1); dx <= fct - 1; ++dx) {
              int fx = x * fct + dx;
              if (fx < 0 || fx >= Fl.vx) continue;
              double w = (double)((fct - std::abs(dx)) * (fct - std::abs(dy)) * (fct - std::abs(dz))) /
                         (double)(fct * fct * fct);
              int64_t fv = Fl.vid(fx, fy, fz);
              for (int c = 0; c < 3; ++c) s[c] += w * Fl.R[c * Fl.nv + fv];
            }
          }
        }
        int64_t cv = C.vid(x, y, z);
        for (int c = 0; c < 3; ++c) C.F[c * C.nv + cv] = s[c];
      }
}

extern "C" void orc_prolong(orc_problem* p, int lf) {
  Level& Fl = p->lv[lf];
  const Level& C = p->lv[lf + 1];
  int fct = C.factor;
#pragma omp parallel for collapse(2) schedule(static)
  for (int z = 0; z < Fl.vz; ++z)
    for (int y = 0; y < Fl.vy; ++y)
      for (int x = 0; x < Fl.vx; ++x) {
        int64_t fv = Fl.vid(x, y, z);
        int cx0 = x / fct, cy0 = y / fct, cz0 = z / fct;
        int rx = x % fct, ry = y % fct, rz = z % fct;
        double s[3] = {0, 0, 0};
        for (int k = 0; k < 8; ++k) {
          int ox = k % 2, oy = k / 2 % 2, oz = k / 4;
          double wx = ox ? (double)rx / fct : (double)(fct - rx) / fct;
          double wy = oy ? (double)ry / fct : (double)(fct - ry) / fct;
          double wz = oz ? (double)rz / fct : (double)(fct - rz) / fct;
          double w = wx * wy * wz;
          if (w == 0) continue;
          int64_t cv = C.vid(cx0 + ox, cy0 + oy, cz0 + oz);
          for (int c = 0; c < 3; ++c) s[c] += w * C.U[c * C.nv + cv];
        }
        for (int c = 0; c < 3; ++c)
          if ((Fl.vmask[fv] >> c) & 1) Fl.U[c * Fl.nv + fv] += s[c];
      }
}

// ----------------------------------------------------------------------------
// Galerkin coarse operators.  Level 0 -> first coarse level: coarse element
// matrix K_E = sum_{fine e in E} Q_e^T Ktilde_e Q_e with Ktilde_e = rho^p D Ke D +
// 1e6 * sum_{fixed DOFs of e} e e^T (grid/Grid.cu:1111-1225: fixed rows/columns
// zeroed, 1e6*W on the diagonal, not scaled by rho^p).  Further levels: exact
// K_E = sum_children Q^T K_child Q (grid/Grid.cu:839-896 in stencil form).
// Stencils are assembled from the element matrices.
// ----------------------------------------------------------------------------
static void interp_weights(int fct, int px, int py, int pz, double Q[8][8]) {
  // Q[a][C]: weight of coarse corner C at fine node a of the fine element at local (px,py,pz)
  for (int a = 0; a < 8; ++a) {
    int q[3] = {px + a % 2, py + a / 2 % 2, pz + a / 4};
    for (int C = 0; C < 8; ++C) {
      int cc[3] = {C % 2, C / 2 % 2, C / 4};
      double w = 1;
      for (int k = 0; k < 3; ++k) w *= cc[k] ? (double)q[k] / fct : (double)(fct - q[k]) / fct;
      Q[a][C] = w;
    }
  }
}

static void accumulate_QtKQ(const double Q[8][8], const double* K, double scale, double* out) {
  // out(24x24) += scale * (Q (x) I3)^T K (Q (x) I3)
  double T[24][24];  // K (Q(x)I3): [row][3C+j]
  for (int r = 0; r < 24; ++r)
    for (int C = 0; C < 8; ++C)
      for (int j = 0; j < 3; ++j) {
        double s = 0;
        for (int b = 0; b < 8; ++b) s += K[r * 24 + 3 * b + j] * Q[b][C];
        T[r][3 * C + j] = s;
      }
  for (int A = 0; A < 8; ++A)
    for (int i = 0; i < 3; ++i)
      for (int col = 0; col < 24; ++col) {
        double s = 0;
        for (int a = 0; a < 8; ++a) s += Q[a][A] * T[3 * a + i][col];
        out[(3 * A + i) * 24 + col] += scale * s;
      }
}

static void galerkin_first(orc_problem* p) {
  const Level& Fl = p->lv[0];
  Level& C = p->lv[1];
  int fct = C.factor;
  C.kel.assign(576 * C.ne, 0.0);
#pragma omp parallel for collapse(2) schedule(dynamic, 4)
  for (int cz = 0; cz < C.ez; ++cz)
    for (int cy = 0; cy < C.ey; ++cy)
      for (int cx = 0; cx < C.ex; ++cx) {
        int64_t ce = C.eid(cx, cy, cz);
        if (!C.eactive[ce]) continue;
        double* out = &C.kel[576 * ce];
        for (int pz = 0; pz < fct; ++pz)
          for (int py = 0; py < fct; ++py)
            for (int px = 0; px < fct; ++px) {
              int fx = cx * fct + px, fy = cy * fct + py, fz = cz * fct + pz;
              if (fx >= Fl.ex || fy >= Fl.ey || fz >= Fl.ez) continue;
              int64_t fe = Fl.eid(fx, fy, fz);
              if (!Fl.eactive[fe]) continue;
              double Q[8][8];
              interp_weights(fct, px, py, pz, Q);
              double Kt[576];
              uint8_t freedof[24];
              for (int a = 0; a < 8; ++a) {
                int64_t v = Fl.vid(fx + a % 2, fy + a / 2 % 2, fz + a / 4);
                for (int c = 0; c < 3; ++c) freedof[3 * a + c] = (Fl.vmask[v] >> c) & 1;
              }
              double pe = p->rhop[fe];
              for (int r = 0; r < 24; ++r)
                for (int s = 0; s < 24; ++s) {
                  double k = pe * p->Ke[r * 24 + s];
                  if (!freedof[r] || !freedof[s]) k = (r == s) ? kDirichletWeight : 0.0;
                  Kt[r * 24 + s] = k;
                }
              accumulate_QtKQ(Q, Kt, 1.0, out);
            }
      }
}

static void galerkin_dyadic(orc_problem* p, int lc) {
  const Level& Fl = p->lv[lc - 1];
  Level& C = p->lv[lc];
  C.kel.assign(576 * C.ne, 0.0);
  double Qs[8][8][8];
  for (int c = 0; c < 8; ++c) interp_weights(2, c % 2, c / 2 % 2, c / 4, Qs[c]);
#pragma omp parallel for collapse(2) schedule(dynamic, 4)
  for (int cz = 0; cz < C.ez; ++cz)
    for (int cy = 0; cy < C.ey; ++cy)
      for (int cx = 0; cx < C.ex; ++cx) {
        int64_t ce = C.eid(cx, cy, cz);
        if (!C.eactive[ce]) continue;
        double* out = &C.kel[576 * ce];
        for (int c = 0; c < 8; ++c) {
          int fx = 2 * cx + c % 2, fy = 2 * cy + c / 2 % 2, fz = 2 * cz + c / 4;
          if (fx >= Fl.ex || fy >= Fl.ey || fz >= Fl.ez) continue;
          int64_t fe = Fl.eid(fx, fy, fz);
          if (!Fl.eactive[fe]) continue;
          accumulate_QtKQ(Qs[c], &Fl.kel[576 * fe], 1.0, out);
        }
      }
}

static void assemble_stencil(Level& L) {
  L.stencil.assign(243 * L.nv, 0.0);
#pragma omp parallel for collapse(2) schedule(static)
  for (int z = 0; z < L.vz; ++z)
    for (int y = 0; y < L.vy; ++y)
      for (int x = 0; x < L.vx; ++x) {
        int64_t v = L.vid(x, y, z);
        for (int w = 0; w < 8; ++w) {
          int ex = x - 1 + w % 2, ey = y - 1 + w / 2 % 2, ez = z - 1 + w / 4;
          if (ex < 0 || ey < 0 || ez < 0 || ex >= L.ex || ey >= L.ey || ez >= L.ez) continue;
          int64_t e = L.eid(ex, ey, ez);
          if (!L.eactive[e]) continue;
          int a = 7 - w;
          const double* K = &L.kel[576 * e];
          for (int b = 0; b < 8; ++b) {
            // neighbour offset of node b relative to v
            int dx = (b % 2) - (a % 2), dy = (b / 2 % 2) - (a / 2 % 2), dz = (b / 4) - (a / 4);
            int d = (dx + 1) + 3 * (dy + 1) + 9 * (dz + 1);
            for (int i = 0; i < 3; ++i)
              for (int j = 0; j < 3; ++j)
                L.stencil[(d * 9 + 3 * i + j) * L.nv + v] += K[(3 * a + i) * 24 + 3 * b + j];
          }
        }
        if (!(L.vmask[v] & 0x8))
          for (int i = 0; i < 3; ++i) L.stencil[(13 * 9 + 4 * i) * L.nv + v] = 1.0;
      }
}

// Coarsest level: dense matrix from the stencil (grid/Grid.cpp:3614-3669), Cholesky.
static void factor_coarsest(orc_problem* p) {
  Level& L = p->lv.back();
  int n = (int)(3 * L.nv);
  p->nc_dense = n;
  std::vector<double> A((size_t)n * n, 0.0);
  for (int z = 0; z < L.vz; ++z)
    for (int y = 0; y < L.vy; ++y)
      for (int x = 0; x < L.vx; ++x) {
        int64_t v = L.vid(x, y, z);
        for (int d = 0; d < 27; ++d) {
          int nx_ = x + d % 3 - 1, ny_ = y + d / 3 % 3 - 1, nz_ = z + d / 9 - 1;
          if (nx_ < 0 || ny_ < 0 || nz_ < 0 || nx_ >= L.vx || ny_ >= L.vy || nz_ >= L.vz) continue;
          int64_t nb = L.vid(nx_, ny_, nz_);
          for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j)
              A[(size_t)(3 * v + i) * n + 3 * nb + j] = L.stencil[(d * 9 + 3 * i + j) * L.nv + v];
        }
      }
  // symmetrise (the assembled operator is symmetric up to roundoff)
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < i; ++j) {
      double s = 0.5 * (A[(size_t)i * n + j] + A[(size_t)j * n + i]);
      A[(size_t)i * n + j] = A[(size_t)j * n + i] = s;
    }
  // Cholesky; a pivot below 1e-10 of the largest diagonal entry is a null
  // direction (floating part): the DOF is dropped (row and column of L set to
  // e_k, right-hand side zeroed in the solve), i.e. the inverse of the
  // remaining DOFs, standing in for the reference's pseudo-inverse.
  double dmax = 0.0;
  for (int k = 0; k < n; ++k) dmax = std::max(dmax, std::fabs(A[(size_t)k * n + k]));
  const double tol = 1e-10 * dmax;
  p->dropped.assign(n, 0);
  for (int k = 0; k < n; ++k) {
    double d = A[(size_t)k * n + k];
    for (int j = 0; j < k; ++j) d -= A[(size_t)k * n + j] * A[(size_t)k * n + j];
    if (d <= tol) {
      p->dropped[k] = 1;
      for (int j = 0; j < k; ++j) A[(size_t)k * n + j] = 0.0;
      A[(size_t)k * n + k] = 1.0;
      for (int i = k + 1; i < n; ++i) A[(size_t)i * n + k] = 0.0;
      continue;
    }
    d = std::sqrt(d);
    A[(size_t)k * n + k] = d;
    for (int i = k + 1; i < n; ++i) {
      double s = A[(size_t)i * n + k];
      for (int j = 0; j < k; ++j) s -= A[(size_t)i * n + j] * A[(size_t)k * n + j];
      A[(size_t)i * n + k] = s / d;
    }
  }
  p->Lc.swap(A);
}

extern "C" void orc_coarsest_solve(orc_problem* p) {
  Level& L = p->lv.back();
  int n = p->nc_dense;
  std::vector<double> b(n);
  for (int64_t v = 0; v < L.nv; ++v)
    for (int c = 0; c < 3; ++c) b[3 * v + c] = L.F[c * L.nv + v];
  for (int i = 0; i < n; ++i)
    if (p->dropped[i]) b[i] = 0.0;
  const double* A = p->Lc.data();
  for (int i = 0; i < n; ++i) {
    double s = b[i];
    for (int j = 0; j < i; ++j) s -= A[(size_t)i * n + j] * b[j];
    b[i] = s / A[(size_t)i * n + i];
  }
  for (int i = n - 1; i >= 0; --i) {
    double s = b[i];
    for (int j = i + 1; j < n; ++j) s -= A[(size_t)j * n + i] * b[j];
    b[i] = s / A[(size_t)i * n + i];
  }
  for (int64_t v = 0; v < L.nv; ++v)
    for (int c = 0; c < 3; ++c) L.U[c * L.nv + v] = b[3 * v + c];
}

extern "C" void orc_update_penalised(orc_problem* p) {
  for (size_t e = 0; e < p->rho.size(); ++e)
    p->rhop[e] = p->lv[0].eactive[e] ? std::pow(p->rho[e], p->penal) : 0.0;
}

extern "C" void orc_update_operators(orc_problem* p) {
  orc_update_penalised(p);
  int nl = (int)p->lv.size();
  for (int l = 1; l < nl; ++l) {
    if (l == 1) galerkin_first(p); else galerkin_dyadic(p, l);
    assemble_stencil(p->lv[l]);
  }
  if (nl > 1) factor_coarsest(p);
  for (int l = 0; l < nl; ++l) p->lmax[l] = 0.0;
}

// ----------------------------------------------------------------------------
// V-cycle in the reference order (grid/Grid.cpp:2399-2444).  With `sym`, the
// post-smoothing runs the adjoint (reverse) sweep so the cycle is symmetric.
// smoother 0 = GS, 1 = Chebyshev.
// ----------------------------------------------------------------------------
static double vnorm(const std::vector<double>& a) {
  double s = 0;
#pragma omp parallel for reduction(+ : s)
  for (int64_t i = 0; i < (int64_t)a.size(); ++i) s += a[i] * a[i];
  return std::sqrt(s);
}

static void vcycle_core(orc_problem* p, int pre, int post, bool sym, int smoother,
                        std::vector<std::vector<double>>* dinv) {
  int nl = (int)p->lv.size();
  if (nl == 1) {
    // single level: smoothing only
    if (smoother == 1) for (int s = 0; s < pre + post; ++s) cheb_level(p, 0, (*dinv)[0]);
    else { smooth_level(p, 0, pre, false); smooth_level(p, 0, post, sym); }
    return;
  }
  for (int l = 0; l < nl; ++l) {
    if (l > 0) {
      level_residual(p, l - 1);
      orc_restrict(p, l);
      std::fill(p->lv[l].U.begin(), p->lv[l].U.end(), 0.0);
    }
    if (l < nl - 1) {
      if (smoother == 1) for (int s = 0; s < pre; ++s) cheb_level(p, l, (*dinv)[l]);
      else smooth_level(p, l, pre, false);
    } else {
      orc_coarsest_solve(p);
    }
  }
  for (int l = nl - 2; l >= 0; --l) {
    orc_prolong(p, l);
    if (smoother == 1) for (int s = 0; s < post; ++s) cheb_level(p, l, (*dinv)[l]);
    else smooth_level(p, l, post, sym);
  }
}

extern "C" double orc_vcycle(orc_problem* p, int pre, int post) {
  vcycle_core(p, pre, post, false, 0, nullptr);
  level_residual(p, 0);
  return vnorm(p->lv[0].R) / vnorm(p->lv[0].F);
}

static void prepare_cheb(orc_problem* p, std::vector<std::vector<double>>& dinv) {
  int nl = (int)p->lv.size();
  dinv.resize(nl);
  for (int l = 0; l < nl; ++l) {
    diag_blocks(p, l, dinv[l]);
    if (p->lmax[l] == 0.0) p->lmax[l] = level_lmax(p, l);
  }
}

// Flexible preconditioned CG (Polak-Ribiere beta) on level 0 with a symmetric
// V-cycle preconditioner.  No reference counterpart (the reference iterates
// V-cycles, utils/test_utils.cpp:937-941).  Warm start from U.
extern "C" int orc_pcg(orc_problem* p, int pre, int post, double rtol, int maxit, int smoother,
                       double* relres) {
  Level& L = p->lv[0];
  int64_t n3 = 3 * L.nv;
  std::vector<std::vector<double>> dinv;
  if (smoother == 1) prepare_cheb(p, dinv);
  std::vector<double> x = L.U, r(n3), z(n3), zold(n3), rold(n3), d(n3), q(n3);
  std::vector<double> f = L.F;
  double fn = vnorm(f);
  if (fn == 0) { std::fill(L.U.begin(), L.U.end(), 0.0); *relres = 0; return 0; }
  orc_apply_fine(p, x.data(), q.data());
  for (int64_t i = 0; i < n3; ++i) r[i] = f[i] - q[i];
  double rn = vnorm(r);
  int it = 0;
  double rz_old = 0;
  while (rn / fn > rtol && it < maxit) {
    // z = B r  (V-cycle with zero initial guess on the residual equation)
    L.F = r;
    std::fill(L.U.begin(), L.U.end(), 0.0);
    vcycle_core(p, pre, post, true, smoother, &dinv);
    z = L.U;
    double rz = 0;
    for (int64_t i = 0; i < n3; ++i) rz += r[i] * z[i];
    if (it == 0) {
      d = z;
    } else {
      double num = 0;
      for (int64_t i = 0; i < n3; ++i) num += z[i] * (r[i] - rold[i]);
      double beta = num / rz_old;
      for (int64_t i = 0; i < n3; ++i) d[i] = z[i] + beta * d[i];
    }
    orc_apply_fine(p, d.data(), q.data());
    double dq = 0;
    for (int64_t i = 0; i < n3; ++i) dq += d[i] * q[i];
    double alpha = rz / dq;
    rold = r;
    for (int64_t i = 0; i < n3; ++i) { x[i] += alpha * d[i]; r[i] -= alpha * q[i]; }
    rz_old = rz;
    rn = vnorm(r);
    ++it;
  }
  L.F = f;
  L.U = x;
  level_residual(p, 0);
  *relres = vnorm(L.R) / fn;
  return it;
}

extern "C" double orc_compliance(const orc_problem* p) {
  const Level& L = p->lv[0];
  double s = 0;
  for (int64_t i = 0; i < 3 * L.nv; ++i) s += L.F[i] * L.U[i];
  return s;
}

// ----------------------------------------------------------------------------
// Spline: knots (grid/Grid.cpp:3253-3337, float arithmetic), Cox-de Boor basis
// (grid/Grid.cu:384-466), density at element centres with clamp and the -0.2
// out-of-range value (grid/Grid.cu:3383-3436).
// ----------------------------------------------------------------------------
extern "C" void orc_set_spline(orc_problem* p, int order, const int* part, const double* bmin,
                               const double* bmax) {
  p->order = order;
  for (int a = 0; a < 3; ++a) {
    p->part[a] = part[a];
    p->nbasis[a] = order + part[a];
    float mn = (float)bmin[a], mx = (float)bmax[a];
    float delta = mx - mn;
    mx += 2.0f * delta / (float)(part[a] + 1);
    mn -= 2.0f * delta / (float)(part[a] + 1);
    float step = (mx - mn) / (float)(part[a] + 1);
    p->knots[a].clear();
    float tmp = mn;
    for (int i = 0; i < order; ++i) p->knots[a].push_back(mn);
    for (int i = 0; i < part[a]; ++i) { tmp += step; p->knots[a].push_back(tmp); }
    for (int i = 0; i < order; ++i) p->knots[a].push_back(mx);
    p->kmin[a] = mn;
    p->kstep[a] = step;
  }
  p->coeff.assign((size_t)p->nbasis[0] * p->nbasis[1] * p->nbasis[2], 0.0);
  p->csens.assign(p->coeff.size(), 0.0);
}

extern "C" int orc_num_coeffs(const orc_problem* p) {
  return p->nbasis[0] * p->nbasis[1] * p->nbasis[2];
}

extern "C" void orc_get_knots(const orc_problem* p, int axis, double* out) {
  std::copy(p->knots[axis].begin(), p->knots[axis].end(), out);
}

// Basis values at x: returns the first basis index (span - order + 1) or -1 out of range.
static int spline_basis(const orc_problem* p, int axis, double x, double* N) {
  int k = p->order;
  int i = (int)std::floor((x - p->kmin[axis]) / p->kstep[axis]) + k;  // grid/Grid.cu:3390-3392
  if (i < k || i > p->nbasis[axis]) return -1;
  int l = i - 1;  // span index
  const std::vector<double>& U = p->knots[axis];
  double left[8], right[8];
  N[0] = 1.0;
  for (int j = 1; j < k; ++j) {
    left[j] = x - U[l + 1 - j];
    right[j] = U[l + j] - x;
    double saved = 0.0;
    for (int r = 0; r < j; ++r) {
      double temp = N[r] / (right[r + 1] + left[j - r]);
      N[r] = saved + right[r + 1] * temp;
      saved = left[j - r] * temp;
    }
    N[j] = saved;
  }
  return i - k;
}

// Basis values at an arbitrary coordinate, for the golden vectors of the
// reference's SplineBasisX/Y/Z: N[order], returns the first basis index or -1.
extern "C" int orc_spline_basis(const orc_problem* p, int axis, double x, double* N) {
  return spline_basis(p, axis, x, N);
}

extern "C" void orc_coeff_to_density(orc_problem* p) {
  const Level& L = p->lv[0];
  int k = p->order;
#pragma omp parallel for collapse(2) schedule(static)
  for (int z = 0; z < L.ez; ++z)
    for (int y = 0; y < L.ey; ++y)
      for (int x = 0; x < L.ex; ++x) {
        int64_t e = L.eid(x, y, z);
        if (!L.eactive[e]) { p->rho[e] = 0.0; continue; }
        double pos[3] = {(x + 0.5) * p->h, (y + 0.5) * p->h, (z + 0.5) * p->h};
        double N[3][8];
        int i0[3];
        bool ok = true;
        for (int a = 0; a < 3; ++a) { i0[a] = spline_basis(p, a, pos[a], N[a]); ok = ok && i0[a] >= 0; }
        double val = -0.2;
        if (ok) {
          val = 0;
          for (int r = 0; r < k; ++r)
            for (int s = 0; s < k; ++s)
              for (int t = 0; t < k; ++t) {
                size_t idx = (i0[0] + r) + (size_t)p->nbasis[0] * ((i0[1] + s) + (size_t)p->nbasis[1] * (i0[2] + t));
                val += p->coeff[idx] * N[0][r] * N[1][s] * N[2][t];
              }
        }
        p->rho[e] = std::min(std::max(val, p->rho_min), 1.0);
      }
}

// Spline adjoint (grid/Grid.cu:3671-3724): dc_ijk = sum_e g_e N_i N_j N_k over
// in-range elements, ignoring the clamp.  Restated as a deterministic sum.
extern "C" void orc_spline_adjoint(orc_problem* p) {
  const Level& L = p->lv[0];
  int k = p->order;
  std::fill(p->csens.begin(), p->csens.end(), 0.0);
  for (int z = 0; z < L.ez; ++z)
    for (int y = 0; y < L.ey; ++y)
      for (int x = 0; x < L.ex; ++x) {
        int64_t e = L.eid(x, y, z);
        if (!L.eactive[e]) continue;
        double pos[3] = {(x + 0.5) * p->h, (y + 0.5) * p->h, (z + 0.5) * p->h};
        double N[3][8];
        int i0[3];
        bool ok = true;
        for (int a = 0; a < 3; ++a) { i0[a] = spline_basis(p, a, pos[a], N[a]); ok = ok && i0[a] >= 0; }
        if (!ok) continue;
        double g = p->sens[e];
        for (int r = 0; r < k; ++r)
          for (int s = 0; s < k; ++s)
            for (int t = 0; t < k; ++t) {
              size_t idx = (i0[0] + r) + (size_t)p->nbasis[0] * ((i0[1] + s) + (size_t)p->nbasis[1] * (i0[2] + t));
              p->csens[idx] += g * N[0][r] * N[1][s] * N[2][t];
            }
      }
}

// Volume: sum(rho) / n_gselements (grid/Grid.cu:5462-5470, denominator with the
// per-colour Round<32> padding of grid/Grid.cpp:4129-4137) or / active count.
static int64_t gs_padded_elements(const Level& L) {
  int64_t cnt[8] = {0};
  for (int z = 0; z < L.ez; ++z)
    for (int y = 0; y < L.ey; ++y)
      for (int x = 0; x < L.ex; ++x)
        if (L.eactive[L.eid(x, y, z)]) cnt[x % 2 + 2 * (y % 2) + 4 * (z % 2)]++;
  int64_t s = 0;
  for (int c = 0; c < 8; ++c) s += (cnt[c] + 31) / 32 * 32;
  return s;
}

extern "C" double orc_volume(const orc_problem* p, int refden) {
  const Level& L = p->lv[0];
  double s = 0;
  int64_t n = 0;
  for (int64_t e = 0; e < L.ne; ++e)
    if (L.eactive[e]) { s += p->rho[e]; ++n; }
  return s / (double)(refden ? gs_padded_elements(L) : n);
}

// Sensitivity g_e = -p rho^(p-1) u_e^T Ke u_e (optimization/optimization.cu:96-159).
extern "C" void orc_sensitivity(orc_problem* p) {
  const Level& L = p->lv[0];
#pragma omp parallel for collapse(2) schedule(static)
  for (int z = 0; z < L.ez; ++z)
    for (int y = 0; y < L.ey; ++y)
      for (int x = 0; x < L.ex; ++x) {
        int64_t e = L.eid(x, y, z);
        if (!L.eactive[e]) { p->sens[e] = 0.0; continue; }
        double ue[24];
        for (int a = 0; a < 8; ++a) {
          int64_t v = L.vid(x + a % 2, y + a / 2 % 2, z + a / 4);
          for (int c = 0; c < 3; ++c) ue[3 * a + c] = masked_u(L, L.U.data(), v, c);
        }
        double q = 0;
        for (int i = 0; i < 24; ++i) {
          double s = 0;
          for (int j = 0; j < 24; ++j) s += p->Ke[i * 24 + j] * ue[j];
          q += ue[i] * s;
        }
        p->sens[e] = -p->penal * std::pow(p->rho[e], p->penal - 1) * q;
      }
}

// Sensitivity filter (grid/Grid.cu:4130-4229): normalised average over the ball
// r^2 <= R^2 with R_int = floor(R + 0.5), weight 1 - 6s^2 + 8s^3 - 3s^4, s = r/R.
extern "C" void orc_filter(orc_problem* p, double R) {
  const Level& L = p->lv[0];
  std::vector<double> src = p->sens;
  int Ri = (int)(R + 0.5);
  double R2 = R * R;
#pragma omp parallel for collapse(2) schedule(static)
  for (int z = 0; z < L.ez; ++z)
    for (int y = 0; y < L.ey; ++y)
      for (int x = 0; x < L.ex; ++x) {
        int64_t e = L.eid(x, y, z);
        if (!L.eactive[e]) { p->sens[e] = 0.0; continue; }
        double ws = 0, gs = 0;
        for (int dx = -Ri; dx <= Ri; ++dx) {
          int nx_ = x + dx;
          if (nx_ < 0 || nx_ >= L.ex) continue;
          for (int dy = -Ri; dy <= Ri; ++dy) {
            int ny_ = y + dy;
            if (ny_ < 0 || ny_ >= L.ey) continue;
            for (int dz = -Ri; dz <= Ri; ++dz) {
              int nz_ = z + dz;
              if (nz_ < 0 || nz_ >= L.ez) continue;
              double r2 = dx * dx + dy * dy + dz * dz;
              if (r2 > R2) continue;
              int64_t n = L.eid(nx_, ny_, nz_);
              if (!L.eactive[n]) continue;
              double s = std::sqrt(r2 / R2), s2 = s * s;
              double w = 1 - 6 * s2 + 8 * s2 * s - 3 * s2 * s2;
              gs += w * src[n];
              ws += w;
            }
          }
        }
        p->sens[e] = gs / ws;
      }
}

// OC on coefficients with bisection on the threshold (optimization/optimization.cu:559-695).
static void oc_trial(const orc_problem* p, const std::vector<double>& cold, double thres,
                     double damp, double step, double cmin, double cmax, std::vector<double>& out) {
  for (size_t i = 0; i < cold.size(); ++i) {
    double c = p->csens[i];
    if (c > 0) c = 0;
    c = std::fabs(c);
    double cn = cold[i] * std::pow(c / thres, damp);
    cn = std::min(std::max(cn, cold[i] - step), cold[i] + step);
    cn = std::min(std::max(cn, cmin), cmax);
    out[i] = cn;
  }
}

extern "C" int orc_oc_update(orc_problem* p, double vgoal, double damp, double step, double cmin,
                             double cmax, int apply_twice, int refden, double* lambda_out) {
  double gmax = 0;
  for (double c : p->csens) gmax = std::max(gmax, std::fabs(c));
  double lo = 0, hi = gmax, thres = 0.5 * (lo + hi);
  std::vector<double> cold = p->coeff, trial(cold.size());
  int itn = 0, trials = 0;
  double V;
  do {
    thres = 0.5 * (lo + hi);
    oc_trial(p, cold, thres, damp, step, cmin, cmax, trial);
    p->coeff = trial;
    orc_coeff_to_density(p);
    V = orc_volume(p, refden);
    ++trials;
    if (V > vgoal) lo = thres;
    else if (V < vgoal) hi = thres;
  } while (std::fabs(V - vgoal) > 1e-4 && itn++ < 30);
  if (apply_twice) {
    std::vector<double> again(cold.size());
    oc_trial(p, p->coeff, thres, damp, step, cmin, cmax, again);
    p->coeff = again;
  }
  orc_coeff_to_density(p);
  if (lambda_out) *lambda_out = thres;
  return trials;
}

// ----------------------------------------------------------------------------
// Reference GS ordering (grid/Grid.cpp:4104-4165 with colours from
// grid/Grid.cu:1286-1328): colour subsets in colour order, each padded to a
// multiple of 32, lexicographic order within a colour.
// ----------------------------------------------------------------------------
extern "C" int orc_gs_maps(const orc_problem* p, int l, int* vidmap, int* eidmap, int* gs_num8,
                           int* n_gse) {
  const Level& L = p->lv[l];
  int64_t nvs[8] = {0}, nes[8] = {0};
  for (int z = 0; z < L.vz; ++z)
    for (int y = 0; y < L.vy; ++y)
      for (int x = 0; x < L.vx; ++x)
        if (L.vmask[L.vid(x, y, z)] & 0x8) nvs[x % 2 + 2 * (y % 2) + 4 * (z % 2)]++;
  for (int z = 0; z < L.ez; ++z)
    for (int y = 0; y < L.ey; ++y)
      for (int x = 0; x < L.ex; ++x)
        if (L.eactive[L.eid(x, y, z)]) nes[x % 2 + 2 * (y % 2) + 4 * (z % 2)]++;
  int64_t voff[8], eoff[8], vt = 0, et = 0;
  for (int c = 0; c < 8; ++c) {
    voff[c] = vt; eoff[c] = et;
    int64_t pv = (nvs[c] + 31) / 32 * 32, pe = (nes[c] + 31) / 32 * 32;
    if (gs_num8) gs_num8[c] = (int)pv;
    vt += pv; et += pe;
  }
  int64_t cntv[8] = {0}, cnte[8] = {0};
  int64_t lv_ = 0;
  for (int z = 0; z < L.vz; ++z)
    for (int y = 0; y < L.vy; ++y)
      for (int x = 0; x < L.vx; ++x)
        if (L.vmask[L.vid(x, y, z)] & 0x8) {
          int c = x % 2 + 2 * (y % 2) + 4 * (z % 2);
          if (vidmap) vidmap[lv_] = (int)(voff[c] + cntv[c]);
          cntv[c]++; lv_++;
        }
  int64_t le = 0;
  for (int z = 0; z < L.ez; ++z)
    for (int y = 0; y < L.ey; ++y)
      for (int x = 0; x < L.ex; ++x)
        if (L.eactive[L.eid(x, y, z)]) {
          int c = x % 2 + 2 * (y % 2) + 4 * (z % 2);
          if (eidmap) eidmap[le] = (int)(eoff[c] + cnte[c]);
          cnte[c]++; le++;
        }
  if (n_gse) *n_gse = (int)et;
  return (int)vt;
}

// ----------------------------------------------------------------------------
// Array access.
// ----------------------------------------------------------------------------
extern "C" int64_t orc_size(const orc_problem* p, int which, int l) {
  const Level& L = p->lv[l];
  switch (which) {
    case ORC_RHO: case ORC_RHOP: case ORC_SENS: return p->lv[0].ne;
    case ORC_COEFF: case ORC_CSENS: return (int64_t)p->coeff.size();
    case ORC_U: case ORC_F: case ORC_R: return 3 * L.nv;
    case ORC_STENCIL: return 243 * L.nv;
    case ORC_KELEM: return 576 * L.ne;
    case ORC_VMASK: return L.nv;
    case ORC_EACTIVE: return L.ne;
    case ORC_KE: return 576;
    case ORC_DIAG: return 9 * L.nv;
  }
  return 0;
}

extern "C" void orc_put(orc_problem* p, int which, int l, const void* src) {
  Level& L = p->lv[l];
  const double* d = (const double*)src;
  int64_t n = orc_size(p, which, l);
  switch (which) {
    case ORC_RHO: std::copy(d, d + n, p->rho.begin()); break;
    case ORC_RHOP: std::copy(d, d + n, p->rhop.begin()); break;
    case ORC_COEFF: std::copy(d, d + n, p->coeff.begin()); break;
    case ORC_SENS: std::copy(d, d + n, p->sens.begin()); break;
    case ORC_CSENS: std::copy(d, d + n, p->csens.begin()); break;
    case ORC_U: std::copy(d, d + n, L.U.begin()); break;
    case ORC_F: std::copy(d, d + n, L.F.begin()); break;
    case ORC_R: std::copy(d, d + n, L.R.begin()); break;
    default: break;
  }
}

extern "C" void orc_get(const orc_problem* p, int which, int l, void* dst) {
  const Level& L = p->lv[l];
  double* d = (double*)dst;
  switch (which) {
    case ORC_RHO: std::copy(p->rho.begin(), p->rho.end(), d); break;
    case ORC_RHOP: std::copy(p->rhop.begin(), p->rhop.end(), d); break;
    case ORC_COEFF: std::copy(p->coeff.begin(), p->coeff.end(), d); break;
    case ORC_SENS: std::copy(p->sens.begin(), p->sens.end(), d); break;
    case ORC_CSENS: std::copy(p->csens.begin(), p->csens.end(), d); break;
    case ORC_U: std::copy(L.U.begin(), L.U.end(), d); break;
    case ORC_F: std::copy(L.F.begin(), L.F.end(), d); break;
    case ORC_R: std::copy(L.R.begin(), L.R.end(), d); break;
    case ORC_STENCIL: std::copy(L.stencil.begin(), L.stencil.end(), d); break;
    case ORC_KELEM: std::copy(L.kel.begin(), L.kel.end(), d); break;
    case ORC_VMASK: std::copy(L.vmask.begin(), L.vmask.end(), (uint8_t*)dst); break;
    case ORC_EACTIVE: std::copy(L.eactive.begin(), L.eactive.end(), (uint8_t*)dst); break;
    case ORC_KE: std::copy(p->Ke, p->Ke + 576, d); break;
    case ORC_DIAG: {
      std::vector<double> Dinv;
      orc_problem* pp = const_cast<orc_problem*>(p);
      (void)pp;
      // raw diagonal blocks (not inverted) in [9][nv]
      for (int64_t i = 0; i < 9 * L.nv; ++i) d[i] = 0;
      if (l > 0) {
        for (int k = 0; k < 9; ++k)
          for (int64_t v = 0; v < L.nv; ++v) d[k * L.nv + v] = L.stencil[(13 * 9 + k) * L.nv + v];
      }
      break;
    }
  }
}
