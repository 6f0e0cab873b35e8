// Host-side set-up: element template, multigrid hierarchy, spline knots,
// Galerkin transfer tables and the reference's GS-padded counts.
#include <algorithm>
#include <cmath>
#include <cstring>

#include "topo_internal.h"

namespace topo {

// 24x24 trilinear-hex stiffness, integrated exactly with 1-D integrals.
// Same operator as the 2x2x2 Gauss rule of element/templateMatrix.cpp:31-99
// (Gauss-2 is exact for the bi-quadratic integrand): node a = ax+2ay+4az,
// DOF 3a+c, Ke[(a,i),(b,j)] = sum_kl C_ikjl int dN_a/dx_k dN_b/dx_l.
void element_template(double E, double nu, double h, double* Ke) {
  const double lam = E * nu / ((1 + nu) * (1 - 2 * nu));
  const double mu = E / (2 * (1 + nu));
  // 1-D integrals on [0,h] of the hat functions phi0 = 1-t/h, phi1 = t/h
  auto mass = [&](int a, int b) { return h * (a == b ? 1.0 / 3.0 : 1.0 / 6.0); };
  auto stiff = [&](int a, int b) { return (a == b ? 1.0 : -1.0) / h; };
  auto dl = [&](int a, int /*b*/) { return (2 * a - 1) / 2.0; };  // int phi_a' phi_b
  auto dr = [&](int /*a*/, int b) { return (2 * b - 1) / 2.0; };  // int phi_a phi_b'
  auto G = [&](int a, int b, int k, int l) {
    int pa[3] = {a % 2, a / 2 % 2, a / 4}, pb[3] = {b % 2, b / 2 % 2, b / 4};
    double g = 1.0;
    for (int m = 0; m < 3; ++m) {
      if (m == k && m == l) g *= stiff(pa[m], pb[m]);
      else if (m == k) g *= dl(pa[m], pb[m]);
      else if (m == l) g *= dr(pa[m], pb[m]);
      else g *= mass(pa[m], pb[m]);
    }
    return g;
  };
  for (int a = 0; a < 8; ++a)
    for (int b = 0; b < 8; ++b)
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
          double s = 0;
          for (int k = 0; k < 3; ++k)
            for (int l = 0; l < 3; ++l) {
              double C = lam * (i == k) * (j == l) + mu * ((i == j) * (k == l) + (i == l) * (k == j));
              if (C != 0) s += C * G(a, b, k, l);
            }
          Ke[(3 * a + i) * 24 + 3 * b + j] = s;
        }
}

static void finish(LevelDims& d) {
  d.vx = d.ex + 1; d.vy = d.ey + 1; d.vz = d.ez + 1;
  d.ne = (int64_t)d.ex * d.ey * d.ez;
  d.nv = (int64_t)d.vx * d.vy * d.vz;
}

static std::vector<uint8_t> vertex_active(const LevelDims& d, const std::vector<uint8_t>& ea) {
  std::vector<uint8_t> va(d.nv, 0);
  for (int z = 0; z < d.ez; ++z)
    for (int y = 0; y < d.ey; ++y)
      for (int x = 0; x < d.ex; ++x)
        if (ea[x + (int64_t)d.ex * (y + (int64_t)d.ey * z)])
          for (int a = 0; a < 8; ++a)
            va[(x + a % 2) + (int64_t)d.vx * ((y + a / 2 % 2) + (int64_t)d.vy * (z + a / 4))] = 0x8;
  return va;
}

static void coarsen(const LevelDims& f, const std::vector<uint8_t>& fa, int factor, LevelDims& c,
                    std::vector<uint8_t>& ca) {
  c.ex = (f.ex + factor - 1) / factor;
  c.ey = (f.ey + factor - 1) / factor;
  c.ez = (f.ez + factor - 1) / factor;
  c.factor = factor;
  finish(c);
  ca.assign(c.ne, 0);
  for (int z = 0; z < f.ez; ++z)
    for (int y = 0; y < f.ey; ++y)
      for (int x = 0; x < f.ex; ++x)
        if (fa[x + (int64_t)f.ex * (y + (int64_t)f.ey * z)])
          ca[x / factor + (int64_t)c.ex * (y / factor + (int64_t)c.ey * (z / factor))] = 1;
}

// Level list per grid/Grid.cpp:747-769 (child-OR coarsening while the active
// element count exceeds max_coarse); the reference's dummy level 1 is skipped
// so the first used coarse level is 4x coarser (grid/Grid.cpp:909-911).
Hierarchy build_hierarchy(int nx, int ny, int nz, const uint8_t* eactive, int max_coarse) {
  Hierarchy H;
  LevelDims d0{};
  d0.ex = nx; d0.ey = ny; d0.ez = nz; d0.factor = 1;
  finish(d0);
  std::vector<uint8_t> a0(d0.ne, 1);
  if (eactive)
    for (int64_t i = 0; i < d0.ne; ++i) a0[i] = eactive[i] ? 1 : 0;
  // count reference levels (including level 1)
  int nref = 1;
  {
    LevelDims cur = d0;
    std::vector<uint8_t> ca = a0;
    while (true) {
      int64_t cnt = 0;
      for (auto v : ca) cnt += v;
      if (cnt <= max_coarse) break;
      LevelDims nd{};
      std::vector<uint8_t> na;
      coarsen(cur, ca, 2, nd, na);
      cur = nd;
      ca.swap(na);
      ++nref;
    }
  }
  H.dims.push_back(d0);
  H.eactive.push_back(a0);
  if (nref >= 3) {
    LevelDims c{};
    std::vector<uint8_t> ca;
    coarsen(d0, a0, 4, c, ca);
    H.dims.push_back(c);
    H.eactive.push_back(ca);
    for (int i = 3; i < nref; ++i) {
      LevelDims n{};
      std::vector<uint8_t> na;
      coarsen(H.dims.back(), H.eactive.back(), 2, n, na);
      H.dims.push_back(n);
      H.eactive.push_back(na);
    }
  } else if (nref == 2) {
    LevelDims c{};
    std::vector<uint8_t> ca;
    coarsen(d0, a0, 2, c, ca);
    H.dims.push_back(c);
    H.eactive.push_back(ca);
  }
  for (size_t l = 0; l < H.dims.size(); ++l) H.vactive.push_back(vertex_active(H.dims[l], H.eactive[l]));
  return H;
}

void fine_tile_zrange(const LevelDims& d, const uint8_t* eactive, std::vector<int2>& out) {
  // lowest / highest active z per element column (x, y)
  std::vector<int> lo((size_t)d.ex * d.ey, d.ez), hi((size_t)d.ex * d.ey, -1);
  for (int z = 0; z < d.ez; ++z)
    for (int y = 0; y < d.ey; ++y)
      for (int x = 0; x < d.ex; ++x)
        if (eactive[x + (int64_t)d.ex * (y + (int64_t)d.ey * z)]) {
          const size_t c = x + (size_t)d.ex * y;
          if (lo[c] > z) lo[c] = z;
          hi[c] = z;
        }
  const int tx = (d.vx + FINE_TILE_X - 2) / (FINE_TILE_X - 1), ty = (d.vy + FINE_TILE_Y - 2) / (FINE_TILE_Y - 1);
  out.assign((size_t)tx * ty, make_int2(d.ez, -1));
  for (int by = 0; by < ty; ++by)
    for (int bx = 0; bx < tx; ++bx) {
      int2 r = make_int2(d.ez, -1);
      // the tile's element columns: x0 - 1 .. x0 + FINE_TILE_X - 2 (same in y)
      const int x0 = bx * (FINE_TILE_X - 1), y0 = by * (FINE_TILE_Y - 1);
      for (int y = std::max(0, y0 - 1); y <= std::min(d.ey - 1, y0 + FINE_TILE_Y - 2); ++y)
        for (int x = std::max(0, x0 - 1); x <= std::min(d.ex - 1, x0 + FINE_TILE_X - 2); ++x) {
          const size_t c = x + (size_t)d.ex * y;
          r.x = std::min(r.x, lo[c]);
          r.y = std::max(r.y, hi[c]);
        }
      out[bx + (size_t)tx * by] = r;
    }
}

// Knot vector per grid/Grid.cpp:3253-3337: the box is enlarged by
// 2*delta/(p+1) on each side, step = extent/(p+1); order copies of each end
// and p interior knots accumulated in float, as the reference does.
void spline_knots(int order, int partition, double bmin, double bmax, std::vector<double>& knots,
                  double& kmin, double& kstep) {
  volatile float mn = (float)bmin, mx = (float)bmax;
  float delta = mx - mn;
  float grow = 2.0f * delta / (float)(partition + 1);
  mx = mx + grow;
  mn = mn - grow;
  float step = (mx - mn) / (float)(partition + 1);
  knots.clear();
  for (int i = 0; i < order; ++i) knots.push_back(mn);
  volatile float tmp = mn;
  for (int i = 0; i < partition; ++i) {
    tmp = tmp + step;
    knots.push_back(tmp);
  }
  for (int i = 0; i < order; ++i) knots.push_back(mx);
  kmin = mn;
  kstep = step;
}

void interp_weights(int fct, int px, int py, int pz, double Q[8][8]) {
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

// T[pos][576] = (Q_pos (x) I3)^T Ke (Q_pos (x) I3) for every fine-element
// position inside a coarse element (factor^3 positions).
void galerkin_tables(const double* Ke, int fct, std::vector<double>& T) {
  int npos = fct * fct * fct;
  T.assign((size_t)npos * 576, 0.0);
  for (int pos = 0; pos < npos; ++pos) {
    double Q[8][8];
    interp_weights(fct, pos % fct, pos / fct % fct, pos / (fct * fct), Q);
    double KQ[24][24];
    for (int r = 0; r < 24; ++r)
      for (int C = 0; C < 8; ++C)
        for (int j = 0; j < 3; ++j) {
          double s = 0;
          for (int b = 0; b < 8; ++b) s += Ke[r * 24 + 3 * b + j] * Q[b][C];
          KQ[r][3 * C + j] = s;
        }
    for (int A = 0; A < 8; ++A)
      for (int i = 0; i < 3; ++i)
        for (int col = 0; col < 24; ++col) {
          double s = 0;
          for (int a = 0; a < 8; ++a) s += Q[a][A] * KQ[3 * a + i][col];
          T[(size_t)pos * 576 + (3 * A + i) * 24 + col] = s;
        }
  }
}

// Element (or vertex) count with each parity colour padded to a multiple of 32
// (grid/Grid.cpp:4129-4137).
int64_t gs_padded_count(const LevelDims& d, const uint8_t* active, bool vertices) {
  int64_t cnt[8] = {0};
  int X = vertices ? d.vx : d.ex, Y = vertices ? d.vy : d.ey, Z = vertices ? d.vz : d.ez;
  for (int z = 0; z < Z; ++z)
    for (int y = 0; y < Y; ++y)
      for (int x = 0; x < X; ++x) {
        int64_t i = x + (int64_t)X * (y + (int64_t)Y * z);
        bool on = vertices ? (active[i] & 0x8) != 0 : active[i] != 0;
        if (on) cnt[x % 2 + 2 * (y % 2) + 4 * (z % 2)]++;
      }
  int64_t s = 0;
  for (int c = 0; c < 8; ++c) s += (cnt[c] + 31) / 32 * 32;
  return s;
}

}  // namespace topo

namespace topo {

// Basis tables at element centres (x+0.5)h: first basis index from the span
// formula of grid/Grid.cu:3390-3392 (-1 when out of range, the reference's -0.2
// branch) and the Cox-de Boor values of grid/Grid.cu:384-466.
void spline_tables(int order, const int* partition, const double* bmin, const double* bmax,
                   const int* nelem, double h, SplineTables& t) {
  t.order = order;
  for (int a = 0; a < 3; ++a) {
    t.nb[a] = order + partition[a];
    spline_knots(order, partition[a], bmin[a], bmax[a], t.knots[a], t.kmin[a], t.kstep[a]);
    const std::vector<double>& U = t.knots[a];
    t.i0[a].assign(nelem[a], -1);
    t.N[a].assign((size_t)nelem[a] * order, 0.0);
    for (int x = 0; x < nelem[a]; ++x) {
      const double pos = (x + 0.5) * h;
      const int i = (int)std::floor((pos - t.kmin[a]) / t.kstep[a]) + order;
      if (i < order || i > t.nb[a]) continue;
      const int l = i - 1;
      double N[8], left[8], right[8];
      N[0] = 1.0;
      for (int j = 1; j < order; ++j) {
        left[j] = pos - U[l + 1 - j];
        right[j] = U[l + j] - pos;
        double saved = 0.0;
        for (int r = 0; r < j; ++r) {
          const double temp = N[r] / (right[r + 1] + left[j - r]);
          N[r] = saved + right[r + 1] * temp;
          saved = left[j - r] * temp;
        }
        N[j] = saved;
      }
      t.i0[a][x] = i - order;
      for (int r = 0; r < order; ++r) t.N[a][(size_t)x * order + r] = N[r];
    }
    t.lo[a].assign(t.nb[a], 0);
    t.hi[a].assign(t.nb[a], 0);
    for (int b = 0; b < t.nb[a]; ++b) {
      int lo = -1, hi = -1;
      for (int x = 0; x < nelem[a]; ++x) {
        const int i0 = t.i0[a][x];
        if (i0 < 0 || b < i0 || b >= i0 + order) continue;
        if (lo < 0) lo = x;
        hi = x + 1;
      }
      t.lo[a][b] = lo < 0 ? 0 : lo;
      t.hi[a][b] = hi < 0 ? 0 : hi;
    }
  }
}

}  // namespace topo
