// Heaviside projection of the density and the additive-manufacturing
// constraints of the reference's MMA path (testOrdinarySplineTopoptMMA,
// utils/test_utils.cpp:972-1217): self-support (overhang) and drip.
//
// Projection (optimization/optimization.cu:161-183, 313-353):
//   rho = clamp(H(rho0), rho_min, 1), H(s) = (tanh(b eta) + tanh(b (s - eta))) /
//   (tanh(b eta) + tanh(b (1 - eta))), eta = 1/2, and the chain rule
//   dH/ds = b (1 - tanh^2(b (s - eta))) / (tanh(b eta) + tanh(b (1 - eta)))
//   on the compliance and volume sensitivities before the filter
//   (computeSensitivity2, optimization/optimization.cu:243-311).
//
// Constraints (deal_surface_points, optimization/optimization.cpp:1103-1127;
// grid/Grid.cu:5529-7156): points on the spline's 1/2 level set, the spline
// gradient as their normal, per point an overhang measure of the normal's
// angle with the build direction and a drip measure from the Hessian, the
// mean over the points, and its derivative with respect to the coefficients
// (points held fixed).  The reference finds the points with marching cubes on
// a (64 + 2)^3 lattice of spline values over the part's box and keeps those
// inside the mesh by CGAL ray tests (grid/Grid.cpp:3722-4032).  Here the
// points are the same lattice's edge crossings (the marching-cubes vertex
// positions), kept when they lie in an active element of the domain, taken in
// lattice order and thinned to at most max_points by the reference's
// equidistant pick; all of it runs on the GPU (crossing flags, stable
// compaction, per-point evaluation), and the coefficient gradient is
// accumulated deterministically: per-point contributions are sorted by
// coefficient with a stable radix sort and each coefficient sums its run in
// point order (the reference's scatter `dc[index] += val` races).
#include <algorithm>
#include <cmath>
#include <memory>
#include <vector>

#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_select.cuh>

#include "handle.h"

using namespace topo;

namespace topo {

constexpr int kSupMaxOrder = 4;

struct SupportState {
  // spline as seen by the point kernels
  double* knots = nullptr;       // device [3][kcap] knot vectors
  int kcap = 0;
  // lattice and points
  double* lat = nullptr;         // (M+2)^3 node values (spline - 1/2)
  uint8_t* flag = nullptr;       // 3 (M+2)^3 edge flags
  int* sel = nullptr;            // selected edge ids
  int* iota = nullptr;           // 0, 1, 2, ... (the compaction's input)
  int* nsel = nullptr;           // device count of selected edges
  int64_t lat_cap = 0;
  double* pts = nullptr;         // [3][pcap]
  double* nrm = nullptr;         // [3][pcap] spline gradient (flipped when the test says so)
  double* hes = nullptr;         // [4][pcap] H00 H11 H01 H10
  double* dir = nullptr;         // [pcap] +1 / -1 normal direction votes
  double* val = nullptr;         // [3][pcap] ss value, drip value, nz < 0
  int pcap = 0;
  // gradient accumulation
  int* key = nullptr;  int* key2 = nullptr;
  double* cv = nullptr; double* cv2 = nullptr;
  int64_t ccap = 0;
  void* cub_tmp = nullptr; size_t cub_bytes = 0;
  double* red = nullptr;         // reduction partials (1024) and results (8)
  double* ssc = nullptr;         // [nc] d ss / d coefficient
  double* dripc = nullptr;       // [nc] d drip / d coefficient
  int nc = 0;
  int npts = 0;
  std::vector<void*> extra;
  ~SupportState() {
    for (void* p : {(void*)knots, (void*)lat, (void*)flag, (void*)sel, (void*)iota, (void*)nsel, (void*)pts, (void*)nrm,
                    (void*)hes, (void*)dir, (void*)val, (void*)key, (void*)key2, (void*)cv, (void*)cv2, cub_tmp,
                    (void*)red, (void*)ssc, (void*)dripc})
      if (p) cudaFree(p);
  }
};

void support_free(SupportState* s) { delete s; }

int support_array(SupportState* s, int which, void** ptr, size_t* count) {
  if (!s) return TOPO_E_STATE;
  switch (which) {
    case TOPO_SSCSENS: *ptr = s->ssc; *count = s->nc; return s->ssc ? TOPO_OK : TOPO_E_STATE;
    case TOPO_DRIPCSENS: *ptr = s->dripc; *count = s->nc; return s->dripc ? TOPO_OK : TOPO_E_STATE;
    case TOPO_SURF_POINTS: *ptr = s->pts; *count = 3 * (size_t)s->npts; return s->pts ? TOPO_OK : TOPO_E_STATE;
    case TOPO_SURF_NORMALS: *ptr = s->nrm; *count = 3 * (size_t)s->npts; return s->nrm ? TOPO_OK : TOPO_E_STATE;
    default: return TOPO_E_BAD_INPUT;
  }
}

}  // namespace topo

namespace {

struct Spl {
  int order;
  int nb[3];
  int nk[3];          // knots per axis
  double kmin[3], kstep[3];
  const double* U;    // [3][kstride]
  int kstride;
  const double* c;    // coefficients, x fastest
};

// B-spline basis values and derivatives up to ND at x (The NURBS Book,
// Piegl and Tiller, algorithm A2.3) for order K: ders[k][j], k = 0..ND,
// j = 0..K-1 for the basis functions i0 .. i0 + K - 1.  Returns i0, or -1
// outside the knot range (span rule of grid/Grid.cu:3397-3404).  K and ND are
// compile-time, so every index is a constant and the tables live in registers.
template <int K, int ND>
__device__ __forceinline__ int basis_ders(const Spl& s, int a, double x, double (&ders)[3][K]) {
  constexpr int p = K - 1;
  const int i = (int)floor((x - s.kmin[a]) / s.kstep[a]) + K;
  if (i < K || i > s.nb[a]) return -1;
  const int l = i - 1;
  const double* U = s.U + (size_t)a * s.kstride;
  double ndu[K][K], left[K], right[K];
  ndu[0][0] = 1.0;
#pragma unroll
  for (int j = 1; j <= p; ++j) {
    left[j] = x - U[l + 1 - j];
    right[j] = U[l + j] - x;
    double saved = 0.0;
#pragma unroll
    for (int r = 0; r < j; ++r) {
      ndu[j][r] = right[r + 1] + left[j - r];
      const double temp = ndu[r][j - 1] / ndu[j][r];
      ndu[r][j] = saved + right[r + 1] * temp;
      saved = left[j - r] * temp;
    }
    ndu[j][j] = saved;
  }
#pragma unroll
  for (int j = 0; j <= p; ++j) ders[0][j] = ndu[j][p];
#pragma unroll
  for (int kk = 1; kk < 3; ++kk)
#pragma unroll
    for (int j = 0; j <= p; ++j) ders[kk][j] = 0.0;
  if (ND > 0) {
#pragma unroll
    for (int r = 0; r <= p; ++r) {
      double aa[2][K + 1];
      aa[0][0] = 1.0;
      int s1 = 0, s2 = 1;
#pragma unroll
      for (int kk = 1; kk <= ND && kk <= p; ++kk) {
        double d = 0.0;
        const int rk = r - kk, pk = p - kk;
        if (r >= kk) {
          aa[s2][0] = aa[s1][0] / ndu[pk + 1][rk];
          d = aa[s2][0] * ndu[rk][pk];
        }
        const int j1 = rk >= -1 ? 1 : -rk;
        const int j2 = (r - 1 <= pk) ? kk - 1 : p - r;
#pragma unroll
        for (int j = 1; j <= K; ++j) {
          if (j < j1 || j > j2) continue;
          aa[s2][j] = (aa[s1][j] - aa[s1][j - 1]) / ndu[pk + 1][rk + j];
          d += aa[s2][j] * ndu[rk + j][pk];
        }
        if (r <= pk) {
          aa[s2][kk] = -aa[s1][kk - 1] / ndu[pk + 1][r];
          d += aa[s2][kk] * ndu[r][pk];
        }
        ders[kk][r] = d;
        const int t = s1; s1 = s2; s2 = t;
      }
    }
    double f = p;
#pragma unroll
    for (int kk = 1; kk <= ND; ++kk) {
#pragma unroll
      for (int j = 0; j <= p; ++j) ders[kk][j] *= f;
      f *= (p - kk);
    }
  }
  return i - K;
}

template <int K>
__device__ double spline_at(const Spl& s, const double x[3], double outside) {
  double Dx[3][K], Dy[3][K], Dz[3][K];
  const int ix = basis_ders<K, 0>(s, 0, x[0], Dx);
  const int iy = basis_ders<K, 0>(s, 1, x[1], Dy);
  const int iz = basis_ders<K, 0>(s, 2, x[2], Dz);
  if (ix < 0 || iy < 0 || iz < 0) return outside;
  double v = 0;
#pragma unroll
  for (int r = 0; r < K; ++r)
#pragma unroll
    for (int q = 0; q < K; ++q)
#pragma unroll
      for (int t = 0; t < K; ++t)
        v += s.c[(ix + r) + (size_t)s.nb[0] * ((iy + q) + (size_t)s.nb[1] * (iz + t))] * Dx[0][r] * Dy[0][q] * Dz[0][t];
  return v;
}

struct Lattice {
  int n;              // nodes per axis (M + 2)
  double o[3], e[3];  // first node's corner (box min - e) and spacing
  double bmin[3], bmax[3];
};

__device__ void node_pos(const Lattice& L, int64_t id, double p[3]) {
  const int64_t n = L.n;
  const int64_t c[3] = {id % n, (id / n) % n, id / (n * n)};
  for (int a = 0; a < 3; ++a) p[a] = L.o[a] + (double)c[a] * L.e[a] + 0.5 * L.e[a];
}

// node value: spline - 1/2 inside the box, -1/2 outside (out-of-knot-range -0.7)
template <int K>
__global__ void k_sup_lattice(Spl s, Lattice L, double* __restrict__ lat) {
  const int64_t id = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t n3 = (int64_t)L.n * L.n * L.n;
  if (id >= n3) return;
  double p[3];
  node_pos(L, id, p);
  bool in = true;
  for (int a = 0; a < 3; ++a) in = in && p[a] >= L.bmin[a] && p[a] <= L.bmax[a];
  lat[id] = in ? spline_at<K>(s, p, -0.2) - 0.5 : -0.5;
}

__device__ bool edge_point(const Lattice& L, const double* lat, int64_t eid, double p[3]) {
  const int a = (int)(eid % 3);
  const int64_t id = eid / 3, n = L.n;
  const int64_t c = a == 0 ? id % n : (a == 1 ? (id / n) % n : id / (n * n));
  if (c + 1 >= n) return false;
  const int64_t id1 = id + (a == 0 ? 1 : (a == 1 ? n : n * n));
  const double v0 = lat[id], v1 = lat[id1];
  if ((v0 < 0) == (v1 < 0)) return false;
  const double t = -v0 / (v1 - v0);
  double p1[3];
  node_pos(L, id, p);
  node_pos(L, id1, p1);
  for (int k = 0; k < 3; ++k) p[k] = p[k] + t * (p1[k] - p[k]);
  return true;
}

__global__ void k_sup_edges(Lattice L, const double* __restrict__ lat, LevelDims d, double h,
                            const uint8_t* __restrict__ eactive, uint8_t* __restrict__ flag) {
  const int64_t eid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t ne = 3 * (int64_t)L.n * L.n * L.n;
  if (eid >= ne) return;
  double p[3];
  uint8_t f = 0;
  if (edge_point(L, lat, eid, p)) {
    bool in = true;
    int ec[3];
    const int dims[3] = {d.ex, d.ey, d.ez};
    for (int a = 0; a < 3; ++a) {
      in = in && p[a] >= L.bmin[a] && p[a] <= L.bmax[a];
      ec[a] = min(max((int)floor(p[a] / h), 0), dims[a] - 1);
    }
    f = in && eactive[ec[0] + (int64_t)d.ex * (ec[1] + (int64_t)d.ey * ec[2])] ? 1 : 0;
  }
  flag[eid] = f;
}

// Points, spline gradient and Hessian, and the normal-direction vote
// (correct_spline_surface_point_normal_direction, grid/Grid.cu:5620-5700).
template <int K>
__global__ void k_sup_points(Spl s, Lattice L, const double* __restrict__ lat, const int* __restrict__ sel,
                             const int* __restrict__ nsel, int maxp, double beta, double* __restrict__ pts,
                             double* __restrict__ nrm, double* __restrict__ hes, double* __restrict__ dir, int pcap) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  const int count = *nsel;
  const int np = min(count, maxp);
  if (k >= np) return;
  int pick = k;
  if (count > maxp) {  // equidistant pick (generateEquidistantIntegers, grid/Grid.cpp:3750-3764)
    const double step = (double)count / (double)(maxp - 1);
    pick = min((int)(k * step), count - 1);
  }
  double p[3];
  edge_point(L, lat, sel[pick], p);
  double Dx[3][K], Dy[3][K], Dz[3][K];
  const int ix = basis_ders<K, 2>(s, 0, p[0], Dx);
  const int iy = basis_ders<K, 2>(s, 1, p[1], Dy);
  const int iz = basis_ders<K, 2>(s, 2, p[2], Dz);
  double g[3] = {0, 0, 0}, H00 = 0, H11 = 0, H01 = 0;
  if (ix >= 0 && iy >= 0 && iz >= 0)
#pragma unroll
    for (int r = 0; r < K; ++r)
#pragma unroll
      for (int q = 0; q < K; ++q)
#pragma unroll
        for (int t = 0; t < K; ++t) {
          const double c = s.c[(ix + r) + (size_t)s.nb[0] * ((iy + q) + (size_t)s.nb[1] * (iz + t))];
          g[0] += c * Dx[1][r] * Dy[0][q] * Dz[0][t];
          g[1] += c * Dx[0][r] * Dy[1][q] * Dz[0][t];
          g[2] += c * Dx[0][r] * Dy[0][q] * Dz[1][t];
          H00 += c * Dx[2][r] * Dy[0][q] * Dz[0][t];
          H11 += c * Dx[0][r] * Dy[2][q] * Dz[0][t];
          H01 += c * Dx[1][r] * Dy[1][q] * Dz[0][t];
        }
  // vote: the Heaviside-projected spline a small step along the gradient
  const double qp[3] = {p[0] + 1e-3 * g[0], p[1] + 1e-3 * g[1], p[2] + 1e-3 * g[2]};
  const double sv = spline_at<K>(s, qp, -0.1);
  const double eta = 0.5;
  const double hs = (tanh(beta * eta) + tanh(beta * (sv - eta))) / (tanh(beta * eta) + tanh(beta * (1 - eta)));
  for (int a = 0; a < 3; ++a) {
    pts[(size_t)a * pcap + k] = p[a];
    nrm[(size_t)a * pcap + k] = g[a];
  }
  hes[k] = H00; hes[(size_t)pcap + k] = H11; hes[2 * (size_t)pcap + k] = H01; hes[3 * (size_t)pcap + k] = H01;
  dir[k] = hs < 0.5 ? 1.0 : -1.0;
}

__global__ void k_sup_flip(int np, int pcap, double* __restrict__ nrm) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= np) return;
  for (int a = 0; a < 3; ++a) nrm[(size_t)a * pcap + k] = -nrm[(size_t)a * pcap + k];
}

struct Params {
  int ss_mode, drip_mode, drip_version, quirks;
  double cos_print, cos_drip, drip_angle;
  double p_norm, hc, sc;
  double drip_beta, drip_mu, drip_alpha, drip_scale;
  double direction;
};

__device__ __forceinline__ double fh(double x, double c) { return x >= 1 ? c * (x - 1) * (x - 1) : 0.0; }
__device__ __forceinline__ double dfh(double x, double c) { return x >= 1 ? 2 * c * (x - 1) : 0.0; }
__device__ __forceinline__ double foh(double x, double c) { return 1 / (1 + exp(-(x - 1.5) / c)) + 1; }
__device__ __forceinline__ double dfoh(double x, double c) {
  const double e = exp(-(x - 1.5) / c);
  return 1 / (1 + e) / (1 + e) / c * e;
}
__device__ __forceinline__ double amax1(double x, double b, double s) { return s * x * x / (1 + exp(b * x)); }
__device__ __forceinline__ double damax1(double x, double b, double s) {
  const double e = 1 + exp(b * x);
  return s * (2 * x - x * x * b) / e + s * x * x * b / e / e;
}
__device__ __forceinline__ double amax2(double x, double b, double s) { return s * x * x / (1 + exp(b * (-x))); }
__device__ __forceinline__ double damax2(double x, double b, double s) {
  const double e = 1 + exp(-b * x);
  return s * (2 * x + x * x * b) / e - s * x * x * b / e / e;
}
__device__ __forceinline__ double drip_up(double x, double mu, double tol) {
  const double off = 1.2;
  return tol > 0.5 * M_PI ? 1 / (1 + exp(-(x - off) * mu)) : 1 / (1 + exp(mu * (x + off)));
}
__device__ __forceinline__ double ddrip_up(double x, double mu, double tol) {
  const double off = 1.2;
  if (tol > 0.5 * M_PI) {
    const double e = exp(-(x - off) * mu);
    return 1 / (1 + e) / (1 + e) * mu * e;
  }
  const double e = exp(mu * (x + off));
  return -mu * e / (1 + e) / (1 + e);
}

__device__ double ss_point(const Params& P, double inner, double nz) {
  const bool down = nz < 0;
  switch (P.ss_mode) {
    case 0: return down ? pow(inner, P.p_norm) : 0.0;
    case 1: return pow(inner, P.p_norm);
    case 2: return down ? fh(inner, P.hc) : 0.0;
    case 3: return fh(inner, P.hc);
    case 4: return down ? foh(inner, P.sc) : 0.0;
    default: return foh(inner, P.sc);
  }
}
__device__ double dss_point(const Params& P, double inner, double nz) {
  const bool down = nz < 0;
  switch (P.ss_mode) {
    case 0: return down ? P.p_norm * pow(inner, P.p_norm - 1) : 0.0;
    case 1: return P.p_norm * pow(inner, P.p_norm - 1);
    case 2: return down ? dfh(inner, P.hc) : 0.0;
    case 3: return dfh(inner, P.hc);
    case 4: return down ? dfoh(inner, P.sc) : 0.0;
    default: return dfoh(inner, P.sc);
  }
}

// per point: ss value, drip value, and whether the normal points down
__global__ void k_sup_values(int np, int pcap, Params P, const double* __restrict__ nrm, const double* __restrict__ hes,
                             double* __restrict__ val) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= np) return;
  const double n0 = nrm[k], n1 = nrm[(size_t)pcap + k], n2 = nrm[2 * (size_t)pcap + k];
  const double nn = sqrt(n0 * n0 + n1 * n1 + n2 * n2);
  const double inner = n2 / nn / P.cos_print;
  val[k] = ss_point(P, inner, n2);
  double dv = 0.0;
  if (P.drip_mode == 7 || (P.drip_mode == 6 && n2 < 0)) {
    const double H00 = hes[k], H11 = hes[(size_t)pcap + k], H01 = hes[2 * (size_t)pcap + k],
                 H10 = hes[3 * (size_t)pcap + k];
    const double hinner = n2 / nn / P.cos_drip;
    const double i1 = H00, i2 = H00 * H11 - H01 * H10;
    const double gx = n0 / n2, gy = n1 / n2;
    const double lead = P.drip_version == 1 ? exp(-P.drip_alpha * gx * gx - P.drip_alpha * gy * gy)
                                            : drip_up(hinner, P.drip_mu, P.drip_angle);
    dv = lead * amax1(i1, P.drip_beta, P.drip_scale) * amax2(i2, P.drip_beta, P.drip_scale);
  }
  val[(size_t)pcap + k] = dv;
  val[2 * (size_t)pcap + k] = n2 < 0 ? 1.0 : 0.0;
}

// per point and tap: the derivatives of the point's ss and drip values with
// respect to the coefficient of that tap (compute_spline_selfsupp_constraint_dcoeff
// and compute_spline_drip_constraint_dcoeff_test, grid/Grid.cu:6147-6321, 6928-7156)
template <int K>
__global__ void k_sup_grad(Spl s, int np, int pcap, Params P, const double* __restrict__ pts,
                           const double* __restrict__ nrm, const double* __restrict__ hes, int* __restrict__ key,
                           double* __restrict__ css, double* __restrict__ cdrip) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= np) return;
  constexpr int T = K * K * K;
  const double p[3] = {pts[k], pts[(size_t)pcap + k], pts[2 * (size_t)pcap + k]};
  double Dx[3][K], Dy[3][K], Dz[3][K];
  const int i0[3] = {basis_ders<K, 2>(s, 0, p[0], Dx), basis_ders<K, 2>(s, 1, p[1], Dy),
                     basis_ders<K, 2>(s, 2, p[2], Dz)};
  const bool ok = i0[0] >= 0 && i0[1] >= 0 && i0[2] >= 0;
  const double n0 = nrm[k], n1 = nrm[(size_t)pcap + k], n2 = nrm[2 * (size_t)pcap + k];
  const double nn = sqrt(n0 * n0 + n1 * n1 + n2 * n2);
  const double H00 = hes[k], H11 = hes[(size_t)pcap + k], H01 = hes[2 * (size_t)pcap + k],
               H10 = hes[3 * (size_t)pcap + k];
  const double inner = n2 / nn / P.cos_print, dss = dss_point(P, inner, n2);
  const bool drip_on = P.drip_mode == 7 || (P.drip_mode == 6 && n2 < 0);
  const double hinner = n2 / nn / P.cos_drip;
  const double i1 = H00, i2 = H00 * H11 - H01 * H10;
  const double tq1 = amax1(i1, P.drip_beta, P.drip_scale), tq2 = amax2(i2, P.drip_beta, P.drip_scale);
  const double dtq1 = damax1(i1, P.drip_beta, P.drip_scale), dtq2 = damax2(i2, P.drip_beta, P.drip_scale);
  const double gx = n0 / n2, gy = n1 / n2;
  const double g_ = exp(-P.drip_alpha * gx * gx - P.drip_alpha * gy * gy);
  const double h_ = drip_up(hinner, P.drip_mu, P.drip_angle), dh_ = ddrip_up(hinner, P.drip_mu, P.drip_angle);
  double acc[4] = {0, 0, 0, 0};  // running Hessian derivative sums (the reference's accumulation)
#pragma unroll
  for (int r = 0; r < K; ++r)
#pragma unroll
    for (int q = 0; q < K; ++q)
#pragma unroll
      for (int w = 0; w < K; ++w) {
        const int t = (r * K + q) * K + w;
        const size_t slot = (size_t)k * T + t;
        if (!ok) { key[slot] = 0; css[slot] = 0; cdrip[slot] = 0; continue; }
        key[slot] = (i0[0] + r) + s.nb[0] * ((i0[1] + q) + s.nb[1] * (i0[2] + w));
        const double dn[3] = {P.direction * Dx[1][r] * Dy[0][q] * Dz[0][w],
                              P.direction * Dx[0][r] * Dy[1][q] * Dz[0][w],
                              P.direction * Dx[0][r] * Dy[0][q] * Dz[1][w]};
        const double dnn = (n0 * dn[0] + n1 * dn[1] + n2 * dn[2]) / nn;
        const double up_p = dn[2] * nn - n2 * dnn;
        css[slot] = dss * (up_p / (nn * nn * P.cos_print));
        double dv = 0.0;
        if (drip_on) {
          const double hd = up_p / (nn * nn * P.cos_drip);
          double d00 = Dx[2][r] * Dy[0][q] * Dz[0][w], d11 = Dx[0][r] * Dy[2][q] * Dz[0][w];
          double d01 = Dx[1][r] * Dy[1][q] * Dz[0][w], d10 = d01;
          double gdx = (dn[0] * n2 - n0 * dn[2]) / (n2 * n2), gdy = (dn[1] * n2 - n1 * dn[2]) / (n2 * n2);
          if (P.quirks) {  // Hessian derivatives summed over the taps so far; x slot overwritten by y
            acc[0] += d00; acc[1] += d11; acc[2] += d01; acc[3] += d10;
            d00 = acc[0]; d11 = acc[1]; d01 = acc[2]; d10 = acc[3];
            gdx = gdy;
            gdy = 0.0;
          }
          const double di1 = d00, di2 = d00 * H11 + H00 * d11 - d01 * H10 - H01 * d10;
          const double dg = (-2 * P.drip_alpha * gx * gdx - 2 * P.drip_alpha * gy * gdy) * g_;
          if (P.drip_version == 1)
            dv = (P.quirks ? dg * hd : dg) * tq1 * tq2 + g_ * dtq1 * di1 * tq2 + g_ * tq1 * dtq2 * di2;
          else
            dv = dh_ * hd * tq1 * tq2 + h_ * dtq1 * di1 * tq2 + h_ * tq1 * dtq2 * di2;
        }
        cdrip[slot] = dv;
      }
}

// out[c] = scale * (sum of the sorted run of key c), summed in sorted order
__global__ void k_sup_runs(int nc, int64_t n, const int* __restrict__ key, const double* __restrict__ v, double scale,
                           double* __restrict__ out) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nc) return;
  int64_t lo = 0, hi = n;
  while (lo < hi) { const int64_t m = (lo + hi) / 2; if (key[m] < c) lo = m + 1; else hi = m; }
  double sum = 0.0;
  for (int64_t i = lo; i < n && key[i] == c; ++i) sum += v[i];
  out[c] = scale * sum;
}

__global__ void k_iota(int64_t n, int* __restrict__ a) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) a[i] = (int)i;
}

__global__ void k_heaviside(int64_t ne, const uint8_t* __restrict__ ea, const double* __restrict__ rho0, double beta,
                            double rho_min, double* __restrict__ rho) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ne) return;
  if (!ea[e]) { rho[e] = 0.0; return; }
  const double eta = 0.5;
  const double v = (tanh(beta * eta) + tanh(beta * (rho0[e] - eta))) / (tanh(beta * eta) + tanh(beta * (1 - eta)));
  rho[e] = fmin(fmax(v, rho_min), 1.0);
}

// a[e] = (fill ? c : a[e]) * dH/drho0 on active elements
__global__ void k_dirac(int64_t ne, const uint8_t* __restrict__ ea, const double* __restrict__ rho0, double beta,
                        bool fill, double c, double* __restrict__ a) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ne) return;
  if (!ea[e]) { a[e] = 0.0; return; }
  const double eta = 0.5, th = tanh(beta * (rho0[e] - eta));
  const double dh = beta * (1 - th * th) / (tanh(beta * eta) + tanh(beta * (1 - eta)));
  a[e] = (fill ? c : a[e]) * dh;
}

template <typename T>
int sup_alloc(T** p, size_t n) {
  if (*p) cudaFree(*p);
  *p = nullptr;
  if (cudaMalloc((void**)p, sizeof(T) * std::max<size_t>(n, 1)) != cudaSuccess) {
    cudaGetLastError();
    *p = nullptr;
    return TOPO_E_NOMEM;
  }
  return TOPO_OK;
}

int sfail(topo_handle* h, int code, const char* m) { return handle_fail(h, code, m); }

}  // namespace

extern "C" {

int topo_heaviside_project(topo_handle* h, double beta) {
  DeviceScope scope(h ? h->cfg.device : -1);
  if (!h || !(beta > 0)) return TOPO_E_BAD_INPUT;
  const DevLevel& L = h->lv[0];
  if (!h->rho_init && sup_alloc(&h->rho_init, L.d.ne) != TOPO_OK) return sfail(h, TOPO_E_NOMEM, "rho_init");
  if (cudaMemcpyAsync(h->rho_init, h->rho, sizeof(double) * L.d.ne, cudaMemcpyDeviceToDevice, h->stream) != cudaSuccess)
    return sfail(h, TOPO_E_CUDA, "heaviside copy");
  k_heaviside<<<(unsigned)((L.d.ne + 255) / 256), 256, 0, h->stream>>>(L.d.ne, L.eactive, h->rho_init, beta,
                                                                        h->cfg.min_density, h->rho);
  count_launch();
  h->rhop_stale = true;
  h->rho_projected = true;
  return cudaGetLastError() == cudaSuccess ? TOPO_OK : sfail(h, TOPO_E_CUDA, "heaviside launch");
}

int topo_heaviside_sensitivity(topo_handle* h, double beta) {
  DeviceScope scope(h ? h->cfg.device : -1);
  if (!h || !(beta > 0)) return TOPO_E_BAD_INPUT;
  if (!h->rho_projected) return sfail(h, TOPO_E_STATE, "heaviside sensitivity: density not projected");
  const DevLevel& L = h->lv[0];
  k_dirac<<<(unsigned)((L.d.ne + 255) / 256), 256, 0, h->stream>>>(L.d.ne, L.eactive, h->rho_init, beta, false, 0.0,
                                                                    h->sens);
  count_launch();
  return cudaGetLastError() == cudaSuccess ? TOPO_OK : sfail(h, TOPO_E_CUDA, "dirac launch");
}

int topo_heaviside_volume_csens(topo_handle* h, double beta, int refden, double filter_radius, double scale,
                                double* out_dev) {
  DeviceScope scope(h ? h->cfg.device : -1);
  if (!h || !(beta > 0)) return TOPO_E_BAD_INPUT;
  if (!h->spline_set) return sfail(h, TOPO_E_STATE, "spline not set");
  if (!h->rho_projected) return sfail(h, TOPO_E_STATE, "heaviside volume sensitivity: density not projected");
  if (!out_dev) out_dev = h->volcsens;
  const DevLevel& L = h->lv[0];
  if (!h->vsens && sup_alloc(&h->vsens, L.d.ne) != TOPO_OK) return sfail(h, TOPO_E_NOMEM, "vsens");
  const double den = (double)(refden ? h->gs_padded_elements : h->active_elements);
  k_dirac<<<(unsigned)((L.d.ne + 255) / 256), 256, 0, h->stream>>>(L.d.ne, L.eactive, h->rho_init, beta, true,
                                                                    scale / den, h->vsens);
  count_launch();
  if (filter_radius > 0) {
    const int rc = handle_filter_prepare(h, filter_radius);
    if (rc != TOPO_OK) return rc;
    launch_filter_df(h->stream, L.d, L.eactive, h->vsens, reinterpret_cast<float2*>(h->sens_tmp), h->filt_offs,
                     h->filt_wdf, h->filt_n);
    count_launch(2);
  }
  launch_spline_adjoint(h->stream, L.d, L.eactive, h->sd, h->vsens, out_dev, h->adj1, h->adj2);
  count_launch(3);
  return cudaGetLastError() == cudaSuccess ? TOPO_OK : sfail(h, TOPO_E_CUDA, "volume sensitivity launch");
}

int topo_support_constraints(topo_handle* h, const topo_support_opts* o, topo_support_stats* st) {
  DeviceScope scope(h ? h->cfg.device : -1);
  if (!h || !o) return TOPO_E_BAD_INPUT;
  if (!h->spline_set) return sfail(h, TOPO_E_STATE, "spline not set");
  if (h->sd.order < 2 || h->sd.order > kSupMaxOrder) return sfail(h, TOPO_E_BAD_INPUT, "spline order outside 2..4");
  if (o->lattice < 2 || o->lattice > 1024 || o->max_points < 2 || o->ss_mode < 0 || o->ss_mode > 5 ||
      o->drip_mode < 0 || o->drip_mode > 7 || !(o->beta > 0))
    return sfail(h, TOPO_E_BAD_INPUT, "support constraints: lattice 2..1024, max_points >= 2, ss_mode 0..5, "
                                      "drip_mode 0..7, beta > 0");
  if (!h->support) h->support = new SupportState;
  SupportState& S = *h->support;
  const cudaStream_t s = h->stream;
  const DevLevel& L0 = h->lv[0];
  const int order = h->sd.order;
  const int nc = h->sd.nb[0] * h->sd.nb[1] * h->sd.nb[2];
  // spline knots on the device
  int kmax = 0;
  for (int a = 0; a < 3; ++a) kmax = std::max<int>(kmax, (int)h->st.knots[a].size());
  if (S.kcap < kmax) {
    if (sup_alloc(&S.knots, 3 * (size_t)kmax) != TOPO_OK) return sfail(h, TOPO_E_NOMEM, "knots");
    S.kcap = kmax;
  }
  {
    std::vector<double> kn(3 * (size_t)S.kcap, 0.0);
    for (int a = 0; a < 3; ++a) std::copy(h->st.knots[a].begin(), h->st.knots[a].end(), kn.begin() + (size_t)a * S.kcap);
    cudaMemcpyAsync(S.knots, kn.data(), sizeof(double) * kn.size(), cudaMemcpyHostToDevice, s);
    cudaStreamSynchronize(s);
  }
  Spl sp{};
  sp.order = order;
  for (int a = 0; a < 3; ++a) {
    sp.nb[a] = h->sd.nb[a];
    sp.nk[a] = (int)h->st.knots[a].size();
    sp.kmin[a] = h->st.kmin[a];
    sp.kstep[a] = h->st.kstep[a];
  }
  sp.U = S.knots;
  sp.kstride = S.kcap;
  sp.c = h->coeff;
  // lattice over the domain box [0, n h], padded by one cell per side
  Lattice lat{};
  lat.n = o->lattice + 2;
  const int dims[3] = {L0.d.ex, L0.d.ey, L0.d.ez};
  for (int a = 0; a < 3; ++a) {
    lat.bmin[a] = 0.0;
    lat.bmax[a] = dims[a] * h->cfg.h;
    lat.e[a] = (lat.bmax[a] - lat.bmin[a]) / o->lattice;
    lat.o[a] = lat.bmin[a] - lat.e[a];
  }
  const int64_t n3 = (int64_t)lat.n * lat.n * lat.n;
  if (S.lat_cap < n3) {
    if (sup_alloc(&S.lat, n3) || sup_alloc(&S.flag, 3 * n3) || sup_alloc(&S.sel, 3 * n3) ||
        sup_alloc(&S.iota, 3 * n3) || sup_alloc(&S.nsel, 1))
      return sfail(h, TOPO_E_NOMEM, "lattice");
    S.lat_cap = n3;
    k_iota<<<(unsigned)((3 * n3 + 255) / 256), 256, 0, s>>>(3 * n3, S.iota);
    count_launch();
  }
  switch (order) {
    case 2: k_sup_lattice<2><<<(unsigned)((n3 + 255) / 256), 256, 0, s>>>(sp, lat, S.lat); break;
    case 3: k_sup_lattice<3><<<(unsigned)((n3 + 255) / 256), 256, 0, s>>>(sp, lat, S.lat); break;
    default: k_sup_lattice<4><<<(unsigned)((n3 + 255) / 256), 256, 0, s>>>(sp, lat, S.lat); break;
  }
  k_sup_edges<<<(unsigned)((3 * n3 + 255) / 256), 256, 0, s>>>(lat, S.lat, L0.d, h->cfg.h, L0.eactive, S.flag);
  count_launch(2);
  // stable compaction of the crossing edges (lattice order)
  size_t need = 0;
  cub::DeviceSelect::Flagged(nullptr, need, S.iota, S.flag, S.sel, S.nsel, (int)(3 * n3), s);
  if (need > S.cub_bytes) {
    if (S.cub_tmp) cudaFree(S.cub_tmp);
    S.cub_tmp = nullptr;
    if (cudaMalloc(&S.cub_tmp, need) != cudaSuccess) { cudaGetLastError(); S.cub_bytes = 0; return sfail(h, TOPO_E_NOMEM, "cub"); }
    S.cub_bytes = need;
  }
  cub::DeviceSelect::Flagged(S.cub_tmp, need, S.iota, S.flag, S.sel, S.nsel, (int)(3 * n3), s);
  count_launch();
  int count = 0;
  cudaMemcpyAsync(&count, S.nsel, sizeof(int), cudaMemcpyDeviceToHost, s);
  if (cudaStreamSynchronize(s) != cudaSuccess) return sfail(h, TOPO_E_CUDA, "support: lattice");
  const int np = std::min(count, o->max_points);
  if (S.pcap < np) {
    if (sup_alloc(&S.pts, 3 * (size_t)np) || sup_alloc(&S.nrm, 3 * (size_t)np) || sup_alloc(&S.hes, 4 * (size_t)np) ||
        sup_alloc(&S.dir, np) || sup_alloc(&S.val, 3 * (size_t)np))
      return sfail(h, TOPO_E_NOMEM, "points");
    S.pcap = np;
  }
  if (!S.red && sup_alloc(&S.red, 1032) != TOPO_OK) return sfail(h, TOPO_E_NOMEM, "partials");
  if (S.nc != nc || !S.ssc) {
    if (sup_alloc(&S.ssc, nc) || sup_alloc(&S.dripc, nc)) return sfail(h, TOPO_E_NOMEM, "constraint gradients");
    S.nc = nc;
  }
  S.npts = np;
  topo_support_stats out{};
  out.candidates = count;
  out.points = np;
  if (np == 0) {
    cudaMemsetAsync(S.ssc, 0, sizeof(double) * nc, s);
    cudaMemsetAsync(S.dripc, 0, sizeof(double) * nc, s);
    cudaStreamSynchronize(s);
    if (st) *st = out;
    return TOPO_OK;
  }
  const unsigned pb = (unsigned)((np + 127) / 128);
  switch (order) {
    case 2: k_sup_points<2><<<pb, 128, 0, s>>>(sp, lat, S.lat, S.sel, S.nsel, o->max_points, o->beta, S.pts, S.nrm,
                                               S.hes, S.dir, S.pcap); break;
    case 3: k_sup_points<3><<<pb, 128, 0, s>>>(sp, lat, S.lat, S.sel, S.nsel, o->max_points, o->beta, S.pts, S.nrm,
                                               S.hes, S.dir, S.pcap); break;
    default: k_sup_points<4><<<pb, 128, 0, s>>>(sp, lat, S.lat, S.sel, S.nsel, o->max_points, o->beta, S.pts, S.nrm,
                                                S.hes, S.dir, S.pcap); break;
  }
  launch_sum(s, S.dir, np, S.red, S.red + 1024);
  count_launch(3);
  double votes = 0;
  cudaMemcpyAsync(&votes, S.red + 1024, sizeof(double), cudaMemcpyDeviceToHost, s);
  if (cudaStreamSynchronize(s) != cudaSuccess) return sfail(h, TOPO_E_CUDA, "support: points");
  if (votes < 0) {  // most points see solid along +gradient: the normals point inward
    k_sup_flip<<<pb, 128, 0, s>>>(np, S.pcap, S.nrm);
    count_launch();
    out.flipped = 1;
  }
  Params P{};
  P.ss_mode = o->ss_mode;
  P.drip_mode = o->drip_mode;
  P.drip_version = o->drip_version;
  P.quirks = o->reference_quirks;
  P.cos_print = std::cos(o->print_angle * M_PI);
  P.drip_angle = o->drip_angle > 0 ? o->drip_angle : 160.0 / 180.0 * M_PI;
  P.cos_drip = std::cos(P.drip_angle);
  P.p_norm = o->p_norm > 0 ? o->p_norm : 8.0;
  P.hc = o->hfunction_c > 0 ? o->hfunction_c : 10.0;
  P.sc = o->sigmoid_c > 0 ? o->sigmoid_c : 0.09;
  P.drip_beta = o->drip_beta > 0 ? o->drip_beta : 128.0;
  P.drip_mu = o->drip_mu > 0 ? o->drip_mu : 32.0;
  P.drip_alpha = o->drip_alpha > 0 ? o->drip_alpha : 4.0;
  P.drip_scale = o->drip_beta_scale > 0 ? o->drip_beta_scale : 10.0;
  P.direction = votes > 0 ? 1.0 : -1.0;  // the reference's sign for d normal / d coefficient
  k_sup_values<<<pb, 128, 0, s>>>(np, S.pcap, P, S.nrm, S.hes, S.val);
  double sums[3];
  for (int q = 0; q < 3; ++q) launch_sum(s, S.val + (size_t)q * S.pcap, np, S.red, S.red + 1025 + q);
  count_launch(7);
  cudaMemcpyAsync(sums, S.red + 1025, sizeof(sums), cudaMemcpyDeviceToHost, s);
  if (cudaStreamSynchronize(s) != cudaSuccess) return sfail(h, TOPO_E_CUDA, "support: values");
  const double down = sums[2];
  const double cnt_ss = (o->ss_mode % 2 == 0) ? down : (double)np;
  const double cnt_drip = (o->drip_mode % 2 == 0) ? down : (double)np;
  out.overhang_points = (int)down;
  if (cnt_ss > 0) out.ss_value = o->ss_mode <= 1 ? std::pow(sums[0] / cnt_ss, 1.0 / P.p_norm) - 1.0 : sums[0] / cnt_ss;
  if (cnt_drip > 0) out.drip_value = o->drip_mode <= 1 ? std::pow(sums[1] / cnt_drip, 1.0 / P.p_norm) - 1.0
                                                       : sums[1] / cnt_drip;
  // coefficient gradients: per-point contributions, stable sort by coefficient, run sums
  const int T = order * order * order;
  const int64_t nct = (int64_t)np * T;
  if (S.ccap < nct) {
    if (sup_alloc(&S.key, nct) || sup_alloc(&S.key2, nct) || sup_alloc(&S.cv, 2 * nct) || sup_alloc(&S.cv2, 2 * nct))
      return sfail(h, TOPO_E_NOMEM, "gradient contributions");
    S.ccap = nct;
  }
  switch (order) {
    case 2: k_sup_grad<2><<<pb, 128, 0, s>>>(sp, np, S.pcap, P, S.pts, S.nrm, S.hes, S.key, S.cv, S.cv + nct); break;
    case 3: k_sup_grad<3><<<pb, 128, 0, s>>>(sp, np, S.pcap, P, S.pts, S.nrm, S.hes, S.key, S.cv, S.cv + nct); break;
    default: k_sup_grad<4><<<pb, 128, 0, s>>>(sp, np, S.pcap, P, S.pts, S.nrm, S.hes, S.key, S.cv, S.cv + nct); break;
  }
  count_launch();
  int nbits = 1;
  while ((1 << nbits) <= nc && nbits < 31) ++nbits;
  for (int q = 0; q < 2; ++q) {
    need = 0;
    cub::DeviceRadixSort::SortPairs(nullptr, need, S.key, S.key2, S.cv + q * nct, S.cv2 + q * nct, (int)nct, 0, nbits,
                                    s);
    if (need > S.cub_bytes) {
      if (S.cub_tmp) cudaFree(S.cub_tmp);
      S.cub_tmp = nullptr;
      if (cudaMalloc(&S.cub_tmp, need) != cudaSuccess) { cudaGetLastError(); S.cub_bytes = 0; return sfail(h, TOPO_E_NOMEM, "cub"); }
      S.cub_bytes = need;
    }
    cub::DeviceRadixSort::SortPairs(S.cub_tmp, need, S.key, S.key2, S.cv + q * nct, S.cv2 + q * nct, (int)nct, 0,
                                    nbits, s);
    const double cnt = q == 0 ? cnt_ss : cnt_drip;
    const double scale = cnt > 0 ? 1.0 / cnt : 0.0;
    k_sup_runs<<<(unsigned)((nc + 255) / 256), 256, 0, s>>>(nc, nct, S.key2, S.cv2 + q * nct, scale,
                                                            q == 0 ? S.ssc : S.dripc);
    count_launch(2);
  }
  if (cudaStreamSynchronize(s) != cudaSuccess || cudaGetLastError() != cudaSuccess)
    return sfail(h, TOPO_E_CUDA, "support: gradients");
  if (st) *st = out;
  return TOPO_OK;
}

}  // extern "C"
