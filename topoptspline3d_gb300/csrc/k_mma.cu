// Method of Moving Asymptotes on the GPU (reference optimization/mma_t.h,
// mma_t.cpp, mma_t.cu; driver utils/test_utils.cpp:972-1217).
//
// The reference runs the MMA subproblem's primal-dual interior-point loop from
// the host: every vector expression is its own kernel followed by a
// device-wide synchronise, the m x m reduced system goes through host memory,
// and each line-search trial reads its error back (optimization/mma_t.cu:330-566).
// Here one cooperative kernel runs the whole update:
//   phase 0     approximation p_i, q_i and proxy offsets b (mma_t.cu:15-130),
//               reset of the primal-dual point (mma_t.cu:702-713)
//   per Newton  N1  Psi, Dx, G_i, delta_x and their reductions (the m x m
//   step            matrix sum G_i G_k / Dx, sum G_i delta_x / Dx, the proxy
//                   constraints) plus the KKT error at the current point;
//                   every CTA then solves the (m+1) reduced system
//                   (mma_t.cu:230-327, 357-400)
//               N2  primal direction dx, dxi, deta and the step bound
//                   (mma_t.cu:402-411)
//               LS  backtracking line search on the 2-norm of the KKT error,
//                   one grid-wide reduction per trial (mma_t.cu:510-566, 569-672)
//   final       asymptote and move-limit update (mma_t.cu:156-227)
// One thread owns a fixed set of design variables for the whole launch, so
// per-variable state never crosses threads.  Grid-wide sums use per-CTA
// partials in a ping-pong buffer.  After each grid.sync every CTA adds the
// partials in the same order, so the scalar control flow (Newton steps,
// line-search decisions, epsilon continuation) is bitwise identical in all
// CTAs and no host round trip is needed.  Arithmetic is FP64 (the reference
// uses FP32).
#include <cooperative_groups.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "topo_internal.h"

namespace cg = cooperative_groups;

namespace topo {

constexpr int kMmaMaxM = 4;        // constraints handled by the GPU kernel
constexpr int kMmaBlock = 256;
constexpr int kMmaWarps = kMmaBlock / 32;
constexpr int kMmaSlots = 32;      // reduction slots per grid-wide reduction
constexpr double kStepFrac = 0.99; // asym_clamp_factor, optimization/mma_t.h:20

struct MmaArgs {
  int n, m;
  double *x, *xold, *xmin, *xmax, *L, *U, *alpha, *beta, *lastdx, *xi, *eta;
  double *p, *q;  // [(m+1)][n]
  double *Dx, *dlx, *dx, *dxi, *deta;
  double* part;   // [2][kMmaSlots][gridDim.x]
  double* stats;  // [5]: sub-iterations, KKT inf-norm, last step, |x - x_old|_2, overflow
  const double* df;
  const double* dg[kMmaMaxM];
  double g[kMmaMaxM], a[kMmaMaxM], c[kMmaMaxM], d[kMmaMaxM], a0;
};

// Scalar state of the subproblem, replicated in every CTA.
template <int M>
struct MmaScalars {
  double y[M], lam[M], mu[M], s[M], lampq[M], b[M];
  double dy[M], dl[M], dmu[M], ds[M];
  double z, zeta, eps, dz, dzeta;
  double err, lasterr, damp, step, old_err, new_err, new_inf;
  int stays, nsub, overflow, accept;
};

// Grid-wide reduction of ns sums followed by nm maxima held per thread in
// v[0..ns+nm).  Every CTA ends with the totals in red[].
__device__ __forceinline__ void grid_reduce(cg::grid_group& grid, double* v, int ns, int nm, double* part,
                                            int& rs, double (*wsum)[kMmaSlots], double* red) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nk = ns + nm;
  for (int k = 0; k < nk; ++k) {
    double t = v[k];
    for (int o = 16; o > 0; o >>= 1) {
      const double u = __shfl_down_sync(0xffffffffu, t, o);
      t = k < ns ? t + u : fmax(t, u);
    }
    if (lane == 0) wsum[warp][k] = t;
  }
  __syncthreads();
  double* slot = part + (size_t)(rs & 1) * kMmaSlots * gridDim.x;
  for (int k = threadIdx.x; k < nk; k += blockDim.x) {
    double t = wsum[0][k];
    for (int w = 1; w < kMmaWarps; ++w) t = k < ns ? t + wsum[w][k] : fmax(t, wsum[w][k]);
    slot[(size_t)k * gridDim.x + blockIdx.x] = t;
  }
  grid.sync();
  for (int k = threadIdx.x; k < nk; k += blockDim.x) {
    const double* pk = slot + (size_t)k * gridDim.x;
    double t = __ldcg(pk);
    for (int b = 1; b < (int)gridDim.x; ++b) t = k < ns ? t + __ldcg(pk + b) : fmax(t, __ldcg(pk + b));
    red[k] = t;
  }
  ++rs;
  __syncthreads();
}

// Dense (M+1) system, partial pivoting (one thread).
template <int K>
__device__ void small_solve(double (&A)[K][K], double (&r)[K]) {
  for (int c = 0; c < K; ++c) {
    int piv = c;
    for (int i = c + 1; i < K; ++i)
      if (fabs(A[i][c]) > fabs(A[piv][c])) piv = i;
    if (piv != c) {
      for (int j = 0; j < K; ++j) { const double t = A[c][j]; A[c][j] = A[piv][j]; A[piv][j] = t; }
      const double t = r[c]; r[c] = r[piv]; r[piv] = t;
    }
    const double dinv = 1.0 / A[c][c];
    for (int i = c + 1; i < K; ++i) {
      const double f = A[i][c] * dinv;
      if (f == 0.0) continue;
      for (int j = c; j < K; ++j) A[i][j] -= f * A[c][j];
      r[i] -= f * r[c];
    }
  }
  for (int c = K - 1; c >= 0; --c) {
    double t = r[c];
    for (int j = c + 1; j < K; ++j) t -= A[c][j] * r[j];
    r[c] = t / A[c][c];
  }
}

// Scalar rows of the KKT error at step t (optimization/mma_t.cu:597-660); vsum,
// vmax are the reduced per-variable terms and gsum the proxy constraints.
template <int M>
__device__ void kkt_scalars(const MmaArgs& A, MmaScalars<M>& S, double t, double damp, double vsum,
                            double vmax, const double* gsum, double* err2, double* errinf) {
  double e2 = vsum, ei = fmax(-10.0, vmax);
  double lt[M], la = 0.0;
  for (int i = 0; i < M; ++i) { lt[i] = S.lam[i] + t * S.dl[i]; la += lt[i] * A.a[i]; }
  const double zt = S.z + t * S.dz, zetat = S.zeta + t * S.dzeta;
  for (int i = 0; i < M; ++i) {
    const double yt = S.y[i] + t * S.dy[i], mt = S.mu[i] + t * S.dmu[i], st = S.s[i] + t * S.ds[i];
    const double rey = A.c[i] + A.d[i] * yt - lt[i] - mt;
    const double relam = (gsum[i] - A.a[i] * zt - yt + st - S.b[i]) / damp;
    const double remu = mt * yt - S.eps;
    const double res = lt[i] * st - S.eps;
    e2 += rey * rey + relam * relam + remu * remu + res * res;
    ei = fmax(ei, fmax(fmax(fabs(rey), fabs(relam)), fmax(fabs(remu), fabs(res))));
  }
  const double rez = A.a0 - zetat - la, rezet = zetat * zt - S.eps;
  e2 += rez * rez + rezet * rezet;
  ei = fmax(ei, fmax(fabs(rez), fabs(rezet)));
  *err2 = sqrt(e2);
  *errinf = ei;
}

template <int M>
__global__ void __launch_bounds__(kMmaBlock) k_mma_update(MmaArgs A) {
  static_assert(M * M + 3 * M + 4 <= kMmaSlots, "reduction slots");
  cg::grid_group grid = cg::this_grid();
  __shared__ double wsum[kMmaWarps][kMmaSlots];
  __shared__ double red[kMmaSlots];
  __shared__ MmaScalars<M> S;
  const int n = A.n;
  const int j0 = blockIdx.x * blockDim.x + threadIdx.x, js = gridDim.x * blockDim.x;
  int rs = 0;
  double v[kMmaSlots];

  // ---- phase 0: approximation at the current design, proxy offsets, reset
  for (int i = 0; i < M; ++i) v[i] = 0.0;
  for (int j = j0; j < n; j += js) {
    const double x = A.x[j], ux = A.U[j] - x, xl = x - A.L[j];
    const double reg = 1e-5 / (A.xmax[j] - A.xmin[j]);
    A.xold[j] = x;
#pragma unroll
    for (int i = 0; i <= M; ++i) {
      const double dfi = i == 0 ? A.df[j] : A.dg[i - 1][j];
      const double pos = fmax(dfi, 0.0), neg = fmax(-dfi, 0.0);
      const double pi = ux * ux * (1.001 * pos + 0.001 * neg + reg);
      const double qi = xl * xl * (0.001 * pos + 1.001 * neg + reg);
      A.p[(size_t)i * n + j] = pi;
      A.q[(size_t)i * n + j] = qi;
      if (i > 0) v[i - 1] += pi / ux + qi / xl;
    }
    const double al = A.alpha[j], be = A.beta[j], xn = 0.5 * (al + be);
    A.x[j] = xn;
    A.xi[j] = fmax(1.0 / (xn - al), 1.0);
    A.eta[j] = fmax(1.0 / (be - xn), 1.0);
  }
  grid_reduce(grid, v, M, 0, A.part, rs, wsum, red);
  if (threadIdx.x == 0) {
    for (int i = 0; i < M; ++i) {
      S.b[i] = red[i] - A.g[i];
      S.y[i] = S.lam[i] = S.s[i] = S.lampq[i] = 1.0;
      S.mu[i] = fmax(0.5 * A.c[i], 1.0);
    }
    S.z = S.zeta = S.eps = 1.0;
    S.err = 1e30;
    S.lasterr = 0.0;
    S.nsub = 0;
    S.overflow = 0;
    S.step = 0.0;
  }
  __syncthreads();

  while (S.eps > 1e-6) {
    __syncthreads();
    if (threadIdx.x == 0) { S.err = 1e30; S.damp = 1.0; S.stays = 0; }
    __syncthreads();
    while (S.err > 0.9 * S.eps) {
      // ---- N1: Newton system and the KKT error at the current point
      const double eps = S.eps;
      double lpq[M], lc[M];
      for (int i = 0; i < M; ++i) { lpq[i] = S.lampq[i]; lc[i] = S.lam[i]; }
      constexpr int kA = 0, kB = M * M, kG = M * M + M, kV = M * M + 2 * M, kX = kV + 1;
      for (int k = 0; k < kX; ++k) v[k] = 0.0;
      v[kX] = 0.0;
      for (int j = j0; j < n; j += js) {
        const double x = A.x[j], ux = A.U[j] - x, xl = x - A.L[j];
        const double ux2 = ux * ux, xl2 = xl * xl;
        const double al = A.alpha[j], be = A.beta[j], xij = A.xi[j], etaj = A.eta[j];
        double pl = A.p[j], ql = A.q[j], pc = pl, qc = ql, G[M];
#pragma unroll
        for (int i = 0; i < M; ++i) {
          const double pi = A.p[(size_t)(i + 1) * n + j], qi = A.q[(size_t)(i + 1) * n + j];
          pl += lpq[i] * pi;
          ql += lpq[i] * qi;
          pc += lc[i] * pi;
          qc += lc[i] * qi;
          G[i] = pi / ux2 - qi / xl2;
          v[kG + i] += pi / ux + qi / xl;
        }
        const double psi = 2.0 * pl / (ux2 * ux) + 2.0 * ql / (xl2 * xl);
        const double xa = x - al, bx = be - x;
        const double Dx = psi + xij / xa + etaj / bx;
        const double varphi = pl / ux2 - ql / xl2;
        const double dlx = -(eps / xa - eps / bx - varphi);
        A.Dx[j] = Dx;
        A.dlx[j] = dlx;
#pragma unroll
        for (int i = 0; i < M; ++i) {
#pragma unroll
          for (int k = 0; k < M; ++k) v[kA + i * M + k] += G[i] * (G[k] / Dx);
          v[kB + i] += G[i] * (dlx / Dx);
        }
        const double rex = pc / ux2 - qc / xl2 - xij + etaj;
        const double rexsi = xij * xa - eps;
        const double reeta = etaj * bx - eps;
        v[kV] += rex * rex + rexsi * rexsi + reeta * reeta;
        v[kX] = fmax(v[kX], fmax(fabs(rex), fmax(fabs(rexsi), fabs(reeta))));
      }
      grid_reduce(grid, v, kX, 1, A.part, rs, wsum, red);
      if (threadIdx.x == 0) {
        constexpr int K = M + 1;
        double Ms[K][K], r[K], Dy[M], dely[M], la = 0.0;
        for (int i = 0; i < M; ++i) la += S.lam[i] * A.a[i];
        for (int i = 0; i < M; ++i) {
          Dy[i] = A.d[i] + S.mu[i] / S.y[i];
          const double Dl = S.s[i] / S.lam[i];
          dely[i] = -(S.lam[i] + eps / S.y[i] - A.c[i] - A.d[i] * S.y[i]);
          const double dell = -(S.z * A.a[i] + S.y[i] + S.b[i] - eps / S.lam[i] - red[kG + i]);
          for (int k = 0; k < M; ++k) Ms[i][k] = red[kA + i * M + k];
          Ms[i][i] += Dl + 1.0 / Dy[i];
          Ms[i][M] = A.a[i];
          Ms[M][i] = A.a[i];
          r[i] = (dell + dely[i] / Dy[i]) - red[kB + i];
        }
        Ms[M][M] = -S.zeta / S.z;
        r[M] = -(la + eps / S.z - A.a0);
        small_solve<K>(Ms, r);
        S.dz = r[M];
        for (int i = 0; i < M; ++i) {
          S.dl[i] = r[i];
          S.dy[i] = S.dl[i] / Dy[i] - dely[i] / Dy[i];
          S.dmu[i] = eps / S.y[i] - S.dy[i] * S.mu[i] / S.y[i] - S.mu[i];
          S.ds[i] = eps / S.lam[i] - S.s[i] / S.lam[i] * S.dl[i] - S.s[i];
        }
        S.dzeta = eps / S.z - S.zeta - (S.zeta / S.z) * S.dz;
        // the error at the current point (damping 1) records lambda for p/q lambda
        double e2, ei;
        kkt_scalars<M>(A, S, 0.0, 1.0, red[kV], red[kX], red + kG, &e2, &ei);
        S.old_err = e2;
        for (int i = 0; i < M; ++i) S.lampq[i] = S.lam[i];
      }
      __syncthreads();
      // ---- N2: primal direction and step bound
      double dl[M];
      for (int i = 0; i < M; ++i) dl[i] = S.dl[i];
      v[0] = v[1] = v[2] = -1e300;
      for (int j = j0; j < n; j += js) {
        const double x = A.x[j], ux = A.U[j] - x, xl = x - A.L[j];
        const double ux2 = ux * ux, xl2 = xl * xl;
        const double xa = x - A.alpha[j], bx = A.beta[j] - x, Dx = A.Dx[j];
        const double xij = A.xi[j], etaj = A.eta[j];
        double dxj = -A.dlx[j] / Dx;
#pragma unroll
        for (int i = 0; i < M; ++i) {
          const double Gi = A.p[(size_t)(i + 1) * n + j] / ux2 - A.q[(size_t)(i + 1) * n + j] / xl2;
          dxj -= dl[i] * Gi / Dx;
        }
        const double dxij = eps / xa - dxj / xa * xij - xij;
        const double detaj = eps / bx + etaj / bx * dxj - etaj;
        A.dx[j] = dxj;
        A.dxi[j] = dxij;
        A.deta[j] = detaj;
        v[0] = fmax(v[0], (-1.0 / kStepFrac) * (dxj / xa));
        v[1] = fmax(v[1], (1.0 / kStepFrac) * (dxj / bx));
        v[2] = fmax(v[2], fmax((-1.0 / kStepFrac) * dxij / xij, (-1.0 / kStepFrac) * detaj / etaj));
      }
      grid_reduce(grid, v, 0, 3, A.part, rs, wsum, red);
      if (threadIdx.x == 0) {
        double t3 = red[2];
        for (int i = 0; i < M; ++i) {
          t3 = fmax(t3, (-1.0 / kStepFrac) * S.dy[i] / S.y[i]);
          t3 = fmax(t3, (-1.0 / kStepFrac) * S.dl[i] / S.lam[i]);
          t3 = fmax(t3, (-1.0 / kStepFrac) * S.dmu[i] / S.mu[i]);
          t3 = fmax(t3, (-1.0 / kStepFrac) * S.ds[i] / S.s[i]);
        }
        t3 = fmax(t3, (-1.0 / kStepFrac) * S.dz / S.z);
        t3 = fmax(t3, (-1.0 / kStepFrac) * S.dzeta / S.zeta);
        S.step = 1.0 / fmax(fmax(red[0], red[1]), fmax(t3, 1.0));
        S.new_err = 1e30;
        S.new_inf = 1e30;
        S.accept = 0;
      }
      __syncthreads();
      // ---- LS: backtracking line search
      while (S.step > 1e-12 && S.new_err > S.old_err) {
        const double t = S.step;
        double lt[M];
        for (int i = 0; i < M; ++i) lt[i] = S.lam[i] + t * S.dl[i];
        for (int k = 0; k <= M; ++k) v[k] = 0.0;
        v[M + 1] = 0.0;
        for (int j = j0; j < n; j += js) {
          const double xt = A.x[j] + t * A.dx[j];
          const double xit = A.xi[j] + t * A.dxi[j], etat = A.eta[j] + t * A.deta[j];
          const double ux = A.U[j] - xt, xl = xt - A.L[j];
          double pl = A.p[j], ql = A.q[j];
#pragma unroll
          for (int i = 0; i < M; ++i) {
            const double pi = A.p[(size_t)(i + 1) * n + j], qi = A.q[(size_t)(i + 1) * n + j];
            pl += lt[i] * pi;
            ql += lt[i] * qi;
            v[i] += pi / ux + qi / xl;
          }
          const double rex = pl / (ux * ux) - ql / (xl * xl) - xit + etat;
          const double rexsi = xit * (xt - A.alpha[j]) - eps;
          const double reeta = etat * (A.beta[j] - xt) - eps;
          v[M] += rex * rex + rexsi * rexsi + reeta * reeta;
          v[M + 1] = fmax(v[M + 1], fmax(fabs(rex), fmax(fabs(rexsi), fabs(reeta))));
        }
        grid_reduce(grid, v, M + 1, 1, A.part, rs, wsum, red);
        if (threadIdx.x == 0) {
          double e2, ei;
          kkt_scalars<M>(A, S, t, S.damp, red[M], red[M + 1], red, &e2, &ei);
          S.new_err = e2;
          S.new_inf = ei;
          for (int i = 0; i < M; ++i) S.lampq[i] = lt[i];
          if (e2 < S.old_err) {
            S.accept = 1;
            for (int i = 0; i < M; ++i) {
              S.y[i] = S.y[i] + t * S.dy[i];
              S.lam[i] = S.lam[i] + t * S.dl[i];
              S.mu[i] = S.mu[i] + t * S.dmu[i];
              S.s[i] = S.s[i] + t * S.ds[i];
            }
            S.z = S.z + t * S.dz;
            S.zeta = S.zeta + t * S.dzeta;
          } else {
            S.step = t / 2;
          }
        }
        __syncthreads();
        if (S.accept) {
          for (int j = j0; j < n; j += js) {
            A.x[j] = A.x[j] + t * A.dx[j];
            A.xi[j] = A.xi[j] + t * A.dxi[j];
            A.eta[j] = A.eta[j] + t * A.deta[j];
          }
          break;
        }
      }
      if (threadIdx.x == 0) {
        const double err = S.new_inf;
        S.err = err;
        if ((err - S.lasterr) / err < 1e-5) ++S.stays;
        else S.stays = 0;
        S.lasterr = err;
        if (S.stays > 6) { S.stays = 0; S.damp *= 10.0; }
        if (S.nsub++ > 80) S.overflow = 1;
      }
      __syncthreads();
      if (S.overflow) break;
    }
    if (S.overflow) break;
    __syncthreads();
    if (threadIdx.x == 0) S.eps *= 0.1;
    __syncthreads();
  }

  // ---- asymptotes, move limits, change of the design
  v[0] = 0.0;
  for (int j = j0; j < n; j += js) {
    const double xv = A.x[j], d0 = xv - A.xold[j], d1 = A.lastdx[j];
    double gamma = 1.0;
    if (d0 * d1 > 0) gamma = 1.2;
    if (d0 * d1 < 0) gamma = 0.7;
    const double st = A.xmax[j] - A.xmin[j];
    double nl = xv - gamma * (xv - d0 - A.L[j]);
    double nu = xv + gamma * (A.U[j] - xv + d0);
    nl = fmin(fmax(nl, xv - 10.0 * st), xv - 0.01 * st);
    nu = fmin(fmax(nu, xv + 0.01 * st), xv + 10.0 * st);
    A.L[j] = nl;
    A.U[j] = nu;
    A.alpha[j] = fmax(A.xmin[j], fmax(nl + 0.1 * (xv - nl), xv - 0.5 * st));
    A.beta[j] = fmin(A.xmax[j], fmin(nu - 0.1 * (nu - xv), xv + 0.5 * st));
    A.lastdx[j] = d0;
    v[0] += d0 * d0;
  }
  grid_reduce(grid, v, 1, 0, A.part, rs, wsum, red);
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    A.stats[0] = S.nsub;
    A.stats[1] = S.err;
    A.stats[2] = S.step;
    A.stats[3] = sqrt(red[0]);
    A.stats[4] = S.overflow;
  }
}

// mma_t::init(lb, ub): bounds, asymptotes, move limits, midpoint start
// (optimization/mma_t.cu:715-766).
__global__ void k_mma_init(int n, const double* lb, const double* ub, double lbu, double ubu, double* xmin,
                           double* xmax, double* L, double* U, double* alpha, double* beta, double* x,
                           double* lastdx) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  const double lo = lb ? lb[j] : lbu, hi = ub ? ub[j] : ubu, st = hi - lo;
  const double xm = 0.5 * (lo + hi);
  const double l = fmin(fmax(lo, xm - 10.0 * st), xm - 0.01 * st);
  const double u = fmin(fmax(hi, xm + 0.01 * st), xm + 10.0 * st);
  const double a = fmax(lo, fmax(l + 0.1 * (xm - l), xm - 0.5 * st));
  const double b = fmin(hi, fmin(u - 0.1 * (u - xm), xm + 0.5 * st));
  xmin[j] = lo;
  xmax[j] = hi;
  L[j] = l;
  U[j] = u;
  alpha[j] = a;
  beta[j] = b;
  x[j] = 0.5 * (a + b);
  lastdx[j] = 0.0;
}

}  // namespace topo

using namespace topo;

struct topo_mma {
  int n = 0, m = 0, device = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  double* buf = nullptr;
  double *x, *xold, *xmin, *xmax, *L, *U, *alpha, *beta, *lastdx, *xi, *eta, *p, *q, *Dx, *dlx, *dx, *dxi,
      *deta, *part, *stats, *lbub;
  double c[kMmaMaxM], d[kMmaMaxM];
  int nblocks = 1;
  int stop_counter = 0;
  bool initialised = false;
  std::string err;
};

static int mma_fail(topo_mma* o, int code, const char* msg) {
  if (o) o->err = msg;
  return code;
}

#define MCK(call)                                                                     \
  do {                                                                                \
    cudaError_t e_ = (call);                                                          \
    if (e_ != cudaSuccess) return mma_fail(o, TOPO_E_CUDA, cudaGetErrorString(e_));   \
  } while (0)

template <int M>
static int mma_occupancy(int* per_sm) {
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, k_mma_update<M>, kMmaBlock, 0) == cudaSuccess
             ? TOPO_OK
             : TOPO_E_CUDA;
}

static int mma_alloc(topo_mma* o) {
  int cur = -1;
  MCK(cudaGetDevice(&cur));
  if (cur != o->device) MCK(cudaSetDevice(o->device));
  int sms = 0, per_sm = 0;
  MCK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, o->device));
  int rc = TOPO_OK;
  switch (o->m) {
    case 1: rc = mma_occupancy<1>(&per_sm); break;
    case 2: rc = mma_occupancy<2>(&per_sm); break;
    case 3: rc = mma_occupancy<3>(&per_sm); break;
    default: rc = mma_occupancy<4>(&per_sm); break;
  }
  if (rc != TOPO_OK || per_sm < 1) return mma_fail(o, TOPO_E_CUDA, "cooperative occupancy query failed");
  // One CTA per SM at most: enough threads for the design sizes the spline
  // lattices give, and a cheaper grid barrier than a fully populated grid.
  const long long want = ((long long)o->n + kMmaBlock - 1) / kMmaBlock;
  o->nblocks = (int)std::max(1LL, std::min<long long>(want, (long long)sms * std::min(per_sm, 1)));
  const size_t n = o->n, m1 = o->m + 1;
  const size_t total = 16 * n + 2 * m1 * n + 2 * (size_t)kMmaSlots * o->nblocks + 8 + 2 * n;
  if (cudaMalloc((void**)&o->buf, total * sizeof(double)) != cudaSuccess)
    return mma_fail(o, TOPO_E_NOMEM, "MMA device buffers");
  double* b = o->buf;
  double** vecs[] = {&o->x, &o->xold, &o->xmin, &o->xmax, &o->L, &o->U, &o->alpha, &o->beta,
                     &o->lastdx, &o->xi, &o->eta, &o->Dx, &o->dlx, &o->dx, &o->dxi, &o->deta};
  for (double** v : vecs) { *v = b; b += n; }
  o->p = b; b += m1 * n;
  o->q = b; b += m1 * n;
  o->part = b; b += 2 * (size_t)kMmaSlots * o->nblocks;
  o->stats = b; b += 8;
  o->lbub = b;
  MCK(cudaMemsetAsync(o->buf, 0, total * sizeof(double), o->stream));
  return TOPO_OK;
}

extern "C" {

int topo_mma_create(int n, int m, int device, topo_mma** out) {
  if (!out) return TOPO_E_BAD_INPUT;
  *out = nullptr;
  if (n <= 0 || m < 1 || m > kMmaMaxM) return TOPO_E_BAD_INPUT;
  topo_mma* o = new topo_mma;
  o->n = n;
  o->m = m;
  o->device = device;
  for (int i = 0; i < kMmaMaxM; ++i) { o->c[i] = 10.0; o->d[i] = 1.0; }
  if (cudaSetDevice(device) != cudaSuccess || cudaStreamCreateWithFlags(&o->stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete o;
    return TOPO_E_CUDA;
  }
  o->own_stream = true;
  const int rc = mma_alloc(o);
  if (rc != TOPO_OK) {
    cudaStreamDestroy(o->stream);
    if (o->buf) cudaFree(o->buf);
    delete o;
    return rc;
  }
  *out = o;
  return TOPO_OK;
}

int topo_mma_create_for(topo_handle* h, int m, topo_mma** out) {
  if (!h || !out) return TOPO_E_BAD_INPUT;
  *out = nullptr;
  if (m < 1 || m > kMmaMaxM) return handle_fail(h, TOPO_E_BAD_INPUT, "MMA: 1 <= m <= 4 constraints");
  SplineView sv;
  const int rc0 = handle_spline_view(h, &sv);
  if (rc0 != TOPO_OK) return rc0;
  topo_mma* o = new topo_mma;
  o->n = sv.sp.nb[0] * sv.sp.nb[1] * sv.sp.nb[2];
  o->m = m;
  o->device = sv.device;
  o->stream = sv.stream;
  o->own_stream = false;
  for (int i = 0; i < kMmaMaxM; ++i) { o->c[i] = 10.0; o->d[i] = 1.0; }
  const int rc = mma_alloc(o);
  if (rc != TOPO_OK) {
    handle_fail(h, rc, o->err.c_str());
    if (o->buf) cudaFree(o->buf);
    delete o;
    return rc;
  }
  *out = o;
  return TOPO_OK;
}

void topo_mma_destroy(topo_mma* o) {
  if (!o) return;
  cudaSetDevice(o->device);
  cudaStreamSynchronize(o->stream);
  if (o->buf) cudaFree(o->buf);
  if (o->own_stream) cudaStreamDestroy(o->stream);
  delete o;
}

const char* topo_mma_last_error(const topo_mma* o) { return o ? o->err.c_str() : "null MMA"; }

int topo_mma_size(const topo_mma* o, int* n, int* m) {
  if (!o || !n || !m) return TOPO_E_BAD_INPUT;
  *n = o->n;
  *m = o->m;
  return TOPO_OK;
}

int topo_mma_set_constraint_amplifier(topo_mma* o, double c, double d) {
  if (!o || !(d > 0) || !(c >= 0)) return mma_fail(o, TOPO_E_BAD_INPUT, "MMA: c >= 0, d > 0");
  for (int i = 0; i < kMmaMaxM; ++i) { o->c[i] = c; o->d[i] = d; }
  return TOPO_OK;
}

static int mma_init_impl(topo_mma* o, const double* lb, const double* ub, double lbu, double ubu) {
  DeviceScope device_scope(o->device);
  const double* dlb = nullptr;
  const double* dub = nullptr;
  if (lb && ub) {
    for (int j = 0; j < o->n; ++j)
      if (!(ub[j] > lb[j])) return mma_fail(o, TOPO_E_BAD_INPUT, "MMA: upper bound must exceed lower bound");
    MCK(cudaMemcpyAsync(o->lbub, lb, sizeof(double) * o->n, cudaMemcpyHostToDevice, o->stream));
    MCK(cudaMemcpyAsync(o->lbub + o->n, ub, sizeof(double) * o->n, cudaMemcpyHostToDevice, o->stream));
    dlb = o->lbub;
    dub = o->lbub + o->n;
  }
  k_mma_init<<<(o->n + 255) / 256, 256, 0, o->stream>>>(o->n, dlb, dub, lbu, ubu, o->xmin, o->xmax, o->L, o->U,
                                                         o->alpha, o->beta, o->x, o->lastdx);
  count_launch();
  MCK(cudaGetLastError());
  MCK(cudaStreamSynchronize(o->stream));
  o->stop_counter = 0;
  o->initialised = true;
  return TOPO_OK;
}

int topo_mma_init(topo_mma* o, const double* lb, const double* ub) {
  if (!o || !lb || !ub) return mma_fail(o, TOPO_E_BAD_INPUT, "MMA: null bounds");
  return mma_init_impl(o, lb, ub, 0.0, 0.0);
}

int topo_mma_init_uniform(topo_mma* o, double lb, double ub) {
  if (!o) return TOPO_E_BAD_INPUT;
  if (!(ub > lb)) return mma_fail(o, TOPO_E_BAD_INPUT, "MMA: upper bound must exceed lower bound");
  return mma_init_impl(o, nullptr, nullptr, lb, ub);
}

int topo_mma_update(topo_mma* o, const double* df_dev, const double* const* dg_dev, const double* g,
                    topo_mma_stats* stats) {
  if (!o) return TOPO_E_BAD_INPUT;
  if (!df_dev || !dg_dev || !g) return mma_fail(o, TOPO_E_BAD_INPUT, "MMA: null gradient or constraint");
  if (!o->initialised) return mma_fail(o, TOPO_E_STATE, "MMA: call topo_mma_init first");
  DeviceScope device_scope(o->device);
  MmaArgs A{};
  A.n = o->n;
  A.m = o->m;
  A.x = o->x; A.xold = o->xold; A.xmin = o->xmin; A.xmax = o->xmax; A.L = o->L; A.U = o->U;
  A.alpha = o->alpha; A.beta = o->beta; A.lastdx = o->lastdx; A.xi = o->xi; A.eta = o->eta;
  A.p = o->p; A.q = o->q; A.Dx = o->Dx; A.dlx = o->dlx; A.dx = o->dx; A.dxi = o->dxi; A.deta = o->deta;
  A.part = o->part;
  A.stats = o->stats;
  A.df = df_dev;
  for (int i = 0; i < o->m; ++i) {
    if (!dg_dev[i]) return mma_fail(o, TOPO_E_BAD_INPUT, "MMA: null constraint gradient");
    if (!std::isfinite(g[i])) return mma_fail(o, TOPO_E_BAD_INPUT, "MMA: non-finite constraint value");
    A.dg[i] = dg_dev[i];
    A.g[i] = g[i];
    A.a[i] = 0.0;
    A.c[i] = o->c[i];
    A.d[i] = o->d[i];
  }
  A.a0 = 1.0;
  void* args[] = {&A};
  const void* fn = nullptr;
  switch (o->m) {
    case 1: fn = (const void*)k_mma_update<1>; break;
    case 2: fn = (const void*)k_mma_update<2>; break;
    case 3: fn = (const void*)k_mma_update<3>; break;
    default: fn = (const void*)k_mma_update<4>; break;
  }
  MCK(cudaLaunchCooperativeKernel(fn, dim3(o->nblocks), dim3(kMmaBlock), args, 0, o->stream));
  count_launch();
  double hs[5];
  MCK(cudaMemcpyAsync(hs, o->stats, sizeof(hs), cudaMemcpyDeviceToHost, o->stream));
  MCK(cudaStreamSynchronize(o->stream));
  // mma_t::update (optimization/mma_t.cpp:42-50): converged once the change has
  // stayed below 1e-3 for more than 10 calls
  if (hs[3] < 1e-3) ++o->stop_counter;
  if (stats) {
    stats->subiterations = (int)hs[0];
    stats->kkt_err = hs[1];
    stats->step = hs[2];
    stats->dx_norm = hs[3];
    stats->overflow = (int)hs[4];
    stats->converged = o->stop_counter > 10;
  }
  if (!std::isfinite(hs[3])) return mma_fail(o, TOPO_E_NONFINITE, "MMA: non-finite design change");
  return TOPO_OK;
}

int topo_mma_get_x(topo_mma* o, double* dst_dev) {
  if (!o || !dst_dev) return mma_fail(o, TOPO_E_BAD_INPUT, "MMA: null destination");
  DeviceScope device_scope(o->device);
  MCK(cudaMemcpyAsync(dst_dev, o->x, sizeof(double) * o->n, cudaMemcpyDeviceToDevice, o->stream));
  return TOPO_OK;
}

int topo_mma_read_x(topo_mma* o, double* dst_host) {
  if (!o || !dst_host) return mma_fail(o, TOPO_E_BAD_INPUT, "MMA: null destination");
  DeviceScope device_scope(o->device);
  MCK(cudaMemcpyAsync(dst_host, o->x, sizeof(double) * o->n, cudaMemcpyDeviceToHost, o->stream));
  MCK(cudaStreamSynchronize(o->stream));
  return TOPO_OK;
}

// Persistent MMA state: the iterate and its history (x, xold), the bounds,
// the asymptotes and their last step (the first nine per-variable arrays),
// the bound arrays, the constraint amplifiers and the stop counter.  The
// per-update scratch (subproblem variables, partial sums) is not kept.
static const char kMmaMagic[8] = {'T', 'O', 'P', 'O', 'M', 'M', 'A', '1'};

int topo_mma_checkpoint_save(topo_mma* o, const char* path) {
  if (!o || !path) return mma_fail(o, TOPO_E_BAD_INPUT, "MMA: null path");
  DeviceScope device_scope(o->device);
  const size_t n = o->n;
  std::vector<double> st(11 * n);
  MCK(cudaMemcpyAsync(st.data(), o->x, sizeof(double) * 9 * n, cudaMemcpyDeviceToHost, o->stream));
  MCK(cudaMemcpyAsync(st.data() + 9 * n, o->lbub, sizeof(double) * 2 * n, cudaMemcpyDeviceToHost, o->stream));
  MCK(cudaStreamSynchronize(o->stream));
  FILE* f = std::fopen(path, "wb");
  if (!f) return mma_fail(o, TOPO_E_BAD_INPUT, "MMA: cannot open checkpoint file");
  const int32_t hdr[4] = {o->n, o->m, o->stop_counter, o->initialised ? 1 : 0};
  bool ok = std::fwrite(kMmaMagic, 1, 8, f) == 8 && std::fwrite(hdr, sizeof(hdr), 1, f) == 1 &&
            std::fwrite(o->c, sizeof(o->c), 1, f) == 1 && std::fwrite(o->d, sizeof(o->d), 1, f) == 1 &&
            std::fwrite(st.data(), sizeof(double), st.size(), f) == st.size();
  ok = (std::fclose(f) == 0) && ok;
  return ok ? TOPO_OK : mma_fail(o, TOPO_E_BAD_INPUT, "MMA: checkpoint write failed");
}

int topo_mma_checkpoint_load(topo_mma* o, const char* path) {
  if (!o || !path) return mma_fail(o, TOPO_E_BAD_INPUT, "MMA: null path");
  DeviceScope device_scope(o->device);
  FILE* f = std::fopen(path, "rb");
  if (!f) return mma_fail(o, TOPO_E_BAD_INPUT, "MMA: cannot open checkpoint file");
  char magic[8];
  int32_t hdr[4];
  double c[kMmaMaxM], d[kMmaMaxM];
  std::vector<double> st(11 * (size_t)o->n);
  bool ok = std::fread(magic, 1, 8, f) == 8 && std::memcmp(magic, kMmaMagic, 8) == 0 &&
            std::fread(hdr, sizeof(hdr), 1, f) == 1 && hdr[0] == o->n && hdr[1] == o->m &&
            std::fread(c, sizeof(c), 1, f) == 1 && std::fread(d, sizeof(d), 1, f) == 1 &&
            std::fread(st.data(), sizeof(double), st.size(), f) == st.size();
  std::fclose(f);
  if (!ok) return mma_fail(o, TOPO_E_BAD_INPUT, "MMA: not a checkpoint of this size");
  MCK(cudaMemcpyAsync(o->x, st.data(), sizeof(double) * 9 * o->n, cudaMemcpyHostToDevice, o->stream));
  MCK(cudaMemcpyAsync(o->lbub, st.data() + 9 * (size_t)o->n, sizeof(double) * 2 * o->n, cudaMemcpyHostToDevice,
                      o->stream));
  MCK(cudaStreamSynchronize(o->stream));
  std::memcpy(o->c, c, sizeof(c));
  std::memcpy(o->d, d, sizeof(d));
  o->stop_counter = hdr[2];
  o->initialised = hdr[3] != 0;
  return TOPO_OK;
}

int topo_mma_write_x(topo_mma* o, const double* src_host) {
  if (!o || !src_host) return mma_fail(o, TOPO_E_BAD_INPUT, "MMA: null source");
  DeviceScope device_scope(o->device);
  MCK(cudaMemcpyAsync(o->x, src_host, sizeof(double) * o->n, cudaMemcpyHostToDevice, o->stream));
  MCK(cudaStreamSynchronize(o->stream));
  return TOPO_OK;
}

}  // extern "C"
