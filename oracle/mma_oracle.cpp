/*
 * mma_oracle.cpp -- CPU FP64 restatement of the reference's Method of Moving
 * Asymptotes optimiser (optimization/mma_t.h, mma_t.cpp, mma_t.cu).
 *
 * TEST INFRASTRUCTURE ONLY: the parity checker for the CUDA MMA in
 * libtopo_gb300.so.  Serial, plain loops, no vector library.
 *
 * The algorithm is Svanberg's MMA with the primal-dual interior-point
 * subproblem solver, in the reference's exact order of steps:
 *   - approximation p, q and the proxy constraint offset b:
 *     optimization/mma_t.cu:15-130 (mma_subproblem_t::init)
 *   - reset of the primal-dual point: optimization/mma_t.cu:702-713
 *   - Newton loop with epsilon continuation, step bound, backtracking line
 *     search on the 2-norm of the KKT residual, damping of the lambda rows
 *     when the error stalls, at most 81 Newton steps per update:
 *     optimization/mma_t.cu:330-508 (solve), 510-566 (search_step),
 *     569-672 (kkt_err), 230-327 (solveLinearSystem)
 *   - asymptote and move-limit update: optimization/mma_t.cu:156-227
 *   - convergence counter: optimization/mma_t.cpp:18-51
 * Parameters as in the reference constructor (mma_t.h:202-214):
 * a0 = 1, a = 0, c = 10, d = 1.  The reference computes in FP32; this
 * restatement and the CUDA product compute in FP64.  The (m+1)x(m+1) reduced
 * system is solved by Gaussian elimination with partial pivoting where the
 * reference uses a column-pivoted Householder QR (optimization/mma_t.cpp:88-122);
 * both give the solution of the same nonsingular system.
 */
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "topo_oracle.h"

namespace {
constexpr double kStepFrac = 0.99;  // asym_clamp_factor, optimization/mma_t.h:20

struct Kkt {
  double err2, errinf;
};
}  // namespace

struct orc_mma {
  int n, m;
  std::vector<double> x, xmin, xmax, L, U, alpha, beta, lastdx, xi, eta;
  std::vector<double> p, q;  // [(m+1)][n]
  std::vector<double> a, c, d;
  double a0 = 1.0;
  int stop_counter = 0;
  double stats[5] = {0, 0, 0, 0, 0};
};

extern "C" {

orc_mma* orc_mma_create(int n, int m) {
  if (n <= 0 || m <= 0 || m > ORC_MMA_MAX_M) return nullptr;
  orc_mma* o = new orc_mma;
  o->n = n;
  o->m = m;
  for (auto* v : {&o->x, &o->xmin, &o->xmax, &o->L, &o->U, &o->alpha, &o->beta, &o->lastdx, &o->xi, &o->eta})
    v->assign(n, 0.0);
  o->p.assign((size_t)(m + 1) * n, 0.0);
  o->q.assign((size_t)(m + 1) * n, 0.0);
  o->a.assign(m, 0.0);
  o->c.assign(m, 10.0);
  o->d.assign(m, 1.0);
  return o;
}

void orc_mma_destroy(orc_mma* o) { delete o; }

void orc_mma_set_constraint_amplifier(orc_mma* o, double c, double d) {
  std::fill(o->c.begin(), o->c.end(), c);
  std::fill(o->d.begin(), o->d.end(), d);
}

/* mma_t::init(lb, ub): set_bound + clamp_asymptotes (optimization/mma_t.cu:754-766, 715-730). */
void orc_mma_init(orc_mma* o, const double* lb, const double* ub) {
  for (int j = 0; j < o->n; ++j) {
    const double lo = lb[j], hi = ub[j], st = hi - lo;
    o->xmin[j] = lo;
    o->xmax[j] = hi;
    double x = 0.5 * (lo + hi);
    double l = std::min(std::max(lo, x - 10.0 * st), x - 0.01 * st);
    double u = std::min(std::max(hi, x + 0.01 * st), x + 10.0 * st);
    o->L[j] = l;
    o->U[j] = u;
    o->alpha[j] = std::max(lo, std::max(l + 0.1 * (x - l), x - 0.5 * st));
    o->beta[j] = std::min(hi, std::min(u - 0.1 * (u - x), x + 0.5 * st));
    o->x[j] = 0.5 * (o->alpha[j] + o->beta[j]);
    o->lastdx[j] = 0.0;
  }
  o->stop_counter = 0;
}

void orc_mma_get_x(const orc_mma* o, double* x) { std::memcpy(x, o->x.data(), sizeof(double) * o->n); }
void orc_mma_set_x(orc_mma* o, const double* x) { std::memcpy(o->x.data(), x, sizeof(double) * o->n); }
void orc_mma_get_stats(const orc_mma* o, double* s5) { std::memcpy(s5, o->stats, sizeof(o->stats)); }

/* Solve the dense k x k system M s = r in place (partial pivoting). */
static void gauss_solve(int k, double* M, double* r) {
  for (int c = 0; c < k; ++c) {
    int piv = c;
    for (int i = c + 1; i < k; ++i)
      if (std::fabs(M[i * k + c]) > std::fabs(M[piv * k + c])) piv = i;
    if (piv != c) {
      for (int j = 0; j < k; ++j) std::swap(M[c * k + j], M[piv * k + j]);
      std::swap(r[c], r[piv]);
    }
    const double dinv = 1.0 / M[c * k + c];
    for (int i = c + 1; i < k; ++i) {
      const double f = M[i * k + c] * dinv;
      if (f == 0.0) continue;
      for (int j = c; j < k; ++j) M[i * k + j] -= f * M[c * k + j];
      r[i] -= f * r[c];
    }
  }
  for (int c = k - 1; c >= 0; --c) {
    double s = r[c];
    for (int j = c + 1; j < k; ++j) s -= M[c * k + j] * r[j];
    r[c] = s / M[c * k + c];
  }
}

/*
 * One MMA step (mma_t::update, optimization/mma_t.cpp:18-51).  df[n] is the
 * objective gradient, dg[m*n] the constraint gradients (constraint-major), g[m]
 * the constraint values.  Returns 1 once the design change has stayed below
 * 1e-3 in 2-norm for more than 10 calls.
 */
int orc_mma_update(orc_mma* o, const double* df, const double* dg, const double* g) {
  const int n = o->n, m = o->m;
  std::vector<double> curx(o->x);
  std::vector<double>& x = o->x;
  const double* L = o->L.data();
  const double* U = o->U.data();
  const double* al = o->alpha.data();
  const double* be = o->beta.data();
  double* xi = o->xi.data();
  double* eta = o->eta.data();
  // ---- approximation (mma_subproblem_t::init)
  std::vector<double> b(m, 0.0);
  for (int i = 0; i <= m; ++i) {
    const double* dfi = i == 0 ? df : dg + (size_t)(i - 1) * n;
    for (int j = 0; j < n; ++j) {
      const double ux = U[j] - x[j], xl = x[j] - L[j];
      const double pos = std::max(dfi[j], 0.0), neg = std::max(-dfi[j], 0.0);
      const double reg = 1e-5 / (o->xmax[j] - o->xmin[j]);
      o->p[(size_t)i * n + j] = ux * ux * (1.001 * pos + 0.001 * neg + reg);
      o->q[(size_t)i * n + j] = xl * xl * (0.001 * pos + 1.001 * neg + reg);
    }
  }
  for (int i = 0; i < m; ++i) {
    double s = 0.0;
    for (int j = 0; j < n; ++j)
      s += o->p[(size_t)(i + 1) * n + j] / (U[j] - x[j]) + o->q[(size_t)(i + 1) * n + j] / (x[j] - L[j]);
    b[i] = s - g[i];
  }
  // ---- reset of the primal-dual point
  std::vector<double> y(m, 1.0), lam(m, 1.0), s(m, 1.0), mu(m), lampq(m, 1.0);
  double z = 1.0, zeta = 1.0, eps = 1.0;
  for (int i = 0; i < m; ++i) mu[i] = std::max(0.5 * o->c[i], 1.0);
  for (int j = 0; j < n; ++j) {
    x[j] = 0.5 * (al[j] + be[j]);
    xi[j] = std::max(1.0 / (x[j] - al[j]), 1.0);
    eta[j] = std::max(1.0 / (be[j] - x[j]), 1.0);
  }
  const double* a = o->a.data();
  const double* c = o->c.data();
  const double* d = o->d.data();
  const double a0 = o->a0;
  std::vector<double> dxv(n), dxiv(n), detav(n), Dx(n), dlx(n), G((size_t)m * n);

  // KKT residual at (x + t dx, ...) with lambda rows divided by damp; also
  // records the lambda used for plambda/qlambda (optimization/mma_t.cu:569-585).
  auto kkt = [&](double t, const double* dyv, double dzv, const double* dlv, const double* dmv, double dzetav,
                 const double* dsv, double damp) -> Kkt {
    double err2 = 0.0, errinf = -10.0;
    std::vector<double> lt(m), yt(m), mt(m), st(m), gsum(m, 0.0);
    for (int i = 0; i < m; ++i) {
      lt[i] = lam[i] + t * dlv[i];
      yt[i] = y[i] + t * dyv[i];
      mt[i] = mu[i] + t * dmv[i];
      st[i] = s[i] + t * dsv[i];
      lampq[i] = lt[i];
    }
    const double zt = z + t * dzv, zetat = zeta + t * dzetav;
    double vsum = 0.0, vmax = 0.0;
    for (int j = 0; j < n; ++j) {
      const double xt = x[j] + t * dxv[j], xit = xi[j] + t * dxiv[j], etat = eta[j] + t * detav[j];
      const double ux = U[j] - xt, xl = xt - L[j];
      double pl = o->p[j], ql = o->q[j];
      for (int i = 0; i < m; ++i) {
        pl += lt[i] * o->p[(size_t)(i + 1) * n + j];
        ql += lt[i] * o->q[(size_t)(i + 1) * n + j];
        gsum[i] += o->p[(size_t)(i + 1) * n + j] / ux + o->q[(size_t)(i + 1) * n + j] / xl;
      }
      const double rex = pl / (ux * ux) - ql / (xl * xl) - xit + etat;
      const double rexsi = xit * (xt - al[j]) - eps;
      const double reeta = etat * (be[j] - xt) - eps;
      vsum += rex * rex + rexsi * rexsi + reeta * reeta;
      vmax = std::max(vmax, std::max(std::fabs(rex), std::max(std::fabs(rexsi), std::fabs(reeta))));
    }
    err2 += vsum;
    errinf = std::max(errinf, vmax);
    double la = 0.0;
    for (int i = 0; i < m; ++i) la += lt[i] * a[i];
    for (int i = 0; i < m; ++i) {
      const double rey = c[i] + d[i] * yt[i] - lt[i] - mt[i];
      const double relam = (gsum[i] - a[i] * zt - yt[i] + st[i] - b[i]) / damp;
      const double remu = mt[i] * yt[i] - eps;
      const double res = lt[i] * st[i] - eps;
      err2 += rey * rey + relam * relam + remu * remu + res * res;
      errinf = std::max(errinf, std::max(std::max(std::fabs(rey), std::fabs(relam)),
                                         std::max(std::fabs(remu), std::fabs(res))));
    }
    const double rez = a0 - zetat - la, rezet = zetat * zt - eps;
    err2 += rez * rez + rezet * rezet;
    errinf = std::max(errinf, std::max(std::fabs(rez), std::fabs(rezet)));
    return {std::sqrt(err2), errinf};
  };

  double err = 1e30, lasterr = 0.0, last_step = 0.0;
  int nsub = 0;
  bool overflow = false;
  std::vector<double> dy(m), dl(m), dmu(m), ds(m), A((size_t)m * m), B(m), gp(m);
  while (eps > 1e-6) {
    err = 1e30;
    double damp = 1.0;
    int stays = 0;
    while (err > 0.9 * eps) {
      // ---- Newton system (Psi, Dx, G, gproxy, varphi, delta_x)
      std::fill(A.begin(), A.end(), 0.0);
      std::fill(B.begin(), B.end(), 0.0);
      std::fill(gp.begin(), gp.end(), 0.0);
      for (int j = 0; j < n; ++j) {
        const double ux = U[j] - x[j], xl = x[j] - L[j];
        const double ux2 = ux * ux, xl2 = xl * xl;
        double pl = o->p[j], ql = o->q[j];
        for (int i = 0; i < m; ++i) {
          pl += lampq[i] * o->p[(size_t)(i + 1) * n + j];
          ql += lampq[i] * o->q[(size_t)(i + 1) * n + j];
        }
        const double psi = 2.0 * pl / (ux2 * ux) + 2.0 * ql / (xl2 * xl);
        const double xa = x[j] - al[j], bx = be[j] - x[j];
        Dx[j] = psi + xi[j] / xa + eta[j] / bx;
        const double varphi = pl / ux2 - ql / xl2;
        dlx[j] = -(eps / xa - eps / bx - varphi);
        for (int i = 0; i < m; ++i) {
          const double pi = o->p[(size_t)(i + 1) * n + j], qi = o->q[(size_t)(i + 1) * n + j];
          G[(size_t)i * n + j] = pi / ux2 - qi / xl2;
          gp[i] += pi / ux + qi / xl;
        }
        for (int i = 0; i < m; ++i) {
          const double gi = G[(size_t)i * n + j];
          for (int k = 0; k < m; ++k) A[i * m + k] += gi * (G[(size_t)k * n + j] / Dx[j]);
          B[i] += gi * (dlx[j] / Dx[j]);
        }
      }
      // ---- reduced (m+1) system for (dlambda, dz) (solveLinearSystem)
      const int k = m + 1;
      std::vector<double> M((size_t)k * k, 0.0), r(k, 0.0), Dy(m), dly(m);
      double la = 0.0;
      for (int i = 0; i < m; ++i) la += lam[i] * a[i];
      for (int i = 0; i < m; ++i) {
        Dy[i] = d[i] + mu[i] / y[i];
        const double Dl = s[i] / lam[i];
        const double dely = -(lam[i] + eps / y[i] - c[i] - d[i] * y[i]);
        const double dell = -(z * a[i] + y[i] + b[i] - eps / lam[i] - gp[i]);
        dly[i] = dely;
        for (int q2 = 0; q2 < m; ++q2) M[i * k + q2] = A[i * m + q2];
        M[i * k + i] += Dl + 1.0 / Dy[i];
        M[i * k + m] = a[i];
        M[m * k + i] = a[i];
        r[i] = (dell + dely / Dy[i]) - B[i];
      }
      M[m * k + m] = -zeta / z;
      r[m] = -(la + eps / z - a0);
      gauss_solve(k, M.data(), r.data());
      const double dz = r[m];
      for (int i = 0; i < m; ++i) {
        dl[i] = r[i];
        dy[i] = dl[i] / Dy[i] - dly[i] / Dy[i];
        dmu[i] = eps / y[i] - dy[i] * mu[i] / y[i] - mu[i];
        ds[i] = eps / lam[i] - s[i] / lam[i] * dl[i] - s[i];
      }
      const double dzeta = eps / z - zeta - (zeta / z) * dz;
      // ---- primal direction and step bound
      double t1 = -1e300, t2 = -1e300, t3 = -1e300;
      for (int j = 0; j < n; ++j) {
        const double xa = x[j] - al[j], bx = be[j] - x[j];
        double dxj = -dlx[j] / Dx[j];
        for (int i = 0; i < m; ++i) dxj -= dl[i] * G[(size_t)i * n + j] / Dx[j];
        dxv[j] = dxj;
        dxiv[j] = eps / xa - dxj / xa * xi[j] - xi[j];
        detav[j] = eps / bx + eta[j] / bx * dxj - eta[j];
        t1 = std::max(t1, (-1.0 / kStepFrac) * (dxj / xa));
        t2 = std::max(t2, (1.0 / kStepFrac) * (dxj / bx));
        t3 = std::max(t3, std::max((-1.0 / kStepFrac) * dxiv[j] / xi[j], (-1.0 / kStepFrac) * detav[j] / eta[j]));
      }
      for (int i = 0; i < m; ++i) {
        t3 = std::max(t3, (-1.0 / kStepFrac) * dy[i] / y[i]);
        t3 = std::max(t3, (-1.0 / kStepFrac) * dl[i] / lam[i]);
        t3 = std::max(t3, (-1.0 / kStepFrac) * dmu[i] / mu[i]);
        t3 = std::max(t3, (-1.0 / kStepFrac) * ds[i] / s[i]);
      }
      t3 = std::max(t3, (-1.0 / kStepFrac) * dz / z);
      t3 = std::max(t3, (-1.0 / kStepFrac) * dzeta / zeta);
      double step = 1.0 / std::max(std::max(t1, t2), std::max(t3, 1.0));
      // ---- backtracking line search (search_step)
      const Kkt old = kkt(0.0, dy.data(), dz, dl.data(), dmu.data(), dzeta, ds.data(), 1.0);
      double new_err = 1e30, new_inf = 1e30;
      while (step > 1e-12 && new_err > old.err2) {
        const Kkt nk = kkt(step, dy.data(), dz, dl.data(), dmu.data(), dzeta, ds.data(), damp);
        new_err = nk.err2;
        new_inf = nk.errinf;
        if (new_err < old.err2) {
          for (int j = 0; j < n; ++j) {
            x[j] = x[j] + step * dxv[j];
            xi[j] = xi[j] + step * dxiv[j];
            eta[j] = eta[j] + step * detav[j];
          }
          for (int i = 0; i < m; ++i) {
            y[i] = y[i] + step * dy[i];
            lam[i] = lam[i] + step * dl[i];
            mu[i] = mu[i] + step * dmu[i];
            s[i] = s[i] + step * ds[i];
          }
          z = z + step * dz;
          zeta = zeta + step * dzeta;
          break;
        }
        step /= 2;
      }
      last_step = step;
      err = new_inf;
      if ((err - lasterr) / err < 1e-5) ++stays;
      else stays = 0;
      lasterr = err;
      if (stays > 6) {
        stays = 0;
        damp *= 10.0;
      }
      if (nsub++ > 80) {
        overflow = true;
        break;
      }
    }
    if (overflow) break;
    eps *= 0.1;
  }
  // ---- asymptotes and move limits (adjust_asym), convergence counter
  double dn2 = 0.0;
  for (int j = 0; j < n; ++j) {
    const double d0 = x[j] - curx[j], d1 = o->lastdx[j];
    double gamma = 1.0;
    if (d0 * d1 > 0) gamma = 1.2;
    if (d0 * d1 < 0) gamma = 0.7;
    const double st = o->xmax[j] - o->xmin[j], xv = x[j];
    double nl = xv - gamma * (xv - d0 - o->L[j]);
    double nu = xv + gamma * (o->U[j] - xv + d0);
    nl = std::min(std::max(nl, xv - 10.0 * st), xv - 0.01 * st);
    nu = std::min(std::max(nu, xv + 0.01 * st), xv + 10.0 * st);
    o->L[j] = nl;
    o->U[j] = nu;
    o->alpha[j] = std::max(o->xmin[j], std::max(nl + 0.1 * (xv - nl), xv - 0.5 * st));
    o->beta[j] = std::min(o->xmax[j], std::min(nu - 0.1 * (nu - xv), xv + 0.5 * st));
    o->lastdx[j] = d0;
    dn2 += d0 * d0;
  }
  if (std::sqrt(dn2) < 1e-3) ++o->stop_counter;
  o->stats[0] = nsub;
  o->stats[1] = err;
  o->stats[2] = last_step;
  o->stats[3] = std::sqrt(dn2);
  o->stats[4] = overflow ? 1.0 : 0.0;
  return o->stop_counter > 10 ? 1 : 0;
}

}  // extern "C"
