// Worst-case (robust) compliance over unit loads on a load region.
//
// The reference finds the worst load with a modified power method
// (optimization/optimization.cpp:213-351): one V-cycle on K u = f, then
// f <- normalise(P u) with P the projection onto admissible loads of the load
// region (optimization/projection.cpp:289-360), until f changes by less than
// 1e-4.  The worst compliance is the largest eigenvalue of M = S^T K^-1 S, S
// the scatter from load coordinates (one normal component, or three
// components, per load vertex) to nodal forces, and f its eigenvector.
//
// Here the iteration runs on `block` load vectors at once and takes a
// Rayleigh-Ritz step each time: X (m x k, orthonormal) -> solve K U = S X for
// all k right-hand sides in one multi-RHS solve -> Y = S^T U = M X -> the
// eigenpairs of the k x k matrix X^T Y give the new basis.  The block converges
// at the rate lambda_{k+1} / lambda_1 rather than lambda_2 / lambda_1, which
// matters because the leading loads of a structure often come in near-equal
// pairs.  Every solve is warm-started from the previous displacements mapped
// into the new basis (U C, with C the same k x k map that takes Y to the new
// X), and the inner tolerance tightens as the worst load settles, so the
// solves cost a few FP64 CG iterations each once the subspace has converged.
// The k x k eigenproblem and the Gram-Schmidt orthonormalisation (m x k
// numbers) run on the host; the scatter, gather and basis map are kernels.
#include <algorithm>
#include <cmath>
#include <memory>
#include <random>
#include <vector>

#include "topo_internal.h"

namespace topo {

struct WorstState {
  int n = 0;                       // load vertices
  int* vid = nullptr;              // device [n] level-0 vertex ids
  double* nrm = nullptr;           // device [3][n] unit normals
  std::vector<int> hvid;
  std::vector<double> hnrm;
  int kcap = 0, mcap = 0;          // capacity of the block buffers
  double* X = nullptr;             // device [k][m] load coordinates
  double* Y = nullptr;             // device [k][m] S^T U
  double* C = nullptr;             // device [k][k] basis map of the displacements
  double* tmp = nullptr;           // device [k][3 nv] rotated displacements
  int64_t tmp_n = 0;
  ~WorstState() {
    for (void* p : {(void*)vid, (void*)nrm, (void*)X, (void*)Y, (void*)C, (void*)tmp})
      if (p) cudaFree(p);
  }
};

void worst_free(WorstState* w) { delete w; }

namespace {

// F[j][c][v_i] = X[j][i] n_c(i) (normal loads) or X[j][3i + c] (free), zero on
// fixed DOFs; F is zeroed before.
__global__ void k_scatter_loads(int n, int k, int m, bool free_dir, const int* vid, const double* nrm,
                                const uint8_t* vmask, int64_t nv, const double* X, double* F) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y;
  if (i >= n || j >= k) return;
  const int v = vid[i];
  const uint8_t mk = vmask[v];
  for (int c = 0; c < 3; ++c) {
    const double val = free_dir ? X[(int64_t)j * m + 3 * i + c] : X[(int64_t)j * m + i] * nrm[c * n + i];
    F[(int64_t)j * 3 * nv + c * nv + v] = ((mk >> c) & 1) ? val : 0.0;
  }
}

// Y = S^T U: Y[j][i] = n(i) . U[j][.][v_i] (normal loads) or Y[j][3i + c] = U[j][c][v_i].
__global__ void k_gather_loads(int n, int k, int m, bool free_dir, const int* vid, const double* nrm,
                               const uint8_t* vmask, int64_t nv, const double* U, double* Y) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y;
  if (i >= n || j >= k) return;
  const int v = vid[i];
  const uint8_t mk = vmask[v];
  double s = 0;
  for (int c = 0; c < 3; ++c) {
    const double u = ((mk >> c) & 1) ? U[(int64_t)j * 3 * nv + c * nv + v] : 0.0;
    if (free_dir) Y[(int64_t)j * m + 3 * i + c] = u;
    else s += nrm[c * n + i] * u;
  }
  if (!free_dir) Y[(int64_t)j * m + i] = s;
}

// out[j][e] = sum_l C[l][j] U[l][e] over k vectors of length len.
__global__ void k_basis_map(int64_t len, int k, const double* __restrict__ C, const double* __restrict__ U,
                            double* __restrict__ out) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= len) return;
  double u[32];
  for (int l = 0; l < k; ++l) u[l] = U[(int64_t)l * len + e];
  for (int j = 0; j < k; ++j) {
    double s = 0;
    for (int l = 0; l < k; ++l) s += C[l * k + j] * u[l];
    out[(int64_t)j * len + e] = s;
  }
}

// Symmetric eigenproblem of a k x k matrix by cyclic Jacobi rotations:
// eigenvalues in w (descending), eigenvectors as the columns of V (row-major).
void jacobi_eig(int k, std::vector<double> A, std::vector<double>& w, std::vector<double>& V) {
  V.assign((size_t)k * k, 0.0);
  for (int i = 0; i < k; ++i) V[(size_t)i * k + i] = 1.0;
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0, tot = 0;
    for (int p = 0; p < k; ++p)
      for (int q = 0; q < k; ++q) {
        tot += A[p * k + q] * A[p * k + q];
        if (p != q) off += A[p * k + q] * A[p * k + q];
      }
    if (off <= 1e-30 * std::max(tot, 1e-300)) break;
    for (int p = 0; p < k; ++p)
      for (int q = p + 1; q < k; ++q) {
        const double apq = A[p * k + q];
        if (std::fabs(apq) < 1e-300) continue;
        const double theta = (A[q * k + q] - A[p * k + p]) / (2 * apq);
        const double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1));
        const double c = 1 / std::sqrt(t * t + 1), s = t * c;
        for (int r = 0; r < k; ++r) {  // A <- A J (columns p, q)
          const double arp = A[r * k + p], arq = A[r * k + q];
          A[r * k + p] = c * arp - s * arq;
          A[r * k + q] = s * arp + c * arq;
        }
        for (int r = 0; r < k; ++r) {  // A <- J^T A (rows p, q)
          const double apr = A[p * k + r], aqr = A[q * k + r];
          A[p * k + r] = c * apr - s * aqr;
          A[q * k + r] = s * apr + c * aqr;
        }
        for (int r = 0; r < k; ++r) {
          const double vrp = V[r * k + p], vrq = V[r * k + q];
          V[r * k + p] = c * vrp - s * vrq;
          V[r * k + q] = s * vrp + c * vrq;
        }
      }
  }
  std::vector<int> ord(k);
  for (int i = 0; i < k; ++i) ord[i] = i;
  std::sort(ord.begin(), ord.end(), [&](int a, int b) { return A[a * k + a] > A[b * k + b]; });
  w.resize(k);
  std::vector<double> Vs((size_t)k * k);
  for (int j = 0; j < k; ++j) {
    w[j] = A[ord[j] * k + ord[j]];
    for (int r = 0; r < k; ++r) Vs[(size_t)r * k + j] = V[(size_t)r * k + ord[j]];
  }
  V.swap(Vs);
}

// Modified Gram-Schmidt on the k columns (rows of Z, [k][m]) in place, twice
// for stability; returns R^-1 (upper triangular, row-major) so that
// Z_out = Z_in R^-1.  A column whose norm collapses is replaced by a seeded
// random direction (its R^-1 column is then zero).
std::vector<double> orthonormalise(int k, int m, std::vector<double>& Z, std::mt19937_64& rng) {
  std::vector<double> Rinv((size_t)k * k, 0.0);
  for (int i = 0; i < k; ++i) Rinv[(size_t)i * k + i] = 1.0;
  std::uniform_real_distribution<double> uni(-1.0, 1.0);
  for (int pass = 0; pass < 2; ++pass) {
    for (int j = 0; j < k; ++j) {
      double* zj = &Z[(size_t)j * m];
      for (int l = 0; l < j; ++l) {
        const double* zl = &Z[(size_t)l * m];
        double d = 0;
        for (int i = 0; i < m; ++i) d += zl[i] * zj[i];
        for (int i = 0; i < m; ++i) zj[i] -= d * zl[i];
        for (int r = 0; r < k; ++r) Rinv[(size_t)r * k + j] -= d * Rinv[(size_t)r * k + l];
      }
      double nr = 0;
      for (int i = 0; i < m; ++i) nr += zj[i] * zj[i];
      nr = std::sqrt(nr);
      if (!(nr > 1e-300)) {
        for (int i = 0; i < m; ++i) zj[i] = uni(rng);
        for (int r = 0; r < k; ++r) Rinv[(size_t)r * k + j] = 0.0;
        --j;  // orthogonalise the replacement against the earlier columns
        continue;
      }
      for (int i = 0; i < m; ++i) zj[i] /= nr;
      for (int r = 0; r < k; ++r) Rinv[(size_t)r * k + j] /= nr;
    }
  }
  return Rinv;
}

}  // namespace
}  // namespace topo

using namespace topo;

extern "C" {

int topo_set_load_region(topo_handle* h, int n, const int* vertices, const double* normals) {
  LevelView lv;
  RET_IF(handle_level_view(h, &lv));
  DeviceScope scope(lv.device);
  if (n <= 0 || !vertices) return handle_fail(h, TOPO_E_BAD_INPUT, "load region: no vertices");
  std::unique_ptr<WorstState> w(new WorstState);
  w->n = n;
  w->hvid.assign(vertices, vertices + n);
  w->hnrm.assign((size_t)3 * n, 0.0);
  for (int i = 0; i < n; ++i) {
    if (vertices[i] < 0 || vertices[i] >= lv.d.nv)
      return handle_fail(h, TOPO_E_BAD_INPUT, "load region: vertex id out of range");
    if (normals) {
      const double a = normals[3 * i], b = normals[3 * i + 1], c = normals[3 * i + 2];
      const double nr = std::sqrt(a * a + b * b + c * c);
      if (!(nr > 0)) return handle_fail(h, TOPO_E_BAD_INPUT, "load region: zero normal");
      w->hnrm[i] = a / nr; w->hnrm[n + i] = b / nr; w->hnrm[2 * (size_t)n + i] = c / nr;
    }
  }
  if (cudaMalloc(&w->vid, sizeof(int) * n) != cudaSuccess || cudaMalloc(&w->nrm, sizeof(double) * 3 * n) != cudaSuccess) {
    cudaGetLastError();
    return handle_fail(h, TOPO_E_NOMEM, "load region buffers");
  }
  cudaMemcpyAsync(w->vid, w->hvid.data(), sizeof(int) * n, cudaMemcpyHostToDevice, lv.stream);
  cudaMemcpyAsync(w->nrm, w->hnrm.data(), sizeof(double) * 3 * n, cudaMemcpyHostToDevice, lv.stream);
  if (cudaStreamSynchronize(lv.stream) != cudaSuccess) return handle_fail(h, TOPO_E_CUDA, "load region upload");
  WorstState*& slot = handle_worst_slot(h);
  if (slot) worst_free(slot);
  slot = w.release();
  return TOPO_OK;
}

int topo_worst_compliance(topo_handle* h, const topo_worst_opts* o, topo_worst_stats* stats) {
  LevelView lv;
  RET_IF(handle_level_view(h, &lv));
  DeviceScope scope(lv.device);
  if (!o) return TOPO_E_BAD_INPUT;
  WorstState* w = handle_worst_slot(h);
  if (!w) return handle_fail(h, TOPO_E_STATE, "worst-case compliance: call topo_set_load_region first");
  const int k = o->block;
  if (k < 1 || k > 32 || o->max_iter < 1 || !(o->tol > 0) || !(o->solve.rtol > 0))
    return handle_fail(h, TOPO_E_BAD_INPUT, "worst-case compliance: block 1..32, max_iter >= 1, tol > 0, rtol > 0");
  const bool free_dir = o->free_direction != 0;
  const int n = w->n, m = free_dir ? 3 * n : n;
  if (k > m) return handle_fail(h, TOPO_E_BAD_INPUT, "worst-case compliance: block larger than the load space");
  const cudaStream_t s = lv.stream;
  const int64_t nv = lv.d.nv, n3 = 3 * nv;
  // buffers
  int rc = TOPO_OK;
  void* dptr = nullptr;
  size_t cnt = 0;
  if (topo_device_ptr(h, TOPO_MULTI_F, 0, &dptr) != TOPO_OK || topo_array_size(h, TOPO_MULTI_F, 0, &cnt) != TOPO_OK ||
      cnt < (size_t)k * n3)
    RET_IF(topo_multi_reserve(h, k));
  if (w->kcap < k || w->mcap < m) {
    for (double** p : {&w->X, &w->Y, &w->C, &w->tmp}) { if (*p) cudaFree(*p); *p = nullptr; }
    if (cudaMalloc(&w->X, sizeof(double) * k * m) != cudaSuccess ||
        cudaMalloc(&w->Y, sizeof(double) * k * m) != cudaSuccess ||
        cudaMalloc(&w->C, sizeof(double) * k * k) != cudaSuccess ||
        cudaMalloc(&w->tmp, sizeof(double) * k * n3) != cudaSuccess) {
      cudaGetLastError();
      w->kcap = w->mcap = 0;
      return handle_fail(h, TOPO_E_NOMEM, "worst-case compliance buffers");
    }
    w->kcap = k; w->mcap = m;
  }
  double *F = nullptr, *U = nullptr;
  RET_IF(topo_device_ptr(h, TOPO_MULTI_F, 0, (void**)&F));
  RET_IF(topo_device_ptr(h, TOPO_MULTI_U, 0, (void**)&U));
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  struct Ev { cudaEvent_t a, b; ~Ev() { if (a) cudaEventDestroy(a); if (b) cudaEventDestroy(b); } } ev{e0, e1};
  cudaEventRecord(e0, s);
  // start vectors: seeded uniform(-1, 1) coordinates (the reference draws
  // random nodal forces and projects them), orthonormalised
  std::mt19937_64 rng(o->seed);
  std::uniform_real_distribution<double> uni(-1.0, 1.0);
  std::vector<double> X((size_t)k * m), Y((size_t)k * m);
  for (auto& x : X) x = uni(rng);
  orthonormalise(k, m, X, rng);
  cudaMemsetAsync(U, 0, sizeof(double) * k * n3, s);
  const dim3 lgrid((n + 127) / 128, k);
  topo_solve_opts so = o->solve;
  topo_worst_stats st{};
  std::vector<double> x1_old;
  double change = 1.0, theta1 = 0, theta2 = 0, last_relres = 1.0;
  std::vector<double> relres(k);
  int it = 0;
  bool done = false;  // the next solve is the last one (at the final tolerance)
  for (;;) {
    ++it;
    // F = S X
    cudaMemcpyAsync(w->X, X.data(), sizeof(double) * k * m, cudaMemcpyHostToDevice, s);
    cudaMemsetAsync(F, 0, sizeof(double) * k * n3, s);
    k_scatter_loads<<<lgrid, 128, 0, s>>>(n, k, m, free_dir, w->vid, w->nrm, lv.vmask, nv, w->X, F);
    count_launch();
    // solve K U = F, warm-started; the tolerance tightens as the load settles
    // and is the final one once the change is below tol
    so.rtol = done ? o->solve.rtol : std::max(o->solve.rtol, std::min(1e-2, 0.1 * change));
    topo_multi_stats ms{};
    rc = topo_solve_multi(h, k, &so, &ms, relres.data());
    if (rc != TOPO_OK && rc != TOPO_E_NOT_CONVERGED) return rc;
    st.solve_iterations += ms.iterations;
    last_relres = relres[0];
    // Y = S^T U
    k_gather_loads<<<lgrid, 128, 0, s>>>(n, k, m, free_dir, w->vid, w->nrm, lv.vmask, nv, U, w->Y);
    count_launch();
    if (cudaMemcpyAsync(Y.data(), w->Y, sizeof(double) * k * m, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
      return handle_fail(h, TOPO_E_CUDA, "worst-case compliance: gather");
    if (done) break;  // the final solve of the converged load
    // Rayleigh-Ritz: H = X^T Y (symmetrised), eigenpairs descending
    std::vector<double> H((size_t)k * k);
    for (int a = 0; a < k; ++a)
      for (int b = 0; b < k; ++b) {
        double d = 0;
        const double* xa = &X[(size_t)a * m];
        const double* yb = &Y[(size_t)b * m];
        for (int i = 0; i < m; ++i) d += xa[i] * yb[i];
        H[(size_t)a * k + b] = d;
      }
    for (int a = 0; a < k; ++a)
      for (int b = a + 1; b < k; ++b) {
        const double v = 0.5 * (H[(size_t)a * k + b] + H[(size_t)b * k + a]);
        H[(size_t)a * k + b] = H[(size_t)b * k + a] = v;
      }
    std::vector<double> theta, W;
    jacobi_eig(k, H, theta, W);
    theta1 = theta[0];
    theta2 = k > 1 ? theta[1] : 0.0;
    // new basis Z = Y W, orthonormalised: Z = Y W R^-1; the displacements
    // follow with U <- U (H W R^-1), exact when span X is invariant (Y = X H)
    std::vector<double> Z((size_t)k * m, 0.0);
    for (int j = 0; j < k; ++j)
      for (int l = 0; l < k; ++l) {
        const double c = W[(size_t)l * k + j];
        if (c == 0) continue;
        const double* yl = &Y[(size_t)l * m];
        double* zj = &Z[(size_t)j * m];
        for (int i = 0; i < m; ++i) zj[i] += c * yl[i];
      }
    const std::vector<double> Rinv = orthonormalise(k, m, Z, rng);
    std::vector<double> HW((size_t)k * k, 0.0), Cm((size_t)k * k, 0.0);
    for (int a = 0; a < k; ++a)
      for (int b = 0; b < k; ++b) {
        double d = 0;
        for (int l = 0; l < k; ++l) d += H[(size_t)a * k + l] * W[(size_t)l * k + b];
        HW[(size_t)a * k + b] = d;
      }
    for (int a = 0; a < k; ++a)
      for (int b = 0; b < k; ++b) {
        double d = 0;
        for (int l = 0; l <= b; ++l) d += HW[(size_t)a * k + l] * Rinv[(size_t)l * k + b];
        Cm[(size_t)a * k + b] = d;
      }
    // change of the worst load (sign-aligned)
    if (!x1_old.empty()) {
      double d = 0;
      for (int i = 0; i < m; ++i) d += x1_old[i] * Z[i];
      const double sg = d < 0 ? -1.0 : 1.0;
      double c2 = 0;
      for (int i = 0; i < m; ++i) c2 += (Z[i] - sg * x1_old[i]) * (Z[i] - sg * x1_old[i]);
      change = std::sqrt(c2);
    }
    x1_old.assign(Z.begin(), Z.begin() + m);
    X.swap(Z);
    cudaMemcpyAsync(w->C, Cm.data(), sizeof(double) * k * k, cudaMemcpyHostToDevice, s);
    k_basis_map<<<(unsigned)((n3 + 255) / 256), 256, 0, s>>>(n3, k, w->C, U, w->tmp);
    cudaMemcpyAsync(U, w->tmp, sizeof(double) * k * n3, cudaMemcpyDeviceToDevice, s);
    count_launch();
    // one more solve at the final tolerance once the load has settled (or the
    // iteration cap is reached: the result is then reported as not converged)
    if (change <= o->tol || it >= o->max_iter) done = true;
  }
  // the worst load and its displacement into level 0 (TOPO_F, TOPO_U)
  double *F0 = nullptr, *U0 = nullptr;
  RET_IF(topo_device_ptr(h, TOPO_F, 0, (void**)&F0));
  RET_IF(topo_device_ptr(h, TOPO_U, 0, (void**)&U0));
  cudaMemcpyAsync(F0, F, sizeof(double) * n3, cudaMemcpyDeviceToDevice, s);
  cudaMemcpyAsync(U0, U, sizeof(double) * n3, cudaMemcpyDeviceToDevice, s);
  cudaEventRecord(e1, s);
  if (cudaEventSynchronize(e1) != cudaSuccess) return handle_fail(h, TOPO_E_CUDA, "worst-case compliance");
  float msf = 0;
  cudaEventElapsedTime(&msf, e0, e1);
  // compliance of the unit worst load: x1 . S^T u1
  double c = 0;
  for (int i = 0; i < m; ++i) c += X[i] * Y[i];
  st.compliance = c;
  st.second = theta2;
  st.change = change;
  st.relres = last_relres;
  st.iterations = it;
  st.ms = msf;
  (void)theta1;
  if (stats) *stats = st;
  if (!std::isfinite(c)) return handle_fail(h, TOPO_E_NONFINITE, "worst-case compliance is not finite");
  if (change > o->tol)
    return handle_fail(h, TOPO_E_NOT_CONVERGED, "worst-case compliance: load still changing after max_iter");
  return TOPO_OK;
}

}  // extern "C"
