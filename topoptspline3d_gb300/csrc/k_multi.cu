// Batched vector kernels of the multi-right-hand-side solver: nb vectors of
// length n stored one after another, one set of CG scalars per right-hand side.
// Reductions are two-pass and deterministic (per-(block, rhs) partials summed
// in a fixed order).
#include <algorithm>

#include "topo_internal.h"

namespace topo {

namespace {
constexpr int kThreads = 256;
inline unsigned nblk(int64_t n, int b) { return (unsigned)((n + b - 1) / b); }
}  // namespace

// partial[rhs][blk] = sum over the block's slice of a[rhs] . b[rhs]
template <typename T>
__global__ void k_bdot_partial(const T* __restrict__ a, const T* __restrict__ b, int64_t n, double* __restrict__ part) {
  __shared__ double sh[kThreads];
  const int64_t off = (int64_t)blockIdx.y * n;
  double s = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * kThreads + threadIdx.x; i < n; i += (int64_t)gridDim.x * kThreads)
    s += (double)a[off + i] * (double)b[off + i];
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int o = kThreads / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[(int64_t)blockIdx.y * gridDim.x + blockIdx.x] = sh[0];
}

__global__ void k_bdot_final(const double* __restrict__ part, int nblocks, int nb, double* __restrict__ out) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nb) return;
  double s = 0.0;
  for (int b = 0; b < nblocks; ++b) s += part[(int64_t)k * nblocks + b];
  out[k] = s;
}

template <typename T>
void launch_bdot(cudaStream_t s, const T* a, const T* b, int64_t n, int nb, double* partial, double* out) {
  const int nblocks = (int)std::min<int64_t>(256, std::max<int64_t>(1, (n + kThreads - 1) / kThreads));
  k_bdot_partial<T><<<dim3(nblocks, nb), kThreads, 0, s>>>(a, b, n, partial);
  k_bdot_final<<<nblk(nb, 64), 64, 0, s>>>(partial, nblocks, nb, out);
}
template void launch_bdot<double>(cudaStream_t, const double*, const double*, int64_t, int, double*, double*);
template void launch_bdot<float>(cudaStream_t, const float*, const float*, int64_t, int, double*, double*);

// Per right-hand side: beta = (rz - zrold) / rzold (first: 0).
__global__ void k_bbeta(int nb, const double* rz, const double* zrold, const double* rzold, int first, double* beta) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nb) return;
  beta[k] = first || !(rzold[k] != 0.0) ? 0.0 : (rz[k] - zrold[k]) / rzold[k];
}

// Per right-hand side: alpha = rz / dq while rr > rtol^2 ff, else 0 (the
// right-hand side has converged and its iterate is frozen); rzold = rz.
__global__ void k_balpha(int nb, const double* rz, const double* dq, const double* rr, const double* ff, double rtol2,
                         double* alpha, double* rzold) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nb) return;
  const bool active = rr[k] > rtol2 * ff[k] && dq[k] != 0.0;
  alpha[k] = active ? rz[k] / dq[k] : 0.0;
  rzold[k] = rz[k];
}

// d = z + beta d
template <typename T>
__global__ void k_bdir(int64_t n, int nb, const T* __restrict__ z, T* __restrict__ d, const double* __restrict__ beta) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n * nb) return;
  const T b = (T)beta[i / n];
  d[i] = z[i] + b * d[i];
}

// x += alpha d, rold = r (when kept), r -= alpha q
template <typename T>
__global__ void k_bupdate(int64_t n, int nb, T* __restrict__ x, T* __restrict__ r, T* __restrict__ rold,
                          const T* __restrict__ d, const T* __restrict__ q, const double* __restrict__ alpha) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n * nb) return;
  const T a = (T)alpha[i / n];
  x[i] += a * d[i];
  if (rold) rold[i] = r[i];
  r[i] -= a * q[i];
}

void launch_bbeta(cudaStream_t s, int nb, const double* rz, const double* zrold, const double* rzold, bool first,
                  double* beta) {
  k_bbeta<<<nblk(nb, 64), 64, 0, s>>>(nb, rz, zrold, rzold, first ? 1 : 0, beta);
}
void launch_balpha(cudaStream_t s, int nb, const double* rz, const double* dq, const double* rr, const double* ff,
                   double rtol2, double* alpha, double* rzold) {
  k_balpha<<<nblk(nb, 64), 64, 0, s>>>(nb, rz, dq, rr, ff, rtol2, alpha, rzold);
}
template <typename T>
void launch_bdir(cudaStream_t s, int64_t n, int nb, const T* z, T* d, const double* beta) {
  k_bdir<T><<<nblk(n * nb, kThreads), kThreads, 0, s>>>(n, nb, z, d, beta);
}
template <typename T>
void launch_bupdate(cudaStream_t s, int64_t n, int nb, T* x, T* r, T* rold, const T* d, const T* q,
                    const double* alpha) {
  k_bupdate<T><<<nblk(n * nb, kThreads), kThreads, 0, s>>>(n, nb, x, r, rold, d, q, alpha);
}
template void launch_bdir<double>(cudaStream_t, int64_t, int, const double*, double*, const double*);
template void launch_bdir<float>(cudaStream_t, int64_t, int, const float*, float*, const double*);
template void launch_bupdate<double>(cudaStream_t, int64_t, int, double*, double*, double*, const double*,
                                     const double*, const double*);
template void launch_bupdate<float>(cudaStream_t, int64_t, int, float*, float*, float*, const float*, const float*,
                                    const double*);

}  // namespace topo
