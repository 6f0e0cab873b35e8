// Vector kernels: deterministic two-pass FP64 reductions, axpy-type updates
// and the Chebyshev smoothing step.
#include "topo_internal.h"

namespace topo {

constexpr int RED_THREADS = 256;
constexpr int RED_MAX_BLOCKS = 1024;

static inline unsigned nblk(int64_t n, int bs) { return (unsigned)((n + bs - 1) / bs); }

int reduce_blocks(int64_t n) {
  int64_t b = (n + RED_THREADS * 8 - 1) / (RED_THREADS * 8);
  if (b < 1) b = 1;
  if (b > RED_MAX_BLOCKS) b = RED_MAX_BLOCKS;
  return (int)b;
}

__device__ __forceinline__ double block_sum(double v) {
  __shared__ double ws[RED_THREADS / 32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) ws[w] = v;
  __syncthreads();
  double s = 0.0;
  if (w == 0) {
    s = lane < RED_THREADS / 32 ? ws[lane] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  }
  return s;  // valid in thread 0
}

template <typename T>
__global__ void __launch_bounds__(RED_THREADS) k_dot_partial(const T* __restrict__ a, const T* __restrict__ b,
                                                             int64_t n, double* __restrict__ partial) {
  double s = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    s += (double)a[i] * (b ? (double)b[i] : 1.0);
  s = block_sum(s);
  if (threadIdx.x == 0) partial[blockIdx.x] = s;
}

__global__ void __launch_bounds__(RED_THREADS) k_finalize_sum(const double* __restrict__ partial, int nb,
                                                              double* __restrict__ out) {
  double s = 0.0;
  for (int i = threadIdx.x; i < nb; i += blockDim.x) s += partial[i];
  s = block_sum(s);
  if (threadIdx.x == 0) *out = s;
}

__global__ void __launch_bounds__(RED_THREADS) k_maxabs_partial(const double* __restrict__ a, int64_t n,
                                                                double* __restrict__ partial) {
  double m = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    m = fmax(m, fabs(a[i]));
  __shared__ double ws[RED_THREADS / 32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_down_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    double r = 0.0;
    for (int w = 0; w < RED_THREADS / 32; ++w) r = fmax(r, ws[w]);
    partial[blockIdx.x] = r;
  }
}

__global__ void k_finalize_max(const double* __restrict__ partial, int nb, double* __restrict__ out) {
  if (threadIdx.x == 0) {
    double r = 0.0;
    for (int i = 0; i < nb; ++i) r = fmax(r, partial[i]);
    *out = r;
  }
}

template <typename T>
void launch_dot(cudaStream_t s, const T* a, const T* b, int64_t n, double* partial, double* out) {
  const int nb = reduce_blocks(n);
  k_dot_partial<T><<<nb, RED_THREADS, 0, s>>>(a, b, n, partial);
  k_finalize_sum<<<1, RED_THREADS, 0, s>>>(partial, nb, out);
}

void launch_sum(cudaStream_t s, const double* a, int64_t n, double* partial, double* out) {
  const int nb = reduce_blocks(n);
  k_dot_partial<double><<<nb, RED_THREADS, 0, s>>>(a, nullptr, n, partial);
  k_finalize_sum<<<1, RED_THREADS, 0, s>>>(partial, nb, out);
}

void launch_maxabs(cudaStream_t s, const double* a, int64_t n, double* partial, double* out) {
  const int nb = reduce_blocks(n);
  k_maxabs_partial<<<nb, RED_THREADS, 0, s>>>(a, n, partial);
  k_finalize_max<<<1, 32, 0, s>>>(partial, nb, out);
}

__global__ void k_axpby(double a, const double* __restrict__ x, double b, double* __restrict__ y, int64_t n) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) y[i] = a * x[i] + b * y[i];
}

void launch_axpby(cudaStream_t s, double a, const double* x, double b, double* y, int64_t n) {
  k_axpby<<<nblk(n, 256), 256, 0, s>>>(a, x, b, y, n);
}

template <typename T>
__global__ void k_fill(T* a, T v, int64_t n) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) a[i] = v;
}

template <typename T>
void launch_fill(cudaStream_t s, T* a, T v, int64_t n) {
  k_fill<T><<<nblk(n, 256), 256, 0, s>>>(a, v, n);
}

template <typename T>
void launch_copy(cudaStream_t s, const T* a, T* b, int64_t n) {
  cudaMemcpyAsync(b, a, sizeof(T) * n, cudaMemcpyDeviceToDevice, s);
}

__global__ void k_d2f(const double* __restrict__ a, float* __restrict__ b, int64_t n) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) b[i] = (float)a[i];
}
__global__ void k_f2d_add(const float* __restrict__ a, double* __restrict__ b, int64_t n) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) b[i] += (double)a[i];
}
void launch_d2f(cudaStream_t s, const double* a, float* b, int64_t n) {
  k_d2f<<<nblk(n, 256), 256, 0, s>>>(a, b, n);
}
void launch_f2d_add(cudaStream_t s, const float* a, double* b, int64_t n) {
  k_f2d_add<<<nblk(n, 256), 256, 0, s>>>(a, b, n);
}

// d = z + beta d, beta = (sc[num0] - sc[num1]) / sc[den] (Polak-Ribiere), or d = z.
template <typename T>
__global__ void k_pcg_dir(const T* __restrict__ z, T* __restrict__ d, const double* __restrict__ sc,
                          int num, int den, bool first, int64_t n) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (first) { d[i] = z[i]; return; }
  const double beta = (sc[num] - sc[num + 1]) / sc[den];
  d[i] = (T)((double)z[i] + beta * (double)d[i]);
}

template <typename T>
void launch_pcg_dir(cudaStream_t s, const T* z, T* d, const double* sc, int num, int den, bool first,
                    int64_t n) {
  k_pcg_dir<T><<<nblk(n, 256), 256, 0, s>>>(z, d, sc, num, den, first, n);
}

// alpha = sc[num]/sc[den]; rold = r; x += alpha d; r -= alpha q.
template <typename T>
__global__ void k_pcg_update(T* __restrict__ x, T* __restrict__ r, T* __restrict__ rold,
                             const T* __restrict__ d, const T* __restrict__ q,
                             const double* __restrict__ sc, int num, int den, int64_t n) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double alpha = sc[num] / sc[den];
  const T ri = r[i];
  rold[i] = ri;
  x[i] = (T)((double)x[i] + alpha * (double)d[i]);
  r[i] = (T)((double)ri - alpha * (double)q[i]);
}

template <typename T>
void launch_pcg_update(cudaStream_t s, T* x, T* r, T* rold, const T* d, const T* q, const double* sc,
                       int num, int den, int64_t n) {
  k_pcg_update<T><<<nblk(n, 256), 256, 0, s>>>(x, r, rold, d, q, sc, num, den, n);
}

// Chebyshev step: z = Dinv r (3x3 blocks), d = c_old d + c_new z (first: d = c_new z), u += d.
template <typename T>
__global__ void k_cheb_step(int64_t nv, const T* __restrict__ dinv, const T* __restrict__ r,
                            T* __restrict__ dvec, T* __restrict__ u, T c_old, T c_new, bool first) {
  const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= nv) return;
  const T r0 = r[v], r1 = r[nv + v], r2 = r[2 * nv + v];
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    const T z = dinv[(3 * i) * nv + v] * r0 + dinv[(3 * i + 1) * nv + v] * r1 + dinv[(3 * i + 2) * nv + v] * r2;
    const T dn = first ? c_new * z : c_old * dvec[i * nv + v] + c_new * z;
    dvec[i * nv + v] = dn;
    u[i * nv + v] += dn;
  }
}

template <typename T>
void launch_cheb_step(cudaStream_t s, const LevelDims& dm, const T* dinv, const T* r, T* dvec, T* u,
                      double c_old, double c_new, bool first) {
  k_cheb_step<T><<<nblk(dm.nv, 256), 256, 0, s>>>(dm.nv, dinv, r, dvec, u, (T)c_old, (T)c_new, first);
}

template void launch_dot<double>(cudaStream_t, const double*, const double*, int64_t, double*, double*);
template void launch_dot<float>(cudaStream_t, const float*, const float*, int64_t, double*, double*);
template void launch_fill<double>(cudaStream_t, double*, double, int64_t);
template void launch_fill<float>(cudaStream_t, float*, float, int64_t);
template void launch_copy<double>(cudaStream_t, const double*, double*, int64_t);
template void launch_copy<float>(cudaStream_t, const float*, float*, int64_t);
template void launch_pcg_dir<double>(cudaStream_t, const double*, double*, const double*, int, int, bool,
                                     int64_t);
template void launch_pcg_dir<float>(cudaStream_t, const float*, float*, const double*, int, int, bool,
                                    int64_t);
template void launch_pcg_update<double>(cudaStream_t, double*, double*, double*, const double*,
                                        const double*, const double*, int, int, int64_t);
template void launch_pcg_update<float>(cudaStream_t, float*, float*, float*, const float*, const float*,
                                       const double*, int, int, int64_t);
template void launch_cheb_step<double>(cudaStream_t, const LevelDims&, const double*, const double*,
                                       double*, double*, double, double, bool);
template void launch_cheb_step<float>(cudaStream_t, const LevelDims&, const float*, const float*, float*,
                                      float*, double, double, bool);

}  // namespace topo
