// Vector kernels: deterministic two-pass FP64 reductions, axpy-type updates
// and the Chebyshev smoothing step.
#include <algorithm>

#include "topo_internal.h"

namespace topo {

constexpr int RED_THREADS = 256;

template <typename T, int W>
struct alignas(16) Pack16 {
  T v[W];
};
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

// Completion by the last block: each block's thread 0 has published its partial;
// every block then takes a ticket, and the block with the last one sums all nb
// partials in index order (the order of k_finalize_sum, so the result does not
// depend on which block finishes last) and resets the counter for the next use.
// Saves the separate finalising launch.  ctr: one counter per stream in order.
__device__ __forceinline__ void finish_sum(const double* partial, int nb, double* out, unsigned* ctr) {
  __shared__ bool last;
  if (threadIdx.x == 0) {  // thread 0 wrote the block's partial: fence, then take a ticket
    __threadfence();
    last = atomicAdd(ctr, 1u) == (unsigned)(nb - 1);
    if (last) __threadfence();
  }
  __syncthreads();
  if (!last) return;
  double s = 0.0;
  for (int i = threadIdx.x; i < nb; i += blockDim.x) s += __ldcg(partial + i);
  s = block_sum(s);
  if (threadIdx.x == 0) {
    *out = s;
    *ctr = 0u;
  }
}

// Per-thread partial sums are accumulated in the vector's precision (FP32
// vectors: a few dozen terms per thread, inside the FP32 inner solver only) and
// combined in FP64 across threads and blocks.  With ctr the last block also
// writes the total to out.  With skip_if_zero the whole grid does nothing while
// *skip_if_zero is 0 (a device-side loop's first iteration).
template <typename T>
__global__ void __launch_bounds__(RED_THREADS) k_dot_partial(const T* __restrict__ a, const T* __restrict__ b,
                                                             int64_t n, double* __restrict__ partial,
                                                             double* __restrict__ out = nullptr,
                                                             unsigned* __restrict__ ctr = nullptr,
                                                             const double* __restrict__ skip_if_zero = nullptr) {
  if (skip_if_zero && *skip_if_zero == 0.0) return;
  T s = T(0);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    s += a[i] * (b ? b[i] : T(1));
  const double bs = block_sum((double)s);
  if (threadIdx.x == 0) partial[blockIdx.x] = bs;
  if (ctr) finish_sum(partial, gridDim.x, out, ctr);
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
void launch_dot(cudaStream_t s, const T* a, const T* b, int64_t n, double* partial, double* out, unsigned* ctr,
                const double* skip_if_zero) {
  const int nb = reduce_blocks(n);
  if (ctr) {
    k_dot_partial<T><<<nb, RED_THREADS, 0, s>>>(a, b, n, partial, out, ctr, skip_if_zero);
  } else {
    k_dot_partial<T><<<nb, RED_THREADS, 0, s>>>(a, b, n, partial);
    k_finalize_sum<<<1, RED_THREADS, 0, s>>>(partial, nb, out);
  }
}

void launch_sum_partials(cudaStream_t s, const double* partial, int nb, double* out) {
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

// The CG step scalars are formed once by a one-thread kernel (an FP64 division
// per vector element is expensive on this part) and read by the vector kernels.
// sc[out] = (sc[num] - (sub >= 0 ? sc[sub] : 0)) / sc[den]
__global__ void k_scalar_ratio(double* sc, int num, int sub, int den, int out) {
  if (threadIdx.x == 0 && blockIdx.x == 0) sc[out] = (sc[num] - (sub >= 0 ? sc[sub] : 0.0)) / sc[den];
}

void launch_scalar_ratio(cudaStream_t s, double* sc, int num, int sub, int den, int out) {
  k_scalar_ratio<<<1, 32, 0, s>>>(sc, num, sub, den, out);
}

// d = z + beta d (beta = sc[beta_slot]), or d = z.  With first_if_zero the
// choice is made on the device: d = z when *first_if_zero is 0 (an iteration
// counter).
template <typename T>
__global__ void k_pcg_dir(const T* __restrict__ z, T* __restrict__ d, const double* __restrict__ sc,
                          int beta_slot, bool first_host, int64_t n, int packed,
                          const double* __restrict__ first_if_zero) {
  constexpr int W = 16 / sizeof(T);
  using P = Pack16<T, W>;
  const bool first = first_if_zero ? (*first_if_zero == 0.0) : first_host;
  const T beta = first ? T(0) : (T)sc[beta_slot];
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t npk = packed ? n / W : 0;
  if (i < npk) {
    const P zp = reinterpret_cast<const P*>(z)[i];
    P dp = first ? zp : reinterpret_cast<const P*>(d)[i];
    if (!first) {
#pragma unroll
      for (int k = 0; k < W; ++k) dp.v[k] = zp.v[k] + beta * dp.v[k];
    }
    reinterpret_cast<P*>(d)[i] = dp;
  }
  // scalar elements: the tail past the last pack, or all of them unpacked
  const int64_t j = packed ? npk * W + i : i;
  if ((!packed || i < W) && j < n) d[j] = first ? z[j] : z[j] + beta * d[j];
}

// d = z (first) or z + beta d, in 16-byte packs when both vectors are aligned
template <typename T>
void launch_pcg_dir(cudaStream_t s, const T* z, T* d, const double* sc, int beta_slot, bool first,
                    int64_t n, const double* first_if_zero) {
  constexpr int W = 16 / sizeof(T);
  const bool packed = (((uintptr_t)z | (uintptr_t)d) & 15) == 0;
  const int64_t threads = packed ? std::max<int64_t>(n / W, W) : n;
  k_pcg_dir<T><<<nblk(threads, 256), 256, 0, s>>>(z, d, sc, beta_slot, first, n, packed ? 1 : 0, first_if_zero);
}

// x += alpha d, rold = r, r -= alpha q (alpha = sc[alpha_slot]), fused with the
// new residual's squared norm: per-thread sums
// in the vectors' precision, combined in FP64 in a fixed order (deterministic).
// Each thread moves 16-byte packs (4 floats / 2 doubles) so enough bytes are in
// flight to stream at HBM bandwidth; the tail past the last whole pack is scalar.

template <typename T>
__global__ void __launch_bounds__(RED_THREADS) k_pcg_update_rr(T* __restrict__ x, T* __restrict__ r,
                                                               T* __restrict__ rold, const T* __restrict__ d,
                                                               const T* __restrict__ q, const double* __restrict__ sc,
                                                               int alpha_slot, int64_t n, double* __restrict__ partial,
                                                               int packed, double* __restrict__ rr, unsigned* __restrict__ ctr) {
  constexpr int W = 16 / sizeof(T);
  using P = Pack16<T, W>;
  const T alpha = (T)sc[alpha_slot];
  T acc = T(0);
  const int64_t gid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x, gs = (int64_t)gridDim.x * blockDim.x;
  const int64_t npk = packed ? n / W : 0;
  for (int64_t i = gid; i < npk; i += gs) {
    const P rp = reinterpret_cast<const P*>(r)[i], xp = reinterpret_cast<const P*>(x)[i];
    const P dp = reinterpret_cast<const P*>(d)[i], qp = reinterpret_cast<const P*>(q)[i];
    P xn, rn;
#pragma unroll
    for (int k = 0; k < W; ++k) {
      xn.v[k] = xp.v[k] + alpha * dp.v[k];
      rn.v[k] = rp.v[k] - alpha * qp.v[k];
      acc += rn.v[k] * rn.v[k];
    }
    if (rold) reinterpret_cast<P*>(rold)[i] = rp;
    reinterpret_cast<P*>(x)[i] = xn;
    reinterpret_cast<P*>(r)[i] = rn;
  }
  for (int64_t i = npk * W + gid; i < n; i += gs) {
    const T ri = r[i];
    if (rold) rold[i] = ri;
    x[i] = x[i] + alpha * d[i];
    const T rn = ri - alpha * q[i];
    r[i] = rn;
    acc += rn * rn;
  }
  const double bs = block_sum((double)acc);
  if (threadIdx.x == 0) partial[blockIdx.x] = bs;
  if (ctr) finish_sum(partial, gridDim.x, rr, ctr);
}

template <typename T>
void launch_pcg_update_rr(cudaStream_t s, T* x, T* r, T* rold, const T* d, const T* q, const double* sc,
                          int alpha_slot, int64_t n, double* partial, double* rr, unsigned* ctr) {
  // 16-byte packs when all five vectors start on 16-byte boundaries
  const uintptr_t al = (uintptr_t)x | (uintptr_t)r | (uintptr_t)rold | (uintptr_t)d | (uintptr_t)q;
  const int nb = reduce_blocks(n);
  k_pcg_update_rr<T><<<nb, RED_THREADS, 0, s>>>(x, r, rold, d, q, sc, alpha_slot, n, partial, (al & 15) == 0,
                                                 rr, ctr);
  if (!ctr) k_finalize_sum<<<1, RED_THREADS, 0, s>>>(partial, nb, rr);
}

template void launch_pcg_update_rr<double>(cudaStream_t, double*, double*, double*, const double*, const double*,
                                           const double*, int, int64_t, double*, double*, unsigned*);
template void launch_pcg_update_rr<float>(cudaStream_t, float*, float*, float*, const float*, const float*,
                                          const double*, int, int64_t, double*, double*, unsigned*);



template void launch_dot<double>(cudaStream_t, const double*, const double*, int64_t, double*, double*, unsigned*,
                                  const double*);
template void launch_dot<float>(cudaStream_t, const float*, const float*, int64_t, double*, double*, unsigned*,
                                 const double*);
template void launch_fill<double>(cudaStream_t, double*, double, int64_t);
template void launch_fill<float>(cudaStream_t, float*, float, int64_t);
template void launch_copy<double>(cudaStream_t, const double*, double*, int64_t);
template void launch_copy<float>(cudaStream_t, const float*, float*, int64_t);
template void launch_pcg_dir<double>(cudaStream_t, const double*, double*, const double*, int, bool, int64_t,
                                      const double*);
template void launch_pcg_dir<float>(cudaStream_t, const float*, float*, const double*, int, bool, int64_t,
                                     const double*);

}  // namespace topo
