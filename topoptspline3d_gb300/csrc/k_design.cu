// Design-chain kernels: B-spline density, element sensitivity, sensitivity
// filter, spline adjoint and the OC coefficient trial.
#include <algorithm>
#include <cmath>
#include <cstring>

#include "df.cuh"
#include "topo_internal.h"

namespace topo {

static inline unsigned nblk(int64_t n, int bs) { return (unsigned)((n + bs - 1) / bs); }

constexpr int MAX_ORDER = 4;  // highest spline order (cubic B-splines)

// v^p for the SIMP exponent: repeated products for small integer p (the
// reference default p = 3), the general pow otherwise.
__device__ __forceinline__ double simp_pow(double v, double p) {
  const int ip = (int)p;
  if ((double)ip == p && ip >= 0 && ip <= 8) {
    double r = 1.0;
    for (int k = 0; k < ip; ++k) r *= v;
    return r;
  }
  return pow(v, p);
}

constexpr int VOL_THREADS = 256;

__global__ void k_sum_partials(const double* __restrict__ partial, int nb, double* __restrict__ out) {
  __shared__ double sh[256];
  double s = 0.0;
  for (int i = threadIdx.x; i < nb; i += blockDim.x) s += partial[i];
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = sh[0];
}

// Separable evaluation, pass 1: B[z][y][i] = sum_{s,t} c[i, iy+s, iz+t] Ny[y][s] Nz[z][t]
// for every x-basis index i (0 where y or z is outside the spline range), in
// FP64, stored split into (hi, lo) floats for the double-float pass 2.
__global__ void k_spline_yz(LevelDims d, SplineDev sp, const double* __restrict__ coeff,
                            float2* __restrict__ B) {
  const int64_t gid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int nbx = sp.nb[0];
  if (gid >= (int64_t)nbx * d.ey * d.ez) return;
  const int i = (int)(gid % nbx);
  const int64_t yz = gid / nbx;
  const int y = (int)(yz % d.ey), z = (int)(yz / d.ey);
  const int iy = sp.i0[1][y], iz = sp.i0[2][z];
  double v = 0.0;
  if (iy >= 0 && iz >= 0) {
    const int k = sp.order;
    for (int s = 0; s < k; ++s) {
      const double ns = sp.N[1][y * k + s];
      double a = 0.0;
      for (int t = 0; t < k; ++t)
        a += coeff[i + (int64_t)nbx * ((iy + s) + (int64_t)sp.nb[1] * (iz + t))] * sp.N[2][z * k + t];
      v += ns * a;
    }
  }
  const df vd = df_from(v);
  B[gid] = make_float2(vd.hi, vd.lo);
}

// Pass 1 of an OC trial in double-float, from coefficients already split into
// (hi, lo) floats (FP64 here would be bound by the FP64 pipe on every trial).
__global__ void k_spline_yz_df(LevelDims d, SplineDev sp, const float2* __restrict__ coeff,
                               float2* __restrict__ B) {
  const int64_t gid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int nbx = sp.nb[0];
  if (gid >= (int64_t)nbx * d.ey * d.ez) return;
  const int i = (int)(gid % nbx);
  const int64_t yz = gid / nbx;
  const int y = (int)(yz % d.ey), z = (int)(yz / d.ey);
  const int iy = sp.i0[1][y], iz = sp.i0[2][z];
  df v(0);
  if (iy >= 0 && iz >= 0) {
    const int k = sp.order;
    for (int s2 = 0; s2 < k; ++s2) {
      const float2 ns = sp.Ndf[1][y * k + s2];
      df a(0);
      for (int t = 0; t < k; ++t) {
        const float2 c = coeff[i + (int64_t)nbx * ((iy + s2) + (int64_t)sp.nb[1] * (iz + t))];
        const float2 nz = sp.Ndf[2][z * k + t];
        a += df(c.x, c.y) * df(nz.x, nz.y);
      }
      v += df(ns.x, ns.y) * a;
    }
  }
  B[gid] = make_float2(v.hi, v.lo);
}

// Pass 2: value at element (x,y,z) = sum_r Nx[x][r] B[z][y][ix + r], or -0.2 out of
// range, in double-float arithmetic (about 1e-15 relative; FP64 here would be
// bound by GB300's FP64 pipe, and each OC bisection trial evaluates it on every
// element).
__device__ __forceinline__ df spline_from_B(const SplineDev& sp, const float2* __restrict__ B,
                                            int x, int y, int z, int ey) {
  const int ix = sp.i0[0][x];
  if (ix < 0 || sp.i0[1][y] < 0 || sp.i0[2][z] < 0) return df_from(-0.2);
  const int k = sp.order;
  const float2* b = B + (int64_t)sp.nb[0] * (y + (int64_t)ey * z) + ix;
  df v(0);
  for (int r = 0; r < k; ++r) {
    const float2 n = sp.Ndf[0][x * k + r], bb = b[r];
    v += df(n.x, n.y) * df(bb.x, bb.y);
  }
  return v;
}

// (x, y, z) of element e, in 32-bit arithmetic when the grid allows
__device__ __forceinline__ void elem_xyz(const LevelDims& d, int64_t e, int& x, int& y, int& z) {
  if (d.ne < (int64_t)1 << 31) {
    const unsigned ee = (unsigned)e, ex = (unsigned)d.ex, t = ee / ex;
    x = (int)(ee - t * ex);
    y = (int)(t % (unsigned)d.ey);
    z = (int)(t / (unsigned)d.ey);
  } else {
    x = (int)(e % d.ex);
    const int64_t t = e / d.ex;
    y = (int)(t % d.ey);
    z = (int)(t / d.ey);
  }
}

__device__ __forceinline__ bool df_lt(df a, df b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }

__global__ void k_density_from_B(LevelDims d, const uint8_t* __restrict__ eactive, SplineDev sp,
                                 const float2* __restrict__ B, double rho_min, double penal,
                                 double* __restrict__ rho, double* __restrict__ rhop, float* __restrict__ rhop32) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= d.ne) return;
  if (!eactive[e]) {
    rho[e] = 0.0; rhop[e] = 0.0; rhop32[e] = 0.0f;
    return;
  }
  int x, y, z;
  elem_xyz(d, e, x, y, z);
  const double v = fmin(fmax(df_to(spline_from_B(sp, B, x, y, z, d.ey)), rho_min), 1.0);
  const double vp = simp_pow(v, penal);
  rho[e] = v; rhop[e] = vp; rhop32[e] = (float)vp;
}

__global__ void __launch_bounds__(VOL_THREADS) k_volume_from_B(LevelDims d, const uint8_t* __restrict__ eactive,
                                                               SplineDev sp, const float2* __restrict__ B,
                                                               double rho_min, double* __restrict__ partial) {
  const df lo = df_from(rho_min), one(1.f, 0.f);
  df sd(0);
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < d.ne; e += (int64_t)gridDim.x * blockDim.x) {
    if (!eactive[e]) continue;
    int x, y, z;
    elem_xyz(d, e, x, y, z);
    df v = spline_from_B(sp, B, x, y, z, d.ey);
    if (df_lt(v, lo)) v = lo;
    if (df_lt(one, v)) v = one;
    sd += v;
  }
  double s = df_to(sd);
  __shared__ double ws[VOL_THREADS / 32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double r = 0.0;
    for (int w = 0; w < VOL_THREADS / 32; ++w) r += ws[w];
    partial[blockIdx.x] = r;
  }
}

// (hi, lo) float split of n doubles
__global__ void k_to_df(int64_t n, const double* __restrict__ a, float2* __restrict__ b) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const df v = df_from(a[i]);
  b[i] = make_float2(v.hi, v.lo);
}

// Pass 1 in double-float, separable, one CTA per (element layer z, chunk of
// SEP_Y element rows y): first C[j][i] = sum_t c[i, j, iz+t] Nz[z][t] for the
// y-basis indices j the chunk's rows use, into shared memory, then
// B[z][y][i] = sum_s Ny[y][s] C[iy+s][i] (0 where y or z is outside the spline
// range).  The products and their order are those of k_spline_yz_df (inner
// sum over t, outer over s); each coefficient is read once per CTA instead of
// once per output.  The shared table holds cap_j y-basis rows; a chunk whose
// rows use more (a spline partition finer than the elements) forms its
// outputs straight from the coefficients.
constexpr int SEP_Y = 16;

__device__ __forceinline__ df spline_yz_at(const LevelDims& d, const SplineDev& sp, const float2* __restrict__ coeff,
                                           int i, int y, int iz, const df* nz) {
  const int iy = sp.i0[1][y], k = sp.order, nbx = sp.nb[0];
  df v(0);
  if (iy < 0) return v;
  for (int s2 = 0; s2 < k; ++s2) {
    const float2 ns = sp.Ndf[1][y * k + s2];
    df a(0);
    for (int t = 0; t < k; ++t) {
      const float2 c = coeff[i + (int64_t)nbx * ((iy + s2) + (int64_t)sp.nb[1] * (iz + t))];
      a += df(c.x, c.y) * nz[t];
    }
    v += df(ns.x, ns.y) * a;
  }
  return v;
}

__global__ void __launch_bounds__(256) k_spline_yz_sep(LevelDims d, SplineDev sp, const float2* __restrict__ coeff,
                                                       float2* __restrict__ B, int cap_j) {
  extern __shared__ float2 sC[];  // [j - jlo][nb0]
  __shared__ int sj[2];
  const int z = blockIdx.x, y0 = blockIdx.y * SEP_Y, y1 = min(y0 + SEP_Y, d.ey);
  const int nbx = sp.nb[0], nby = sp.nb[1], k = sp.order;
  const int iz = sp.i0[2][z];
  float2* Bz = B + (int64_t)nbx * d.ey * z;
  if (iz < 0) {
    for (int q = threadIdx.x; q < nbx * (y1 - y0); q += blockDim.x) Bz[nbx * y0 + q] = make_float2(0.f, 0.f);
    return;
  }
  if (threadIdx.x == 0) {  // y-basis indices of the chunk's rows
    int lo = nby, hi = -1;
    for (int y = y0; y < y1; ++y) {
      const int iy = sp.i0[1][y];
      if (iy >= 0) { lo = min(lo, iy); hi = max(hi, iy + k - 1); }
    }
    sj[0] = lo;
    sj[1] = hi;
  }
  __syncthreads();
  const int jlo = sj[0], nj = sj[1] - sj[0] + 1;
  df nz[MAX_ORDER];
#pragma unroll
  for (int t = 0; t < MAX_ORDER; ++t) {
    const float2 n = t < k ? sp.Ndf[2][z * k + t] : make_float2(0.f, 0.f);
    nz[t] = df(n.x, n.y);
  }
  if (nj > cap_j) {  // (uniform over the CTA)
    for (int q = threadIdx.x; q < nbx * (y1 - y0); q += blockDim.x) {
      const df v = spline_yz_at(d, sp, coeff, q % nbx, y0 + q / nbx, iz, nz);
      Bz[nbx * y0 + q] = make_float2(v.hi, v.lo);
    }
    return;
  }
  for (int q = threadIdx.x; q < nbx * nj; q += blockDim.x) {
    const int i = q % nbx, j = jlo + q / nbx;
    df a(0);
    for (int t = 0; t < k; ++t) {
      const float2 c = coeff[i + (int64_t)nbx * (j + (int64_t)nby * (iz + t))];
      a += df(c.x, c.y) * nz[t];
    }
    sC[q] = make_float2(a.hi, a.lo);
  }
  __syncthreads();
  for (int q = threadIdx.x; q < nbx * (y1 - y0); q += blockDim.x) {
    const int i = q % nbx, y = y0 + q / nbx;
    const int iy = sp.i0[1][y];
    df v(0);
    if (iy >= 0) {
      for (int s2 = 0; s2 < k; ++s2) {
        const float2 ns = sp.Ndf[1][y * k + s2];
        const float2 a = sC[i + nbx * (iy - jlo + s2)];
        v += df(ns.x, ns.y) * df(a.x, a.y);
      }
    }
    Bz[nbx * y0 + q] = make_float2(v.hi, v.lo);
  }
}

// Pass 2 one element row (y, z) at a time, one thread per element column x
// (the CTA is the row's width rounded up to whole warps): the row's pass-1
// values B[z][y][:] are staged in shared memory, the next row's values and
// activity flags are loaded while this row's elements are evaluated, and each
// thread keeps its column's basis index and weights in registers for all rows
// (values as spline_from_B).  Rows of at most ROW_MAX elements.
constexpr int ROW_MAX = 1024;

__device__ __forceinline__ df row_value(const float2* sB, int ix, const df* nx, int k, bool in) {
  if (!in) return df_from(-0.2);
  df v(0);
  for (int r = 0; r < k; ++r) {
    const float2 bb = sB[ix + r];
    v += nx[r] * df(bb.x, bb.y);
  }
  return v;
}

// MODE 0: volume partial sums (clamped values of active elements, per CTA);
// MODE 1: densities rho, rho^p (FP64 and FP32) of every element.
template <int MODE>
__global__ void __launch_bounds__(ROW_MAX) k_spline_rows(LevelDims d, const uint8_t* __restrict__ eactive,
                                                         SplineDev sp, const float2* __restrict__ B,
                                                         double rho_min, double penal,
                                                         double* __restrict__ partial, double* __restrict__ rho,
                                                         double* __restrict__ rhop, float* __restrict__ rhop32) {
  extern __shared__ float2 sB[];  // nb0
  const int nbx = sp.nb[0], ex = d.ex, nrows = d.ey * d.ez, k = sp.order;
  const int x = threadIdx.x;
  const bool col = x < ex;
  // the column's basis index and weights, for every row
  int ix = -1;
  df nx[MAX_ORDER];
#pragma unroll
  for (int r = 0; r < MAX_ORDER; ++r) nx[r] = df(0);
  if (col) {
    ix = sp.i0[0][x];
    for (int r = 0; r < k; ++r) {
      const float2 n = sp.Ndf[0][x * k + r];
      nx[r] = df(n.x, n.y);
    }
  }
  const df lo = df_from(rho_min), one(1.f, 0.f);
  df sd(0);
  float2 pb[4];
  uint8_t pa = 0;
  auto fetch = [&](int row) {
    const float2* b = B + (int64_t)nbx * row;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int i = x + q * (int)blockDim.x;
      pb[q] = i < nbx ? b[i] : make_float2(0.f, 0.f);
    }
    pa = col ? eactive[x + (int64_t)ex * row] : 0;
  };
  int row = blockIdx.x;
  if (row < nrows) fetch(row);
  for (; row < nrows; row += gridDim.x) {
    __syncthreads();  // the previous row's readers are done with sB
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int i = x + q * (int)blockDim.x;
      if (i < nbx) sB[i] = pb[q];
    }
    const uint8_t act = pa;
    __syncthreads();
    if (row + (int)gridDim.x < nrows) fetch(row + gridDim.x);
    if (!col) continue;
    const int y = row % d.ey, z = row / d.ey;
    const bool in = ix >= 0 && sp.i0[1][y] >= 0 && sp.i0[2][z] >= 0;
    if (MODE == 0) {
      if (!act) continue;
      df v = row_value(sB, ix, nx, k, in);
      if (df_lt(v, lo)) v = lo;
      if (df_lt(one, v)) v = one;
      sd += v;
    } else {
      const int64_t e = x + (int64_t)ex * row;
      if (!act) {
        rho[e] = 0.0; rhop[e] = 0.0; rhop32[e] = 0.0f;
        continue;
      }
      const double v = fmin(fmax(df_to(row_value(sB, ix, nx, k, in)), rho_min), 1.0);
      const double vp = simp_pow(v, penal);
      rho[e] = v; rhop[e] = vp; rhop32[e] = (float)vp;
    }
  }
  if (MODE != 0) return;
  double s = df_to(sd);
  __shared__ double ws[ROW_MAX / 32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double r = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) r += ws[w];
    partial[blockIdx.x] = r;
  }
}

// Pass 1 through the separable kernel when its layer table fits in shared
// memory (returns false otherwise).
static bool spline_yz_sep(cudaStream_t s, const LevelDims& d, const SplineDev& sp, const float2* coeff_df,
                          float2* B) {
  // rows of SEP_Y elements span SEP_Y + order - 1 y-basis indices when the
  // partition is no finer than the elements (the kernel checks each chunk)
  const int cap_j = std::min(sp.nb[1], SEP_Y + sp.order - 1);
  const size_t smem = sizeof(float2) * (size_t)sp.nb[0] * cap_j;
  if (sp.order > MAX_ORDER || smem > 200 * 1024) return false;
  if (smem > 48 * 1024 &&
      cudaFuncSetAttribute(k_spline_yz_sep, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  k_spline_yz_sep<<<dim3(d.ez, (d.ey + SEP_Y - 1) / SEP_Y), 256, smem, s>>>(d, sp, coeff_df, B, cap_j);
  return true;
}

static int rows_threads(const LevelDims& d) { return std::min(ROW_MAX, (d.ex + 31) / 32 * 32); }

// Rows fit the row kernel: at most ROW_MAX elements, a staged row of basis
// values within 4 per thread, spline order at most MAX_ORDER.
static bool rows_fit(const LevelDims& d, const SplineDev& sp) {
  return d.ex <= ROW_MAX && sp.nb[0] <= 4 * rows_threads(d) && sp.order <= MAX_ORDER;
}

static int rows_blocks(const LevelDims& d) { return (int)std::min<int64_t>(1024, (int64_t)d.ey * d.ez); }

void launch_coeff_to_density(cudaStream_t s, const LevelDims& d, const uint8_t* eactive,
                             const SplineDev& sp, const double* coeff, double rho_min, double penal,
                             double* rho, double* rhop, float* rhop32, double* Btmp, float2* coeff_df) {
  const int64_t nB = (int64_t)sp.nb[0] * d.ey * d.ez;
  const int64_t nc = (int64_t)sp.nb[0] * sp.nb[1] * sp.nb[2];
  float2* B = reinterpret_cast<float2*>(Btmp);  // nB (hi, lo) pairs in the nB-double scratch
  bool sep = false;
  if (coeff_df) {
    k_to_df<<<nblk(nc, 256), 256, 0, s>>>(nc, coeff, coeff_df);
    sep = spline_yz_sep(s, d, sp, coeff_df, B);
  }
  if (!sep) k_spline_yz<<<nblk(nB, 256), 256, 0, s>>>(d, sp, coeff, B);
  if (rows_fit(d, sp))
    k_spline_rows<1><<<rows_blocks(d), rows_threads(d), sizeof(float2) * sp.nb[0], s>>>(
        d, eactive, sp, B, rho_min, penal, nullptr, rho, rhop, rhop32);
  else
    k_density_from_B<<<nblk(d.ne, 256), 256, 0, s>>>(d, eactive, sp, B, rho_min, penal, rho, rhop, rhop32);
}

void launch_trial_volume(cudaStream_t s, const LevelDims& d, const uint8_t* eactive,
                         const SplineDev& sp, const float2* coeff_df, double rho_min, double* partial,
                         double* out, double* Btmp) {
  const int64_t nB = (int64_t)sp.nb[0] * d.ey * d.ez;
  float2* B = reinterpret_cast<float2*>(Btmp);  // nB (hi, lo) pairs in the nB-double scratch
  if (!spline_yz_sep(s, d, sp, coeff_df, B)) k_spline_yz_df<<<nblk(nB, 256), 256, 0, s>>>(d, sp, coeff_df, B);
  int nb;
  if (rows_fit(d, sp)) {
    nb = rows_blocks(d);
    k_spline_rows<0><<<nb, rows_threads(d), sizeof(float2) * sp.nb[0], s>>>(d, eactive, sp, B, rho_min, 0.0, partial,
                                                                           nullptr, nullptr, nullptr);
  } else {  // two elements per thread at most (up to 2048 partials)
    nb = (int)std::min<int64_t>(2048, (d.ne + VOL_THREADS * 2 - 1) / (VOL_THREADS * 2));
    if (nb < 1) nb = 1;
    k_volume_from_B<<<nb, VOL_THREADS, 0, s>>>(d, eactive, sp, B, rho_min, partial);
  }
  k_sum_partials<<<1, 256, 0, s>>>(partial, nb, out);
}

// Element sensitivity g_e = -p rho^(p-1) u_e^T Ke u_e (optimization/optimization.cu:96-159),
// with u_e^T Ke u_e evaluated in the sum-factorised modal form: Walsh-Hadamard
// coefficients of the nodal values, the displacement gradient split over the
// orthogonal functions {1, X, Y, Z, YZ, XZ, XY} of the reference cube, and the
// isotropic energy of each part weighted by the function's L2 norm.  The
// energy is formed in double-float arithmetic (about 1e-14 relative, on the
// FP32 pipe); only the final scaling by -p rho^(p-1) (h/2)^3 runs in FP64.
template <typename T>
__device__ __forceinline__ T cst(double v);
template <>
__device__ __forceinline__ double cst<double>(double v) { return v; }
template <>
__device__ __forceinline__ df cst<df>(double v) { return df_from(v); }
__device__ __forceinline__ double to_double(double v) { return v; }
__device__ __forceinline__ double to_double(df v) { return df_to(v); }

template <typename T>
__device__ __forceinline__ void hadamard8(T v[8]) {
#pragma unroll
  for (int h = 1; h < 8; h <<= 1)
#pragma unroll
    for (int i = 0; i < 8; ++i)
      if (!(i & h)) {
        const T a = v[i], b = v[i | h];
        v[i] = a + b;
        v[i | h] = b - a;
      }
}

// 0.5 lam tr(G)^2 + mu |sym G|^2 with lam2 = lam / 2
template <typename T>
__device__ __forceinline__ T energy_part(const T G[3][3], T lam2, T mu) {
  const T half = cst<T>(0.5), two = cst<T>(2.0);
  const T tr = G[0][0] + G[1][1] + G[2][2];
  T ee = G[0][0] * G[0][0] + G[1][1] * G[1][1] + G[2][2] * G[2][2];
  const T e01 = half * (G[0][1] + G[1][0]), e02 = half * (G[0][2] + G[2][0]), e12 = half * (G[1][2] + G[2][1]);
  ee += two * (e01 * e01 + e02 * e02 + e12 * e12);
  return lam2 * tr * tr + mu * ee;
}

template <typename T>
__global__ void k_sensitivity(LevelDims d, const uint8_t* __restrict__ eactive,
                              const double* __restrict__ rho, const double* __restrict__ u,
                              double penal, double lam, double mu, double h, double* __restrict__ sens) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= d.ne) return;
  if (!eactive[e]) { sens[e] = 0.0; return; }
  const int x = (int)(e % d.ex);
  const int64_t t = e / d.ex;
  const int y = (int)(t % d.ey), z = (int)(t / d.ey);
  // c[i][S]: modal coefficient of component i for mode S (bit0 x, bit1 y, bit2 z),
  // with sign convention H[a][S] = prod_{k in S} (2 a_k - 1); scaled by 2/h * 1/8.
  T c[3][8];
#pragma unroll
  for (int i = 0; i < 3; ++i) {
#pragma unroll
    for (int a = 0; a < 8; ++a) {
      const int64_t v = (x + (a & 1)) + (int64_t)d.vx * ((y + ((a >> 1) & 1)) + (int64_t)d.vy * (z + (a >> 2)));
      c[i][a] = cst<T>(u[i * d.nv + v]);
    }
    hadamard8<T>(c[i]);
  }
  const T sc = cst<T>(2.0 / h / 8.0), lam2 = cst<T>(0.5 * lam), muT = cst<T>(mu), zero = cst<T>(0.0);
  T tot = zero;
#pragma unroll
  for (int f = 0; f < 7; ++f) {
    T G[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j)
        G[i][j] = ((f >> j) & 1) ? zero : sc * c[i][f | (1 << j)];
    const int nbits = (f & 1) + ((f >> 1) & 1) + ((f >> 2) & 1);
    const T nf = cst<T>(nbits == 0 ? 8.0 : (nbits == 1 ? 8.0 / 3.0 : 8.0 / 9.0));
    tot += nf * energy_part<T>(G, lam2, muT);
  }
  const double hh = 0.5 * h;
  const double q = 2.0 * hh * hh * hh * to_double(tot);  // u_e^T Ke u_e
  sens[e] = -penal * simp_pow(rho[e], penal - 1.0) * q;
}

void launch_sensitivity(cudaStream_t s, const LevelDims& d, const uint8_t* eactive,
                        const double* rho, const double* u, double penal, double lam, double mu,
                        double h, double* sens) {
  k_sensitivity<df><<<nblk(d.ne, 128), 128, 0, s>>>(d, eactive, rho, u, penal, lam, mu, h, sens);
}

// The same sensitivity from element energies E = u_e . (rho^p Ke u_e) that the
// solve's final residual kernel wrote: -p rho^(p-1) u_e^T Ke u_e = -p E / rho.
__global__ void k_sensitivity_from_energy(int64_t ne, const uint8_t* __restrict__ eactive,
                                          const double* __restrict__ rho, double penal, double* __restrict__ sens) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ne) return;
  const double r = rho[e];
  sens[e] = (eactive[e] && r > 0.0) ? -penal * sens[e] / r : 0.0;
}

void launch_sensitivity_from_energy(cudaStream_t s, int64_t ne, const uint8_t* eactive, const double* rho,
                                    double penal, double* sens) {
  k_sensitivity_from_energy<<<nblk(ne, 256), 256, 0, s>>>(ne, eactive, rho, penal, sens);
}

// Sensitivity filter (grid/Grid.cu:4130-4229): normalised average over the ball
// r^2 <= R^2, R_int = floor(R + 0.5), weight 1 - 6s^2 + 8s^3 - 3s^4 with s = r/R.
// The ball's offsets and weights depend only on R; they come precomputed (in the
// reference's loop order dx, dy, dz) so no square root is taken per neighbour.
// It runs in double-float arithmetic (about 1e-14 relative): the sensitivities
// and weights arrive split into (hi, lo) floats, the weighted sums run on the
// FP32 pipe, and the quotient is a double-float division (FP32 quotient, one
// correction from the double-float remainder; Dekker 1971).  An FP64 form is
// bound by GB300's FP64 pipe (66 FP64 operations per element).
__device__ __forceinline__ df df_div(df a, df b) {
  const float q1 = __fdiv_rn(a.hi, b.hi);
  const df r = a - b * df(q1, 0.f);
  const float q2 = __fdiv_rn(r.hi, b.hi);
  return df_fast2sum(q1, q2);
}

__global__ void k_filter_df(LevelDims d, const uint8_t* __restrict__ eactive, const float2* __restrict__ src,
                            double* __restrict__ dst, const int4* __restrict__ offs,
                            const float2* __restrict__ wts, int noffs) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= d.ne) return;
  if (!eactive[e]) { dst[e] = 0.0; return; }
  int x, y, z;
  if (d.ne < (int64_t)1 << 31) {  // 32-bit index arithmetic
    const unsigned ee = (unsigned)e, ex = (unsigned)d.ex, t = ee / ex;
    x = (int)(ee - t * ex);
    y = (int)(t % (unsigned)d.ey);
    z = (int)(t / (unsigned)d.ey);
  } else {
    x = (int)(e % d.ex);
    const int64_t t = e / d.ex;
    y = (int)(t % d.ey);
    z = (int)(t / d.ey);
  }
  df ws(0), gs(0);
  for (int k = 0; k < noffs; ++k) {
    const int4 o = offs[k];
    const int nx = x + o.x, ny = y + o.y, nz = z + o.z;
    if (nx < 0 || ny < 0 || nz < 0 || nx >= d.ex || ny >= d.ey || nz >= d.ez) continue;
    const int64_t n = nx + (int64_t)d.ex * (ny + (int64_t)d.ey * nz);
    if (!eactive[n]) continue;
    const float2 wv = wts[k], sv = src[n];
    const df w(wv.x, wv.y);
    gs += w * df(sv.x, sv.y);
    ws += w;
  }
  dst[e] = df_to(df_div(gs, ws));
}

void launch_filter_df(cudaStream_t s, const LevelDims& d, const uint8_t* eactive, double* sens,
                      float2* sens_df, const int4* offs, const float2* wts, int noffs) {
  k_to_df<<<nblk(d.ne, 256), 256, 0, s>>>(d.ne, sens, sens_df);
  k_filter_df<<<nblk(d.ne, 128), 128, 0, s>>>(d, eactive, sens_df, sens, offs, wts, noffs);
}

// Ball offsets within r^2 <= R^2, R_int = floor(R + 0.5), weight
// 1 - 6s^2 + 8s^3 - 3s^4 with s = r/R (grid/Grid.cu:4156-4209, 4226-4229).
void filter_table(double R, std::vector<int4>& offs, std::vector<double>& w) {
  const int Ri = (int)(R + 0.5);
  const double R2 = R * R;
  offs.clear();
  w.clear();
  for (int dx = -Ri; dx <= Ri; ++dx)
    for (int dy = -Ri; dy <= Ri; ++dy)
      for (int dz = -Ri; dz <= Ri; ++dz) {
        const double r2 = (double)(dx * dx + dy * dy + dz * dz);
        if (r2 > R2) continue;
        const double sv = std::sqrt(r2 / R2), s2 = sv * sv;
        w.push_back(1.0 - 6.0 * s2 + 8.0 * s2 * sv - 3.0 * s2 * s2);
        offs.push_back(make_int4(dx, dy, dz, 0));
      }
}

// Spline adjoint (grid/Grid.cu:3671-3724) as a deterministic separable gather:
// T1[i][y][z] = sum_x g Nx, T2[i][j][z] = sum_y T1 Ny, dc[i][j][k] = sum_z T2 Nz.
// Elements outside the spline range (any axis) and inactive elements contribute 0.
__global__ void k_adj_x(LevelDims d, const uint8_t* __restrict__ eactive, SplineDev sp,
                        const double* __restrict__ g, double* __restrict__ T1) {
  const int64_t gid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int nbx = sp.nb[0];
  if (gid >= (int64_t)nbx * d.ey * d.ez) return;
  const int i = (int)(gid % nbx);
  const int64_t yz = gid / nbx;
  const int y = (int)(yz % d.ey), z = (int)(yz / d.ey);
  double s = 0.0;
  if (sp.i0[1][y] >= 0 && sp.i0[2][z] >= 0) {
    const int k = sp.order;
    for (int x = sp.lo[0][i]; x < sp.hi[0][i]; ++x) {
      const int ix = sp.i0[0][x];
      if (ix < 0) continue;
      const int r = i - ix;
      if (r < 0 || r >= k) continue;
      const int64_t e = x + (int64_t)d.ex * (y + (int64_t)d.ey * z);
      if (!eactive[e]) continue;
      s += g[e] * sp.N[0][x * k + r];
    }
  }
  T1[gid] = s;  // layout [z][y][i]
}

__global__ void k_adj_y(LevelDims d, SplineDev sp, const double* __restrict__ T1, double* __restrict__ T2) {
  const int64_t gid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int nbx = sp.nb[0], nby = sp.nb[1];
  if (gid >= (int64_t)nbx * nby * d.ez) return;
  const int i = (int)(gid % nbx);
  const int64_t t = gid / nbx;
  const int j = (int)(t % nby), z = (int)(t / nby);
  const int k = sp.order;
  double s = 0.0;
  for (int y = sp.lo[1][j]; y < sp.hi[1][j]; ++y) {
    const int iy = sp.i0[1][y];
    if (iy < 0) continue;
    const int r = j - iy;
    if (r < 0 || r >= k) continue;
    s += T1[i + (int64_t)nbx * (y + (int64_t)d.ey * z)] * sp.N[1][y * k + r];
  }
  T2[gid] = s;  // layout [z][j][i]
}

__global__ void k_adj_z(LevelDims d, SplineDev sp, const double* __restrict__ T2, double* __restrict__ dc) {
  const int64_t gid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int nbx = sp.nb[0], nby = sp.nb[1], nbz = sp.nb[2];
  if (gid >= (int64_t)nbx * nby * nbz) return;
  const int i = (int)(gid % nbx);
  const int64_t t = gid / nbx;
  const int j = (int)(t % nby), kk = (int)(t / nby);
  const int k = sp.order;
  double s = 0.0;
  for (int z = sp.lo[2][kk]; z < sp.hi[2][kk]; ++z) {
    const int iz = sp.i0[2][z];
    if (iz < 0) continue;
    const int r = kk - iz;
    if (r < 0 || r >= k) continue;
    s += T2[i + (int64_t)nbx * (j + (int64_t)nby * z)] * sp.N[2][z * k + r];
  }
  dc[gid] = s;
}

void launch_spline_adjoint(cudaStream_t s, const LevelDims& d, const uint8_t* eactive,
                           const SplineDev& sp, const double* sens, double* csens, double* tmp1,
                           double* tmp2) {
  const int64_t n1 = (int64_t)sp.nb[0] * d.ey * d.ez;
  const int64_t n2 = (int64_t)sp.nb[0] * sp.nb[1] * d.ez;
  const int64_t n3 = (int64_t)sp.nb[0] * sp.nb[1] * sp.nb[2];
  k_adj_x<<<nblk(n1, 256), 256, 0, s>>>(d, eactive, sp, sens, tmp1);
  k_adj_y<<<nblk(n2, 256), 256, 0, s>>>(d, sp, tmp1, tmp2);
  k_adj_z<<<nblk(n3, 256), 256, 0, s>>>(d, sp, tmp2, csens);
}

__global__ void k_penalise(int64_t ne, const uint8_t* __restrict__ eactive, const double* __restrict__ rho,
                           double penal, double* __restrict__ rhop, float* __restrict__ rhop32) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ne) return;
  const double v = eactive[e] ? simp_pow(rho[e], penal) : 0.0;
  rhop[e] = v;
  rhop32[e] = (float)v;
}

void launch_penalise(cudaStream_t s, int64_t ne, const uint8_t* eactive, const double* rho,
                     double penal, double* rhop, float* rhop32) {
  k_penalise<<<nblk(ne, 256), 256, 0, s>>>(ne, eactive, rho, penal, rhop, rhop32);
}

// Reference precision (the reference keeps rho in FP32 and takes rho^p with
// powf, grid/Grid.cu:1739): rho rounded to FP32, rho^p = powf(rho, p) in FP32.
__global__ void k_penalise_ref32(int64_t ne, const uint8_t* __restrict__ eactive, double* __restrict__ rho,
                                 float penal, double* __restrict__ rhop, float* __restrict__ rhop32) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ne) return;
  const float r = (float)rho[e];
  rho[e] = (double)r;
  const float v = eactive[e] ? powf(r, penal) : 0.f;
  rhop[e] = (double)v;
  rhop32[e] = v;
}

void launch_penalise_ref32(cudaStream_t s, int64_t ne, const uint8_t* eactive, double* rho, double penal,
                           double* rhop, float* rhop32) {
  k_penalise_ref32<<<nblk(ne, 256), 256, 0, s>>>(ne, eactive, rho, (float)penal, rhop, rhop32);
}

// x[i] rounded to FP32 in place: the arrays the reference stores as float.
__global__ void k_round_f32(int64_t n, double* __restrict__ x) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) x[i] = (double)(float)x[i];
}

void launch_round_f32(cudaStream_t s, int64_t n, double* x) {
  if (n > 0) k_round_f32<<<nblk(n, 256), 256, 0, s>>>(n, x);
}

// OC trial on the coefficients (optimization/optimization.cu:559-587):
// c' = clamp(clamp(c (max(-dc,0)/thres)^damp, c-step, c+step), cmin, cmax).
// The threshold is thres, or *thres_p when that is given (the device-side
// bisection).  For damp = 1/2 the power is the correctly rounded square root.
__global__ void k_oc_trial(int64_t nc, const double* __restrict__ cold, const double* __restrict__ csens,
                           double thres, const double* __restrict__ thres_p, double damp, double step,
                           double cmin, double cmax, double* __restrict__ cnew, float2* __restrict__ cnew_df) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nc) return;
  if (thres_p) thres = *thres_p;
  double g = csens[i];
  if (g > 0) g = 0;
  g = fabs(g);
  const double co = cold[i];
  const double q = g / thres;
  double cn = co * (damp == 0.5 ? sqrt(q) : pow(q, damp));
  cn = fmin(fmax(cn, co - step), co + step);
  cn = fmin(fmax(cn, cmin), cmax);
  cnew[i] = cn;
  if (cnew_df) {
    const df v = df_from(cn);
    cnew_df[i] = make_float2(v.hi, v.lo);
  }
}

void launch_oc_trial(cudaStream_t s, int64_t nc, const double* cold, const double* csens, double thres,
                     double damp, double step, double cmin, double cmax, double* cnew, float2* cnew_df,
                     const double* thres_p) {
  k_oc_trial<<<nblk(nc, 256), 256, 0, s>>>(nc, cold, csens, thres, thres_p, damp, step, cmin, cmax, cnew,
                                           cnew_df);
}

}  // namespace topo
