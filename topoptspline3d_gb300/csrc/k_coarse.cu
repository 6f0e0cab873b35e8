// Coarse-level kernels: 27-point 3x3-block stencil apply / Gauss-Seidel,
// trilinear transfers, Galerkin coarse operators and the coarsest dense solve.
#include <cooperative_groups.h>

#include <mutex>

#include "df.cuh"
#include "topo_internal.h"

namespace cg = cooperative_groups;

namespace topo {

static inline unsigned nblk(int64_t n, int bs) { return (unsigned)((n + bs - 1) / bs); }

// Coarse levels below this vertex count run the warp-per-vertex stencil kernels.
constexpr int64_t STENCIL_WARP_MAX_NV = 32768;

// Where stencil coefficient q (neighbour k times 9 plus block entry, 0..242) of
// vertex v lives: base(v) + q * stride().  [243][nv] for FP64 and for the small
// levels; tiled for the FP32 levels the row kernels serve (vertex count at
// least STENCIL_WARP_MAX_NV): the 243 x 32 coefficients of each group of 32
// vertices lie together, so a warp of consecutive vertices reads one
// contiguous block instead of 243 arrays.  A tiled array holds 243 x 32
// values per started group of 32 vertices.
struct StIdx {
  int64_t nv;
  bool tiled;
  __device__ __forceinline__ int64_t base(int64_t v) const { return tiled ? (v >> 5) * (243 * 32) + (v & 31) : v; }
  __device__ __forceinline__ int64_t stride() const { return tiled ? 32 : nv; }
};

template <typename T>
StIdx st_idx(const LevelDims& d) {
  return StIdx{d.nv, sizeof(T) == 4 && d.nv >= STENCIL_WARP_MAX_NV};
}

// ---------------------------------------------------------------------------
// Stencil apply: y_v = sum_d S(v,d) u_{v+d}  (grid/Grid.cu:2126-2224 residual form).
// ---------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ void stencil_row(const LevelDims& d, const T* __restrict__ st, StIdx si,
                                            const T* __restrict__ u, int x, int y, int z, int64_t v,
                                            T o[3]) {
  o[0] = o[1] = o[2] = T(0);
  const int64_t nv = d.nv, ss = si.stride();
  const T* sb = st + si.base(v);
#pragma unroll
  for (int k = 0; k < 27; ++k) {
    const int nx = x + k % 3 - 1, ny = y + k / 3 % 3 - 1, nz = z + k / 9 - 1;
    if (nx < 0 || ny < 0 || nz < 0 || nx >= d.vx || ny >= d.vy || nz >= d.vz) continue;
    const int64_t n = nx + (int64_t)d.vx * (ny + (int64_t)d.vy * nz);
    const T u0 = u[n], u1 = u[nv + n], u2 = u[2 * nv + n];
    const T* s = sb + (int64_t)(k * 9) * ss;
    o[0] += s[0] * u0 + s[ss] * u1 + s[2 * ss] * u2;
    o[1] += s[3 * ss] * u0 + s[4 * ss] * u1 + s[5 * ss] * u2;
    o[2] += s[6 * ss] * u0 + s[7 * ss] * u1 + s[8 * ss] * u2;
  }
}


template <typename T>
__global__ void k_stencil_gs(LevelDims d, const T* __restrict__ st, StIdx si, const uint8_t* __restrict__ vmask,
                             T* u, const T* __restrict__ f, int cx, int cy, int cz, int hx, int hy,
                             int64_t cnt, bool reverse) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= cnt) return;
  const int x = cx + 2 * (int)(t % hx);
  const int64_t t2 = t / hx;
  const int y = cy + 2 * (int)(t2 % hy), z = cz + 2 * (int)(t2 / hy);
  const int64_t v = x + (int64_t)d.vx * (y + (int64_t)d.vy * z);
  if (!(vmask[v] & 8)) return;
  T o[3], S[9], r[3];
  stencil_row<T>(d, st, si, u, x, y, z, v, o);
#pragma unroll
  for (int k = 0; k < 9; ++k) S[k] = st[si.base(v) + (int64_t)(13 * 9 + k) * si.stride()];
#pragma unroll
  for (int c = 0; c < 3; ++c) r[c] = f[c * d.nv + v] - o[c];
  T du[3] = {T(0), T(0), T(0)};
  if (!reverse) {
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      T s = r[i];
#pragma unroll
      for (int j = 0; j < i; ++j) s -= S[3 * i + j] * du[j];
      du[i] = s / S[4 * i];
    }
  } else {
#pragma unroll
    for (int i = 2; i >= 0; --i) {
      T s = r[i];
#pragma unroll
      for (int j = i + 1; j < 3; ++j) s -= S[3 * i + j] * du[j];
      du[i] = s / S[4 * i];
    }
  }
#pragma unroll
  for (int i = 0; i < 3; ++i) u[i * d.nv + v] += du[i];
}

template <typename T>
__global__ void k_stencil_diag_inv(LevelDims d, const T* __restrict__ st, StIdx si,
                                   const uint8_t* __restrict__ vmask, T* __restrict__ dinv) {
  const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= d.nv) return;
  T S[9];
#pragma unroll
  for (int k = 0; k < 9; ++k) S[k] = st[si.base(v) + (int64_t)(13 * 9 + k) * si.stride()];
  const T a = S[0], b = S[1], c = S[2], dd = S[4], e = S[5], f = S[8];
  const T A0 = dd * f - e * e, A1 = c * e - b * f, A2 = b * e - c * dd;
  const T det = a * A0 + b * A1 + c * A2;
  const T inv[9] = {A0, A1, A2, A1, a * f - c * c, b * c - a * e, A2, b * c - a * e, a * dd - b * b};
  const T rd = T(1) / det;
  const bool act = (vmask[v] & 8) != 0;
#pragma unroll
  for (int k = 0; k < 9; ++k) dinv[k * d.nv + v] = act ? inv[k] * rd : T(0);
}

// Row-split stencil kernels: a CTA of 3 x SV threads covers SV vertices, one
// thread per (vertex, row); the three rows of a vertex share its neighbours'
// values through L1.  Three times the threads of a vertex-per-thread kernel keep
// enough loads in flight on the small coarse levels.
constexpr int SV = 64;

template <typename T>
__device__ __forceinline__ T stencil_row_i(const LevelDims& d, const T* __restrict__ st, StIdx si,
                                           const T* __restrict__ u, int x, int y, int z, int64_t v, int row) {
  T o = T(0);
  const int64_t nv = d.nv, ss = si.stride();
  const T* sb = st + si.base(v);
#pragma unroll
  for (int k = 0; k < 27; ++k) {
    const int nx = x + k % 3 - 1, ny = y + k / 3 % 3 - 1, nz = z + k / 9 - 1;
    if (nx < 0 || ny < 0 || nz < 0 || nx >= d.vx || ny >= d.vy || nz >= d.vz) continue;
    const int64_t n = nx + (int64_t)d.vx * (ny + (int64_t)d.vy * nz);
    const T* s = sb + (int64_t)(k * 9 + 3 * row) * ss;
    o += s[0] * u[n] + s[ss] * u[nv + n] + s[2 * ss] * u[2 * nv + n];
  }
  return o;
}

template <typename T>
__global__ void __launch_bounds__(3 * SV) k_stencil_apply3(LevelDims d, const T* __restrict__ st, StIdx si,
                                                           const T* __restrict__ u, const T* __restrict__ f,
                                                           T* __restrict__ out, bool residual) {
  const int64_t bo = (int64_t)blockIdx.y * 3 * d.nv;  // right-hand side of the batch
  u += bo;
  if (f) f += bo;
  out += bo;
  const int row = threadIdx.x / SV;
  const int64_t v = (int64_t)blockIdx.x * SV + threadIdx.x % SV;
  if (v >= d.nv) return;
  const int x = (int)(v % d.vx);
  const int64_t t = v / d.vx;
  const int y = (int)(t % d.vy), z = (int)(t / d.vy);
  const T o = stencil_row_i<T>(d, st, si, u, x, y, z, v, row);
  const int64_t i = row * d.nv + v;
  out[i] = residual ? f[i] - o : o;
}

// One Chebyshev step on a stencil level: uout = u + d, d = c_old d + c_new Dinv (f - A u).
template <typename T>
__global__ void __launch_bounds__(3 * SV) k_stencil_cheb(LevelDims d, const T* __restrict__ st, StIdx si,
                                                         const T* __restrict__ u, const T* __restrict__ f,
                                                         T* __restrict__ uout, const T* __restrict__ dinv,
                                                         T* __restrict__ dv, const double* __restrict__ coef,
                                                         bool first) {
  __shared__ T sr[3][SV];
  const int64_t bo = (int64_t)blockIdx.y * 3 * d.nv;  // right-hand side of the batch
  u += bo;
  f += bo;
  uout += bo;
  dv += bo;
  const int row = threadIdx.x / SV, lv = threadIdx.x % SV;
  const int64_t v = (int64_t)blockIdx.x * SV + lv;
  const int64_t nv = d.nv;
  const bool ok = v < nv;
  if (ok) {
    const int x = (int)(v % d.vx);
    const int64_t t = v / d.vx;
    const int y = (int)(t % d.vy), z = (int)(t / d.vy);
    sr[row][lv] = f[row * nv + v] - stencil_row_i<T>(d, st, si, u, x, y, z, v, row);
  }
  __syncthreads();
  if (!ok) return;
  const T zz = dinv[(3 * row) * nv + v] * sr[0][lv] + dinv[(3 * row + 1) * nv + v] * sr[1][lv] +
               dinv[(3 * row + 2) * nv + v] * sr[2][lv];
  const int64_t i = row * nv + v;
  const T c_old = (T)__ldg(coef), c_new = (T)__ldg(coef + 1);
  const T dn = first ? c_new * zz : c_old * dv[i] + c_new * zz;
  dv[i] = dn;
  uout[i] = u[i] + dn;
}

// Warp-per-vertex forms for the small coarse levels, whose row-per-thread
// kernels are latency-bound (a thread walks 27 neighbours in sequence while
// only a few warps per SM are resident): lane k < 27 takes neighbour k, forms
// its three row contributions from 9 stencil and 3 vector loads, and the warp
// sums them with shuffles.  One round of independent loads per vertex.  Small
// levels' stencils stay in L2, so the lanes' scattered stencil reads are cheap.
constexpr int WV = 8;  // vertices (warps) per 256-thread CTA

template <typename T>
__device__ __forceinline__ void stencil_warp_rows(const LevelDims& d, const T* __restrict__ st,
                                                  const T* __restrict__ u, int64_t v, int lane, T o[3]) {
  const int x = (int)(v % d.vx);
  const int64_t t = v / d.vx;
  const int y = (int)(t % d.vy), z = (int)(t / d.vy);
  o[0] = o[1] = o[2] = T(0);
  if (lane < 27) {
    const int nx = x + lane % 3 - 1, ny = y + lane / 3 % 3 - 1, nz = z + lane / 9 - 1;
    if (nx >= 0 && ny >= 0 && nz >= 0 && nx < d.vx && ny < d.vy && nz < d.vz) {
      const int64_t n = nx + (int64_t)d.vx * (ny + (int64_t)d.vy * nz), nv = d.nv;
      const T u0 = u[n], u1 = u[nv + n], u2 = u[2 * nv + n];
      const T* sk = st + (int64_t)(lane * 9) * nv + v;
#pragma unroll
      for (int row = 0; row < 3; ++row)
        o[row] = sk[(3 * row) * nv] * u0 + sk[(3 * row + 1) * nv] * u1 + sk[(3 * row + 2) * nv] * u2;
    }
  }
#pragma unroll
  for (int row = 0; row < 3; ++row)
#pragma unroll
    for (int m = 16; m > 0; m >>= 1) o[row] += __shfl_xor_sync(0xffffffffu, o[row], m);
}

template <typename T>
__global__ void __launch_bounds__(32 * WV) k_stencil_apply_warp(LevelDims d, const T* __restrict__ st,
                                                                const T* __restrict__ u, const T* __restrict__ f,
                                                                T* __restrict__ out, bool residual) {
  const int64_t bo = (int64_t)blockIdx.y * 3 * d.nv;  // right-hand side of the batch
  u += bo;
  if (f) f += bo;
  out += bo;
  const int lane = threadIdx.x & 31;
  const int64_t v = (int64_t)blockIdx.x * WV + (threadIdx.x >> 5);
  if (v >= d.nv) return;  // whole warp
  T o[3];
  stencil_warp_rows<T>(d, st, u, v, lane, o);
  if (lane < 3) {
    const int64_t i = lane * d.nv + v;
    const T ol = lane == 0 ? o[0] : (lane == 1 ? o[1] : o[2]);
    out[i] = residual ? f[i] - ol : ol;
  }
}

template <typename T>
__global__ void __launch_bounds__(32 * WV) k_stencil_cheb_warp(LevelDims d, const T* __restrict__ st,
                                                               const T* __restrict__ u, const T* __restrict__ f,
                                                               T* __restrict__ uout, const T* __restrict__ dinv,
                                                               T* __restrict__ dv, const double* __restrict__ coef,
                                                               bool first) {
  const int64_t bo = (int64_t)blockIdx.y * 3 * d.nv;  // right-hand side of the batch
  u += bo;
  f += bo;
  uout += bo;
  dv += bo;
  const int lane = threadIdx.x & 31;
  const int64_t v = (int64_t)blockIdx.x * WV + (threadIdx.x >> 5);
  if (v >= d.nv) return;  // whole warp
  T o[3];
  stencil_warp_rows<T>(d, st, u, v, lane, o);
  if (lane < 3) {
    const int64_t nv = d.nv;
    const T r0 = f[v] - o[0], r1 = f[nv + v] - o[1], r2 = f[2 * nv + v] - o[2];
    const T zz = dinv[(3 * lane) * nv + v] * r0 + dinv[(3 * lane + 1) * nv + v] * r1 +
                 dinv[(3 * lane + 2) * nv + v] * r2;
    const int64_t i = lane * nv + v;
    const T c_old = (T)__ldg(coef), c_new = (T)__ldg(coef + 1);
    const T dn = first ? c_new * zz : c_old * dv[i] + c_new * zz;
    dv[i] = dn;
    uout[i] = u[i] + dn;
  }
}

// Levels with fewer vertices than this use the warp-per-vertex kernels.

template <typename T>
void launch_stencil_apply(cudaStream_t s, const LevelDims& d, const T* st, const T* u, const T* f,
                          T* out, bool residual, int nb) {
  if (d.nv < STENCIL_WARP_MAX_NV)
    k_stencil_apply_warp<T><<<dim3(nblk(d.nv, WV), nb), 32 * WV, 0, s>>>(d, st, u, f, out, residual);
  else
    k_stencil_apply3<T><<<dim3(nblk(d.nv, SV), nb), 3 * SV, 0, s>>>(d, st, st_idx<T>(d), u, f, out, residual);
}

template <typename T>
void launch_stencil_cheb(cudaStream_t s, const LevelDims& d, const T* st, const T* u, const T* f, T* uout,
                         const T* dinv, T* dvec, const double* coef, bool first, int nb) {
  if (d.nv < STENCIL_WARP_MAX_NV)
    k_stencil_cheb_warp<T><<<dim3(nblk(d.nv, WV), nb), 32 * WV, 0, s>>>(d, st, u, f, uout, dinv, dvec, coef, first);
  else
    k_stencil_cheb<T><<<dim3(nblk(d.nv, SV), nb), 3 * SV, 0, s>>>(d, st, st_idx<T>(d), u, f, uout, dinv, dvec, coef,
                                                                  first);
}

template void launch_stencil_cheb<double>(cudaStream_t, const LevelDims&, const double*, const double*,
                                          const double*, double*, const double*, double*, const double*, bool, int);
template void launch_stencil_cheb<float>(cudaStream_t, const LevelDims&, const float*, const float*,
                                         const float*, float*, const float*, float*, const double*, bool, int);

// First Chebyshev step from a zero iterate with a stored block-Jacobi inverse
// (coarse levels; FP64 level 0 with its free-DOF mask): r = f, d = c_new D^-1 r,
// u_out = d.  Equals the full step on u = 0, since A 0 = 0 exactly.
template <typename T>
__global__ void k_cheb_zero_stored(int64_t nv, const uint8_t* __restrict__ vmask, const T* __restrict__ dinv,
                                   const T* __restrict__ f, T* __restrict__ dv, T* __restrict__ uout,
                                   const double* __restrict__ coef) {
  const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= nv) return;
  const int64_t bo = (int64_t)blockIdx.y * 3 * nv;
  f += bo;
  dv += bo;
  uout += bo;
  const uint8_t m = vmask ? vmask[v] : 7;
  T r[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) r[c] = ((m >> c) & 1) ? f[c * nv + v] : T(0);
  const T c_new = (T)__ldg(coef + 1);
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const T zz = dinv[(3 * c) * nv + v] * r[0] + dinv[(3 * c + 1) * nv + v] * r[1] + dinv[(3 * c + 2) * nv + v] * r[2];
    const T dn = c_new * zz;
    dv[c * nv + v] = dn;
    uout[c * nv + v] = dn;
  }
}

template <typename T>
void launch_cheb_zero_stored(cudaStream_t s, int64_t nv, const uint8_t* vmask, const T* dinv, const T* f, T* dvec,
                             T* uout, const double* coef, int nb) {
  k_cheb_zero_stored<T><<<dim3(nblk(nv, 256), nb), 256, 0, s>>>(nv, vmask, dinv, f, dvec, uout, coef);
}

template void launch_cheb_zero_stored<double>(cudaStream_t, int64_t, const uint8_t*, const double*, const double*,
                                              double*, double*, const double*, int);
template void launch_cheb_zero_stored<float>(cudaStream_t, int64_t, const uint8_t*, const float*, const float*,
                                             float*, float*, const double*, int);

template <typename T>
void launch_stencil_gs(cudaStream_t s, const LevelDims& d, const T* st, const uint8_t* vmask, T* u,
                       const T* f, int colour, bool reverse) {
  const int cx = colour & 1, cy = (colour >> 1) & 1, cz = colour >> 2;
  const int hx = (d.vx - cx + 1) / 2, hy = (d.vy - cy + 1) / 2, hz = (d.vz - cz + 1) / 2;
  const int64_t cnt = (int64_t)hx * hy * hz;
  if (cnt <= 0) return;
  k_stencil_gs<T><<<nblk(cnt, 128), 128, 0, s>>>(d, st, st_idx<T>(d), vmask, u, f, cx, cy, cz, hx, hy, cnt, reverse);
}

template <typename T>
void launch_stencil_diag_inv(cudaStream_t s, const LevelDims& d, const T* st, const uint8_t* vmask,
                             T* dinv) {
  k_stencil_diag_inv<T><<<nblk(d.nv, 256), 256, 0, s>>>(d, st, st_idx<T>(d), vmask, dinv);
}

// ---------------------------------------------------------------------------
// Transfers.  Prolongation is trilinear interpolation from the coarse element
// corners, masked on fixed fine DOFs; restriction is its exact transpose
// (factor 4: grid/Grid.cu:2509-2570 and 2635-2671; factor 2: 2456-2507, 2594-2632).
// ---------------------------------------------------------------------------
template <typename T, int FCT>
__global__ void k_restrict(LevelDims fd, LevelDims cd, const T* __restrict__ rf, T* __restrict__ fc) {
  rf += (int64_t)blockIdx.y * 3 * fd.nv;  // right-hand side of the batch
  fc += (int64_t)blockIdx.y * 3 * cd.nv;
  const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= cd.nv) return;
  const int x = (int)(v % cd.vx);
  const int64_t t = v / cd.vx;
  const int y = (int)(t % cd.vy), z = (int)(t / cd.vy);
  T s0 = T(0), s1 = T(0), s2 = T(0);
  const T inv = T(1) / T(FCT * FCT * FCT);
  for (int dz = -(FCT - 1); dz <= FCT - 1; ++dz) {
    const int fz = z * FCT + dz;
    if (fz < 0 || fz >= fd.vz) continue;
    const int wz = FCT - (dz < 0 ? -dz : dz);
    for (int dy = -(FCT - 1); dy <= FCT - 1; ++dy) {
      const int fy = y * FCT + dy;
      if (fy < 0 || fy >= fd.vy) continue;
      const int wyz = wz * (FCT - (dy < 0 ? -dy : dy));
#pragma unroll
      for (int dx = -(FCT - 1); dx <= FCT - 1; ++dx) {
        const int fx = x * FCT + dx;
        if (fx < 0 || fx >= fd.vx) continue;
        const T w = T(wyz * (FCT - (dx < 0 ? -dx : dx))) * inv;
        const int64_t fv = fx + (int64_t)fd.vx * (fy + (int64_t)fd.vy * fz);
        s0 += w * rf[fv];
        s1 += w * rf[fd.nv + fv];
        s2 += w * rf[2 * fd.nv + fv];
      }
    }
  }
  fc[v] = s0; fc[cd.nv + v] = s1; fc[2 * cd.nv + v] = s2;
}

// Restriction by a factor of 4 with the fine z taps split across warps: a CTA
// of 7 warps covers 32 consecutive coarse vertices; warp w gathers the fine
// plane z = 4 cz + w - 3 (7 x 7 taps, weights (4 - |d|) per axis) for its lane's
// vertex, and warp 0 sums the seven partial sums in a fixed order.  Seven
// times the threads of a vertex-per-thread gather keep the loads in flight.
constexpr int R4_WARPS = 7;

template <typename T>
__global__ void __launch_bounds__(32 * R4_WARPS) k_restrict4(LevelDims fd, LevelDims cd, const T* __restrict__ rf,
                                                             T* __restrict__ fc) {
  __shared__ T part[R4_WARPS][3][32];
  rf += (int64_t)blockIdx.y * 3 * fd.nv;  // right-hand side of the batch
  fc += (int64_t)blockIdx.y * 3 * cd.nv;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int64_t v = (int64_t)blockIdx.x * 32 + lane;
  T s0 = T(0), s1 = T(0), s2 = T(0);
  if (v < cd.nv) {
    const int x = (int)(v % cd.vx);
    const int64_t t = v / cd.vx;
    const int y = (int)(t % cd.vy), z = (int)(t / cd.vy);
    const int dz = w - 3, fz = 4 * z + dz;
    if (fz >= 0 && fz < fd.vz) {
      const T wz = T(4 - (dz < 0 ? -dz : dz));
      for (int dy = -3; dy <= 3; ++dy) {
        const int fy = 4 * y + dy;
        if (fy < 0 || fy >= fd.vy) continue;
        const T wyz = wz * T(4 - (dy < 0 ? -dy : dy));
        const int64_t rowv = (int64_t)fd.vx * (fy + (int64_t)fd.vy * fz);
#pragma unroll
        for (int dx = -3; dx <= 3; ++dx) {
          const int fx = 4 * x + dx;
          if (fx < 0 || fx >= fd.vx) continue;
          const T wt = wyz * T(4 - (dx < 0 ? -dx : dx));
          const int64_t fv = rowv + fx;
          s0 += wt * rf[fv];
          s1 += wt * rf[fd.nv + fv];
          s2 += wt * rf[2 * fd.nv + fv];
        }
      }
    }
  }
  part[w][0][lane] = s0;
  part[w][1][lane] = s1;
  part[w][2][lane] = s2;
  __syncthreads();
  if (w == 0 && v < cd.nv) {
    const T inv = T(1) / T(64);
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      T a = T(0);
#pragma unroll
      for (int k = 0; k < R4_WARPS; ++k) a += part[k][c][lane];
      fc[c * cd.nv + v] = a * inv;
    }
  }
}

template <typename T, int FCT>
__global__ void k_prolong(LevelDims fd, LevelDims cd, const T* __restrict__ uc, T* __restrict__ uf,
                          const uint8_t* __restrict__ vmask) {
  uc += (int64_t)blockIdx.y * 3 * cd.nv;  // right-hand side of the batch
  uf += (int64_t)blockIdx.y * 3 * fd.nv;
  const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= fd.nv) return;
  int x, y, z;
  if (fd.nv < (int64_t)1 << 31) {  // 32-bit index arithmetic
    const unsigned vv = (unsigned)v, vx = (unsigned)fd.vx, vy = (unsigned)fd.vy, tt = vv / vx;
    x = (int)(vv - tt * vx);
    y = (int)(tt % vy);
    z = (int)(tt / vy);
  } else {
    x = (int)(v % fd.vx);
    const int64_t t = v / fd.vx;
    y = (int)(t % fd.vy);
    z = (int)(t / fd.vy);
  }
  const uint8_t m = vmask[v];
  if (!(m & 7) || !(m & 8)) return;
  const int cx = x / FCT, cy = y / FCT, cz = z / FCT;
  const int rx = x % FCT, ry = y % FCT, rz = z % FCT;
  T s0 = T(0), s1 = T(0), s2 = T(0);
  const T inv = T(1) / T(FCT * FCT * FCT);
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    const int ox = k & 1, oy = (k >> 1) & 1, oz = k >> 2;
    const int wx = ox ? rx : FCT - rx, wy = oy ? ry : FCT - ry, wz = oz ? rz : FCT - rz;
    const int wi = wx * wy * wz;
    if (wi == 0) continue;
    const T w = T(wi) * inv;
    const int64_t cv = (cx + ox) + (int64_t)cd.vx * ((cy + oy) + (int64_t)cd.vy * (cz + oz));
    s0 += w * uc[cv];
    s1 += w * uc[cd.nv + cv];
    s2 += w * uc[2 * cd.nv + cv];
  }
  if (m & 1) uf[v] += s0;
  if (m & 2) uf[fd.nv + v] += s1;
  if (m & 4) uf[2 * fd.nv + v] += s2;
}

template <typename T>
void launch_restrict(cudaStream_t s, const LevelDims& fine, const LevelDims& coarse, const T* rf,
                     T* fc, int nb) {
  if (coarse.factor == 4) {
    k_restrict4<T><<<dim3(nblk(coarse.nv, 32), nb), 32 * R4_WARPS, 0, s>>>(fine, coarse, rf, fc);
  } else {
    k_restrict<T, 2><<<dim3(nblk(coarse.nv, 128), nb), 128, 0, s>>>(fine, coarse, rf, fc);
  }
}

// Prolongation by a factor of 4 with one thread per 4 fine vertices along x
// (x = 4 cx .. 4 cx + 3 share the coarse corners cx, cx + 1): the 24 coarse
// values are read once per 4 fine vertices instead of once per vertex.
template <typename T>
__global__ void __launch_bounds__(256) k_prolong4x(LevelDims fd, LevelDims cd, const T* __restrict__ uc,
                                                   T* __restrict__ uf, const uint8_t* __restrict__ vmask) {
  uc += (int64_t)blockIdx.y * 3 * cd.nv;  // right-hand side of the batch
  uf += (int64_t)blockIdx.y * 3 * fd.nv;
  const int nqx = (fd.vx + 3) / 4;  // 4-vertex groups per fine row
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t nq = (int64_t)nqx * fd.vy * fd.vz;
  if (q >= nq) return;
  const int cx = (int)(q % nqx);
  const int64_t t = q / nqx;
  const int y = (int)(t % fd.vy), z = (int)(t / fd.vy);
  const int cy = y / 4, cz = z / 4, ry = y % 4, rz = z % 4;
  // coarse corners (cx + ox, cy + oy, cz + oz) weighted in y and z; corners
  // with a zero weight are not read (they may lie outside the coarse grid)
  T cyz[2][3];  // [ox][component]: sum over oy, oz of wy wz u_c
#pragma unroll
  for (int ox = 0; ox < 2; ++ox) {
    cyz[ox][0] = cyz[ox][1] = cyz[ox][2] = T(0);
    if (cx + ox >= cd.vx) continue;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int oy = k & 1, oz = k >> 1;
      const int w = (oy ? ry : 4 - ry) * (oz ? rz : 4 - rz);
      if (w == 0) continue;
      const int64_t cv = (cx + ox) + (int64_t)cd.vx * ((cy + oy) + (int64_t)cd.vy * (cz + oz));
      cyz[ox][0] += T(w) * uc[cv];
      cyz[ox][1] += T(w) * uc[cd.nv + cv];
      cyz[ox][2] += T(w) * uc[2 * cd.nv + cv];
    }
  }
  const T inv = T(1) / T(64);
  const int64_t row = (int64_t)fd.vx * (y + (int64_t)fd.vy * z);
  // masks and fine values of the four vertices are loaded together (a vertex
  // past the row's end reads the group's first), then the corrections added
  uint8_t mm[4];
  T uo[4][3];
#pragma unroll
  for (int rx = 0; rx < 4; ++rx) {
    const int x = 4 * cx + rx;
    const int64_t v = row + (x < fd.vx ? x : 4 * cx);
    mm[rx] = x < fd.vx ? vmask[v] : 0;
#pragma unroll
    for (int c = 0; c < 3; ++c) uo[rx][c] = uf[c * fd.nv + v];
  }
#pragma unroll
  for (int rx = 0; rx < 4; ++rx) {
    const uint8_t m = mm[rx];
    if (!(m & 7) || !(m & 8)) continue;
    const int64_t v = row + 4 * cx + rx;
    const T w0 = T(4 - rx), w1 = T(rx);
#pragma unroll
    for (int c = 0; c < 3; ++c)
      if ((m >> c) & 1) uf[c * fd.nv + v] = uo[rx][c] + (w0 * cyz[0][c] + w1 * cyz[1][c]) * inv;
  }
}

template <typename T>
void launch_prolong(cudaStream_t s, const LevelDims& fine, const LevelDims& coarse, const T* uc,
                    T* uf, const uint8_t* vmask_fine, int nb) {
  if (coarse.factor == 4) {
    const int64_t nq = (int64_t)((fine.vx + 3) / 4) * fine.vy * fine.vz;
    k_prolong4x<T><<<dim3(nblk(nq, 256), nb), 256, 0, s>>>(fine, coarse, uc, uf, vmask_fine);
  } else
    k_prolong<T, 2><<<dim3(nblk(fine.nv, 256), nb), 256, 0, s>>>(fine, coarse, uc, uf, vmask_fine);
}

// ---------------------------------------------------------------------------
// Galerkin, first coarse level (grid/Grid.cu:1111-1225 restated per element):
// K_E = sum_pos rho^p_pos T_pos over fine elements without fixed DOFs (a
// [N_E x 64] x [64 x 300] product over the symmetric entries), plus the exact
// Q^T Ktilde Q of fine elements that touch fixed DOFs, where Ktilde has the
// fixed rows/columns zeroed and 1e6 on their diagonal (grid/Grid.cu:1196-1207).
// ---------------------------------------------------------------------------
constexpr int GAL_CE = 16;    // coarse elements per CTA
constexpr int GAL_THREADS = 320;

template <typename T, int FCT>
__global__ void __launch_bounds__(GAL_THREADS) k_galerkin_gemm(LevelDims fd, LevelDims cd,
                                                               const double* __restrict__ rhop,
                                                               const uint8_t* __restrict__ vmask,
                                                               const T* __restrict__ Ttab,
                                                               T* __restrict__ kel) {
  constexpr int NPOS = FCT * FCT * FCT;
  __shared__ T rp[GAL_CE][NPOS];
  const int64_t ce0 = (int64_t)blockIdx.x * GAL_CE;
  for (int i = threadIdx.x; i < GAL_CE * NPOS; i += blockDim.x) {
    const int k = i / NPOS, pos = i % NPOS;
    const int64_t ce = ce0 + k;
    T val = T(0);
    if (ce < cd.ne) {
      const int cx = (int)(ce % cd.ex);
      const int64_t t = ce / cd.ex;
      const int cy = (int)(t % cd.ey), cz = (int)(t / cd.ey);
      const int fx = cx * FCT + pos % FCT, fy = cy * FCT + pos / FCT % FCT, fz = cz * FCT + pos / (FCT * FCT);
      if (fx < fd.ex && fy < fd.ey && fz < fd.ez) {
        const int64_t fe = fx + (int64_t)fd.ex * (fy + (int64_t)fd.ey * fz);
        bool fixed = false;
#pragma unroll
        for (int a = 0; a < 8; ++a) {
          const int64_t vv = (fx + (a & 1)) + (int64_t)fd.vx * ((fy + ((a >> 1) & 1)) + (int64_t)fd.vy * (fz + (a >> 2)));
          const uint8_t m = vmask[vv];
          fixed |= (m & 7) != 7;
        }
        val = fixed ? T(0) : T(rhop[fe]);
      }
    }
    rp[k][pos] = val;
  }
  __syncthreads();
  const int ent = threadIdx.x;
  if (ent >= 300) return;
  // upper-triangle index -> (i, j), i <= j
  int i = 0, rem = ent;
  while (rem >= 24 - i) { rem -= 24 - i; ++i; }
  const int j = i + rem;
  T acc[GAL_CE];
#pragma unroll
  for (int k = 0; k < GAL_CE; ++k) acc[k] = T(0);
  for (int pos = 0; pos < NPOS; ++pos) {
    const T tv = Ttab[pos * 576 + i * 24 + j];
#pragma unroll
    for (int k = 0; k < GAL_CE; ++k) acc[k] += rp[k][pos] * tv;
  }
#pragma unroll
  for (int k = 0; k < GAL_CE; ++k) {
    const int64_t ce = ce0 + k;
    if (ce >= cd.ne) break;
    kel[ce * 576 + i * 24 + j] = acc[k];
    kel[ce * 576 + j * 24 + i] = acc[k];
  }
}

// Fixed-DOF fine elements: K_E += Q^T Ktilde_e Q, one CTA per coarse element,
// one thread per entry; fine elements are visited in a fixed order.
template <typename T, int FCT>
__global__ void __launch_bounds__(576) k_galerkin_fixed(LevelDims fd, LevelDims cd,
                                                        const double* __restrict__ rhop,
                                                        const uint8_t* __restrict__ eactive,
                                                        const uint8_t* __restrict__ vmask,
                                                        const double* __restrict__ Ke,
                                                        const int* __restrict__ list,
                                                        T* __restrict__ kel) {
  // products in the operator's precision: FP32 for the FP32 preconditioner's
  // operators (the FP64 form is bound by GB300's FP64 pipe), FP64 for FP64
  constexpr int NP = FCT * FCT * FCT;  // fine elements in the coarse element
  __shared__ T sK[576];
  __shared__ T sQ[8][8];
  __shared__ uint8_t sfree[NP][24];
  __shared__ uint8_t sflag[NP];
  const int64_t ce = list[blockIdx.x];
  const int cx = (int)(ce % cd.ex);
  const int64_t t = ce / cd.ex;
  const int cy = (int)(t % cd.ey), cz = (int)(t / cd.ey);
  const int ent = threadIdx.x;
  const int R = ent / 24, S = ent % 24;
  const int A = R / 3, i = R % 3, B = S / 3, j = S % 3;
  // free-DOF pattern of every fine element at once (one thread each); the
  // fine elements with all 24 DOFs free are left to the GEMM pass
  if (ent < NP) {
    const int px = ent % FCT, py = ent / FCT % FCT, pz = ent / (FCT * FCT);
    const int fx = cx * FCT + px, fy = cy * FCT + py, fz = cz * FCT + pz;
    int flag = 0;
    if (fx < fd.ex && fy < fd.ey && fz < fd.ez && eactive[fx + (int64_t)fd.ex * (fy + (int64_t)fd.ey * fz)]) {
      for (int a = 0; a < 8; ++a) {
        const int64_t vv = (fx + (a & 1)) + (int64_t)fd.vx * ((fy + ((a >> 1) & 1)) + (int64_t)fd.vy * (fz + (a >> 2)));
        const uint8_t m = vmask[vv];
        for (int c = 0; c < 3; ++c) sfree[ent][3 * a + c] = (m >> c) & 1;
        if ((m & 7) != 7) flag = 1;
      }
    }
    sflag[ent] = (uint8_t)flag;
  }
  __syncthreads();
  T acc = T(0);
  for (int pos = 0; pos < NP; ++pos) {
    if (!sflag[pos]) continue;  // the same for the whole CTA
    const int px = pos % FCT, py = pos / FCT % FCT, pz = pos / (FCT * FCT);
    const int fx = cx * FCT + px, fy = cy * FCT + py, fz = cz * FCT + pz;
    const double pe = rhop[fx + (int64_t)fd.ex * (fy + (int64_t)fd.ey * fz)];
    {
      const int r = ent / 24, s2 = ent % 24;
      double k = pe * Ke[ent];
      if (!sfree[pos][r] || !sfree[pos][s2]) k = (r == s2) ? 1e6 : 0.0;
      sK[ent] = T(k);
    }
    if (ent < 64) {
      const int a = ent / 8, C = ent % 8;
      const int q[3] = {px + (a & 1), py + ((a >> 1) & 1), pz + (a >> 2)};
      const int cc[3] = {C & 1, (C >> 1) & 1, C >> 2};
      double w = 1.0;
      for (int k = 0; k < 3; ++k) w *= cc[k] ? (double)q[k] / FCT : (double)(FCT - q[k]) / FCT;
      sQ[a][C] = T(w);
    }
    __syncthreads();
    T s = T(0);
    for (int a = 0; a < 8; ++a) {
      const T qa = sQ[a][A];
      if (qa == T(0)) continue;
      T inner = T(0);
      for (int b = 0; b < 8; ++b) inner += sK[(3 * a + i) * 24 + 3 * b + j] * sQ[b][B];
      s += qa * inner;
    }
    acc += s;
    __syncthreads();  // sK and sQ are rewritten for the next fine element
  }
  if (acc != T(0)) kel[ce * 576 + ent] += acc;
}

// Dyadic Galerkin: K_E = sum_children Q_c^T K_child Q_c (grid/Grid.cu:839-896 in
// element form).  One CTA per coarse element, two-stage product per child.
template <typename T>
__global__ void __launch_bounds__(576) k_galerkin_dyadic(LevelDims fd, LevelDims cd,
                                                         const uint8_t* __restrict__ eactive_f,
                                                         const T* __restrict__ kel_f,
                                                         T* __restrict__ kel_c) {
  __shared__ T sK[576];
  __shared__ T sT[576];
  __shared__ T sQ[8][8];
  const int64_t ce = blockIdx.x;
  const int cx = (int)(ce % cd.ex);
  const int64_t t = ce / cd.ex;
  const int cy = (int)(t % cd.ey), cz = (int)(t / cd.ey);
  const int ent = threadIdx.x;
  const int R = ent / 24, S = ent % 24;
  T acc = T(0);
  for (int c = 0; c < 8; ++c) {
    const int ox = c & 1, oy = (c >> 1) & 1, oz = c >> 2;
    const int fx = 2 * cx + ox, fy = 2 * cy + oy, fz = 2 * cz + oz;
    const bool on = fx < fd.ex && fy < fd.ey && fz < fd.ez &&
                    eactive_f[fx + (int64_t)fd.ex * (fy + (int64_t)fd.ey * fz)];
    if (!on) continue;  // uniform across the CTA
    const int64_t fe = fx + (int64_t)fd.ex * (fy + (int64_t)fd.ey * fz);
    __syncthreads();
    sK[ent] = kel_f[fe * 576 + ent];
    if (ent < 64) {
      const int a = ent / 8, C = ent % 8;
      const int q[3] = {ox + (a & 1), oy + ((a >> 1) & 1), oz + (a >> 2)};
      const int cc[3] = {C & 1, (C >> 1) & 1, C >> 2};
      T w = T(1);
      for (int k = 0; k < 3; ++k) w *= cc[k] ? T(q[k]) / T(2) : T(2 - q[k]) / T(2);
      sQ[a][C] = w;
    }
    __syncthreads();
    {  // stage 1: sT[r][3C+jj] = sum_b K[r][3b+jj] Q[b][C]
      const int r = ent / 24, col = ent % 24, C = col / 3, jj = col % 3;
      T s = T(0);
#pragma unroll
      for (int b = 0; b < 8; ++b) s += sK[r * 24 + 3 * b + jj] * sQ[b][C];
      sT[ent] = s;
    }
    __syncthreads();
    {  // stage 2: acc[(A,i),S] += sum_a Q[a][A] T[3a+i][S]
      const int A = R / 3, i = R % 3;
      T s = T(0);
#pragma unroll
      for (int a = 0; a < 8; ++a) s += sQ[a][A] * sT[(3 * a + i) * 24 + S];
      acc += s;
    }
  }
  kel_c[ce * 576 + ent] = acc;
}

// Stencil assembly from element matrices: thread per (neighbour d, vertex v).
template <typename T>
__global__ void k_assemble_stencil(LevelDims d, const uint8_t* __restrict__ eactive,
                                   const uint8_t* __restrict__ vmask, const T* __restrict__ kel,
                                   T* __restrict__ st, StIdx si) {
  const int64_t gid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= 27 * d.nv) return;
  const int k = (int)(gid / d.nv);
  const int64_t v = gid % d.nv;
  const int x = (int)(v % d.vx);
  const int64_t t = v / d.vx;
  const int y = (int)(t % d.vy), z = (int)(t / d.vy);
  const int dx = k % 3 - 1, dy = k / 3 % 3 - 1, dz = k / 9 - 1;
  T blk[9];
#pragma unroll
  for (int q = 0; q < 9; ++q) blk[q] = T(0);
  // elements containing both v and v+(dx,dy,dz)
  for (int ez = z - 1; ez <= z; ++ez) {
    if (ez < 0 || ez >= d.ez) continue;
    const int az = z - ez, bz = az + dz;
    if (bz < 0 || bz > 1) continue;
    for (int ey = y - 1; ey <= y; ++ey) {
      if (ey < 0 || ey >= d.ey) continue;
      const int ay = y - ey, by = ay + dy;
      if (by < 0 || by > 1) continue;
      for (int ex = x - 1; ex <= x; ++ex) {
        if (ex < 0 || ex >= d.ex) continue;
        const int ax = x - ex, bx = ax + dx;
        if (bx < 0 || bx > 1) continue;
        const int64_t e = ex + (int64_t)d.ex * (ey + (int64_t)d.ey * ez);
        if (!eactive[e]) continue;
        const int a = ax + 2 * ay + 4 * az, b = bx + 2 * by + 4 * bz;
        const T* K = kel + e * 576;
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
          for (int j = 0; j < 3; ++j) blk[3 * i + j] += K[(3 * a + i) * 24 + 3 * b + j];
      }
    }
  }
  if (k == 13 && !(vmask[v] & 8)) {
    blk[0] = T(1); blk[4] = T(1); blk[8] = T(1);
  }
#pragma unroll
  for (int q = 0; q < 9; ++q) st[si.base(v) + (int64_t)(k * 9 + q) * si.stride()] = blk[q];
}

__global__ void k_dense_from_stencil(LevelDims d, const double* __restrict__ st,
                                     double* __restrict__ A) {
  const int64_t n = 3 * d.nv;
  const int64_t gid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= 243 * d.nv) return;
  const int q = (int)(gid / d.nv);  // k*9 + 3i + j
  const int64_t v = gid % d.nv;
  const int k = q / 9, i = (q % 9) / 3, j = q % 3;
  const int x = (int)(v % d.vx);
  const int64_t t = v / d.vx;
  const int y = (int)(t % d.vy), z = (int)(t / d.vy);
  const int nx = x + k % 3 - 1, ny = y + k / 3 % 3 - 1, nz = z + k / 9 - 1;
  if (nx < 0 || ny < 0 || nz < 0 || nx >= d.vx || ny >= d.vy || nz >= d.vz) return;
  const int64_t nb = nx + (int64_t)d.vx * (ny + (int64_t)d.vy * nz);
  A[(3 * v + i) * n + 3 * nb + j] = st[(int64_t)q * d.nv + v];
}

__global__ void k_symmetrize(int n, double* A) {
  const int64_t gid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= (int64_t)n * n) return;
  const int i = (int)(gid / n), j = (int)(gid % n);
  if (j >= i) return;
  const double s = 0.5 * (A[(int64_t)i * n + j] + A[(int64_t)j * n + i]);
  A[(int64_t)i * n + j] = s;
  A[(int64_t)j * n + i] = s;
}

// In-place Gauss-Jordan inverse of a symmetric positive (semi-)definite matrix
// (no pivoting needed), one cooperative launch; two grid barriers per pivot.
// A pivot below 1e-10 of the largest diagonal entry belongs to a null
// direction (a floating part of the domain): its row and column are dropped,
// which gives the inverse of the remaining DOFs, as the reference's
// pseudo-inverse does for its coarsest system (grid/Grid.cpp:3657, 4072).
// status[0] counts dropped pivots; a clearly negative pivot sets status[1] = k+1
// and every block stops at the same step (all threads read the same pivot).
__global__ void k_gauss_jordan(int n, double* A, int* status) {
  cg::grid_group grid = cg::this_grid();
  const int64_t nn = (int64_t)n * n;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const int64_t tid0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  double dmax = 0.0;
  for (int k = 0; k < n; ++k) dmax = fmax(dmax, fabs(A[(int64_t)k * n + k]));
  const double tol = 1e-10 * dmax;
  for (int k = 0; k < n; ++k) {
    const double p = A[(int64_t)k * n + k];
    if (p < -tol) {
      if (tid0 == 0) status[1] = k + 1;
      return;
    }
    if (p <= tol) {  // drop DOF k
      for (int64_t g = tid0; g < 2 * (int64_t)n; g += stride) {
        if (g < n) A[(int64_t)k * n + g] = 0.0;
        else A[(g - n) * n + k] = 0.0;
      }
      if (tid0 == 0) status[0] += 1;
      grid.sync();
      continue;
    }
    const double rp = 1.0 / p;
    for (int64_t g = tid0; g < nn; g += stride) {
      const int i = (int)(g / n), j = (int)(g % n);
      if (i == k || j == k) continue;
      A[g] -= A[(int64_t)i * n + k] * A[(int64_t)k * n + j] * rp;
    }
    grid.sync();
    for (int64_t g = tid0; g < 2 * (int64_t)n; g += stride) {
      if (g < n) {
        const int j = (int)g;
        if (j != k) A[(int64_t)k * n + j] *= rp;
        else A[(int64_t)k * n + k] = rp;
      } else {
        const int i = (int)(g - n);
        if (i != k) A[(int64_t)i * n + k] *= -rp;
      }
    }
    grid.sync();
  }
}

// Blocked Gauss-Jordan inversion (in place, SPD matrix, same pivot-drop rule as
// k_gauss_jordan).  For each panel K of GJB pivots: one CTA inverts the
// diagonal block D = A[K,K] pivot by pivot in shared memory (dropping pivots
// <= tol); all CTAs form the row panel P = D^-1 A[K,:] and copy the column panel
// C = A[:,K]; then every element gets its rank-GJB update
//   A[i,c] = D^-1 | P | -C D^-1 | A[i,c] - C[i,:] P[:,c]
// for (i in K, c in K) | (i in K) | (c in K) | otherwise.  Three grid barriers
// per panel instead of two per pivot.
constexpr int GJB = 32;

//
// DFC: the rank-GJB updates of phase C (n^3 of the n^3 + O(n^2 GJB) work) run
// in double-float arithmetic on the FP32 pipe (58x the FP64 rate on GB300),
// with the panels split into (hi, lo) floats once per panel; the panel
// factorisation stays FP64, where its serial latency matters more than its
// rate.  Used when the coarsest matrix comes from FP32 stencils.  (Measured
// at n = 1617, 304 CTAs: splitting the panels as each tile is staged kept the
// FP64 pipe 55% busy with conversions, 6.6 ms against 5.2 ms; also holding the
// matrix split in place for the whole inversion took the FP64 pipe to 18% but
// ran 5.4 ms, and the update on packed two-lane FP32 instructions cut the
// instructions by a quarter but ran 5.6 ms: the panel barriers and the serial
// panel work then set the pace.)
template <bool DFC>
__global__ void __launch_bounds__(256) k_gj_blocked(int n, double* __restrict__ A, double* __restrict__ work,
                                                    int* __restrict__ status) {
  cg::grid_group grid = cg::this_grid();
  __shared__ double sd[GJB][GJB + 1];
  __shared__ df scd[DFC ? GJB : 1][GJB + 1];
  __shared__ df spd[DFC ? GJB : 1][GJB + 1];
  __shared__ double sc[GJB][GJB + 1];
  __shared__ double sp[GJB][GJB + 1];
  double* P = work + GJB * GJB;      // [GJB][n]
  double* Cp = P + (int64_t)GJB * n; // [n][GJB]
  df* Pdf = reinterpret_cast<df*>(Cp + (int64_t)GJB * n);  // P split, [GJB][n]
  df* Cdf = Pdf + (int64_t)GJB * n;                          // Cp split, [n][GJB]
  const int tid = threadIdx.x;
  double dmax = 0.0;
  for (int k = 0; k < n; ++k) dmax = fmax(dmax, fabs(A[(int64_t)k * n + k]));
  const double tol = 1e-10 * dmax;
  const int nblk_tiles = (n + GJB - 1) / GJB;
  // ---- A: CTA 0 inverts a diagonal block D = A[K,K] (K = [k0, k0 + GJB)) in
  // FP64 and publishes it through the work array.  The block of panel k + 1
  // is inverted during panel k's update (look-ahead): CTA 0 updates that one
  // tile first and inverts it while the other CTAs update the rest.
  // (Measured alternatives on GB300 at n = 675: every CTA inverting its own
  // copy saves a grid barrier but ran at 2.4 ms in FP64, every SM's narrow
  // FP64 pipe then carrying the panel work, and at 2.6 ms in double-float,
  // whose pivot steps lengthen the serial chain; inverting between the update
  // phases, with its own grid barrier, ran at 1.9 ms; this form at 1.56 ms.)
  auto panel_invert = [&](int k0) {
    const int kb = min(GJB, n - k0);
    for (int e = tid; e < GJB * GJB; e += blockDim.x) {
      const int r = e / GJB, c = e % GJB;
      sd[r][c] = (r < kb && c < kb) ? A[(int64_t)(k0 + r) * n + k0 + c] : 0.0;
    }
    __syncthreads();
    for (int j = 0; j < kb; ++j) {
      const double p = sd[j][j];
      if (p < -tol) {
        if (tid == 0) status[1] = k0 + j + 1;
        break;
      }
      __syncthreads();
      if (p <= tol) {  // drop DOF k0 + j
        for (int e = tid; e < 2 * GJB; e += blockDim.x) {
          if (e < GJB) sd[j][e] = 0.0;
          else sd[e - GJB][j] = 0.0;
        }
        if (tid == 0) status[0] += 1;
        __syncthreads();
        continue;
      }
      // 1/p: FP32 estimate refined by two Newton steps r <- r + r (1 - p r)
      double rp = (double)__frcp_rn((float)p);
      rp = fma(rp, fma(-p, rp, 1.0), rp);
      rp = fma(rp, fma(-p, rp, 1.0), rp);
      for (int e = tid; e < GJB * GJB; e += blockDim.x) {
        const int r = e / GJB, c = e % GJB;
        if (r < kb && c < kb && r != j && c != j) sd[r][c] -= sd[r][j] * sd[j][c] * rp;
      }
      __syncthreads();
      for (int e = tid; e < 2 * kb; e += blockDim.x) {
        if (e < kb) { if (e != j) sd[j][e] *= rp; else sd[j][j] = rp; }
        else { const int r = e - kb; if (r != j) sd[r][j] *= -rp; }
      }
      __syncthreads();
    }
    __syncthreads();
    for (int e = tid; e < GJB * GJB; e += blockDim.x) work[e] = sd[e / GJB][e % GJB];
  };
  if (blockIdx.x == 0) panel_invert(0);
  grid.sync();
  for (int k0 = 0; k0 < n; k0 += GJB) {
    const int kb = min(GJB, n - k0);
    if (status[1]) return;  // indefinite pivot: every CTA sees it after the barrier
    for (int e = tid; e < GJB * GJB; e += blockDim.x) sd[e / GJB][e % GJB] = work[e];
    __syncthreads();
    // ---- B: row panel P = D^-1 A[K,:] (columns outside K) and column panel C = A[:,K]
    const int64_t gt = (int64_t)blockIdx.x * blockDim.x + tid, gs = (int64_t)gridDim.x * blockDim.x;
    for (int64_t e = gt; e < (int64_t)kb * n; e += gs) {
      const int r = (int)(e / n), c = (int)(e % n);
      double v = 0.0;
      if (c < k0 || c >= k0 + kb) {
#pragma unroll 8
        for (int m = 0; m < kb; ++m) v += sd[r][m] * A[(int64_t)(k0 + m) * n + c];
      }
      P[(int64_t)r * n + c] = v;
      if constexpr (DFC) Pdf[(int64_t)r * n + c] = df_from(v);
    }
    for (int64_t e = gt; e < (int64_t)n * kb; e += gs) {
      const int i = (int)(e / kb), m = (int)(e % kb);
      const double v = (i < k0 || i >= k0 + kb) ? A[(int64_t)i * n + k0 + m] : 0.0;
      Cp[(int64_t)i * GJB + m] = v;
      if constexpr (DFC) Cdf[(int64_t)i * GJB + m] = df_from(v);
    }
    grid.sync();
    // ---- C: rank-kb update, GJB x GJB tiles of A.  With a next panel, CTA 0
    // takes only its diagonal tile and then inverts it; the others share the
    // rest.
    const int k1 = k0 + GJB, tn = k1 < n ? (k1 / GJB) * (nblk_tiles + 1) : -1;
    const bool ahead = tn >= 0 && gridDim.x > 1;
    const int t_first = ahead ? (blockIdx.x == 0 ? tn : (int)blockIdx.x - 1) : (int)blockIdx.x;
    const int t_step = ahead ? (blockIdx.x == 0 ? nblk_tiles * nblk_tiles : (int)gridDim.x - 1) : (int)gridDim.x;
    for (int t0 = t_first; t0 < nblk_tiles * nblk_tiles; t0 += t_step) {
      // the CTAs other than 0 skip the diagonal tile of the next panel
      const int t = (ahead && blockIdx.x != 0 && t0 >= tn) ? t0 + 1 : t0;
      if (t >= nblk_tiles * nblk_tiles) break;
      const int ti = (t / nblk_tiles) * GJB, tc = (t % nblk_tiles) * GJB;
      // a tile outside the panel's rows and columns: every element gets the update
      const bool band = (ti < k0 + kb && ti + GJB > k0) || (tc < k0 + kb && tc + GJB > k0);
      __syncthreads();
      for (int e = tid; e < GJB * GJB; e += blockDim.x) {
        const int r = e / GJB, c = e % GJB;
        const bool inc = ti + r < n && c < kb, inp = r < kb && tc + c < n;
        if (!DFC || band) {
          sc[r][c] = inc ? Cp[(int64_t)(ti + r) * GJB + c] : 0.0;
          sp[r][c] = inp ? P[(int64_t)r * n + tc + c] : 0.0;
        }
        if constexpr (DFC) {
          scd[r][c] = inc ? Cdf[(int64_t)(ti + r) * GJB + c] : df(0.f, 0.f);
          spd[r][c] = inp ? Pdf[(int64_t)r * n + tc + c] : df(0.f, 0.f);
        }
      }
      __syncthreads();
      if (!band && blockDim.x == 8 * GJB) {
        // four rows of one column per thread: four independent chains share
        // each panel value (per element the operations and order of the loop
        // below)
        const int c = tid % GJB, r0 = tid / GJB, col = tc + c;
        double* a[4];
        bool in[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const int i = ti + r0 + 8 * q;
          in[q] = i < n && col < n;
          a[q] = A + (int64_t)(in[q] ? i : 0) * n + (in[q] ? col : 0);
        }
        if constexpr (DFC) {
          df v[4];
#pragma unroll
          for (int q = 0; q < 4; ++q) v[q] = df_from(in[q] ? *a[q] : 0.0);
#pragma unroll 4
          for (int m = 0; m < kb; ++m) {
            const df pm = spd[m][c];
#pragma unroll
            for (int q = 0; q < 4; ++q) v[q] = v[q] - scd[r0 + 8 * q][m] * pm;
          }
#pragma unroll
          for (int q = 0; q < 4; ++q)
            if (in[q]) *a[q] = df_to(v[q]);
        } else {
          double v[4];
#pragma unroll
          for (int q = 0; q < 4; ++q) v[q] = in[q] ? *a[q] : 0.0;
#pragma unroll 4
          for (int m = 0; m < kb; ++m) {
            const double pm = sp[m][c];
#pragma unroll
            for (int q = 0; q < 4; ++q) v[q] -= sc[r0 + 8 * q][m] * pm;
          }
#pragma unroll
          for (int q = 0; q < 4; ++q)
            if (in[q]) *a[q] = v[q];
        }
        continue;
      }
      for (int e = tid; e < GJB * GJB; e += blockDim.x) {
        const int r = e / GJB, c = e % GJB;
        const int i = ti + r, col = tc + c;
        if (i >= n || col >= n) continue;
        const bool iK = i >= k0 && i < k0 + kb, cK = col >= k0 && col < k0 + kb;
        double& a = A[(int64_t)i * n + col];
        if (iK && cK) {
          a = sd[i - k0][col - k0];
        } else if (iK) {
          a = sp[i - k0][c];
        } else if (cK) {
          double v = 0.0;
          for (int m = 0; m < kb; ++m) v += sc[r][m] * sd[m][col - k0];
          a = -v;
        } else if constexpr (DFC) {
          df v = df_from(a);
          for (int m = 0; m < kb; ++m) v = v - scd[r][m] * spd[m][c];
          a = df_to(v);
        } else {
          double v = a;
          for (int m = 0; m < kb; ++m) v -= sc[r][m] * sp[m][c];
          a = v;
        }
      }
    }
    if (k1 < n && blockIdx.x == 0) {
      __syncthreads();  // the tile's updates are visible to the whole CTA
      panel_invert(k1);
    }
    grid.sync();
  }
}

__global__ void k_to_float(const double* __restrict__ a, float* __restrict__ b, int64_t n) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) b[i] = (float)a[i];
}

// u_soa = Ainv * f_soa over the dense DOF ordering 3v+c; one warp per row.
template <typename T>
__global__ void k_dense_gemv(int n, const T* __restrict__ Ainv, const T* __restrict__ f, T* __restrict__ u,
                             int64_t nv) {
  f += (int64_t)blockIdx.y * 3 * nv;  // right-hand side of the batch
  u += (int64_t)blockIdx.y * 3 * nv;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (warp >= n) return;
  T s = T(0);
  for (int j = lane; j < n; j += 32) s += Ainv[(int64_t)warp * n + j] * f[(j % 3) * nv + j / 3];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) u[(warp % 3) * nv + warp / 3] = s;
}

void launch_galerkin_first_impl(cudaStream_t s, const LevelDims& fd, const LevelDims& cd,
                                const double* rhop, const uint8_t* eactive_f, const uint8_t* vmask_f,
                                const double* Ttab64, const float* Ttab32, const double* Ke,
                                const int* fixed_list, int nfixed, double* kel, float* kel32) {
  const unsigned g = nblk(cd.ne, GAL_CE);
  const unsigned nf = (unsigned)nfixed;
  if (cd.factor == 4) {
    if (kel) {
      k_galerkin_gemm<double, 4><<<g, GAL_THREADS, 0, s>>>(fd, cd, rhop, vmask_f, Ttab64, kel);
      if (nf) k_galerkin_fixed<double, 4><<<nf, 576, 0, s>>>(fd, cd, rhop, eactive_f, vmask_f, Ke, fixed_list, kel);
    }
    if (kel32) {
      k_galerkin_gemm<float, 4><<<g, GAL_THREADS, 0, s>>>(fd, cd, rhop, vmask_f, Ttab32, kel32);
      if (nf) k_galerkin_fixed<float, 4><<<nf, 576, 0, s>>>(fd, cd, rhop, eactive_f, vmask_f, Ke, fixed_list, kel32);
    }
  } else {
    if (kel) {
      k_galerkin_gemm<double, 2><<<g, GAL_THREADS, 0, s>>>(fd, cd, rhop, vmask_f, Ttab64, kel);
      if (nf) k_galerkin_fixed<double, 2><<<nf, 576, 0, s>>>(fd, cd, rhop, eactive_f, vmask_f, Ke, fixed_list, kel);
    }
    if (kel32) {
      k_galerkin_gemm<float, 2><<<g, GAL_THREADS, 0, s>>>(fd, cd, rhop, vmask_f, Ttab32, kel32);
      if (nf) k_galerkin_fixed<float, 2><<<nf, 576, 0, s>>>(fd, cd, rhop, eactive_f, vmask_f, Ke, fixed_list, kel32);
    }
  }
}

template <typename T>
void launch_galerkin_dyadic_t(cudaStream_t s, const LevelDims& fd, const LevelDims& cd,
                              const uint8_t* eactive_f, const T* kel_f, T* kel_c) {
  k_galerkin_dyadic<T><<<(unsigned)cd.ne, 576, 0, s>>>(fd, cd, eactive_f, kel_f, kel_c);
}

template <typename T>
void launch_assemble_stencil_t(cudaStream_t s, const LevelDims& d, const uint8_t* eactive,
                               const uint8_t* vmask, const T* kel, T* st) {
  k_assemble_stencil<T><<<nblk(27 * d.nv, 256), 256, 0, s>>>(d, eactive, vmask, kel, st, st_idx<T>(d));
}

void launch_dense_from_stencil(cudaStream_t s, const LevelDims& d, const double* st, double* A) {
  const int64_t n = 3 * d.nv;
  cudaMemsetAsync(A, 0, sizeof(double) * n * n, s);
  k_dense_from_stencil<<<nblk(243 * d.nv, 256), 256, 0, s>>>(d, st, A);
  k_symmetrize<<<nblk(n * n, 256), 256, 0, s>>>((int)n, A);
}

int coarsest_invert(cudaStream_t s, int n, double* A, double* work, int* status_dev, bool df_update,
                    int max_per_sm) {
  int dev = 0, nsm = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  const int threads = 256;
  if (work) {  // blocked form: GJB-pivot panels, rank-GJB updates
    void* fn = df_update ? (void*)k_gj_blocked<true> : (void*)k_gj_blocked<false>;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, threads, 0);
    if (per_sm < 1) return (int)cudaErrorCooperativeLaunchTooLarge;
    const int tiles = ((n + GJB - 1) / GJB) * ((n + GJB - 1) / GJB);
    const int blocks = std::max(1, std::min(tiles, nsm * std::min(per_sm, std::max(1, max_per_sm))));
    cudaMemsetAsync(status_dev, 0, 2 * sizeof(int), s);
    void* args[] = {&n, &A, &work, &status_dev};
    return (int)cudaLaunchCooperativeKernel(fn, dim3(blocks), dim3(threads), args, 0, s);
  }
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_gauss_jordan, threads, 0);
  if (per_sm < 1) return (int)cudaErrorCooperativeLaunchTooLarge;
  int64_t want = ((int64_t)n * n + threads - 1) / threads;
  int blocks = (int)std::min<int64_t>(want, (int64_t)nsm * std::min(per_sm, 2));
  if (blocks < 1) blocks = 1;
  cudaMemsetAsync(status_dev, 0, 2 * sizeof(int), s);
  void* args[] = {&n, &A, &status_dev};
  return (int)cudaLaunchCooperativeKernel((void*)k_gauss_jordan, dim3(blocks), dim3(threads), args,
                                          0, s);
}

void launch_to_float(cudaStream_t s, const double* a, float* b, int64_t n) {
  k_to_float<<<nblk(n, 256), 256, 0, s>>>(a, b, n);
}

template <typename T>
void launch_dense_gemv(cudaStream_t s, int n, const T* Ainv, const T* f_soa, T* u_soa, int64_t nv, int nb) {
  k_dense_gemv<T><<<dim3(nblk((int64_t)n * 32, 256), nb), 256, 0, s>>>(n, Ainv, f_soa, u_soa, nv);
}

template void launch_stencil_apply<double>(cudaStream_t, const LevelDims&, const double*, const double*,
                                           const double*, double*, bool, int);
template void launch_stencil_apply<float>(cudaStream_t, const LevelDims&, const float*, const float*,
                                          const float*, float*, bool, int);
template void launch_stencil_gs<double>(cudaStream_t, const LevelDims&, const double*, const uint8_t*,
                                        double*, const double*, int, bool);
template void launch_stencil_gs<float>(cudaStream_t, const LevelDims&, const float*, const uint8_t*,
                                       float*, const float*, int, bool);
template void launch_stencil_diag_inv<double>(cudaStream_t, const LevelDims&, const double*,
                                              const uint8_t*, double*);
template void launch_stencil_diag_inv<float>(cudaStream_t, const LevelDims&, const float*,
                                             const uint8_t*, float*);
template void launch_restrict<double>(cudaStream_t, const LevelDims&, const LevelDims&, const double*,
                                      double*, int);
template void launch_restrict<float>(cudaStream_t, const LevelDims&, const LevelDims&, const float*,
                                     float*, int);
template void launch_prolong<double>(cudaStream_t, const LevelDims&, const LevelDims&, const double*,
                                     double*, const uint8_t*, int);
template void launch_prolong<float>(cudaStream_t, const LevelDims&, const LevelDims&, const float*,
                                    float*, const uint8_t*, int);
template void launch_galerkin_dyadic_t<double>(cudaStream_t, const LevelDims&, const LevelDims&,
                                               const uint8_t*, const double*, double*);
template void launch_galerkin_dyadic_t<float>(cudaStream_t, const LevelDims&, const LevelDims&,
                                              const uint8_t*, const float*, float*);
template void launch_assemble_stencil_t<double>(cudaStream_t, const LevelDims&, const uint8_t*,
                                                const uint8_t*, const double*, double*);
template void launch_assemble_stencil_t<float>(cudaStream_t, const LevelDims&, const uint8_t*,
                                               const uint8_t*, const float*, float*);
template void launch_dense_gemv<double>(cudaStream_t, int, const double*, const double*, double*,
                                        int64_t, int);
template void launch_dense_gemv<float>(cudaStream_t, int, const float*, const float*, float*, int64_t, int);

}  // namespace topo
