// Fine-level (level 0) matrix-free elasticity kernels on the dense voxel grid.
//
// The operator is y = K(rho) u with K = sum_e rho_e^p Ke, Ke the 24x24 template
// (element/templateMatrix.cpp:31-99).  Rows of fixed DOFs and inactive vertices
// are zero; vectors are kept zero on fixed DOFs, which removes the fixed columns
// exactly as the reference's WS kernels do (grid/Grid.cu:2277-2333, 1699-1842).
#include <mutex>
#include <type_traits>

#include "df.cuh"
#include "topo_internal.h"

namespace topo {

__constant__ double cKe64[576];
__constant__ float cKe32[576];

template <typename T>
__device__ __forceinline__ T ke(int i);
template <>
__device__ __forceinline__ double ke<double>(int i) { return cKe64[i]; }
template <>
__device__ __forceinline__ float ke<float>(int i) { return cKe32[i]; }

// Modal constants: lambda, mu, k0 = h/16, k1 = h/48, k2 = h/144 (see k_fine_modal).
__constant__ double cModal64[5];
__constant__ float cModal32[5];

template <typename T>
__device__ __forceinline__ T modal_c(int i);
template <>
__device__ __forceinline__ double modal_c<double>(int i) { return cModal64[i]; }
template <>
__device__ __forceinline__ float modal_c<float>(int i) { return cModal32[i]; }

// Modal constants split into hi + lo floats.
__constant__ float2 cModalDF[5];
template <>
__device__ __forceinline__ df modal_c<df>(int i) {
  const float2 c = cModalDF[i];
  return df(c.x, c.y);
}

void upload_template(const double* Ke576, double lam, double mu, double h) {
  float k32[576];
  for (int i = 0; i < 576; ++i) k32[i] = (float)Ke576[i];
  cudaMemcpyToSymbol(cKe64, Ke576, sizeof(double) * 576);
  cudaMemcpyToSymbol(cKe32, k32, sizeof(float) * 576);
  const double m64[5] = {lam, mu, h / 16.0, h / 48.0, h / 144.0};
  const float m32[5] = {(float)m64[0], (float)m64[1], (float)m64[2], (float)m64[3], (float)m64[4]};
  cudaMemcpyToSymbol(cModal64, m64, sizeof(m64));
  cudaMemcpyToSymbol(cModal32, m32, sizeof(m32));
  float2 mdf[5];
  for (int i = 0; i < 5; ++i) {
    mdf[i].x = (float)m64[i];
    mdf[i].y = (float)(m64[i] - (double)mdf[i].x);
  }
  cudaMemcpyToSymbol(cModalDF, mdf, sizeof(mdf));
}

// ---------------------------------------------------------------------------
// Sum-factorised ("modal") element operator.  The nodal values of one
// displacement component are Walsh-Hadamard transformed (c_S = sum_a H[a][S] u_a,
// H[a][S] = prod_{k in S} (2a_k - 1)), which splits the trilinear field into the
// orthogonal functions {1, X, Y, Z, XY, XZ, YZ, XYZ} of the reference cube.  The
// displacement gradient restricted to each orthogonal function gives one
// isotropic stress, and the element forces are the transposed transform of the
// modal forces.  The result equals rho^p Ke u_e (Ke integrated exactly, as the
// 2x2x2 Gauss rule of element/templateMatrix.cpp:31-99 does) with about 240
// flops per element instead of the 1152 of the dense 24x24 product.
// ---------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ void wht_fwd(T v[8]) {
#pragma unroll
  for (int hb = 1; hb < 8; hb <<= 1)
#pragma unroll
    for (int i = 0; i < 8; ++i)
      if (!(i & hb)) {
        const T a = v[i], b = v[i | hb];
        v[i] = a + b;
        v[i | hb] = b - a;
      }
}

template <typename T>
__device__ __forceinline__ void wht_bwd(T v[8]) {
#pragma unroll
  for (int hb = 1; hb < 8; hb <<= 1)
#pragma unroll
    for (int i = 0; i < 8; ++i)
      if (!(i & hb)) {
        const T a = v[i], b = v[i | hb];
        v[i] = a - b;
        v[i | hb] = a + b;
      }
}

// The transforms of the three displacement components.  FP32: components 0
// and 1 go through the packed two-lane FP32 instructions of sm_100 and later
// (__fadd2_rn, __ffma2_rn; per lane the same rounding as the scalar forms, so
// the results are identical), which halves their instruction count in an
// issue-bound kernel.
template <typename T>
__device__ __forceinline__ void wht3_fwd(T c[3][8]) {
  wht_fwd<T>(c[0]); wht_fwd<T>(c[1]); wht_fwd<T>(c[2]);
}
template <typename T>
__device__ __forceinline__ void wht3_bwd(T g[3][8]) {
  wht_bwd<T>(g[0]); wht_bwd<T>(g[1]); wht_bwd<T>(g[2]);
}
template <>
__device__ __forceinline__ void wht3_fwd<float>(float c[3][8]) {
  const float2 m1 = make_float2(-1.f, -1.f);
  float2 p[8];
#pragma unroll
  for (int a = 0; a < 8; ++a) p[a] = make_float2(c[0][a], c[1][a]);
#pragma unroll
  for (int hb = 1; hb < 8; hb <<= 1)
#pragma unroll
    for (int i = 0; i < 8; ++i)
      if (!(i & hb)) {
        const float2 a = p[i], b = p[i | hb];
        p[i] = __fadd2_rn(a, b);
        p[i | hb] = __ffma2_rn(a, m1, b);  // b - a
      }
#pragma unroll
  for (int a = 0; a < 8; ++a) { c[0][a] = p[a].x; c[1][a] = p[a].y; }
  wht_fwd<float>(c[2]);
}
template <>
__device__ __forceinline__ void wht3_bwd<float>(float g[3][8]) {
  const float2 m1 = make_float2(-1.f, -1.f);
  float2 p[8];
#pragma unroll
  for (int a = 0; a < 8; ++a) p[a] = make_float2(g[0][a], g[1][a]);
#pragma unroll
  for (int hb = 1; hb < 8; hb <<= 1)
#pragma unroll
    for (int i = 0; i < 8; ++i)
      if (!(i & hb)) {
        const float2 a = p[i], b = p[i | hb];
        p[i] = __ffma2_rn(b, m1, a);  // a - b
        p[i | hb] = __fadd2_rn(a, b);
      }
#pragma unroll
  for (int a = 0; a < 8; ++a) { g[0][a] = p[a].x; g[1][a] = p[a].y; }
  wht_bwd<float>(g[2]);
}

// Double-float: components 0 and 1 in the lanes of df2.
template <>
__device__ __forceinline__ void wht3_fwd<df>(df c[3][8]) {
  df2 p[8];
#pragma unroll
  for (int a = 0; a < 8; ++a)
    p[a] = {make_float2(c[0][a].hi, c[1][a].hi), make_float2(c[0][a].lo, c[1][a].lo)};
#pragma unroll
  for (int hb = 1; hb < 8; hb <<= 1)
#pragma unroll
    for (int i = 0; i < 8; ++i)
      if (!(i & hb)) {
        const df2 a = p[i], b = p[i | hb];
        p[i] = df2_add(a, b);
        p[i | hb] = df2_add(b, df2_neg(a));  // b - a
      }
#pragma unroll
  for (int a = 0; a < 8; ++a) {
    c[0][a] = df(p[a].hi.x, p[a].lo.x);
    c[1][a] = df(p[a].hi.y, p[a].lo.y);
  }
  wht_fwd<df>(c[2]);
}
template <>
__device__ __forceinline__ void wht3_bwd<df>(df g[3][8]) {
  df2 p[8];
#pragma unroll
  for (int a = 0; a < 8; ++a)
    p[a] = {make_float2(g[0][a].hi, g[1][a].hi), make_float2(g[0][a].lo, g[1][a].lo)};
#pragma unroll
  for (int hb = 1; hb < 8; hb <<= 1)
#pragma unroll
    for (int i = 0; i < 8; ++i)
      if (!(i & hb)) {
        const df2 a = p[i], b = p[i | hb];
        p[i] = df2_add(a, df2_neg(b));  // a - b
        p[i | hb] = df2_add(a, b);
      }
#pragma unroll
  for (int a = 0; a < 8; ++a) {
    g[0][a] = df(p[a].hi.x, p[a].lo.x);
    g[1][a] = df(p[a].hi.y, p[a].lo.y);
  }
  wht_bwd<df>(g[2]);
}

// In: c[3][8] nodal values per component.  Out: c[3][8] nodal forces of pe*Ke*u.
// EN: also *energy = u . (pe Ke u) = sum over modes of (transformed u) . (modal
// force), since the backward transform is the forward one's transpose.
template <typename T, bool EN = false>
__device__ __forceinline__ void modal_element(T c[3][8], T pe, T* energy = nullptr) {
  wht3_fwd<T>(c);
  const T L = modal_c<T>(0) * pe, M = modal_c<T>(1) * pe;
  const T k0 = modal_c<T>(2), k1 = modal_c<T>(3), k2 = modal_c<T>(4);
  T g[3][8];
#pragma unroll
  for (int i = 0; i < 3; ++i) g[i][0] = T(0);
  {  // constant part of the gradient
    const T tr = c[0][1] + c[1][2] + c[2][4];
    const T sxy = M * (c[0][2] + c[1][1]), sxz = M * (c[0][4] + c[2][1]), syz = M * (c[1][4] + c[2][2]);
    g[0][1] = k0 * (L * tr + T(2) * M * c[0][1]);
    g[1][2] = k0 * (L * tr + T(2) * M * c[1][2]);
    g[2][4] = k0 * (L * tr + T(2) * M * c[2][4]);
    g[0][2] = k0 * sxy; g[1][1] = k0 * sxy;
    g[0][4] = k0 * sxz; g[2][1] = k0 * sxz;
    g[1][4] = k0 * syz; g[2][2] = k0 * syz;
  }
  {  // X part (modes XY -> 3, XZ -> 5)
    const T tr = c[1][3] + c[2][5];
    const T syz = M * (c[1][5] + c[2][3]);
    g[0][3] = k1 * M * c[0][3];
    g[1][3] = k1 * (L * tr + T(2) * M * c[1][3]);
    g[2][3] = k1 * syz;
    g[0][5] = k1 * M * c[0][5];
    g[1][5] = k1 * syz;
    g[2][5] = k1 * (L * tr + T(2) * M * c[2][5]);
  }
  {  // Y part (XY -> 3, YZ -> 6)
    const T tr = c[0][3] + c[2][6];
    const T sxz = M * (c[0][6] + c[2][3]);
    g[0][3] += k1 * (L * tr + T(2) * M * c[0][3]);
    g[1][3] += k1 * M * c[1][3];
    g[2][3] += k1 * sxz;
    g[0][6] = k1 * sxz;
    g[1][6] = k1 * M * c[1][6];
    g[2][6] = k1 * (L * tr + T(2) * M * c[2][6]);
  }
  {  // Z part (XZ -> 5, YZ -> 6)
    const T tr = c[0][5] + c[1][6];
    const T sxy = M * (c[0][6] + c[1][5]);
    g[0][5] += k1 * (L * tr + T(2) * M * c[0][5]);
    g[1][5] += k1 * sxy;
    g[2][5] += k1 * M * c[2][5];
    g[0][6] += k1 * sxy;
    g[1][6] += k1 * (L * tr + T(2) * M * c[1][6]);
    g[2][6] += k1 * M * c[2][6];
  }
  {  // YZ, XZ, XY parts all act on the XYZ mode
    const T kk = k2 * (L + T(4) * M);
    g[0][7] = kk * c[0][7]; g[1][7] = kk * c[1][7]; g[2][7] = kk * c[2][7];
  }
  if constexpr (EN) {
    T e = T(0);
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int a = 1; a < 8; ++a) e += c[i][a] * g[i][a];  // g[i][0] = 0: rigid translation
    *energy = e;
  }
  wht3_bwd<T>(g);
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int a = 0; a < 8; ++a) c[i][a] = g[i][a];
}

// The vertex planes [zb0, zb1) of a fine-tile CTA narrowed to [z0, zend), the
// planes next to the tile's active elements (LevelDims::colz): a plane sees
// non-zero forces only from an active element layer directly below or above
// it.  The planes cut away get the operator's output for zero forces, which
// is what the full march would give there, without staging planes or
// computing (void) elements.  The kernels are instantiated twice: VOID for
// levels with void planes, and without the narrowing (and its code, which
// costs registers in the z march) for fully active boxes.
template <bool VOID>
__device__ __forceinline__ void fine_active_planes(const LevelDims& d, int zb0, int zb1, int& z0, int& zend) {
  z0 = zb0;
  zend = zb1;
  if (VOID) {
    const int2 cz = d.colz[blockIdx.x + gridDim.x * blockIdx.y];
    z0 = min(max(zb0, cz.x), zb1);
    zend = max(z0, min(zb1, cz.y + 2));
  }
}

// y = K(rho) u (or f - K u) on level 0.  A CTA owns a (TXE-1) x (TYE-1) column of
// vertices over TZ vertex planes and marches in z.  Vertex planes are staged in
// shared memory by asynchronous copies (cp.async, zero-filled outside the
// domain) two planes ahead of use in a 3-slot ring; per element layer the CTA
// computes its TXE x TYE elements (one per thread) into shared memory, and each
// owned vertex adds its four in-layer elements' bottom-node forces to the
// top-node forces carried in registers from the layer below.  Shared arrays
// hold one 4-vector per vertex / element node so each gather is one access.
// MODE 0: out = K u; 1: out = f - K u; 2: one Chebyshev step, r = f - K u,
// z = Dinv r, d = c_old d + c_new z (first: c_new z), out = u + d (out != u).
struct ChebArgs {
  const void* dinv;  // block inverse: [9][nv] (FP64), packed symmetric (FP32, dinv_sym_apply)
  void* dvec;        // [3][nv]
  const double* coef;  // (c_old, c_new) of the step, in device memory
  int first;
  double* dotp;      // per-CTA partial sums: MODE 0 u.out, FP32 MODE 3 f.out (null: none)
  int d_is_u;        // MODE 2, FP32: d equals u on entry (the step after a zero start); dvec is not read
  double* dot;       // with ctr: the last CTA sums the partials into *dot
  unsigned* ctr;     // zeroed ticket counter (reset by the last CTA)
};

// Sum of v over the CTA (valid in thread 0); every thread must call it.
__device__ __forceinline__ double modal_block_sum(double v);

// After thread 0 of every CTA published its partial: the CTA that takes the last
// ticket sums the n partials in index order (independent of which CTA is last)
// into *out and resets the counter.  Every thread must call it.
__device__ __forceinline__ void modal_finish_sum(const double* partial, int64_t n, double* out, unsigned* ctr) {
  __shared__ bool last;
  if (threadIdx.x == 0) {  // thread 0 wrote the block's partial: fence, then take a ticket
    __threadfence();
    last = atomicAdd(ctr, 1u) == (unsigned)(n - 1);
    if (last) __threadfence();
  }
  __syncthreads();
  if (!last) return;
  double s = 0.0;
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) s += __ldcg(partial + i);
  s = modal_block_sum(s);
  if (threadIdx.x == 0) {
    *out = s;
    *ctr = 0u;
  }
}

__device__ __forceinline__ double modal_block_sum(double v) {
  __shared__ double ws[32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  if (lane == 0) ws[w] = v;
  __syncthreads();
  double r = 0.0;
  if (w == 0) {
    r = lane < nw ? ws[lane] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) r += __shfl_down_sync(0xffffffffu, r, o);
  }
  return r;
}

template <typename T>
struct alignas(4 * sizeof(T)) Vec4 {
  T x, y, z, w;
};

__device__ __forceinline__ void cp_async_4(void* smem, const void* gmem, bool valid) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(s), "l"(gmem), "r"(valid ? 4 : 0));
}
__device__ __forceinline__ void cp_async_8(void* smem, const void* gmem, bool valid) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(s), "l"(gmem), "r"(valid ? 8 : 0));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
__device__ __forceinline__ void cp_async_wait1() { asm volatile("cp.async.wait_group 1;\n" ::: "memory"); }

template <typename T>
__device__ __forceinline__ void cp_async_elem(T* smem, const T* gmem, bool valid) {
  if (sizeof(T) == 4) cp_async_4(smem, gmem, valid);
  else cp_async_8(smem, gmem, valid);
}

template <typename T, int TXE, int TYE>
struct ModalSmem {
  static constexpr int NT = TXE * TYE, PX = TXE + 1, PY = TYE + 1, NP = PX * PY;
  Vec4<T> plane[3][NP];  // vertex planes (u0, u1, u2, -) in a 3-slot ring
  Vec4<T> fe[8][NT];     // nodal forces of the layer's elements, per local node
};

// z = D^-1 r with level 0's FP32 block inverse in its packed symmetric layout:
// float4 (d00, d01, d02, d11) per vertex, then float2 (d12, d22) per vertex
// (24 bytes and two loads per vertex instead of nine; the same products in the
// same order as the [9][nv] form, since the stored block is symmetric).
template <typename I>
__device__ __forceinline__ void dinv_sym_apply(const float* __restrict__ dinv, I nv, I v, const float r[3],
                                               float z[3]) {
  const float4 a = reinterpret_cast<const float4*>(dinv)[v];
  const float2 b = reinterpret_cast<const float2*>(dinv + 4 * nv)[v];
  z[0] = a.x * r[0] + a.y * r[1] + a.z * r[2];
  z[1] = a.y * r[0] + a.w * r[1] + b.x * r[2];
  z[2] = a.z * r[0] + b.x * r[1] + b.y * r[2];
}

// Build-time choices for the FP32 kernel, measured on GB300 (half-MBB
// 256x128x128, Chebyshev step per launch):
//  - the Chebyshev step reads the stored FP32 block-Jacobi inverse (36 bytes per
//    vertex); rebuilding the diagonal blocks from rho^p and solving them costs
//    about 150 instructions per vertex, and the kernel is issue-bound, so
//    reading wins: 143 us against 154 us (two-barrier form).
//  - resident threads per SM (launch bounds): 1024 for all three modes (64
//    registers per thread, no spills).
//  - TOPO_MODAL32_TYE 8: element rows (warps) of a 32-wide CTA tile.  16 rows
//    halve the halo overhead but ran slower (162 us, two-barrier form).
// FP64 variants ask for 512 resident threads (two 256-thread CTAs, at most
// 128 registers per thread).
#ifndef TOPO_FINE32_THREADS_PER_SM
#define TOPO_FINE32_THREADS_PER_SM 1024
#endif
#ifndef TOPO_FINE32_CHEB_THREADS_PER_SM
#define TOPO_FINE32_CHEB_THREADS_PER_SM 1024
#endif
#ifndef TOPO_MODAL32_TYE
#define TOPO_MODAL32_TYE 8
#endif

constexpr int modal_min_ctas(int threads, int per_sm) { return per_sm / threads > 0 ? per_sm / threads : 1; }

template <typename T, int TXE, int TYE, int MODE, bool VOID>
__global__ void __launch_bounds__(TXE* TYE, sizeof(T) == 4 ? modal_min_ctas(TXE * TYE, MODE == 2
                                                                                          ? TOPO_FINE32_CHEB_THREADS_PER_SM
                                                                                          : TOPO_FINE32_THREADS_PER_SM)
                                                           : modal_min_ctas(TXE * TYE, 512))
    k_fine_modal(LevelDims d, const T* __restrict__ rhop,
                                                         const uint8_t* __restrict__ vmask,
                                                         const T* __restrict__ u, const T* __restrict__ f,
                                                         T* __restrict__ out, int TZ, ChebArgs ch) {
  using S = ModalSmem<T, TXE, TYE>;
  constexpr int NT = S::NT, PX = S::PX, NP = S::NP;
  extern __shared__ __align__(32) unsigned char modal_smem[];
  S& sm = *reinterpret_cast<S*>(modal_smem);
  const int t = threadIdx.x, i = t % TXE, j = t / TXE;
  // blockIdx.z enumerates (right-hand side, z block): vectors of a batch of
  // right-hand sides are stored one after another, the operator is shared
  const int zblk = fine_zblocks(d.vz, TZ);
  const int rhs = blockIdx.z / zblk;
  const int kz = blockIdx.z - rhs * zblk;
  const int x0 = blockIdx.x * (TXE - 1), y0 = blockIdx.y * (TYE - 1), zb0 = kz * TZ;
  const int64_t nv = d.nv;
  u += (int64_t)rhs * 3 * nv;
  if (f) f += (int64_t)rhs * 3 * nv;
  out += (int64_t)rhs * 3 * nv;
  const int gx = x0 + i, gy = y0 + j;  // owned vertex (x, y) and element (x-1, y-1)
  const bool own = (i < TXE - 1) && (j < TYE - 1) && gx < d.vx && gy < d.vy;
  const int zb1 = fine_zblock_end(d.vz, TZ, kz);
  int z0, zend;  // the planes marched: [zb0, zb1) less the void
  fine_active_planes<VOID>(d, zb0, zb1, z0, zend);
  T acc0 = T(0), acc1 = T(0), acc2 = T(0);
  T dsum = T(0);  // MODE 0 with ch.dotp: this thread's share of u.out
  // This thread's plane slots k = t + s NT and their in-plane vertex offsets
  // (-1 outside the domain), fixed for the whole z march.
  constexpr int KS = (NP + NT - 1) / NT;
  int pxy[KS];
#pragma unroll
  for (int s = 0; s < KS; ++s) {
    const int k = t + s * NT, px = k % PX, py = k / PX;
    const int vx = x0 - 1 + px, vy = y0 - 1 + py;
    pxy[s] = (k < NP && vx >= 0 && vy >= 0 && vx < d.vx && vy < d.vy) ? vx + d.vx * vy : -1;
  }
  const int64_t plane_n = (int64_t)d.vx * d.vy;
  // asynchronous copy of vertex plane z into its ring slot (z + 3) % 3
  auto prefetch = [&](int z) {
    if (z <= zend) {
      Vec4<T>* dst = sm.plane[(z + 3) % 3];
      const bool zok = z >= 0 && z < d.vz;
      const int64_t zoff = (int64_t)z * plane_n;
#pragma unroll
      for (int s = 0; s < KS; ++s) {
        const int k = t + s * NT;
        if (k < NP) {
          const bool ok = zok && pxy[s] >= 0;
          const int64_t v = ok ? zoff + pxy[s] : 0;
          cp_async_elem<T>(&dst[k].x, u + v, ok);
          cp_async_elem<T>(&dst[k].y, u + nv + v, ok);
          cp_async_elem<T>(&dst[k].z, u + 2 * nv + v, ok);
        }
      }
    }
    cp_async_commit();
  };
  // Per-layer global operands (the element's rho^p; the owned vertex's mask,
  // load and Chebyshev direction) are read one layer ahead into registers, so
  // their latency overlaps the current layer's work instead of stalling it.
  const int pex = gx - 1, pey = gy - 1;
  const bool pe_xy = pex >= 0 && pey >= 0 && pex < d.ex && pey < d.ey;
  auto load_pe = [&](int ez) -> T {
    return (pe_xy && ez >= 0 && ez < d.ez) ? rhop[pex + (int64_t)d.ex * (pey + (int64_t)d.ey * ez)] : T(0);
  };
  const T* __restrict__ dvin =
      (MODE == 2 && !ch.first) ? static_cast<const T*>(ch.dvec) + (int64_t)rhs * 3 * nv : nullptr;
  uint8_t vm_n = 0;
  T f_n[3] = {T(0), T(0), T(0)}, dv_n[3] = {T(0), T(0), T(0)};
  auto load_vertex = [&](int z) {
    if (!own || z < z0 || z >= zend) return;
    const int64_t v = gx + (int64_t)d.vx * (gy + (int64_t)d.vy * z);
    vm_n = vmask[v];
    if (MODE >= 1) {
#pragma unroll
      for (int c = 0; c < 3; ++c) f_n[c] = f[c * nv + v];
    }
    if (MODE == 2 && dvin) {
#pragma unroll
      for (int c = 0; c < 3; ++c) dv_n[c] = dvin[c * nv + v];
    }
  };
  // owned vertices of void planes [pa, pb): the output for zero forces
  auto void_planes = [&](int pa, int pb) {
    if (!own) return;
    for (int p = pa; p < pb; ++p) {
      const int64_t v = gx + (int64_t)d.vx * (gy + (int64_t)d.vy * p);
      const uint8_t m = vmask[v];
      if (MODE < 2) {
#pragma unroll
        for (int c = 0; c < 3; ++c) out[c * nv + v] = (MODE == 1 && ((m >> c) & 1)) ? f[c * nv + v] : T(0);
      } else {
        const T* __restrict__ dinv = static_cast<const T*>(ch.dinv);
        T* __restrict__ dv = static_cast<T*>(ch.dvec) + (int64_t)rhs * 3 * nv;
        T r[3], zc[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) r[c] = ((m >> c) & 1) ? f[c * nv + v] : T(0);
#pragma unroll
        for (int c = 0; c < 3; ++c)
          zc[c] = dinv[(3 * c) * nv + v] * r[0] + dinv[(3 * c + 1) * nv + v] * r[1] + dinv[(3 * c + 2) * nv + v] * r[2];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          const T c_old = T(__ldg(ch.coef)), c_new = T(__ldg(ch.coef + 1));
          const T dn = ch.first ? c_new * zc[c] : c_old * (dvin ? dvin[c * nv + v] : T(0)) + c_new * zc[c];
          dv[c * nv + v] = dn;
          out[c * nv + v] = u[c * nv + v] + dn;
        }
      }
    }
  };
  if (VOID) {
    void_planes(zb0, z0);
    void_planes(zend, zb1);
  }
  T pe_n = load_pe(z0 - 1);
  if (z0 < zend) {
    prefetch(z0 - 1);
    prefetch(z0);
    for (int ez = z0 - 1; ez < zend; ++ez) {
      prefetch(ez + 2);
      const T pe = pe_n;
      const uint8_t vm_c = vm_n;
      T f_c[3], dv_c[3];
#pragma unroll
      for (int c = 0; c < 3; ++c) { f_c[c] = f_n[c]; dv_c[c] = dv_n[c]; }
      if (ez + 1 < zend) pe_n = load_pe(ez + 1);
      load_vertex(ez + 1);
      cp_async_wait1();
      __syncthreads();
      // the owned vertex's own value at plane ez (Chebyshev update); read here,
      // before the slot can be refilled by the next layer's prefetch
      Vec4<T> uo{T(0), T(0), T(0), T(0)};
      if (MODE == 2 || (MODE == 0 && ch.dotp)) uo = sm.plane[(ez + 3) % 3][(i + 1) + PX * (j + 1)];
      {
        if (pe != T(0)) {
          T c[3][8];
#pragma unroll
          for (int a = 0; a < 8; ++a) {
            const int k = (i + (a & 1)) + PX * (j + ((a >> 1) & 1));
            const Vec4<T> p = sm.plane[(ez + (a >> 2) + 3) % 3][k];
            c[0][a] = p.x; c[1][a] = p.y; c[2][a] = p.z;
          }
          modal_element<T>(c, pe);
#pragma unroll
          for (int a = 0; a < 8; ++a) sm.fe[a][t] = Vec4<T>{c[0][a], c[1][a], c[2][a], T(0)};
        } else {
#pragma unroll
          for (int a = 0; a < 8; ++a) sm.fe[a][t] = Vec4<T>{T(0), T(0), T(0), T(0)};
        }
      }
      __syncthreads();
      if (own) {
        T b0 = acc0, b1 = acc1, b2 = acc2, t0 = T(0), t1 = T(0), t2 = T(0);
#pragma unroll
        for (int w = 0; w < 4; ++w) {
          const int wx = w & 1, wy = w >> 1;
          const int te = (i + wx) + TXE * (j + wy);
          const int a = (1 - wx) + 2 * (1 - wy);  // bottom node of that element
          const Vec4<T> bo = sm.fe[a][te], to = sm.fe[a + 4][te];
          b0 += bo.x; b1 += bo.y; b2 += bo.z;
          t0 += to.x; t1 += to.y; t2 += to.z;
        }
        if (ez >= z0) {
          const int64_t v = gx + (int64_t)d.vx * (gy + (int64_t)d.vy * ez);
          const uint8_t m = vm_c;
          const T y[3] = {b0, b1, b2};
          if (MODE < 2) {
            const T uv[3] = {uo.x, uo.y, uo.z};
#pragma unroll
            for (int c = 0; c < 3; ++c) {
              const bool fr = (m >> c) & 1;
              const int64_t idx = c * nv + v;
              const T o = MODE == 1 ? (fr ? f_c[c] - y[c] : T(0)) : (fr ? y[c] : T(0));
              out[idx] = o;
              if (MODE == 0) dsum += uv[c] * o;
            }
          } else {
            const T* __restrict__ dinv = static_cast<const T*>(ch.dinv);
            T* __restrict__ dv = static_cast<T*>(ch.dvec) + (int64_t)rhs * 3 * nv;
            T r[3];
#pragma unroll
            for (int c = 0; c < 3; ++c) r[c] = ((m >> c) & 1) ? f_c[c] - y[c] : T(0);
            const T uv[3] = {uo.x, uo.y, uo.z};
            T zc[3];
#pragma unroll
            for (int c = 0; c < 3; ++c)
              zc[c] = dinv[(3 * c) * nv + v] * r[0] + dinv[(3 * c + 1) * nv + v] * r[1] + dinv[(3 * c + 2) * nv + v] * r[2];
#pragma unroll
            for (int c = 0; c < 3; ++c) {
              const T c_old = T(__ldg(ch.coef)), c_new = T(__ldg(ch.coef + 1));
              const T dn = ch.first ? c_new * zc[c] : c_old * dv_c[c] + c_new * zc[c];
              dv[c * nv + v] = dn;
              out[c * nv + v] = uv[c] + dn;
            }
          }
        }
        acc0 = t0; acc1 = t1; acc2 = t2;
      }
    }
  }
  // drain the (empty) trailing copy groups before the CTA exits
  asm volatile("cp.async.wait_all;\n" ::: "memory");
  if (MODE == 0 && ch.dotp) {
    const double bs = modal_block_sum((double)dsum);
    if (t == 0) ch.dotp[blockIdx.x + (int64_t)gridDim.x * (blockIdx.y + (int64_t)gridDim.y * blockIdx.z)] = bs;
  }
}

// ---------------------------------------------------------------------------
// FP32 form with one barrier per element layer.  A CTA is TYE warps; lane i of
// warp j computes element (i, j) of the layer and owns vertex (i, j), the
// element's (+x, +y) corner.  The element's nodal forces are combined along x
// with a warp shuffle (vertex column i takes the x = 1 nodes of element i and
// the x = 0 nodes of element i + 1); the y = 1 half stays in the lane's
// registers and the y = 0 half (6 floats) goes through a double-buffered
// shared exchange to warp j - 1.  The owned vertex's sum for plane ez is then
// formed in the next layer's step, after its single barrier: its own y = 1
// part, row j + 1's exchanged y = 0 part, and the top-node part carried from
// the layer below.  Vertex planes sit in a 4-slot ring and only the element
// phase reads them (the owned vertex's own value is taken into registers
// there), so the copy issued at the top of a step never lands in a plane that
// a warp still in the previous step may read.
// Against the 2-barrier form: a quarter of the shared-memory traffic per
// element, half the barriers.
// ---------------------------------------------------------------------------
// Owned vertex (gx, gy) of the FP32 kernel over void planes [pa, pb): the
// output of MODE for zero forces (kept out of line: inlined, its live values
// pushed the z march past its register budget).
template <int MODE>
__device__ __noinline__ void fine32_void_planes(const LevelDims& d, const uint8_t* __restrict__ vmask,
                                                const float* __restrict__ u, const float* __restrict__ f,
                                                float* __restrict__ out, const ChebArgs& ch, int rhs, int gx, int gy,
                                                int pa, int pb, const float* coef, float& dsum) {
  constexpr bool CHEB = MODE >= 2, DOTS = MODE == 3;
  const int64_t nv = d.nv;
  const float* __restrict__ dvin =
      (CHEB && !ch.first && !ch.d_is_u) ? static_cast<const float*>(ch.dvec) + (int64_t)rhs * 3 * nv : nullptr;
  for (int p = pa; p < pb; ++p) {
    const int64_t v = gx + (int64_t)d.vx * (gy + (int64_t)d.vy * p);
    const uint8_t m = vmask[v];
    if (!CHEB) {
#pragma unroll
      for (int c = 0; c < 3; ++c) out[c * nv + v] = (MODE == 1 && ((m >> c) & 1)) ? f[c * nv + v] : 0.f;
    } else {
      float* __restrict__ dv = static_cast<float*>(ch.dvec) + (int64_t)rhs * 3 * nv;
      float r[3], zc[3], uv[3];
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        r[c] = ((m >> c) & 1) ? f[c * nv + v] : 0.f;
        uv[c] = u[c * nv + v];
      }
      dinv_sym_apply(static_cast<const float*>(ch.dinv), nv, v, r, zc);
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const float dold = ch.d_is_u ? uv[c] : (dvin ? dvin[c * nv + v] : 0.f);
        const float dn = ch.first ? coef[1] * zc[c] : coef[0] * dold + coef[1] * zc[c];
        dv[c * nv + v] = dn;
        const float o = uv[c] + dn;
        out[c * nv + v] = o;
        if (DOTS) dsum += f[c * nv + v] * o;
      }
    }
  }
}

template <int TYE>
struct Modal32Smem {
  static constexpr int TXE = 32, NT = TXE * TYE, PX = TXE + 1, PY = TYE + 1, NP = PX * PY;
  float4 plane[4][NP];  // vertex planes (u0, u1, u2, -) in a 4-slot ring
  float4 xa[2][NT];     // exchanged y = 0 forces: (z = 0: c0, c1, c2; z = 1: c0)
  float2 xb[2][NT];     //                         (z = 1: c1, c2)
  float coef[2];        // Chebyshev (c_old, c_new), read after each plane's barrier
};

template <int TYE, int MODE, bool I32, bool VOID>
__global__ void __launch_bounds__(32 * TYE, modal_min_ctas(32 * TYE, MODE >= 2 ? TOPO_FINE32_CHEB_THREADS_PER_SM
                                                                               : TOPO_FINE32_THREADS_PER_SM))
    k_fine_modal32(LevelDims d, const float* __restrict__ rhop, const uint8_t* __restrict__ vmask,
                   const float* __restrict__ u, const float* __restrict__ f, float* __restrict__ out, int TZ,
                   ChebArgs ch) {
  // MODE 3: the Chebyshev step of MODE 2 that also sums f.out.  I32: vertex and
  // element offsets within one right-hand side in 32-bit arithmetic (3 nv and
  // ne below 2^31), one instruction per address instead of two.
  constexpr bool CHEB = MODE >= 2, DOTS = MODE == 3;
  using I = typename std::conditional<I32, int, int64_t>::type;
  using S = Modal32Smem<TYE>;
  constexpr int TXE = 32, NT = S::NT, PX = S::PX, NP = S::NP;
  extern __shared__ __align__(16) unsigned char m32_smem[];
  S& sm = *reinterpret_cast<S*>(m32_smem);
  const int t = threadIdx.x, i = t & 31, j = t >> 5;
  if (CHEB && t == 0) {
    sm.coef[0] = float(ch.coef[0]);
    sm.coef[1] = float(ch.coef[1]);
  }
  const int zblk = fine_zblocks(d.vz, TZ);
  const int rhs = blockIdx.z / zblk;
  const int kz = blockIdx.z - rhs * zblk;
  const int x0 = blockIdx.x * (TXE - 1), y0 = blockIdx.y * (TYE - 1), zb0 = kz * TZ;
  const int zb1 = zb0 + TZ + (kz + 1 == zblk ? d.vz - zblk * TZ : 0);  // fine_zblock_end
  const I nv = (I)d.nv;
  u += (int64_t)rhs * 3 * d.nv;
  if (f) f += (int64_t)rhs * 3 * d.nv;
  out += (int64_t)rhs * 3 * d.nv;
  const int gx = x0 + i, gy = y0 + j;
  const bool own = (i < TXE - 1) && (j < TYE - 1) && gx < d.vx && gy < d.vy;
  int z0, zend;  // the planes marched: [zb0, zb1) less the void
  fine_active_planes<VOID>(d, zb0, zb1, z0, zend);
  constexpr int KS = (NP + NT - 1) / NT;
  int pxy[KS];
#pragma unroll
  for (int s = 0; s < KS; ++s) {
    const int k = t + s * NT, px = k % PX, py = k / PX;
    const int vx = x0 - 1 + px, vy = y0 - 1 + py;
    pxy[s] = (k < NP && vx >= 0 && vy >= 0 && vx < d.vx && vy < d.vy) ? vx + d.vx * vy : -1;
  }
  const I plane_n = (I)d.vx * d.vy;
  auto prefetch = [&](int z) {
    if (z <= zend) {
      float4* dst = sm.plane[(z + 4) & 3];
      const bool zok = z >= 0 && z < d.vz;
      const I zoff = (I)z * plane_n;
#pragma unroll
      for (int s = 0; s < KS; ++s) {
        const int k = t + s * NT;
        if (k < NP) {
          const bool ok = zok && pxy[s] >= 0;
          const I v = ok ? zoff + pxy[s] : 0;
          cp_async_4(&dst[k].x, u + v, ok);
          cp_async_4(&dst[k].y, u + nv + v, ok);
          cp_async_4(&dst[k].z, u + 2 * nv + v, ok);
        }
      }
    }
    cp_async_commit();
  };
  const int pex = gx - 1, pey = gy - 1;
  const bool pe_xy = pex >= 0 && pey >= 0 && pex < d.ex && pey < d.ey;
  auto load_pe = [&](int ez) -> float {
    return (pe_xy && ez >= 0 && ez < d.ez) ? rhop[pex + (I)d.ex * (pey + (I)d.ey * ez)] : 0.f;
  };
  const float* __restrict__ dvin =
      (CHEB && !ch.first && !ch.d_is_u) ? static_cast<const float*>(ch.dvec) + (int64_t)rhs * 3 * d.nv : nullptr;
  // operands of the owned vertex at plane z, read in step z and used in step z + 1
  uint8_t vm_n = 0;
  float f_n[3] = {0.f, 0.f, 0.f}, dv_n[3] = {0.f, 0.f, 0.f};
  auto load_vertex = [&](int z) {
    if (!own || z < z0 || z >= zend) return;
    const I v = gx + (I)d.vx * (gy + (I)d.vy * z);
    vm_n = vmask[v];
    if (MODE >= 1) {
#pragma unroll
      for (int c = 0; c < 3; ++c) f_n[c] = f[c * nv + v];
    }
    if (CHEB && dvin) {
#pragma unroll
      for (int c = 0; c < 3; ++c) dv_n[c] = dvin[c * nv + v];
    }
  };
  float own1[2][3] = {{0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}};  // own y = 1 forces of the last layer, z = 0 / 1
  float top[3] = {0.f, 0.f, 0.f};                          // z = 1 forces of the layer below the last
  float uo[3] = {0.f, 0.f, 0.f};                           // owned vertex's own value at the last layer's plane
  float dsum = 0.f;
  if (VOID && (zb0 < z0 || zend < zb1)) {  // void planes: the step's output for zero forces
    if (CHEB) __syncthreads();      // the step coefficients in shared memory
    if (own) {
      fine32_void_planes<MODE>(d, vmask, u, f, out, ch, rhs, gx, gy, zb0, z0, sm.coef, dsum);
      fine32_void_planes<MODE>(d, vmask, u, f, out, ch, rhs, gx, gy, zend, zb1, sm.coef, dsum);
    }
  }
  float pe_n = load_pe(z0 - 1);
  if (z0 < zend) {
    prefetch(z0 - 1);
    prefetch(z0);
    // step st: finish vertex plane st - 1 (layers st - 2, st - 1), then compute element layer st
    for (int st = z0 - 1; st <= zend; ++st) {
      prefetch(st + 2);
      const float pe = pe_n;
      const uint8_t vm_c = vm_n;
      float f_c[3], dv_c[3];
#pragma unroll
      for (int c = 0; c < 3; ++c) { f_c[c] = f_n[c]; dv_c[c] = dv_n[c]; }
      if (st + 1 < zend) pe_n = load_pe(st + 1);
      load_vertex(st);
      cp_async_wait1();
      __syncthreads();
      // ---- vertex plane p = st - 1
      if (st >= z0) {
        const int p = st - 1, xs = (st - 1) & 1;
        float y[3];
        if (own) {
          const float4 ra = sm.xa[xs][t + TXE];
          const float2 rb = sm.xb[xs][t + TXE];
          const float r0[3] = {ra.x, ra.y, ra.z}, r1[3] = {ra.w, rb.x, rb.y};
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            y[c] = top[c] + (own1[0][c] + r0[c]);
            top[c] = own1[1][c] + r1[c];
          }
          if (p >= z0) {
            const I v = gx + (I)d.vx * (gy + (I)d.vy * p);
            const uint8_t m = vm_c;
            const float uv[3] = {uo[0], uo[1], uo[2]};
            if (!CHEB) {
#pragma unroll
              for (int c = 0; c < 3; ++c) {
                const bool fr = (m >> c) & 1;
                const float o = MODE == 1 ? (fr ? f_c[c] - y[c] : 0.f) : (fr ? y[c] : 0.f);
                out[c * nv + v] = o;
                if (MODE == 0) dsum += uv[c] * o;
              }
            } else {
              float* __restrict__ dv = static_cast<float*>(ch.dvec) + (int64_t)rhs * 3 * d.nv;
              float r[3], zc[3];
#pragma unroll
              for (int c = 0; c < 3; ++c) r[c] = ((m >> c) & 1) ? f_c[c] - y[c] : 0.f;
              dinv_sym_apply(static_cast<const float*>(ch.dinv), nv, v, r, zc);
#pragma unroll
              for (int c = 0; c < 3; ++c) {
                const float dold = ch.d_is_u ? uv[c] : dv_c[c];
                const float c_old = sm.coef[0], c_new = sm.coef[1];
                const float dn = ch.first ? c_new * zc[c] : c_old * dold + c_new * zc[c];
                dv[c * nv + v] = dn;
                const float o = uv[c] + dn;
                out[c * nv + v] = o;
                if (DOTS) dsum += f_c[c] * o;
              }
            }
          }
        }
      }
      // ---- element layer st
      if (st < zend) {
        if (CHEB || (MODE == 0 && ch.dotp)) {
          const float4 q = sm.plane[(st + 4) & 3][(i + 1) + PX * (j + 1)];
          uo[0] = q.x; uo[1] = q.y; uo[2] = q.z;
        }
        float c[3][8];
        if (pe != 0.f) {
#pragma unroll
          for (int a = 0; a < 8; ++a) {
            const int k = (i + (a & 1)) + PX * (j + ((a >> 1) & 1));
            const float4 q = sm.plane[(st + (a >> 2) + 4) & 3][k];
            c[0][a] = q.x; c[1][a] = q.y; c[2][a] = q.z;
          }
          modal_element<float>(c, pe);
        } else {
#pragma unroll
          for (int a = 0; a < 8; ++a) c[0][a] = c[1][a] = c[2][a] = 0.f;
        }
        // x combine: vertex column i takes the x = 1 nodes of element i and the
        // x = 0 nodes of element i + 1 (lane 31's column is not owned)
        float xc[2][2][3];  // [y bit][z bit][component]
#pragma unroll
        for (int yb = 0; yb < 2; ++yb)
#pragma unroll
          for (int zb = 0; zb < 2; ++zb)
#pragma unroll
            for (int cc = 0; cc < 3; ++cc)
              xc[yb][zb][cc] = c[cc][1 + 2 * yb + 4 * zb] +
                               __shfl_down_sync(0xffffffffu, c[cc][2 * yb + 4 * zb], 1);
#pragma unroll
        for (int zb = 0; zb < 2; ++zb)
#pragma unroll
          for (int cc = 0; cc < 3; ++cc) own1[zb][cc] = xc[1][zb][cc];
        sm.xa[st & 1][t] = make_float4(xc[0][0][0], xc[0][0][1], xc[0][0][2], xc[0][1][0]);
        sm.xb[st & 1][t] = make_float2(xc[0][1][1], xc[0][1][2]);
      }
    }
  }
  asm volatile("cp.async.wait_all;\n" ::: "memory");
  const int64_t cta = blockIdx.x + (int64_t)gridDim.x * (blockIdx.y + (int64_t)gridDim.y * blockIdx.z);
  if ((MODE == 0 || DOTS) && ch.dotp) {
    const double bs = modal_block_sum((double)dsum);
    if (t == 0) ch.dotp[cta] = bs;
    if (ch.ctr) modal_finish_sum(ch.dotp, (int64_t)gridDim.x * gridDim.y * gridDim.z, ch.dot, ch.ctr);
  }
}

// ---------------------------------------------------------------------------
// The FP32 z march with the element products on the tensor cores (tcgen05,
// kind::tf32, fp32 accumulators in tensor memory), in three-term TF32
// arithmetic: u = u_hi + u_lo and Ke = K_hi + K_lo with u_hi, K_hi exact in
// TF32, and u.Ke ~ u_hi K_hi + u_hi K_lo + u_lo K_hi (the dropped u_lo K_lo is
// 2^-22 of the product), which keeps the FP32 kernel's accuracy.
//
// Per element layer the products are one GEMM per half tile: M = 128 elements
// (32 along x by 4 rows of y), N = 32 (8 nodes x (3 force components + 1
// zero)), K = 32 (8 nodes x (3 displacement components + 1 zero)), issued as
// 4 K steps of 8, one per (dy, dz) node pair: the A operand of K step (dy,
// dz) is the staged vertex plane z + dz, rows y + dy, read straight from
// shared memory (float4 per vertex, 32 vertices per row: core matrices of 8
// consecutive x, 128 bytes apart; the second 4 K values are the x + 1 vertex,
// 16 bytes on -- the leading-dimension offset).  Lane i of warp j reads the
// 32 columns of its element (i, j) from tensor-memory lane i + 32 (j % 4), so
// after the read-back the thread holds exactly what the SIMT kernel's
// modal_element leaves (times rho^p), and the rest of the step (x combine,
// y exchange, vertex update) is the SIMT kernel's.
//
// A 32-vertex plane row has no halo column: lane 31's element reads the next
// row's first vertex (or a zero padding row) for its x + 1 nodes and is not
// used, so a CTA owns 30 vertex columns (the SIMT kernel: 31).
//
// Software pipeline, one barrier per step st:
//   before the barrier: cp.async of plane st + 2 (2-slot raw ring), TF32 split
//     of this thread's staged vertices of plane st + 1 (3-slot ring);
//   after it: one thread issues the 24 MMAs of layer st into accumulator
//     st % 2 and commits them to mbarrier st % 2; all threads update the
//     vertices of plane st - 2 and read back layer st - 1 (issued one step
//     earlier, so its products are normally complete by then).
// The owned vertex's own value is read from global memory one step ahead.
// ---------------------------------------------------------------------------
template <int TYE>
struct Modal32TcSmem {
  static constexpr int TXE = 32, NT = TXE * TYE, PX = 32, PY = TYE + 1, NP = PX * PY, NPA = NP + PX;
  float4 raw[2][NP];     // cp.async ring of vertex planes (u0, u1, u2, -)
  float4 ahi[3][NPA];    // TF32 high parts (u0, u1, u2, 0); one zero row of padding
  float4 alo[3][NPA];    // low parts u - hi
  float4 bhi[4][2][32];  // Ke per K step (dy, dz): [dx][n = 4 node + component][4 displacement components]
  float4 blo[4][2][32];
  float4 xa[2][NT];      // exchanged y = 0 forces (as Modal32Smem)
  float2 xb[2][NT];
  float coef[2];
  unsigned long long bar[2];
  uint32_t tmem;
};

__device__ __forceinline__ float tf32_hi(float x) { return __uint_as_float(__float_as_uint(x) & 0xFFFFE000u); }

__device__ __forceinline__ uint64_t tc_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  // tcgen05 shared-memory descriptor, no swizzle: start, leading- and
  // stride-dimension byte offsets (>> 4), version 0b001 at bit 46
  return (uint64_t)((addr & 0x3FFFF) >> 4) | ((uint64_t)((lbo >> 4) & 0x3FFF) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFF) << 32) | (1ull << 46);
}

__device__ __forceinline__ bool tc_bar_wait(unsigned long long* bar, uint32_t parity) {
  const uint32_t a = (uint32_t)__cvta_generic_to_shared(bar);
  for (int it = 0; it < (1 << 24); ++it) {
    uint32_t done;
    asm volatile(
        "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

__device__ int g_fine_tc_err;

// Reads (and clears) the flag of k_fine_tc32's bounded waits: 0 when no wait
// gave up since the last call.
cudaError_t fine_tc_error(int* flag) {
  int zero = 0;
  cudaError_t e = cudaMemcpyFromSymbol(flag, g_fine_tc_err, sizeof(int));
  if (e != cudaSuccess) return e;
  return *flag ? cudaMemcpyToSymbol(g_fine_tc_err, &zero, sizeof(int)) : cudaSuccess;
}

template <int TYE, int MODE, bool I32>
__global__ void __launch_bounds__(32 * TYE, 3)
    k_fine_tc32(LevelDims d, const float* __restrict__ rhop, const uint8_t* __restrict__ vmask,
                const float* __restrict__ u, const float* __restrict__ f, float* __restrict__ out, int TZ,
                ChebArgs ch) {
  static_assert(TYE == 8, "two M = 128 tiles of 32 x 4 elements per layer");
  constexpr bool CHEB = MODE >= 2, DOTS = MODE == 3;
  using I = typename std::conditional<I32, int, int64_t>::type;
  using S = Modal32TcSmem<TYE>;
  constexpr int TXE = 32, NT = S::NT, PX = S::PX, NP = S::NP, NPA = S::NPA;
  // D fp32, A and B tf32 (format 2), K-major, N = 32, M = 128
  constexpr uint32_t IDESC = (1u << 4) | (2u << 7) | (2u << 10) | ((32u >> 3) << 17) | ((128u >> 4) << 24);
  constexpr uint32_t SLOT = NPA * 16;  // bytes of one plane slot
  extern __shared__ __align__(16) unsigned char tc_smem[];
  S& sm = *reinterpret_cast<S*>(tc_smem);
  const int t = threadIdx.x, i = t & 31, j = t >> 5;
  if (t == 0) {
    if (CHEB) {
      sm.coef[0] = float(ch.coef[0]);
      sm.coef[1] = float(ch.coef[1]);
    }
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"((uint32_t)__cvta_generic_to_shared(&sm.bar[0])));
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"((uint32_t)__cvta_generic_to_shared(&sm.bar[1])));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (j == 0) {  // two accumulators of 2 x 32 columns
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 128;" ::"r"(
        (uint32_t)__cvta_generic_to_shared(&sm.tmem)));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  // Ke operand: entry (s, dx, n, c) = Ke[(3 b + comp) 24 + 3 a + c], node a =
  // dx + 2 dy + 4 dz of K step s = dy + 2 dz, n = 4 b + comp; zero rows and
  // columns for the fourth components
  for (int e = t; e < 4 * 2 * 32 * 4; e += NT) {
    const int c = e & 3, n = (e >> 2) & 31, dx = (e >> 7) & 1, s = e >> 8;
    const int a = dx + 2 * (s & 1) + 4 * (s >> 1), b = n >> 2, comp = n & 3;
    const double k = (comp < 3 && c < 3) ? cKe64[(3 * b + comp) * 24 + 3 * a + c] : 0.0;
    const float hi = tf32_hi((float)k);
    reinterpret_cast<float*>(&sm.bhi[s][dx][n])[c] = hi;
    reinterpret_cast<float*>(&sm.blo[s][dx][n])[c] = (float)(k - (double)hi);
  }
  for (int e = NP + t; e < NPA; e += NT) {
#pragma unroll
    for (int q = 0; q < 3; ++q) sm.ahi[q][e] = sm.alo[q][e] = make_float4(0.f, 0.f, 0.f, 0.f);
  }
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = sm.tmem;

  const int zblk = fine_zblocks(d.vz, TZ);
  const int rhs = blockIdx.z / zblk;
  const int kz = blockIdx.z - rhs * zblk;
  const int x0 = blockIdx.x * (TXE - 2), y0 = blockIdx.y * (TYE - 1), zb0 = kz * TZ;
  const int zb1 = zb0 + TZ + (kz + 1 == zblk ? d.vz - zblk * TZ : 0);  // fine_zblock_end
  const I nv = (I)d.nv;
  u += (int64_t)rhs * 3 * d.nv;
  if (f) f += (int64_t)rhs * 3 * d.nv;
  out += (int64_t)rhs * 3 * d.nv;
  const int gx = x0 + i, gy = y0 + j;
  const bool own = (i < TXE - 2) && (j < TYE - 1) && gx < d.vx && gy < d.vy;
  const int z0 = zb0, zend = zb1;
  constexpr int KS = (NP + NT - 1) / NT;
  int pxy[KS];
#pragma unroll
  for (int s = 0; s < KS; ++s) {
    const int k = t + s * NT, px = k % PX, py = k / PX;
    const int vx = x0 - 1 + px, vy = y0 - 1 + py;
    pxy[s] = (k < NP && vx >= 0 && vy >= 0 && vx < d.vx && vy < d.vy) ? vx + d.vx * vy : -1;
  }
  const I plane_n = (I)d.vx * d.vy;
  auto prefetch = [&](int z) {
    if (z <= zend) {
      float4* dst = sm.raw[z & 1];
      const bool zok = z >= 0 && z < d.vz;
      const I zoff = (I)z * plane_n;
#pragma unroll
      for (int s = 0; s < KS; ++s) {
        const int k = t + s * NT;
        if (k < NP) {
          const bool ok = zok && pxy[s] >= 0;
          const I v = ok ? zoff + pxy[s] : 0;
          cp_async_4(&dst[k].x, u + v, ok);
          cp_async_4(&dst[k].y, u + nv + v, ok);
          cp_async_4(&dst[k].z, u + 2 * nv + v, ok);
        }
      }
    }
    cp_async_commit();
  };
  // TF32 split of this thread's staged vertices of plane z (own cp.async
  // copies, complete after cp_async_wait1) into slot (z + 3) % 3
  auto split = [&](int z) {
    const int q = (z + 3) % 3;
#pragma unroll
    for (int s = 0; s < KS; ++s) {
      const int k = t + s * NT;
      if (k < NP) {
        const float4 v = sm.raw[z & 1][k];
        const float h0 = tf32_hi(v.x), h1 = tf32_hi(v.y), h2 = tf32_hi(v.z);
        sm.ahi[q][k] = make_float4(h0, h1, h2, 0.f);
        sm.alo[q][k] = make_float4(v.x - h0, v.y - h1, v.z - h2, 0.f);
      }
    }
  };
  const int pex = gx - 1, pey = gy - 1;
  const bool pe_xy = pex >= 0 && pey >= 0 && pex < d.ex && pey < d.ey;
  auto load_pe = [&](int ez) -> float {
    return (pe_xy && ez >= 0 && ez < d.ez) ? rhop[pex + (I)d.ex * (pey + (I)d.ey * ez)] : 0.f;
  };
  const float* __restrict__ dvin =
      (CHEB && !ch.first && !ch.d_is_u) ? static_cast<const float*>(ch.dvec) + (int64_t)rhs * 3 * d.nv : nullptr;
  constexpr bool NEED_U = CHEB || MODE == 0;
  // operands of the owned vertex at plane z, read in step z + 1 and used in step z + 2
  uint8_t vm_n = 0;
  float f_n[3] = {0.f, 0.f, 0.f}, dv_n[3] = {0.f, 0.f, 0.f}, u_n[3] = {0.f, 0.f, 0.f};
  auto load_vertex = [&](int z) {
    if (!own || z < z0 || z >= zend) return;
    const I v = gx + (I)d.vx * (gy + (I)d.vy * z);
    vm_n = vmask[v];
    if (MODE >= 1) {
#pragma unroll
      for (int c = 0; c < 3; ++c) f_n[c] = f[c * nv + v];
    }
    if (CHEB && dvin) {
#pragma unroll
      for (int c = 0; c < 3; ++c) dv_n[c] = dvin[c * nv + v];
    }
    if (NEED_U && (CHEB || ch.dotp)) {
#pragma unroll
      for (int c = 0; c < 3; ++c) u_n[c] = u[c * nv + v];
    }
  };
  // descriptors of slot 0 / K step 0; the others by adding the byte offset >> 4
  // to the start-address field (shared addresses stay below 2^18 bytes)
  const uint64_t dah0 = tc_desc((uint32_t)__cvta_generic_to_shared(&sm.ahi[0][0]), 16, 128);
  const uint64_t dal0 = tc_desc((uint32_t)__cvta_generic_to_shared(&sm.alo[0][0]), 16, 128);
  const uint64_t dbh0 = tc_desc((uint32_t)__cvta_generic_to_shared(&sm.bhi[0][0][0]), 512, 128);
  const uint64_t dbl0 = tc_desc((uint32_t)__cvta_generic_to_shared(&sm.blo[0][0][0]), 512, 128);
  float own1[2][3] = {{0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}};
  float top[3] = {0.f, 0.f, 0.f};
  float dsum = 0.f;
  bool tc_ok = true;
  float pe_n = 0.f;  // rho^p of layer st - 1, read in step st - 1
  if (z0 < zend) {
    prefetch(z0 - 1);
    prefetch(z0);
    asm volatile("cp.async.wait_group 1;\n" ::: "memory");
    split(z0 - 1);
    for (int st = z0 - 1; st <= zend + 1; ++st) {
      prefetch(st + 2);
      const float pe = pe_n;  // layer st - 1
      const uint8_t vm_c = vm_n;
      float f_c[3], dv_c[3], u_c[3];  // plane st - 2
#pragma unroll
      for (int c = 0; c < 3; ++c) { f_c[c] = f_n[c]; dv_c[c] = dv_n[c]; u_c[c] = u_n[c]; }
      pe_n = load_pe(st);
      load_vertex(st - 1);
      cp_async_wait1();
      split(st + 1);
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      asm volatile("tcgen05.fence::before_thread_sync;");
      __syncthreads();
      asm volatile("tcgen05.fence::after_thread_sync;");
      const int q = st - (z0 - 1);  // layer index in this CTA
      // ---- the products of layer st into accumulator q % 2, issued by lane 0 of
      // the last warp (its row owns no vertices, so it has the least to do)
      if (st < zend && t == NT - 32 && tc_ok) {
        const uint32_t s0 = (uint32_t)((st + 3) % 3), s1 = (uint32_t)((st + 4) % 3);
#pragma unroll
        for (int T = 0; T < 2; ++T) {
#pragma unroll
          for (int s = 0; s < 4; ++s) {
            const int dy = s & 1, dz = s >> 1;
            const uint32_t off = ((dz ? s1 : s0) * SLOT + (uint32_t)((4 * T + dy) * PX) * 16) >> 4;
            const uint32_t boff = (uint32_t)(s * 1024) >> 4;
            const uint32_t dt = tmem + 64 * (q & 1) + 32 * T;
            // hi.hi (overwrites D at the first K step), hi.lo, lo.hi
            asm volatile(
                "{\n.reg .pred p, r;\nsetp.ne.b32 p, %6, 0;\nsetp.eq.b32 r, %6, %6;\n"
                "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %5, p;\n"
                "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %3, %5, r;\n"
                "tcgen05.mma.cta_group::1.kind::tf32 [%0], %4, %2, %5, r;\n}\n" ::"r"(dt),
                "l"(dah0 + off), "l"(dbh0 + boff), "l"(dbl0 + boff), "l"(dal0 + off), "r"(IDESC), "r"(s));
          }
        }
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                         (uint32_t)__cvta_generic_to_shared(&sm.bar[q & 1]))
                     : "memory");
      }
      // ---- vertex plane p = st - 2 (layers st - 3 and st - 2 read back)
      if (st >= z0 + 1) {
        const int p = st - 2, xs = p & 1;
        float y[3];
        if (own) {
          const float4 ra = sm.xa[xs][t + TXE];
          const float2 rb = sm.xb[xs][t + TXE];
          const float r0[3] = {ra.x, ra.y, ra.z}, r1[3] = {ra.w, rb.x, rb.y};
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            y[c] = top[c] + (own1[0][c] + r0[c]);
            top[c] = own1[1][c] + r1[c];
          }
          if (p >= z0) {
            const I v = gx + (I)d.vx * (gy + (I)d.vy * p);
            const uint8_t m = vm_c;
            const float uv[3] = {u_c[0], u_c[1], u_c[2]};  // the owned vertex's value at plane p
            if (!CHEB) {
#pragma unroll
              for (int c = 0; c < 3; ++c) {
                const bool fr = (m >> c) & 1;
                const float o = MODE == 1 ? (fr ? f_c[c] - y[c] : 0.f) : (fr ? y[c] : 0.f);
                out[c * nv + v] = o;
                if (MODE == 0) dsum += uv[c] * o;
              }
            } else {
              float* __restrict__ dv = static_cast<float*>(ch.dvec) + (int64_t)rhs * 3 * d.nv;
              float r[3], zc[3];
#pragma unroll
              for (int c = 0; c < 3; ++c) r[c] = ((m >> c) & 1) ? f_c[c] - y[c] : 0.f;
              dinv_sym_apply(static_cast<const float*>(ch.dinv), nv, v, r, zc);
#pragma unroll
              for (int c = 0; c < 3; ++c) {
                const float dold = ch.d_is_u ? uv[c] : dv_c[c];
                const float c_old = sm.coef[0], c_new = sm.coef[1];
                const float dn = ch.first ? c_new * zc[c] : c_old * dold + c_new * zc[c];
                dv[c * nv + v] = dn;
                const float o = uv[c] + dn;
                out[c * nv + v] = o;
                if (DOTS) dsum += f_c[c] * o;
              }
            }
          }
        }
      }
      // ---- read back layer st - 1 from accumulator (q - 1) % 2
      if (st >= z0 && st <= zend) {
        const int qp = q - 1;
        if (tc_ok) {
          tc_ok = tc_bar_wait(&sm.bar[qp & 1], (uint32_t)((qp >> 1) & 1));
          if (!tc_ok) atomicExch(&g_fine_tc_err, 1);
        }
        asm volatile("tcgen05.fence::after_thread_sync;");
        uint32_t r[32];
        const uint32_t ta = tmem + ((uint32_t)(32 * (j & 3)) << 16) + 64 * (qp & 1) + 32 * (j >> 2);
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,"
            "%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
            : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
              "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
              "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
              "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
            : "r"(ta));
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
        float c[3][8];
        const float pw = tc_ok ? pe : 0.f;
#pragma unroll
        for (int a = 0; a < 8; ++a)
#pragma unroll
          for (int cc = 0; cc < 3; ++cc) c[cc][a] = pw * __uint_as_float(r[4 * a + cc]);
        float xc[2][2][3];  // [y bit][z bit][component]
#pragma unroll
        for (int yb = 0; yb < 2; ++yb)
#pragma unroll
          for (int zb = 0; zb < 2; ++zb)
#pragma unroll
            for (int cc = 0; cc < 3; ++cc)
              xc[yb][zb][cc] = c[cc][1 + 2 * yb + 4 * zb] +
                               __shfl_down_sync(0xffffffffu, c[cc][2 * yb + 4 * zb], 1);
#pragma unroll
        for (int zb = 0; zb < 2; ++zb)
#pragma unroll
          for (int cc = 0; cc < 3; ++cc) own1[zb][cc] = xc[1][zb][cc];
        sm.xa[(st - 1) & 1][t] = make_float4(xc[0][0][0], xc[0][0][1], xc[0][0][2], xc[0][1][0]);
        sm.xb[(st - 1) & 1][t] = make_float2(xc[0][1][1], xc[0][1][2]);
      }
    }
  }
  asm volatile("cp.async.wait_all;\n" ::: "memory");
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (j == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 128;" ::"r"(tmem));
  const int64_t cta = blockIdx.x + (int64_t)gridDim.x * (blockIdx.y + (int64_t)gridDim.y * blockIdx.z);
  if ((MODE == 0 || DOTS) && ch.dotp) {
    const double bs = modal_block_sum((double)dsum);
    if (t == 0) ch.dotp[cta] = bs;
    if (ch.ctr) modal_finish_sum(ch.dotp, (int64_t)gridDim.x * gridDim.y * gridDim.z, ch.dot, ch.ctr);
  }
}

// The same operator (MODE 0: out = K u, MODE 1: out = f - K u) on FP64 vectors
// computed in double-float arithmetic.  Vertex planes arrive as doubles by
// cp.async and are split into (hi, lo) float pairs once per plane, so the only
// FP64 instructions left are about eight conversions per vertex; the element
// operator runs on the FP32 pipe.
//
// Shared memory of the double-float kernel.  High and low parts live in
// separate 16-byte arrays, so each lane's access is one contiguous 16 bytes and
// a warp's access touches the minimum of banks (a 32-byte (hi, lo) entry per
// lane made every access take twice the wavefronts).  Vertex planes arrive as
// doubles in a 3-slot staging ring and are split into two converted slots.
template <int TXE, int TYE>
struct DfSmem {
  static constexpr int NT = TXE * TYE, PX = TXE + 1, PY = TYE + 1, NP = PX * PY;
  float4 phi[2][NP], plo[2][NP];  // converted planes: (u0, u1, u2) high / low parts
  float4 fhi[8][NT], flo[8][NT];  // nodal forces of the layer's elements, high / low parts
  double raw[3][3][NP];           // cp.async staging: [slot][component][vertex]
};

template <int TXE, int TYE, int MODE, bool VOID>
__global__ void __launch_bounds__(TXE* TYE) k_fine_modal_df(LevelDims d, const double* __restrict__ rhop,
                                                            const uint8_t* __restrict__ vmask,
                                                            const double* __restrict__ u,
                                                            const double* __restrict__ f, double* __restrict__ out,
                                                            int TZ, double* __restrict__ energy) {
  using S = DfSmem<TXE, TYE>;
  constexpr int NT = S::NT, PX = S::PX, NP = S::NP;
  extern __shared__ __align__(32) unsigned char modal_smem[];
  S& sm = *reinterpret_cast<S*>(modal_smem);
  const int t = threadIdx.x, i = t % TXE, j = t / TXE;
  const int zblk = fine_zblocks(d.vz, TZ);
  const int rhs = blockIdx.z / zblk;
  const int kz = blockIdx.z - rhs * zblk;
  const int x0 = blockIdx.x * (TXE - 1), y0 = blockIdx.y * (TYE - 1), zb0 = kz * TZ;
  const int64_t nv = d.nv;
  u += (int64_t)rhs * 3 * nv;
  if (f) f += (int64_t)rhs * 3 * nv;
  out += (int64_t)rhs * 3 * nv;
  const int gx = x0 + i, gy = y0 + j;
  const bool own = (i < TXE - 1) && (j < TYE - 1) && gx < d.vx && gy < d.vy;
  const int zb1 = fine_zblock_end(d.vz, TZ, kz);
  int z0, zend;  // the planes marched: [zb0, zb1) less the void
  fine_active_planes<VOID>(d, zb0, zb1, z0, zend);
  // Void planes [pa, pb): the owned vertices get the output for zero forces;
  // MODE 3 writes zero energy for this thread's owned elements of those layers.
  auto void_planes = [&](int pa, int pb) {
    for (int p = pa; p < pb; ++p) {
      if (own) {
        const int64_t v = gx + (int64_t)d.vx * (gy + (int64_t)d.vy * p);
        const uint8_t m = vmask[v];
#pragma unroll
        for (int c = 0; c < 3; ++c) out[c * nv + v] = (MODE >= 1 && ((m >> c) & 1)) ? f[c * nv + v] : 0.0;
      }
      const int ex = gx - 1, ey = gy - 1;
      if (MODE == 3 && i > 0 && j > 0 && ex < d.ex && ey < d.ey && p < d.ez)
        energy[ex + (int64_t)d.ex * (ey + (int64_t)d.ey * p)] = 0.0;
    }
  };
  if (VOID) {
    void_planes(zb0, z0);
    void_planes(zend, zb1);
  }
  df acc0(0), acc1(0), acc2(0);
  auto prefetch = [&](int z) {
    if (z <= zend) {
      double (*dst)[NP] = sm.raw[(z + 3) % 3];
      for (int k = t; k < NP; k += NT) {
        const int px = k % PX, py = k / PX;
        const int vx = x0 - 1 + px, vy = y0 - 1 + py;
        const bool ok = vx >= 0 && vy >= 0 && z >= 0 && vx < d.vx && vy < d.vy && z < d.vz;
        const int64_t v = ok ? vx + (int64_t)d.vx * (vy + (int64_t)d.vy * z) : 0;
        cp_async_8(&dst[0][k], u + v, ok);
        cp_async_8(&dst[1][k], u + nv + v, ok);
        cp_async_8(&dst[2][k], u + 2 * nv + v, ok);
      }
    }
    cp_async_commit();
  };
  // split staged plane z's doubles into high and low parts (converted slot (z + 2) & 1)
  auto convert = [&](int z) {
    if (z > zend) return;
    const double (*src)[NP] = sm.raw[(z + 3) % 3];
    const int cs = (z + 2) & 1;
    for (int k = t; k < NP; k += NT) {
      const df a = df_from(src[0][k]), b = df_from(src[1][k]), c = df_from(src[2][k]);
      sm.phi[cs][k] = make_float4(a.hi, b.hi, c.hi, 0.f);
      sm.plo[cs][k] = make_float4(a.lo, b.lo, c.lo, 0.f);
    }
  };
  if (z0 < zend) {
    prefetch(z0 - 1);
    prefetch(z0);
    for (int ez = z0 - 1; ez < zend; ++ez) {
      prefetch(ez + 2);
      cp_async_wait1();
      __syncthreads();
      if (ez == z0 - 1) convert(ez);
      convert(ez + 1);
      __syncthreads();
      {
        const int ex = gx - 1, ey = gy - 1;
        df pe(0);
        if (ex >= 0 && ey >= 0 && ez >= 0 && ex < d.ex && ey < d.ey && ez < d.ez)
          pe = df_from(rhop[ex + (int64_t)d.ex * (ey + (int64_t)d.ey * ez)]);
        // MODE 3 writes u_e . (rho^p Ke u_e) of the elements this CTA owns (its
        // first element row / column and layer belong to the neighbouring tiles)
        const bool own_e = MODE == 3 && i > 0 && j > 0 && ez >= z0 && ex < d.ex && ey < d.ey && ez < d.ez;
        if (pe != df(0)) {
          df c[3][8];
#pragma unroll
          for (int a = 0; a < 8; ++a) {
            const int k = (i + (a & 1)) + PX * (j + ((a >> 1) & 1));
            const int cs = (ez + (a >> 2) + 2) & 1;
            const float4 h = sm.phi[cs][k], l = sm.plo[cs][k];
            c[0][a] = df(h.x, l.x); c[1][a] = df(h.y, l.y); c[2][a] = df(h.z, l.z);
          }
          if (MODE == 3) {
            df en;
            modal_element<df, true>(c, pe, &en);
            if (own_e) energy[ex + (int64_t)d.ex * (ey + (int64_t)d.ey * ez)] = df_to(en);
          } else {
            modal_element<df>(c, pe);
          }
#pragma unroll
          for (int a = 0; a < 8; ++a) {
            sm.fhi[a][t] = make_float4(c[0][a].hi, c[1][a].hi, c[2][a].hi, 0.f);
            sm.flo[a][t] = make_float4(c[0][a].lo, c[1][a].lo, c[2][a].lo, 0.f);
          }
        } else {
#pragma unroll
          for (int a = 0; a < 8; ++a) {
            sm.fhi[a][t] = make_float4(0.f, 0.f, 0.f, 0.f);
            sm.flo[a][t] = make_float4(0.f, 0.f, 0.f, 0.f);
          }
          if (own_e) energy[ex + (int64_t)d.ex * (ey + (int64_t)d.ey * ez)] = 0.0;
        }
      }
      __syncthreads();
      if (own) {
        df b0 = acc0, b1 = acc1, b2 = acc2, t0(0), t1(0), t2(0);
#pragma unroll
        for (int w = 0; w < 4; ++w) {
          const int wx = w & 1, wy = w >> 1;
          const int te = (i + wx) + TXE * (j + wy);
          const int a = (1 - wx) + 2 * (1 - wy);
          const float4 bh = sm.fhi[a][te], bl = sm.flo[a][te], th = sm.fhi[a + 4][te], tl = sm.flo[a + 4][te];
          b0 += df(bh.x, bl.x); b1 += df(bh.y, bl.y); b2 += df(bh.z, bl.z);
          t0 += df(th.x, tl.x); t1 += df(th.y, tl.y); t2 += df(th.z, tl.z);
        }
        if (ez >= z0) {
          const int64_t v = gx + (int64_t)d.vx * (gy + (int64_t)d.vy * ez);
          const uint8_t m = vmask[v];
          const double y[3] = {df_to(b0), df_to(b1), df_to(b2)};
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            const bool fr = (m >> c) & 1;
            const int64_t idx = c * nv + v;
            out[idx] = MODE >= 1 ? (fr ? f[idx] - y[c] : 0.0) : (fr ? y[c] : 0.0);
          }
        }
        acc0 = t0; acc1 = t1; acc2 = t2;
      }
    }
  }
  asm volatile("cp.async.wait_all;\n" ::: "memory");
}

// Row block of vertex (x,y,z): out = sum over incident elements of rho^p Ke[a,:] u_e,
// S = diagonal 3x3 block.  Template arguments fix whether S is needed.
template <typename T, bool NEED_S>
__device__ __forceinline__ void fine_row(const LevelDims& d, const T* __restrict__ rhop,
                                         const T* __restrict__ u, int x, int y, int z, T out[3],
                                         T S[9]) {
  out[0] = out[1] = out[2] = T(0);
  if (NEED_S)
#pragma unroll
    for (int i = 0; i < 9; ++i) S[i] = T(0);
  const int64_t nv = d.nv;
#pragma unroll
  for (int w = 0; w < 8; ++w) {
    const int ex = x - 1 + (w & 1), ey = y - 1 + ((w >> 1) & 1), ez = z - 1 + (w >> 2);
    if (ex < 0 || ey < 0 || ez < 0 || ex >= d.ex || ey >= d.ey || ez >= d.ez) continue;
    const T pe = rhop[ex + (int64_t)d.ex * (ey + (int64_t)d.ey * ez)];
    if (pe == T(0)) continue;
    const int a = 7 - w;
    T s0 = T(0), s1 = T(0), s2 = T(0);
#pragma unroll
    for (int b = 0; b < 8; ++b) {
      const int64_t vb = (ex + (b & 1)) + (int64_t)d.vx * ((ey + ((b >> 1) & 1)) + (int64_t)d.vy * (ez + (b >> 2)));
      const T u0 = u[vb], u1 = u[nv + vb], u2 = u[2 * nv + vb];
      const int r0 = (3 * a) * 24 + 3 * b;
      s0 += ke<T>(r0) * u0 + ke<T>(r0 + 1) * u1 + ke<T>(r0 + 2) * u2;
      s1 += ke<T>(r0 + 24) * u0 + ke<T>(r0 + 25) * u1 + ke<T>(r0 + 26) * u2;
      s2 += ke<T>(r0 + 48) * u0 + ke<T>(r0 + 49) * u1 + ke<T>(r0 + 50) * u2;
    }
    out[0] += pe * s0; out[1] += pe * s1; out[2] += pe * s2;
    if (NEED_S) {
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) S[3 * i + j] += pe * ke<T>((3 * a + i) * 24 + 3 * a + j);
    }
  }
}

template <typename T>
__global__ void __launch_bounds__(256) k_fine_apply(LevelDims d, const T* __restrict__ rhop,
                                                    const uint8_t* __restrict__ vmask,
                                                    const T* __restrict__ u, const T* __restrict__ f,
                                                    T* __restrict__ out, bool residual) {
  const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= d.nv) return;
  const int x = (int)(v % d.vx);
  const int64_t t = v / d.vx;
  const int y = (int)(t % d.vy), z = (int)(t / d.vy);
  const uint8_t m = vmask[v];
  T o[3] = {T(0), T(0), T(0)};
  if (m & 7) fine_row<T, false>(d, rhop, u, x, y, z, o, nullptr);
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const bool fr = (m >> c) & 1;
    const int64_t i = c * d.nv + v;
    out[i] = residual ? (fr ? f[i] - o[c] : T(0)) : (fr ? o[c] : T(0));
  }
}

// One colour of the 8-colour point-block Gauss-Seidel sweep.  Forward: DOFs
// 0,1,2 (grid/Grid.cu:1830-1838); reverse: DOFs 2,1,0 (adjoint sweep).
template <typename T>
__device__ __forceinline__ void block_update(T* u, int64_t nv, int64_t v, const T r[3], const T S[9],
                                             uint8_t fb, bool reverse) {
  T du[3] = {T(0), T(0), T(0)};
  if (!reverse) {
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      if (!((fb >> i) & 1)) continue;
      T s = r[i];
#pragma unroll
      for (int j = 0; j < i; ++j) s -= S[3 * i + j] * du[j];
      du[i] = s / S[4 * i];
    }
  } else {
#pragma unroll
    for (int i = 2; i >= 0; --i) {
      if (!((fb >> i) & 1)) continue;
      T s = r[i];
#pragma unroll
      for (int j = i + 1; j < 3; ++j) s -= S[3 * i + j] * du[j];
      du[i] = s / S[4 * i];
    }
  }
#pragma unroll
  for (int i = 0; i < 3; ++i)
    if ((fb >> i) & 1) u[i * nv + v] += du[i];
}

template <typename T>
__global__ void __launch_bounds__(256) k_fine_gs(LevelDims d, const T* __restrict__ rhop,
                                                 const uint8_t* __restrict__ vmask, T* u,
                                                 const T* __restrict__ f, int cx, int cy, int cz,
                                                 int hx, int hy, int64_t cnt, bool reverse) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= cnt) return;
  const int x = cx + 2 * (int)(t % hx);
  const int64_t t2 = t / hx;
  const int y = cy + 2 * (int)(t2 % hy), z = cz + 2 * (int)(t2 / hy);
  const int64_t v = x + (int64_t)d.vx * (y + (int64_t)d.vy * z);
  const uint8_t m = vmask[v];
  const uint8_t fb = (m & 8) ? (m & 7) : 0;
  if (!fb) return;
  T o[3], S[9], r[3];
  fine_row<T, true>(d, rhop, u, x, y, z, o, S);
#pragma unroll
  for (int c = 0; c < 3; ++c) r[c] = f[c * d.nv + v] - o[c];
  block_update<T>(u, d.nv, v, r, S, fb, reverse);
}

// Inverse of the free-DOF part of each diagonal 3x3 block (Chebyshev): [9][nv]
// in FP64, the packed symmetric layout of dinv_sym_apply in FP32.
template <typename T>
__device__ __forceinline__ void invert_block(const T S_in[9], uint8_t fb, T* dinv, int64_t nv,
                                             int64_t v) {
  T S[9];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j)
      S[3 * i + j] = (((fb >> i) & 1) && ((fb >> j) & 1)) ? S_in[3 * i + j] : (i == j ? T(1) : T(0));
  const T a = S[0], b = S[1], c = S[2], dd = S[4], e = S[5], f = S[8];
  const T A0 = dd * f - e * e, A1 = c * e - b * f, A2 = b * e - c * dd;
  const T det = a * A0 + b * A1 + c * A2;
  const T inv[9] = {A0, A1, A2, A1, a * f - c * c, b * c - a * e, A2, b * c - a * e, a * dd - b * b};
  const T rd = T(1) / det;
  T o[9];
#pragma unroll
  for (int k = 0; k < 9; ++k) {
    const int i = k / 3, j = k % 3;
    const bool keep = ((fb >> i) & 1) && ((fb >> j) & 1);
    o[k] = keep ? inv[k] * rd : T(0);
  }
  if constexpr (sizeof(T) == 4) {  // FP32: the packed symmetric layout (the block is symmetric entry for entry)
    reinterpret_cast<float4*>(dinv)[v] = make_float4(o[0], o[1], o[2], o[4]);
    reinterpret_cast<float2*>(dinv + 4 * nv)[v] = make_float2(o[5], o[8]);
  } else {
#pragma unroll
    for (int k = 0; k < 9; ++k) dinv[k * nv + v] = o[k];
  }
}

template <typename T>
__global__ void k_fine_diag_inv(LevelDims d, const T* __restrict__ rhop,
                                const uint8_t* __restrict__ vmask, T* __restrict__ dinv) {
  const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= d.nv) return;
  const int x = (int)(v % d.vx);
  const int64_t t = v / d.vx;
  const int y = (int)(t % d.vy), z = (int)(t / d.vy);
  const uint8_t m = vmask[v];
  const uint8_t fb = (m & 8) ? (m & 7) : 0;
  T S[9];
#pragma unroll
  for (int i = 0; i < 9; ++i) S[i] = T(0);
#pragma unroll
  for (int w = 0; w < 8; ++w) {
    const int ex = x - 1 + (w & 1), ey = y - 1 + ((w >> 1) & 1), ez = z - 1 + (w >> 2);
    if (ex < 0 || ey < 0 || ez < 0 || ex >= d.ex || ey >= d.ey || ez >= d.ez) continue;
    const T pe = rhop[ex + (int64_t)d.ex * (ey + (int64_t)d.ey * ez)];
    const int a = 7 - w;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) S[3 * i + j] += pe * ke<T>((3 * a + i) * 24 + 3 * a + j);
  }
  invert_block<T>(S, fb, dinv, d.nv, v);
}

static inline unsigned blocks_for(int64_t n, int bs) { return (unsigned)((n + bs - 1) / bs); }

constexpr int MODAL_TXE = 32, MODAL_TYE = 8, MODAL_TZ = 16;
// the per-tile active z ranges (LevelDims::colz) are laid out for this tile
static_assert(MODAL_TXE == FINE_TILE_X && MODAL_TYE == FINE_TILE_Y && TOPO_MODAL32_TYE == FINE_TILE_Y,
              "fine kernel tiles and LevelDims::colz disagree");
// CTA tile rows of the FP32 / FP64 modal kernels
template <typename T>
constexpr int modal_tye() { return sizeof(T) == 4 ? TOPO_MODAL32_TYE : MODAL_TYE; }

// Whether an FP32 launch with depth argument tz runs the tensor-core kernel
// (TOPO_FINE_TC_FLAG, and no void planes: the per-tile z ranges are laid out
// for the modal kernel's tiles).
template <typename T>
bool modal_tc(const LevelDims& d, int tz) {
  return sizeof(T) == 4 && (tz & TOPO_FINE_TC_FLAG) && !(d.colz && d.colz_void);
}
inline int modal_depth(int tz) {
  tz &= ~TOPO_FINE_FLAGS;
  return tz <= 0 ? MODAL_TZ : tz;
}
// Element rows (warps) of the launch's CTA tile: the ROWS flags choose 4 or 16
// for the FP32 modal kernel on levels without void planes.
template <typename T>
int modal_rows(const LevelDims& d, int tz) {
  if (sizeof(T) != 4 || modal_tc<T>(d, tz) || (d.colz && d.colz_void)) return modal_tye<T>();
  return (tz & TOPO_FINE_ROWS4_FLAG) ? 4 : (tz & TOPO_FINE_ROWS16_FLAG) ? 16 : modal_tye<T>();
}

template <typename T>
dim3 modal_grid(const LevelDims& d, int tz, int nb) {
  const int rows = modal_rows<T>(d, tz);
  const int xs = modal_tc<T>(d, tz) ? MODAL_TXE - 2 : MODAL_TXE - 1;  // owned vertex columns per CTA
  return dim3((d.vx + xs - 1) / xs, (d.vy + rows - 2) / (rows - 1), fine_zblocks(d.vz, modal_depth(tz)) * nb);
}

// One launch of the FP32 modal kernel with a CTA tile of ROWS element rows.
template <int ROWS, int MODE, bool VOID>
void launch_modal32_rows(cudaStream_t s, const LevelDims& d, const float* rhop, const uint8_t* vmask, const float* u,
                         const float* f, float* out, int tz, const dim3& grid, const ChebArgs& ch) {
  const size_t smem = sizeof(Modal32Smem<ROWS>);
  static PerDeviceOnce once;
  once_per_device(once, [smem] {
    cudaError_t e = cudaFuncSetAttribute(k_fine_modal32<ROWS, MODE, true, VOID>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(k_fine_modal32<ROWS, MODE, false, VOID>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)smem);
    return e;
  });
  // (MODE 3 keeps 64-bit offsets: with 32-bit ones it spilled 32 bytes and
  // ran 122 against 118 us at 256x128x128, where modes 0-2 gained 4-9 us)
  if (MODE != 3 && 3 * d.nv < ((int64_t)1 << 31) && d.ne < ((int64_t)1 << 31))
    k_fine_modal32<ROWS, MODE, true, VOID><<<grid, 32 * ROWS, smem, s>>>(d, rhop, vmask, u, f, out, tz, ch);
  else
    k_fine_modal32<ROWS, MODE, false, VOID><<<grid, 32 * ROWS, smem, s>>>(d, rhop, vmask, u, f, out, tz, ch);
}

// One launch of the modal operator in mode MODE: the single-barrier kernel for
// FP32, the generic kernel for FP64; the VOID instantiations where level 0 has
// void planes.  Kernels are opted into their dynamic shared memory once per
// device.
template <typename T, int MODE, bool VOID>
void launch_modal_v(cudaStream_t s, const LevelDims& d, const T* rhop, const uint8_t* vmask, const T* u, const T* f,
                    T* out, int tz, int nb, const ChebArgs& ch) {
  const dim3 grid = modal_grid<T>(d, tz, nb);
  const bool tc = modal_tc<T>(d, tz) && !VOID;
  const int rows = modal_rows<T>(d, tz);
  tz = modal_depth(tz);
  constexpr int TYE = modal_tye<T>();
  if constexpr (sizeof(T) == 4 && !VOID) {
    if (!tc && rows == 4) {
      launch_modal32_rows<4, MODE, false>(s, d, rhop, vmask, u, f, out, tz, grid, ch);
      return;
    }
    if (!tc && rows == 16) {
      launch_modal32_rows<16, MODE, false>(s, d, rhop, vmask, u, f, out, tz, grid, ch);
      return;
    }
  }
  if constexpr (sizeof(T) == 4 && TYE == 8 && !VOID) {
    if (tc) {
      const size_t smem = sizeof(Modal32TcSmem<TYE>);
      static PerDeviceOnce once;
      once_per_device(once, [smem] {
        cudaError_t e = cudaFuncSetAttribute(k_fine_tc32<TYE, MODE, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem);
        if (e == cudaSuccess)
          e = cudaFuncSetAttribute(k_fine_tc32<TYE, MODE, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)smem);
        return e;
      });
      if (MODE != 3 && 3 * d.nv < ((int64_t)1 << 31) && d.ne < ((int64_t)1 << 31))
        k_fine_tc32<TYE, MODE, true><<<grid, 32 * TYE, smem, s>>>(d, rhop, vmask, u, f, out, tz, ch);
      else
        k_fine_tc32<TYE, MODE, false><<<grid, 32 * TYE, smem, s>>>(d, rhop, vmask, u, f, out, tz, ch);
      return;
    }
  }
  if constexpr (sizeof(T) == 4) {
    launch_modal32_rows<TYE, MODE, VOID>(s, d, rhop, vmask, u, f, out, tz, grid, ch);
  } else {
    const size_t smem = sizeof(ModalSmem<T, MODAL_TXE, TYE>);
    static PerDeviceOnce once;
    once_per_device(once, [smem] {
      return cudaFuncSetAttribute(k_fine_modal<T, MODAL_TXE, TYE, MODE, VOID>,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    });
    k_fine_modal<T, MODAL_TXE, TYE, MODE, VOID><<<grid, MODAL_TXE * TYE, smem, s>>>(d, rhop, vmask, u, f, out, tz,
                                                                                     ch);
  }
}

template <typename T, int MODE>
void launch_modal(cudaStream_t s, const LevelDims& d, const T* rhop, const uint8_t* vmask, const T* u, const T* f,
                  T* out, int tz, int nb, const ChebArgs& ch) {
  if (d.colz && d.colz_void) launch_modal_v<T, MODE, true>(s, d, rhop, vmask, u, f, out, tz, nb, ch);
  else launch_modal_v<T, MODE, false>(s, d, rhop, vmask, u, f, out, tz, nb, ch);
}

template <typename T>
void launch_fine_apply(cudaStream_t s, const LevelDims& d, const T* rhop, const uint8_t* vmask,
                       const T* u, const T* f, T* out, bool residual, int nb, int tz) {
  const ChebArgs ch{nullptr, nullptr, nullptr, 0, nullptr, 0, nullptr, nullptr};
  if (residual) launch_modal<T, 1>(s, d, rhop, vmask, u, f, out, tz, nb, ch);
  else launch_modal<T, 0>(s, d, rhop, vmask, u, f, out, tz, nb, ch);
}

// out = K u with the per-CTA partial sums of u.out in partial[0, n) (one
// right-hand side).  Returns n, or 0, launching nothing, when the grid has more
// CTAs than the cap partial slots.
template <typename T>
int launch_fine_apply_dot(cudaStream_t s, const LevelDims& d, const T* rhop, const uint8_t* vmask, const T* u,
                          T* out, int tz, double* partial, int cap, double* dot, unsigned* ctr) {
  const dim3 grid = modal_grid<T>(d, tz, 1);
  const int64_t nparts = (int64_t)grid.x * grid.y * grid.z;
  if (nparts > cap) return 0;
  const ChebArgs ch{nullptr, nullptr, nullptr, 0, partial, 0, dot, dot ? ctr : nullptr};
  launch_modal<T, 0>(s, d, rhop, vmask, u, nullptr, out, tz, 1, ch);
  return (int)nparts;
}

template int launch_fine_apply_dot<float>(cudaStream_t, const LevelDims&, const float*, const uint8_t*,
                                          const float*, float*, int, double*, int, double*, unsigned*);
template int launch_fine_apply_dot<double>(cudaStream_t, const LevelDims&, const double*, const uint8_t*,
                                           const double*, double*, int, double*, int, double*, unsigned*);

template <bool VOID>
static void launch_fine_apply_df_v(cudaStream_t s, const LevelDims& d, const double* rhop, const uint8_t* vmask,
                                   const double* u, const double* f, double* out, bool residual, int nb, int tz,
                                   double* energy) {
  if (tz <= 0) tz = MODAL_TZ;
  const dim3 grid((d.vx + MODAL_TXE - 2) / (MODAL_TXE - 1), (d.vy + MODAL_TYE - 2) / (MODAL_TYE - 1),
                  fine_zblocks(d.vz, tz) * nb);
  constexpr int NT = MODAL_TXE * MODAL_TYE;
  const size_t smem = sizeof(DfSmem<MODAL_TXE, MODAL_TYE>);
  static PerDeviceOnce once;
  once_per_device(once, [smem] {
    cudaError_t e = cudaFuncSetAttribute(k_fine_modal_df<MODAL_TXE, MODAL_TYE, 0, VOID>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(k_fine_modal_df<MODAL_TXE, MODAL_TYE, 1, VOID>,
                               cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(k_fine_modal_df<MODAL_TXE, MODAL_TYE, 3, VOID>,
                               cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    return e;
  });
  if (residual && energy)
    k_fine_modal_df<MODAL_TXE, MODAL_TYE, 3, VOID><<<grid, NT, smem, s>>>(d, rhop, vmask, u, f, out, tz, energy);
  else if (residual)
    k_fine_modal_df<MODAL_TXE, MODAL_TYE, 1, VOID><<<grid, NT, smem, s>>>(d, rhop, vmask, u, f, out, tz, nullptr);
  else
    k_fine_modal_df<MODAL_TXE, MODAL_TYE, 0, VOID><<<grid, NT, smem, s>>>(d, rhop, vmask, u, f, out, tz, nullptr);
}

void launch_fine_apply_df(cudaStream_t s, const LevelDims& d, const double* rhop, const uint8_t* vmask,
                          const double* u, const double* f, double* out, bool residual, int nb, int tz,
                          double* energy) {
  if (d.colz && d.colz_void) launch_fine_apply_df_v<true>(s, d, rhop, vmask, u, f, out, residual, nb, tz, energy);
  else launch_fine_apply_df_v<false>(s, d, rhop, vmask, u, f, out, residual, nb, tz, energy);
}

// One fused Chebyshev step on level 0: uout = u + d with d = c_old d + c_new Dinv (f - K u)
// and (c_old, c_new) = coef[0..1] in device memory.
template <typename T>
int launch_fine_cheb(cudaStream_t s, const LevelDims& d, const T* rhop, const uint8_t* vmask, const T* u,
                     const T* f, T* uout, const T* dinv, T* dvec, const double* coef, bool first, int nb,
                     int tz, bool d_is_u, double* dot_fo, int cap, double* dot, unsigned* ctr) {
  // the FP64 kernel always reads d and has no fused dots
  int nparts = 0;
  if (sizeof(T) == 4 && dot_fo && nb == 1) {
    const dim3 grid = modal_grid<T>(d, tz, 1);
    nparts = (int64_t)grid.x * grid.y * grid.z <= cap ? (int)(grid.x * grid.y * grid.z) : 0;
  }
  const ChebArgs ch{dinv, dvec, coef, first ? 1 : 0, nparts ? dot_fo : nullptr,
                    (d_is_u && sizeof(T) == 4) ? 1 : 0, dot, (nparts && dot) ? ctr : nullptr};
  if constexpr (sizeof(T) == 4) {
    if (nparts) {  // the step with the fused sums is its own instantiation
      launch_modal<T, 3>(s, d, rhop, vmask, u, f, uout, tz, nb, ch);
      return nparts;
    }
  }
  launch_modal<T, 2>(s, d, rhop, vmask, u, f, uout, tz, nb, ch);
  return nparts;
}

template int launch_fine_cheb<double>(cudaStream_t, const LevelDims&, const double*, const uint8_t*,
                                      const double*, const double*, double*, const double*, double*,
                                      const double*, bool, int, int, bool, double*, int, double*, unsigned*);
template int launch_fine_cheb<float>(cudaStream_t, const LevelDims&, const float*, const uint8_t*,
                                     const float*, const float*, float*, const float*, float*, const double*,
                                     bool, int, int, bool, double*, int, double*, unsigned*);

// First Chebyshev step from a zero iterate (every pre-smoothing sweep of a
// preconditioning V-cycle starts from u = 0): K u vanishes, so r = f on the
// free DOFs, d = c_new D^-1 r and u_out = d.  No vertex planes are read and no
// element operator is applied; with the stored FP32 block inverse (packed
// symmetric layout) the result equals the fused step's on u = 0.  Rebuilding
// the blocks from the eight incident elements' rho^p here took about 350
// instructions per vertex and ran issue-bound (47 us at 256x128x128).
// blockIdx.y is the right-hand side of a batch.
__global__ void k_fine_cheb_zero32(int64_t nv, const uint8_t* __restrict__ vmask, const float* __restrict__ dinv,
                                   const float* __restrict__ f, float* __restrict__ dv, float* __restrict__ out,
                                   const double* __restrict__ coef) {
  const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= nv) return;
  const int64_t bo = (int64_t)blockIdx.y * 3 * nv;
  f += bo;
  if (dv) dv += bo;
  out += bo;
  const uint8_t m = vmask[v];
  float r[3], zc[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) r[c] = ((m >> c) & 1) ? f[c * nv + v] : 0.f;
  dinv_sym_apply(dinv, nv, v, r, zc);
  const float c_new = (float)__ldg(coef + 1);
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const float dn = c_new * zc[c];
    if (dv) dv[c * nv + v] = dn;
    out[c * nv + v] = dn;
  }
}

template <typename T>
void launch_fine_cheb_zero(cudaStream_t s, const LevelDims& d, const T* rhop, const uint8_t* vmask, const T* f,
                           T* uout, const T* dinv, T* dvec, const double* coef, int nb) {
  if (sizeof(T) == 4) {  // dvec may be null: d is not stored (the next step takes d = u)
    k_fine_cheb_zero32<<<dim3(blocks_for(d.nv, 256), nb), 256, 0, s>>>(
        d.nv, vmask, reinterpret_cast<const float*>(dinv), reinterpret_cast<const float*>(f),
        reinterpret_cast<float*>(dvec), reinterpret_cast<float*>(uout), coef);
  } else {
    launch_cheb_zero_stored<T>(s, d.nv, vmask, dinv, f, dvec, uout, coef, nb);
  }
}

template void launch_fine_cheb_zero<double>(cudaStream_t, const LevelDims&, const double*, const uint8_t*,
                                            const double*, double*, const double*, double*, const double*, int);
template void launch_fine_cheb_zero<float>(cudaStream_t, const LevelDims&, const float*, const uint8_t*,
                                           const float*, float*, const float*, float*, const double*, int);

// Dense-row form of the same operator (thread per vertex, 8 x 3 x 24 products);
// kept as the cross-check of the modal kernel.
template <typename T>
void launch_fine_apply_dense(cudaStream_t s, const LevelDims& d, const T* rhop, const uint8_t* vmask,
                             const T* u, const T* f, T* out, bool residual) {
  k_fine_apply<T><<<blocks_for(d.nv, 256), 256, 0, s>>>(d, rhop, vmask, u, f, out, residual);
}

template void launch_fine_apply_dense<double>(cudaStream_t, const LevelDims&, const double*,
                                              const uint8_t*, const double*, const double*, double*, bool);
template void launch_fine_apply_dense<float>(cudaStream_t, const LevelDims&, const float*,
                                             const uint8_t*, const float*, const float*, float*, bool);

template <typename T>
void launch_fine_gs(cudaStream_t s, const LevelDims& d, const T* rhop, const uint8_t* vmask, T* u,
                    const T* f, int colour, bool reverse) {
  const int cx = colour & 1, cy = (colour >> 1) & 1, cz = colour >> 2;
  const int hx = (d.vx - cx + 1) / 2, hy = (d.vy - cy + 1) / 2, hz = (d.vz - cz + 1) / 2;
  const int64_t cnt = (int64_t)hx * hy * hz;
  if (cnt <= 0) return;
  k_fine_gs<T><<<blocks_for(cnt, 256), 256, 0, s>>>(d, rhop, vmask, u, f, cx, cy, cz, hx, hy, cnt,
                                                    reverse);
}

template <typename T>
void launch_fine_diag_inv(cudaStream_t s, const LevelDims& d, const T* rhop, const uint8_t* vmask,
                          T* dinv) {
  k_fine_diag_inv<T><<<blocks_for(d.nv, 256), 256, 0, s>>>(d, rhop, vmask, dinv);
}

template void launch_fine_apply<double>(cudaStream_t, const LevelDims&, const double*, const uint8_t*,
                                        const double*, const double*, double*, bool, int, int);
template void launch_fine_apply<float>(cudaStream_t, const LevelDims&, const float*, const uint8_t*,
                                       const float*, const float*, float*, bool, int, int);
template void launch_fine_gs<double>(cudaStream_t, const LevelDims&, const double*, const uint8_t*,
                                     double*, const double*, int, bool);
template void launch_fine_gs<float>(cudaStream_t, const LevelDims&, const float*, const uint8_t*,
                                    float*, const float*, int, bool);
template void launch_fine_diag_inv<double>(cudaStream_t, const LevelDims&, const double*,
                                           const uint8_t*, double*);
template void launch_fine_diag_inv<float>(cudaStream_t, const LevelDims&, const float*,
                                          const uint8_t*, float*);

}  // namespace topo
