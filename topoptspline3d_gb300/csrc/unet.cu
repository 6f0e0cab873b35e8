// Learned preconditioner: network definition, training and application.
//
// U-Net on the vertex grid (3 levels, 16/32/64 channels, 3x3x3 kernels):
//   L0a conv 16->16 relu (input: r/lr xyz, z/lz xyz, log-density, 9 zero channels)
//   L0b conv 16->16 relu                      -> s0
//   pool -> L1a conv 16->32 relu, L1b conv 32->32 relu -> s1
//   pool -> L2a conv 32->64 relu, L2b conv 64->32 relu -> b2
//   D1a conv [up(b2), s1] 64->32 relu, D1b conv 32->16 relu -> d1
//   D0a conv [up(d1), s0] 32->16 relu, D0b conv 16->16 (channels 0-2 used)
// 246,931 effective parameters (3x3x3 kernels on the real input and output
// channels plus biases).  Weights are stored in fp32 (Adam master copy) and
// bf16 (what the tensor cores read); activations are bf16, accumulation fp32.
//
// The network corrects the FP32 multigrid preconditioner of the mixed solver:
//   z' = z + beta lz * N(s(r / lr), s(z / lz), log rho),  z = V(r),  s(x) = x / (1 + |x|/8)
// with lr, lz the local rms of r and z (over blocks of 8^3 vertices, floored at
// 1e-2 of the global rms), and the correction c = lz * N taken in the amount
// that minimises the energy norm of the error: beta = c.(r - A z) / c.(A c)
// (two FP32 operator applications; beta = 0 keeps z, so the correction never
// makes the error larger in that norm).  Every input and the target are in
// local units, so crops from stiff and soft regions, loads and far field have
// targets of the same size, and the network sees the V-cycle output it
// corrects.  It is trained on pairs harvested from the solver's own iterates:
// for a residual r_k with V-cycle output z_k and error e_k = u* - u_k, the
// target is (e_k - z_k) / lz_k.  Its last layer starts at zero, so an untrained
// network leaves the V-cycle unchanged.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <vector>

#include "topo_internal.h"

namespace topo {

// k_unet.cu
cudaError_t unet_conv(cudaStream_t s, int cin, int cout, const __nv_bfloat16* s1, const __nv_bfloat16* s2, int c1,
                      int up1, const __nv_bfloat16* W, const float* bias, int X, int Y, int Z, int nb, int relu,
                      int out_mode, void* out);
cudaError_t unet_wgrad(cudaStream_t s, int cin, int cout, const __nv_bfloat16* s1, const __nv_bfloat16* s2, int c1,
                       int up1, const __nv_bfloat16* G, int X, int Y, int Z, int nb, int groups, float* part,
                       float* dW);
// k_conv_tc.cu: the same convolution on the tcgen05 tensor cores
cudaError_t unet_conv_tc(cudaStream_t s, int cin, int cout, const __nv_bfloat16* s1, const __nv_bfloat16* s2, int c1,
                         int up1, const __nv_bfloat16* W, const float* bias, int X, int Y, int Z, int nb, int relu,
                         int out_mode, void* out);
cudaError_t conv_tc_error(int* flag);
void unet_bias_grad(cudaStream_t s, const __nv_bfloat16* G, int64_t nvox, int C, float* part, int nblk, float* db);
void unet_relu_grad(cudaStream_t s, const float* dY, const __nv_bfloat16* Y, int64_t n, int relu, __nv_bfloat16* G);
void unet_pool(cudaStream_t s, const __nv_bfloat16* in, int X, int Y, int Z, int nb, int C, __nv_bfloat16* out);
void unet_pool_bwd(cudaStream_t s, const float* dout, int X, int Y, int Z, int nb, int C, int accumulate, float* din);
void unet_up_bwd(cudaStream_t s, const float* dfull, int X, int Y, int Z, int nb, int cfull, int c, float* dhalf);
void unet_slice(cudaStream_t s, const float* src, int64_t nvox, int cfull, int c0, int c, int accumulate, float* dst);
void unet_flip(cudaStream_t s, const __nv_bfloat16* W, int cin, int cout, __nv_bfloat16* Wt);
void unet_adam(cudaStream_t s, int64_t n, const float* grad, float lr, float b1, float b2, float eps, int step,
               float* w, float* m, float* v, __nv_bfloat16* wb, const double* gn2 = nullptr, float clip = 1.f);
void unet_to_bf16(cudaStream_t s, const float* a, int64_t n, __nv_bfloat16* b);

namespace {

constexpr int kIn = 16;     // padded input channels
constexpr int kInUsed = 8;  // stored input channels: r xyz, z xyz, log-density, 0
constexpr int kBlk = 8;     // vertex block side of the local rms
enum { L0A, L0B, L1A, L1B, L2A, L2B, D1A, D1B, D0A, D0B, NLAYER };
struct LayerDef { int cin, cout, relu, cin_real, cout_real; };
constexpr LayerDef kDef[NLAYER] = {{kIn, 16, 1, kInUsed, 16},  {16, 16, 1, 16, 16}, {16, 32, 1, 16, 32},
                                   {32, 32, 1, 32, 32},  {32, 64, 1, 32, 64}, {64, 32, 1, 64, 32},
                                   {64, 32, 1, 64, 32},  {32, 16, 1, 32, 16}, {32, 16, 1, 32, 16},
                                   {16, 16, 0, 16, 3}};

inline unsigned nb256(int64_t n) { return (unsigned)((n + 255) / 256); }

uint64_t splitmix(uint64_t& s) {
  uint64_t z = (s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
double uniform01(uint64_t& s) { return (double)(splitmix(s) >> 11) * (1.0 / 9007199254740992.0); }

// ---- kernels ---------------------------------------------------------------

// Network input of a normalised residual component: linear near zero,
// saturating at +-8 (the residual of a solve concentrates on loads and
// supports, so r / rms(r) reaches the thousands there).  Applied identically
// to training crops and at inference.
__device__ __forceinline__ float squash(float x) { return x / (1.f + fabsf(x) * 0.125f); }

// log10(rho) averaged over the active elements around each vertex, mapped to
// log10(rho)/3 + 0.5 (rho in [1e-3, 1] -> [-0.5, 0.5]).
__global__ void k_vertex_logrho(LevelDims d, const uint8_t* __restrict__ eactive, const double* __restrict__ rho,
                                double rho_min, float* __restrict__ lr) {
  const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= d.nv) return;
  const int x = (int)(v % d.vx), y = (int)((v / d.vx) % d.vy), z = (int)(v / ((int64_t)d.vx * d.vy));
  double s = 0;
  int n = 0;
  for (int k = 0; k < 8; ++k) {
    const int ex = x - 1 + (k & 1), ey = y - 1 + ((k >> 1) & 1), ez = z - 1 + (k >> 2);
    if (ex < 0 || ey < 0 || ez < 0 || ex >= d.ex || ey >= d.ey || ez >= d.ez) continue;
    const int64_t e = ex + (int64_t)d.ex * (ey + (int64_t)d.ey * ez);
    if (!eactive[e]) continue;
    s += log10(fmax(rho[e], 1e-12));
    ++n;
  }
  const double l = n ? s / n : log10(rho_min);
  lr[v] = (float)(l / 3.0 + 0.5);
}

// z[c][v] += lz[v] * out[v'][c] on free DOFs.
__global__ void k_unpack_add(LevelDims d, int X, int Y, const __nv_bfloat16* __restrict__ out, const uint8_t* vmask,
                             const float* __restrict__ lz, float* __restrict__ z) {
  const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= d.nv) return;
  const int x = (int)(v % d.vx), y = (int)((v / d.vx) % d.vy), zz = (int)(v / ((int64_t)d.vx * d.vy));
  const int64_t u = ((int64_t)zz * Y + y) * X + x;
  const uint8_t m = vmask[v];
  const float s = lz[v];
  for (int k = 0; k < 3; ++k)
    if ((m >> k) & 1) z[k * d.nv + v] += s * __bfloat162float(out[u * 16 + k]);
}

// Mean square of a [3][nv] field over each block of kBlk^3 vertices.
__global__ void k_block_ms(LevelDims d, const float* __restrict__ f, float* __restrict__ blk) {
  const int nbx = (d.vx + kBlk - 1) / kBlk, nby = (d.vy + kBlk - 1) / kBlk, nbz = (d.vz + kBlk - 1) / kBlk;
  const int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= (int64_t)nbx * nby * nbz) return;
  const int bx = (int)(b % nbx), by = (int)((b / nbx) % nby), bz = (int)(b / ((int64_t)nbx * nby));
  double s = 0;
  int n = 0;
  for (int z = bz * kBlk; z < min(d.vz, (bz + 1) * kBlk); ++z)
    for (int y = by * kBlk; y < min(d.vy, (by + 1) * kBlk); ++y)
      for (int x = bx * kBlk; x < min(d.vx, (bx + 1) * kBlk); ++x) {
        const int64_t v = x + (int64_t)d.vx * (y + (int64_t)d.vy * z);
        for (int k = 0; k < 3; ++k) s += (double)f[k * d.nv + v] * f[k * d.nv + v];
        n += 3;
      }
  blk[b] = (float)(s / max(n, 1));
}

// Local rms per vertex: its block's rms, floored at 1e-2 of the global rms
// (gsum = sum of squares over the 3 nv entries).
__global__ void k_local_rms(LevelDims d, const float* __restrict__ blk, const double* __restrict__ gsum,
                            float* __restrict__ out) {
  const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= d.nv) return;
  const int nbx = (d.vx + kBlk - 1) / kBlk, nby = (d.vy + kBlk - 1) / kBlk;
  const int x = (int)(v % d.vx), y = (int)((v / d.vx) % d.vy), z = (int)(v / ((int64_t)d.vx * d.vy));
  const int64_t b = x / kBlk + (int64_t)nbx * (y / kBlk + (int64_t)nby * (z / kBlk));
  const double floor2 = 1e-4 * (*gsum / (3.0 * d.nv));
  const double ms = fmax((double)blk[b], floor2);
  out[v] = ms > 0 ? (float)sqrt(ms) : 1.f;
}

// a <- b - a
__global__ void k_sub_into(int64_t n, const float* __restrict__ b, float* __restrict__ a) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) a[i] = b[i] - a[i];
}

// z += beta c, beta = num / den clamped to [-2, 2] (0 if den <= 0); beta kept in *beta_out.
__global__ void k_axpy_ratio(int64_t n, const double* __restrict__ num, const double* __restrict__ den,
                             const float* __restrict__ c, float* __restrict__ z, double* __restrict__ beta_out) {
  const double dd = *den;
  double beta = dd > 0 ? *num / dd : 0.0;
  beta = fmin(fmax(beta, -2.0), 2.0);
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) z[i] += (float)beta * c[i];
  if (i == 0) *beta_out = beta;
}

// Positivity guard: if r.z <= 0 after the correction, restore the plain
// V-cycle output and set the sticky rejection flag.
__global__ void k_guard(int64_t n, const double* __restrict__ rz, const float* __restrict__ zsave,
                        float* __restrict__ z, int* __restrict__ flag) {
  if (!(*rz > 0.0)) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) z[i] = zsave[i];
    if (i == 0) *flag = 1;
  }
}

// Full-grid network input: channels 0-2 = s(r / lr), 3-5 = s(z / lz),
// 6 = log-density, 7-15 = 0.
__global__ void k_pack_input_dev(LevelDims d, int X, int Y, int Z, const float* __restrict__ r,
                                 const float* __restrict__ zin, const float* __restrict__ lrr,
                                 const float* __restrict__ lzz, const float* __restrict__ lr,
                                 __nv_bfloat16* __restrict__ x0) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (int64_t)X * Y * Z) return;
  const int x = (int)(i % X), y = (int)((i / X) % Y), z = (int)(i / ((int64_t)X * Y));
  __align__(16) __nv_bfloat16 c[16];
  for (int k = 0; k < 16; ++k) c[k] = __float2bfloat16_rn(0.f);
  if (x < d.vx && y < d.vy && z < d.vz) {
    const int64_t v = x + (int64_t)d.vx * (y + (int64_t)d.vy * z);
    const float ir = 1.f / lrr[v], iz = 1.f / lzz[v];
    for (int k = 0; k < 3; ++k) {
      c[k] = __float2bfloat16_rn(squash(r[k * d.nv + v] * ir));
      c[3 + k] = __float2bfloat16_rn(squash(zin[k * d.nv + v] * iz));
    }
    c[6] = __float2bfloat16_rn(lr[v]);
  }
  uint4* dst = reinterpret_cast<uint4*>(x0 + i * 16);
  dst[0] = reinterpret_cast<const uint4*>(c)[0];
  dst[1] = reinterpret_cast<const uint4*>(c)[1];
}

// Crop extraction: crop j (origin org[j]) of side S into dataset slot slot0 + j:
// X[slot][v][8] = (s(r/lr), s(z/lz), log-density, 0), T[slot][v][3] = t / lz, M[slot][v] = vmask.
__global__ void k_crop(LevelDims d, int S, const int* __restrict__ org, int ncrop, int slot0,
                       const float* __restrict__ r, const float* __restrict__ zk, const float* __restrict__ t,
                       const float* __restrict__ lrr, const float* __restrict__ lzz, const float* __restrict__ lr,
                       const uint8_t* __restrict__ vmask, __nv_bfloat16* __restrict__ DX, float* __restrict__ DT,
                       uint8_t* __restrict__ DM) {
  const int64_t per = (int64_t)S * S * S;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= per * ncrop) return;
  const int j = (int)(i / per);
  const int64_t q = i - j * per;
  const int cx = (int)(q % S), cy = (int)((q / S) % S), cz = (int)(q / ((int64_t)S * S));
  const int x = org[3 * j] + cx, y = org[3 * j + 1] + cy, z = org[3 * j + 2] + cz;
  const int64_t o = (int64_t)(slot0 + j) * per + q;
  float in[kInUsed] = {0, 0, 0, 0, 0, 0, 0, 0}, tv[3] = {0, 0, 0};
  uint8_t m = 0;
  if (x < d.vx && y < d.vy && z < d.vz) {
    const int64_t v = x + (int64_t)d.vx * (y + (int64_t)d.vy * z);
    m = vmask[v];
    const float ir = 1.f / lrr[v], iz = 1.f / lzz[v];
    for (int k = 0; k < 3; ++k) {
      in[k] = squash(r[k * d.nv + v] * ir);
      in[3 + k] = squash(zk[k * d.nv + v] * iz);
      tv[k] = t[k * d.nv + v] * iz;
    }
    in[6] = lr[v];
  }
  for (int k = 0; k < kInUsed; ++k) DX[o * kInUsed + k] = __float2bfloat16_rn(in[k]);
  for (int k = 0; k < 3; ++k) DT[o * 3 + k] = tv[k];
  DM[o] = m;
}

// Training batch from dataset slots idx[b].
__global__ void k_gather(int64_t per, const int* __restrict__ idx, int nb, const __nv_bfloat16* __restrict__ DX,
                         const float* __restrict__ DT, const uint8_t* __restrict__ DM,
                         __nv_bfloat16* __restrict__ x0, float* __restrict__ T, uint8_t* __restrict__ M) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= per * nb) return;
  const int b = (int)(i / per);
  const int64_t q = i - b * per, s = (int64_t)idx[b] * per + q;
  __align__(16) __nv_bfloat16 c[16];
  for (int k = 0; k < 16; ++k) c[k] = __float2bfloat16_rn(0.f);
  for (int k = 0; k < kInUsed; ++k) c[k] = DX[s * kInUsed + k];
  uint4* dst = reinterpret_cast<uint4*>(x0 + i * 16);
  dst[0] = reinterpret_cast<const uint4*>(c)[0];
  dst[1] = reinterpret_cast<const uint4*>(c)[1];
  for (int k = 0; k < 3; ++k) T[i * 3 + k] = DT[s * 3 + k];
  M[i] = DM[s];
}

// Host-tensor input: x[v][8] fp32 -> x0[v][16] bf16.
__global__ void k_expand_input(int64_t n, const float* __restrict__ x, __nv_bfloat16* __restrict__ x0) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  for (int k = 0; k < 16; ++k) x0[i * 16 + k] = __float2bfloat16_rn(k < kInUsed ? x[i * kInUsed + k] : 0.f);
}

__global__ void k_extract_output(int64_t n, const __nv_bfloat16* __restrict__ out, float* __restrict__ y) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  for (int k = 0; k < 3; ++k) y[i * 3 + k] = __bfloat162float(out[i * 16 + k]);
}

// Relative squared error sum m (p - t)^2 / sum m t^2 over free DOFs (mask bits
// 0-2): pass 1 writes per-block partials (num, den).
__global__ void k_loss_partial(int64_t n, const __nv_bfloat16* __restrict__ out, const float* __restrict__ T,
                               const uint8_t* __restrict__ M, double* __restrict__ part) {
  __shared__ double sn[256], sd[256];
  double a = 0, b = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const uint8_t m = M[i];
    for (int k = 0; k < 3; ++k) {
      if (!((m >> k) & 1)) continue;
      const double p = __bfloat162float(out[i * 16 + k]), t = T[i * 3 + k];
      a += (p - t) * (p - t);
      b += t * t;
    }
  }
  sn[threadIdx.x] = a;
  sd[threadIdx.x] = b;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) { sn[threadIdx.x] += sn[threadIdx.x + o]; sd[threadIdx.x] += sd[threadIdx.x + o]; }
    __syncthreads();
  }
  if (threadIdx.x == 0) { part[2 * blockIdx.x] = sn[0]; part[2 * blockIdx.x + 1] = sd[0]; }
}

// res[0..2] = numerator, denominator and their ratio (the reported loss).
// With ema, the gradient's normaliser res[3] is a running average of the
// batch denominators (heavy-tailed targets make a per-batch one erratic).
__global__ void k_loss_final(const double* __restrict__ part, int nblk, double* __restrict__ res, double* loss_log,
                             double* ema) {
  double a = 0, b = 0;
  for (int i = 0; i < nblk; ++i) { a += part[2 * i]; b += part[2 * i + 1]; }
  res[0] = a;
  res[1] = b;
  res[2] = b > 0 ? a / b : 0.0;
  res[3] = b;
  if (ema) {
    *ema = *ema > 0 ? 0.98 * *ema + 0.02 * b : b;
    res[3] = *ema;
  }
  if (loss_log) *loss_log = res[2];
}

// dL/dout = 2 m (p - t) / res[3] on channels 0-2, 0 elsewhere (fp32 [n][16]).
__global__ void k_loss_grad(int64_t n, const __nv_bfloat16* __restrict__ out, const float* __restrict__ T,
                            const uint8_t* __restrict__ M, const double* __restrict__ res, float* __restrict__ g) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double den = res[3];
  const float s = den > 0 ? (float)(2.0 / den) : 0.f;
  const uint8_t m = M[i];
  for (int k = 0; k < 16; ++k) {
    float v = 0.f;
    if (k < 3 && ((m >> k) & 1)) v = s * (__bfloat162float(out[i * 16 + k]) - T[i * 3 + k]);
    g[i * 16 + k] = v;
  }
}

// t = (u* - x_k) - z_k (fp32, [3][nv])
__global__ void k_harvest_target(int64_t n, const double* __restrict__ ustar, const float* __restrict__ xk,
                                 const float* __restrict__ zk, float* __restrict__ t) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  t[i] = (float)(ustar[i] - (double)xk[i]) - zk[i];
}

template <typename T>
__global__ void k_to_f32(int64_t n, const T* __restrict__ a, float* __restrict__ b) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) b[i] = (float)a[i];
}

}  // namespace

// ---- network state ---------------------------------------------------------

struct UNetWork {
  int X = 0, Y = 0, Z = 0, nb = 0;
  __nv_bfloat16 *x0 = nullptr, *a[NLAYER] = {nullptr}, *p0 = nullptr, *p1 = nullptr, *G = nullptr;
  float *gout = nullptr, *gA = nullptr, *gB = nullptr, *gs0 = nullptr, *gs1 = nullptr;
  float* T = nullptr;
  uint8_t* M = nullptr;
  std::vector<void*> blocks;
  bool training = false;
  ~UNetWork() { for (void* p : blocks) cudaFree(p); }
  template <typename P>
  cudaError_t alloc(P** p, size_t count) {
    void* q = nullptr;
    const cudaError_t e = cudaMalloc(&q, std::max<size_t>(count * sizeof(P), 256));
    if (e != cudaSuccess) return e;
    blocks.push_back(q);
    *p = static_cast<P*>(q);
    return cudaSuccess;
  }
};

struct UNetState {
  size_t woff[NLAYER], boff[NLAYER], nparam = 0;
  float *w = nullptr, *m = nullptr, *v = nullptr, *grad = nullptr;
  __nv_bfloat16 *wb = nullptr, *wt = nullptr;
  float* part = nullptr;    // weight-gradient partials
  float* bpart = nullptr;   // bias-gradient partials
  double *lpart = nullptr, *lres = nullptr, *loss_log = nullptr;
  double* dsum = nullptr;   // reduction outputs (4 doubles)
  double* dpart = nullptr;  // reduction partials
  int step = 0;
  int groups = 16;
  int conv_kind = 0;        // 3x3x3 convolutions: 0 mma.sync (measured faster here), 1 tcgen05 + TMA
  std::unique_ptr<UNetWork> full, batch;
  // dataset of crops
  int S = 32, cap = 0, count = 0, next = 0;
  __nv_bfloat16* DX = nullptr;
  float* DT = nullptr;
  uint8_t* DM = nullptr;
  int* dorg = nullptr;
  int* didx = nullptr;
  // harvest buffers
  float* lr = nullptr;     // vertex log-density [nv]
  float *lfr = nullptr, *lfz = nullptr;  // local rms of r and z per vertex [nv]
  float* blk = nullptr;                  // block mean squares
  float *cbuf = nullptr, *az = nullptr, *ac = nullptr;  // correction, A z, A c [3nv]
  float* zsave = nullptr;  // plain V-cycle output kept for the positivity guard [3nv]
  int* reject = nullptr;   // sticky flag: the guard restored the plain output
  std::vector<float*> hr, hz, hx;
  int hcount = 0, hcap = 0;
  uint64_t rng = 0x5eedull;
  std::vector<void*> blocks;
  ~UNetState() {
    for (void* p : blocks) cudaFree(p);
    for (auto* vv : {&hr, &hz, &hx})
      for (float* p : *vv) cudaFree(p);
  }
  template <typename P>
  cudaError_t alloc(P** p, size_t count) {
    void* q = nullptr;
    const cudaError_t e = cudaMalloc(&q, std::max<size_t>(count * sizeof(P), 256));
    if (e != cudaSuccess) return e;
    blocks.push_back(q);
    *p = static_cast<P*>(q);
    return cudaSuccess;
  }
};

#define UCK(call)                                   \
  do {                                              \
    cudaError_t e_ = (call);                        \
    if (e_ != cudaSuccess) return e_;               \
  } while (0)

size_t unet_param_count() {
  size_t n = 0;
  for (int l = 0; l < NLAYER; ++l) n += (size_t)kDef[l].cout * 27 * kDef[l].cin + kDef[l].cout;
  return n;
}

static cudaError_t unet_new(UNetState** out) {
  std::unique_ptr<UNetState> u(new UNetState);
  size_t o = 0;
  for (int l = 0; l < NLAYER; ++l) {
    u->woff[l] = o;
    o += (size_t)kDef[l].cout * 27 * kDef[l].cin;
    u->boff[l] = o;
    o += kDef[l].cout;
  }
  u->nparam = o;
  UCK(u->alloc(&u->w, o));
  UCK(u->alloc(&u->m, o));
  UCK(u->alloc(&u->v, o));
  UCK(u->alloc(&u->grad, o));
  UCK(u->alloc(&u->wb, o));
  UCK(u->alloc(&u->wt, o));
  UCK(u->alloc(&u->part, (size_t)u->groups * 27 * 64 * 32));
  UCK(u->alloc(&u->bpart, (size_t)512 * 64));
  UCK(u->alloc(&u->lpart, 2 * 1024));
  UCK(u->alloc(&u->lres, 8));
  UCK(cudaMemset(u->lres, 0, 8 * sizeof(double)));
  UCK(u->alloc(&u->loss_log, 1 << 16));
  UCK(u->alloc(&u->dsum, 4));
  UCK(u->alloc(&u->dpart, 4096));
  *out = u.release();
  return cudaSuccess;
}

void unet_free(UNetState* u) { delete u; }

// He-normal weights on the real channels, zero last layer and biases.
static cudaError_t unet_init_host(UNetState* u, cudaStream_t s, uint64_t seed) {
  std::vector<float> w(u->nparam, 0.f);
  uint64_t st = seed ? seed : 1;
  for (int l = 0; l < NLAYER; ++l) {
    if (l == D0B) continue;
    const LayerDef& L = kDef[l];
    const double sd = std::sqrt(2.0 / (27.0 * L.cin_real));
    for (int n = 0; n < L.cout_real; ++n)
      for (int t = 0; t < 27; ++t)
        for (int c = 0; c < L.cin_real; ++c) {
          const double u1 = std::max(uniform01(st), 1e-300), u2 = uniform01(st);
          w[u->woff[l] + ((size_t)n * 27 + t) * L.cin + c] = (float)(sd * std::sqrt(-2 * std::log(u1)) * std::cos(2 * M_PI * u2));
        }
  }
  UCK(cudaMemcpyAsync(u->w, w.data(), sizeof(float) * u->nparam, cudaMemcpyHostToDevice, s));
  UCK(cudaMemsetAsync(u->m, 0, sizeof(float) * u->nparam, s));
  UCK(cudaMemsetAsync(u->v, 0, sizeof(float) * u->nparam, s));
  unet_to_bf16(s, u->w, (int64_t)u->nparam, u->wb);
  u->step = 0;
  return cudaStreamSynchronize(s);
}

static cudaError_t work_alloc(UNetWork* w, int X, int Y, int Z, int nb, bool training) {
  w->X = X; w->Y = Y; w->Z = Z; w->nb = nb; w->training = training;
  const size_t V0 = (size_t)nb * X * Y * Z, V1 = V0 / 8, V2 = V0 / 64;
  UCK(w->alloc(&w->x0, V0 * 16));
  const size_t sizes[NLAYER] = {V0 * 16, V0 * 16, V1 * 32, V1 * 32, V2 * 64, V2 * 32, V1 * 32, V1 * 16, V0 * 16, V0 * 16};
  for (int l = 0; l < NLAYER; ++l) UCK(w->alloc(&w->a[l], sizes[l]));
  UCK(w->alloc(&w->p0, V1 * 16));
  UCK(w->alloc(&w->p1, V2 * 32));
  if (training) {
    UCK(w->alloc(&w->G, V0 * 32));
    UCK(w->alloc(&w->gout, V0 * 16));
    UCK(w->alloc(&w->gA, V0 * 32));
    UCK(w->alloc(&w->gB, V0 * 32));
    UCK(w->alloc(&w->gs0, V0 * 16));
    UCK(w->alloc(&w->gs1, V1 * 32));
    UCK(w->alloc(&w->T, V0 * 3));
    UCK(w->alloc(&w->M, V0));
  }
  return cudaSuccess;
}

// One 3x3x3 convolution through the kernel the state selects.
static cudaError_t conv_any(const UNetState* u, cudaStream_t s, int cin, int cout, const __nv_bfloat16* s1,
                            const __nv_bfloat16* s2, int c1, int up1, const __nv_bfloat16* W, const float* bias, int X,
                            int Y, int Z, int nb, int relu, int out_mode, void* out) {
  if (u->conv_kind == 1) return unet_conv_tc(s, cin, cout, s1, s2, c1, up1, W, bias, X, Y, Z, nb, relu, out_mode, out);
  return unet_conv(s, cin, cout, s1, s2, c1, up1, W, bias, X, Y, Z, nb, relu, out_mode, out);
}

static cudaError_t conv_layer(UNetState* u, cudaStream_t s, int l, const __nv_bfloat16* s1, const __nv_bfloat16* s2,
                              int c1, int up1, int X, int Y, int Z, int nb, __nv_bfloat16* out) {
  const LayerDef& L = kDef[l];
  return conv_any(u, s, L.cin, L.cout, s1, s2, c1, up1, u->wb + u->woff[l], u->w + u->boff[l], X, Y, Z, nb, L.relu,
                  0, out);
}

// Forward pass on w->x0 (dims X, Y, Z per volume, nb volumes); output w->a[D0B].
static cudaError_t unet_forward(UNetState* u, cudaStream_t s, UNetWork* w) {
  const int X = w->X, Y = w->Y, Z = w->Z, nb = w->nb;
  const int X1 = X / 2, Y1 = Y / 2, Z1 = Z / 2, X2 = X / 4, Y2 = Y / 4, Z2 = Z / 4;
  UCK(conv_layer(u, s, L0A, nullptr, w->x0, 0, 0, X, Y, Z, nb, w->a[L0A]));
  UCK(conv_layer(u, s, L0B, nullptr, w->a[L0A], 0, 0, X, Y, Z, nb, w->a[L0B]));
  unet_pool(s, w->a[L0B], X, Y, Z, nb, 16, w->p0);
  UCK(conv_layer(u, s, L1A, nullptr, w->p0, 0, 0, X1, Y1, Z1, nb, w->a[L1A]));
  UCK(conv_layer(u, s, L1B, nullptr, w->a[L1A], 0, 0, X1, Y1, Z1, nb, w->a[L1B]));
  unet_pool(s, w->a[L1B], X1, Y1, Z1, nb, 32, w->p1);
  UCK(conv_layer(u, s, L2A, nullptr, w->p1, 0, 0, X2, Y2, Z2, nb, w->a[L2A]));
  UCK(conv_layer(u, s, L2B, nullptr, w->a[L2A], 0, 0, X2, Y2, Z2, nb, w->a[L2B]));
  UCK(conv_layer(u, s, D1A, w->a[L2B], w->a[L1B], 32, 1, X1, Y1, Z1, nb, w->a[D1A]));
  UCK(conv_layer(u, s, D1B, nullptr, w->a[D1A], 0, 0, X1, Y1, Z1, nb, w->a[D1B]));
  UCK(conv_layer(u, s, D0A, w->a[D1B], w->a[L0B], 16, 1, X, Y, Z, nb, w->a[D0A]));
  UCK(conv_layer(u, s, D0B, nullptr, w->a[D0A], 0, 0, X, Y, Z, nb, w->a[D0B]));
  count_launch(12);
  return cudaGetLastError();
}

// One layer's backward: G = dY (.) relu'(Y); weight and bias gradients; data
// gradient into dX (fp32, cin channels) when dX != nullptr.
static cudaError_t layer_bwd(UNetState* u, cudaStream_t s, UNetWork* w, int l, const float* dY,
                             const __nv_bfloat16* Yact, const __nv_bfloat16* s1, const __nv_bfloat16* s2, int c1,
                             int up1, int X, int Y, int Z, float* dX) {
  const LayerDef& L = kDef[l];
  const int64_t nvox = (int64_t)w->nb * X * Y * Z;
  unet_relu_grad(s, dY, Yact, nvox * L.cout, L.relu, w->G);
  UCK(unet_wgrad(s, L.cin, L.cout, s1, s2, c1, up1, w->G, X, Y, Z, w->nb, u->groups, u->part, u->grad + u->woff[l]));
  const int nblk = (int)std::min<int64_t>(512, std::max<int64_t>(1, nvox / 64));
  unet_bias_grad(s, w->G, nvox, L.cout, u->bpart, nblk, u->grad + u->boff[l]);
  count_launch(5);
  if (dX) {
    unet_flip(s, u->wb + u->woff[l], L.cin, L.cout, u->wt + u->woff[l]);
    UCK(conv_any(u, s, L.cout, L.cin, nullptr, w->G, 0, 0, u->wt + u->woff[l], nullptr, X, Y, Z, w->nb, 0, 1, dX));
    count_launch(2);
  }
  return cudaGetLastError();
}

// Backward from w->gout (dL/d output, fp32 [V0][16]); gradients into u->grad.
static cudaError_t unet_backward(UNetState* u, cudaStream_t s, UNetWork* w) {
  const int X = w->X, Y = w->Y, Z = w->Z, nb = w->nb;
  const int X1 = X / 2, Y1 = Y / 2, Z1 = Z / 2, X2 = X / 4, Y2 = Y / 4, Z2 = Z / 4;
  const int64_t V0 = (int64_t)nb * X * Y * Z, V1 = V0 / 8;
  UCK(layer_bwd(u, s, w, D0B, w->gout, w->a[D0B], nullptr, w->a[D0A], 0, 0, X, Y, Z, w->gA));
  UCK(layer_bwd(u, s, w, D0A, w->gA, w->a[D0A], w->a[D1B], w->a[L0B], 16, 1, X, Y, Z, w->gB));
  unet_slice(s, w->gB, V0, 32, 16, 16, 0, w->gs0);
  unet_up_bwd(s, w->gB, X, Y, Z, nb, 32, 16, w->gA);  // d d1 [V1][16]
  UCK(layer_bwd(u, s, w, D1B, w->gA, w->a[D1B], nullptr, w->a[D1A], 0, 0, X1, Y1, Z1, w->gB));
  UCK(layer_bwd(u, s, w, D1A, w->gB, w->a[D1A], w->a[L2B], w->a[L1B], 32, 1, X1, Y1, Z1, w->gA));
  unet_slice(s, w->gA, V1, 64, 32, 32, 0, w->gs1);
  unet_up_bwd(s, w->gA, X1, Y1, Z1, nb, 64, 32, w->gB);  // d b2 [V2][32]
  UCK(layer_bwd(u, s, w, L2B, w->gB, w->a[L2B], nullptr, w->a[L2A], 0, 0, X2, Y2, Z2, w->gA));
  UCK(layer_bwd(u, s, w, L2A, w->gA, w->a[L2A], nullptr, w->p1, 0, 0, X2, Y2, Z2, w->gB));
  unet_pool_bwd(s, w->gB, X1, Y1, Z1, nb, 32, 1, w->gs1);
  UCK(layer_bwd(u, s, w, L1B, w->gs1, w->a[L1B], nullptr, w->a[L1A], 0, 0, X1, Y1, Z1, w->gA));
  UCK(layer_bwd(u, s, w, L1A, w->gA, w->a[L1A], nullptr, w->p0, 0, 0, X1, Y1, Z1, w->gB));
  unet_pool_bwd(s, w->gB, X, Y, Z, nb, 16, 1, w->gs0);
  UCK(layer_bwd(u, s, w, L0B, w->gs0, w->a[L0B], nullptr, w->a[L0A], 0, 0, X, Y, Z, w->gA));
  UCK(layer_bwd(u, s, w, L0A, w->gA, w->a[L0A], nullptr, w->x0, 0, 0, X, Y, Z, nullptr));
  count_launch(6);
  return cudaGetLastError();
}

static cudaError_t unet_loss(UNetState* u, cudaStream_t s, UNetWork* w, double* loss_slot, bool ema) {
  const int64_t n = (int64_t)w->nb * w->X * w->Y * w->Z;
  const int nblk = (int)std::min<int64_t>(1024, std::max<int64_t>(1, (n + 255) / 256));
  k_loss_partial<<<nblk, 256, 0, s>>>(n, w->a[D0B], w->T, w->M, u->lpart);
  k_loss_final<<<1, 1, 0, s>>>(u->lpart, nblk, u->lres, loss_slot, ema ? u->lres + 4 : nullptr);
  k_loss_grad<<<nb256(n), 256, 0, s>>>(n, w->a[D0B], w->T, w->M, u->lres, w->gout);
  count_launch(3);
  return cudaGetLastError();
}

static cudaError_t ensure_work(std::unique_ptr<UNetWork>& w, int X, int Y, int Z, int nb, bool training) {
  if (w && w->X == X && w->Y == Y && w->Z == Z && w->nb == nb && (w->training || !training)) return cudaSuccess;
  w.reset(new UNetWork);
  return work_alloc(w.get(), X, Y, Z, nb, training);
}

static inline int pad8(int v) { return (v + 7) / 8 * 8; }

// ---- solver hooks ------------------------------------------------------------

// Vertex log-density of the current design (called once per solve).
cudaError_t unet_prepare(UNetState* u, cudaStream_t s, const LevelDims& d, const uint8_t* eactive, const double* rho,
                         double rho_min) {
  if (!u->lr) UCK(u->alloc(&u->lr, d.nv));
  if (!u->zsave) UCK(u->alloc(&u->zsave, 3 * d.nv));
  if (!u->reject) UCK(u->alloc(&u->reject, 1));
  if (!u->lfr) UCK(u->alloc(&u->lfr, d.nv));
  if (!u->lfz) UCK(u->alloc(&u->lfz, d.nv));
  if (!u->cbuf) UCK(u->alloc(&u->cbuf, 3 * d.nv));
  if (!u->az) UCK(u->alloc(&u->az, 3 * d.nv));
  if (!u->ac) UCK(u->alloc(&u->ac, 3 * d.nv));
  if (!u->blk) {
    const int64_t nb = (int64_t)((d.vx + kBlk - 1) / kBlk) * ((d.vy + kBlk - 1) / kBlk) * ((d.vz + kBlk - 1) / kBlk);
    UCK(u->alloc(&u->blk, nb));
  }
  UCK(cudaMemsetAsync(u->reject, 0, sizeof(int), s));
  k_vertex_logrho<<<nb256(d.nv), 256, 0, s>>>(d, eactive, rho, rho_min, u->lr);
  count_launch();
  UCK(ensure_work(u->full, pad8(d.vx), pad8(d.vy), pad8(d.vz), 1, false));
  return cudaGetLastError();
}

// out[v] = local rms of the [3][nv] field f (blocks of kBlk^3 vertices, floored
// at 1e-2 of the global rms); gsum: a device double for the global sum of squares.
static void local_rms(UNetState* u, cudaStream_t s, const LevelDims& d, const float* f, float* out, double* partial,
                      double* gsum) {
  const int64_t nb = (int64_t)((d.vx + kBlk - 1) / kBlk) * ((d.vy + kBlk - 1) / kBlk) * ((d.vz + kBlk - 1) / kBlk);
  k_block_ms<<<nb256(nb), 256, 0, s>>>(d, f, u->blk);
  launch_dot<float>(s, f, f, 3 * d.nv, partial, gsum);
  k_local_rms<<<nb256(d.nv), 256, 0, s>>>(d, u->blk, gsum, out);
  count_launch(4);
}

// z += beta lz N(s(r / lr), s(z / lz), log rho) on free DOFs (fp32 [3][nv]
// vectors), beta energy-optimal; rhop32 and tz: the FP32 fine operator.
cudaError_t unet_apply(UNetState* u, cudaStream_t s, const LevelDims& d, const uint8_t* vmask, const float* rhop32,
                       int tz, const float* r, float* z, double* partial) {
  UNetWork* w = u->full.get();
  const int64_t n3 = 3 * d.nv;
  UCK(cudaMemcpyAsync(u->zsave, z, sizeof(float) * n3, cudaMemcpyDeviceToDevice, s));
  local_rms(u, s, d, r, u->lfr, partial, u->dsum);
  local_rms(u, s, d, z, u->lfz, partial, u->dsum + 1);
  k_pack_input_dev<<<nb256((int64_t)w->X * w->Y * w->Z), 256, 0, s>>>(d, w->X, w->Y, w->Z, r, z, u->lfr, u->lfz,
                                                                      u->lr, w->x0);
  count_launch();
  UCK(unet_forward(u, s, w));
  UCK(cudaMemsetAsync(u->cbuf, 0, sizeof(float) * n3, s));
  k_unpack_add<<<nb256(d.nv), 256, 0, s>>>(d, w->X, w->Y, w->a[D0B], vmask, u->lfz, u->cbuf);
  // energy-optimal amount of the correction
  launch_fine_apply<float>(s, d, rhop32, vmask, z, nullptr, u->az, false, 1, tz);
  launch_fine_apply<float>(s, d, rhop32, vmask, u->cbuf, nullptr, u->ac, false, 1, tz);
  k_sub_into<<<nb256(n3), 256, 0, s>>>(n3, r, u->az);  // az <- r - A z
  launch_dot<float>(s, u->cbuf, u->az, n3, partial, u->dsum);
  launch_dot<float>(s, u->cbuf, u->ac, n3, partial, u->dsum + 1);
  k_axpy_ratio<<<nb256(n3), 256, 0, s>>>(n3, u->dsum, u->dsum + 1, u->cbuf, z, u->dsum + 3);
  launch_dot<float>(s, r, z, n3, partial, u->dsum + 2);
  k_guard<<<nb256(n3), 256, 0, s>>>(n3, u->dsum + 2, u->zsave, z, u->reject);
  count_launch(12);
  return cudaGetLastError();
}

// Whether the positivity guard fired since unet_prepare (blocking read).
cudaError_t unet_rejected(UNetState* u, cudaStream_t s, int* out) {
  *out = 0;
  if (!u->reject) return cudaSuccess;
  UCK(cudaMemcpyAsync(out, u->reject, sizeof(int), cudaMemcpyDeviceToHost, s));
  return cudaStreamSynchronize(s);
}

// Record one outer iterate for harvesting: r_k (fp64), z_k = V(r_k) (fp32), x_k (fp64).
cudaError_t unet_harvest_record(UNetState* u, cudaStream_t s, int64_t n3, const double* r, const float* z,
                                const double* x, int cap) {
  if (u->hcount >= cap) return cudaSuccess;
  if ((int)u->hr.size() <= u->hcount) {
    float *a = nullptr, *b = nullptr, *c = nullptr;
    UCK(cudaMalloc(&a, sizeof(float) * n3));
    UCK(cudaMalloc(&b, sizeof(float) * n3));
    UCK(cudaMalloc(&c, sizeof(float) * n3));
    u->hr.push_back(a);
    u->hz.push_back(b);
    u->hx.push_back(c);
  }
  k_to_f32<double><<<nb256(n3), 256, 0, s>>>(n3, r, u->hr[u->hcount]);
  UCK(cudaMemcpyAsync(u->hz[u->hcount], z, sizeof(float) * n3, cudaMemcpyDeviceToDevice, s));
  k_to_f32<double><<<nb256(n3), 256, 0, s>>>(n3, x, u->hx[u->hcount]);
  count_launch(2);
  ++u->hcount;
  return cudaGetLastError();
}

// After the solve: targets from u*, crops into the dataset (ring buffer).
cudaError_t unet_harvest_finish(UNetState* u, cudaStream_t s, const LevelDims& d, const uint8_t* vmask,
                                const double* ustar, int crops_per_iterate, double* partial) {
  const int64_t n3 = 3 * d.nv;
  if (u->cap == 0 || u->hcount == 0) { u->hcount = 0; return cudaSuccess; }
  const int S = u->S;
  std::vector<int> org(3 * crops_per_iterate);
  for (int k = 0; k < u->hcount; ++k) {
    float* t = u->hx[k];  // reuse x_k's buffer for the target
    k_harvest_target<<<nb256(n3), 256, 0, s>>>(n3, ustar, u->hx[k], u->hz[k], t);
    count_launch();
    local_rms(u, s, d, u->hr[k], u->lfr, partial, u->dsum);
    local_rms(u, s, d, u->hz[k], u->lfz, partial, u->dsum + 1);
    for (int j = 0; j < crops_per_iterate; ++j) {
      org[3 * j] = (int)(uniform01(u->rng) * std::max(1, d.vx - S / 2)) - S / 4;
      org[3 * j + 1] = (int)(uniform01(u->rng) * std::max(1, d.vy - S / 2)) - S / 4;
      org[3 * j + 2] = (int)(uniform01(u->rng) * std::max(1, d.vz - S / 2)) - S / 4;
      for (int a = 0; a < 3; ++a) org[3 * j + a] = std::max(0, org[3 * j + a]);
    }
    int done = 0;
    while (done < crops_per_iterate) {
      const int slot = u->next;
      const int nc = std::min(crops_per_iterate - done, u->cap - slot);
      UCK(cudaMemcpyAsync(u->dorg, org.data() + 3 * done, sizeof(int) * 3 * nc, cudaMemcpyHostToDevice, s));
      const int64_t tot = (int64_t)S * S * S * nc;
      k_crop<<<nb256(tot), 256, 0, s>>>(d, S, u->dorg, nc, slot, u->hr[k], u->hz[k], t, u->lfr, u->lfz, u->lr,
                                        vmask, u->DX, u->DT, u->DM);
      count_launch();
      UCK(cudaStreamSynchronize(s));  // dorg is reused
      u->next = (slot + nc) % u->cap;
      u->count = std::min(u->cap, u->count + nc);
      done += nc;
    }
  }
  u->hcount = 0;
  return cudaGetLastError();
}

cudaError_t unet_dataset_reserve(UNetState* u, int cap, int S) {
  if (u->cap) return cudaErrorInvalidValue;
  const size_t per = (size_t)S * S * S;
  u->S = S;
  UCK(u->alloc(&u->DX, per * cap * kInUsed));
  UCK(u->alloc(&u->DT, per * cap * 3));
  UCK(u->alloc(&u->DM, per * cap));
  UCK(u->alloc(&u->dorg, 3 * 4096));
  UCK(u->alloc(&u->didx, 4096));
  u->cap = cap;
  u->count = u->next = 0;
  return cudaSuccess;
}

// Training steps on random batches of the first `limit` dataset crops (all if
// limit <= 0); lr = Adam step size.  loss_out: mean relative loss of the steps.
// After a synchronisation: whether a bounded wait of the tensor-core
// convolution gave up (cudaErrorLaunchTimeout) since the last check.
static cudaError_t conv_wait_status(const UNetState* u) {
  if (u->conv_kind != 1) return cudaSuccess;
  int flag = 0;
  UCK(conv_tc_error(&flag));
  return flag ? cudaErrorLaunchTimeout : cudaSuccess;
}

cudaError_t unet_train(UNetState* u, cudaStream_t s, int steps, int batch, double lr, uint64_t seed, int lo, int hi,
                       bool update, double* loss_out) {
  if (u->count == 0 || steps <= 0 || batch <= 0 || steps > (1 << 16) || batch > 4096) return cudaErrorInvalidValue;
  hi = hi <= 0 ? u->count : std::min(hi, u->count);
  lo = std::max(0, std::min(lo, hi - 1));
  const int S = u->S;
  UCK(ensure_work(u->batch, S, S, S, batch, true));
  UNetWork* w = u->batch.get();
  const int64_t per = (int64_t)S * S * S;
  uint64_t st = seed ? seed : 7;
  std::vector<int> idx(batch);
  // step size: linear warm-up over the first tenth of the steps (at most 100),
  // then a cosine decay to a tenth; gradients clipped to a global norm of 1
  const int warm = std::max(1, std::min(100, steps / 10));
  for (int it = 0; it < steps; ++it) {
    for (int b = 0; b < batch; ++b) idx[b] = lo + (int)(uniform01(st) * (hi - lo));
    UCK(cudaMemcpyAsync(u->didx, idx.data(), sizeof(int) * batch, cudaMemcpyHostToDevice, s));
    k_gather<<<nb256(per * batch), 256, 0, s>>>(per, u->didx, batch, u->DX, u->DT, u->DM, w->x0, w->T, w->M);
    count_launch();
    UCK(unet_forward(u, s, w));
    UCK(unet_loss(u, s, w, u->loss_log + it, update));
    if (update) {
      UCK(unet_backward(u, s, w));
      ++u->step;
      const double frac = it < warm ? (it + 1.0) / warm
                                    : 0.1 + 0.45 * (1.0 + std::cos(M_PI * (it - warm) / std::max(1, steps - warm)));
      launch_dot<float>(s, u->grad, u->grad, (int64_t)u->nparam, u->dpart, u->dsum + 3);
      unet_adam(s, (int64_t)u->nparam, u->grad, (float)(lr * frac), 0.9f, 0.999f, 1e-8f, u->step, u->w, u->m, u->v,
                u->wb, u->dsum + 3, 1.0f);
      count_launch(3);
    }
    UCK(cudaStreamSynchronize(s));  // idx is reused
  }
  UCK(conv_wait_status(u));
  std::vector<double> l(steps);
  UCK(cudaMemcpy(l.data(), u->loss_log, sizeof(double) * steps, cudaMemcpyDeviceToHost));
  double m = 0;
  for (double x : l) m += x;
  *loss_out = m / steps;
  return cudaSuccess;
}

// Host-tensor forward/loss/backward (checks and tools): x [nb][Z][Y][X][8].
cudaError_t unet_host_pass(UNetState* u, cudaStream_t s, int X, int Y, int Z, int nb, const float* x, const float* t,
                           const uint8_t* m, float* y, double* loss, float* grad) {
  const bool train = t != nullptr;
  std::unique_ptr<UNetWork> w;
  UCK(ensure_work(w, X, Y, Z, nb, train));
  const int64_t n = (int64_t)nb * X * Y * Z;
  float* xd = nullptr;
  UCK(cudaMalloc(&xd, sizeof(float) * n * kInUsed));
  cudaError_t e = cudaMemcpyAsync(xd, x, sizeof(float) * n * kInUsed, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) {
    k_expand_input<<<nb256(n), 256, 0, s>>>(n, xd, w->x0);
    count_launch();
    e = unet_forward(u, s, w.get());
  }
  if (e == cudaSuccess && y) {
    k_extract_output<<<nb256(n), 256, 0, s>>>(n, w->a[D0B], xd);
    count_launch();
    e = cudaMemcpyAsync(y, xd, sizeof(float) * n * 3, cudaMemcpyDeviceToHost, s);
  }
  if (e == cudaSuccess && train) {
    e = cudaMemcpyAsync(w->T, t, sizeof(float) * n * 3, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(w->M, m, n, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = unet_loss(u, s, w.get(), nullptr, false);
    if (e == cudaSuccess) e = unet_backward(u, s, w.get());
    if (e == cudaSuccess) e = cudaMemcpyAsync(grad, u->grad, sizeof(float) * u->nparam, cudaMemcpyDeviceToHost, s);
    double res[4];
    if (e == cudaSuccess) e = cudaMemcpyAsync(res, u->lres, sizeof(res), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e == cudaSuccess && loss) *loss = res[2];
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e == cudaSuccess) e = conv_wait_status(u);
  cudaFree(xd);
  return e;
}

int unet_conv_kernel(const UNetState* u) { return u->conv_kind; }
void unet_set_conv_kernel(UNetState* u, int kind) { u->conv_kind = kind; }

cudaError_t unet_create(UNetState** out, cudaStream_t s, uint64_t seed) {
  UNetState* u = nullptr;
  UCK(unet_new(&u));
  const cudaError_t e = unet_init_host(u, s, seed);
  if (e != cudaSuccess) { delete u; return e; }
  u->rng = seed ^ 0xC0FFEEull;
  *out = u;
  return cudaSuccess;
}

cudaError_t unet_set_params(UNetState* u, cudaStream_t s, const float* host) {
  UCK(cudaMemcpyAsync(u->w, host, sizeof(float) * u->nparam, cudaMemcpyHostToDevice, s));
  UCK(cudaMemsetAsync(u->m, 0, sizeof(float) * u->nparam, s));
  UCK(cudaMemsetAsync(u->v, 0, sizeof(float) * u->nparam, s));
  unet_to_bf16(s, u->w, (int64_t)u->nparam, u->wb);
  UCK(cudaMemsetAsync(u->lres, 0, 8 * sizeof(double), s));
  u->step = 0;
  return cudaStreamSynchronize(s);
}

cudaError_t unet_get_params(UNetState* u, cudaStream_t s, float* host) {
  UCK(cudaMemcpyAsync(host, u->w, sizeof(float) * u->nparam, cudaMemcpyDeviceToHost, s));
  return cudaStreamSynchronize(s);
}

int unet_dataset_count(const UNetState* u) { return u->count; }
int unet_crop_side(const UNetState* u) { return u->S; }

// Copy dataset crop `slot` to the host: x [S^3][8], t [S^3][3], m [S^3].
cudaError_t unet_dataset_get(UNetState* u, cudaStream_t s, int slot, float* x, float* t, uint8_t* m) {
  if (slot < 0 || slot >= u->count) return cudaErrorInvalidValue;
  const int64_t per = (int64_t)u->S * u->S * u->S;
  std::vector<__nv_bfloat16> xb(per * kInUsed);
  UCK(cudaMemcpyAsync(xb.data(), u->DX + slot * per * kInUsed, sizeof(__nv_bfloat16) * per * kInUsed,
                      cudaMemcpyDeviceToHost, s));
  UCK(cudaMemcpyAsync(t, u->DT + slot * per * 3, sizeof(float) * per * 3, cudaMemcpyDeviceToHost, s));
  UCK(cudaMemcpyAsync(m, u->DM + slot * per, per, cudaMemcpyDeviceToHost, s));
  UCK(cudaStreamSynchronize(s));
  for (int64_t i = 0; i < per * kInUsed; ++i) x[i] = __bfloat162float(xb[i]);
  return cudaSuccess;
}

}  // namespace topo
