// Learned preconditioner: a 3-level 3D convolutional U-Net on the vertex grid,
// trained on the GPU by the kernels in this file.
//
// Tensors are channels-last bf16 ("NDHWC"): element (b, z, y, x, c) at
// (((b*Z + z)*Y + y)*X + x)*C + c, several equal volumes stacked along z.  Each
// volume has its own zero padding, so training crops and the full grid use the
// same kernels.
//
// 3x3x3 convolution as an implicit GEMM on the tensor cores (mma.sync
// m16n8k16, bf16 x bf16 -> fp32):
//   M = output voxels (16 consecutive x per warp), N = output channels,
//   K = 27 taps x input channels.
// A CTA computes a 16(x) x 8(y) x 2(z) output tile.  It stages the input halo
// (18 x 10 x 4 voxels, all input channels) and the whole weight matrix
// [Cout][27*Cin] in shared memory with cp.async (zero fill outside the volume),
// then feeds the tensor cores with ldmatrix.  Rows of both smem arrays are
// padded by 8 bf16 so the 8 row addresses of every ldmatrix fall in distinct
// 16-byte bank groups.  Input channels may come from two tensors, a half-
// resolution one read through nearest upsampling and a full-resolution skip
// tensor, so the U-Net's upsample + concat never touches memory.
//
// Backward: the data gradient is the same convolution with flipped, transposed
// weights; the weight gradient is a GEMM over voxels (one CTA column per tap,
// per-CTA partials summed in a fixed order, so training is deterministic).
#include <cuda_bf16.h>

#include <cstdint>
#include <mutex>

#include "topo_internal.h"

namespace topo {

namespace {

constexpr int kTX = 16, kTY = 8, kTZ = 2;             // output tile
constexpr int kHX = kTX + 2, kHY = kTY + 2, kHZ = kTZ + 2;
constexpr int kHalo = kHX * kHY * kHZ;                 // 720 voxels
constexpr int kConvThreads = 256;                      // 8 warps, one y row each

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void cp_async16(void* dst, const void* src, bool valid) {
  const int n = valid ? 16 : 0;
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(smem_u32(dst)), "l"(src), "r"(n));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::); }

__device__ __forceinline__ void ldsm_x4(uint32_t& r0, uint32_t& r1, uint32_t& r2, uint32_t& r3, const void* p) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
               : "r"(smem_u32(p)));
}
__device__ __forceinline__ void ldsm_x4_t(uint32_t& r0, uint32_t& r1, uint32_t& r2, uint32_t& r3, const void* p) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
               : "r"(smem_u32(p)));
}

__device__ __forceinline__ void mma_bf16(float (&d)[4], uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3,
                                         uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

// Source of input channel block [c0, c0+8) at voxel (b, x, y, z): either the
// half-resolution tensor (channels [0, c1), nearest upsampling) or the skip
// tensor (channels [c1, cin)).  Returns nullptr outside the volume.
struct ConvIn {
  const __nv_bfloat16* s1;  // c1 channels; half resolution if up1
  const __nv_bfloat16* s2;  // cin - c1 channels, full resolution
  int c1, up1;
};

__device__ __forceinline__ const __nv_bfloat16* in_ptr(const ConvIn& in, int cin, int X, int Y, int Z, int b, int x,
                                                      int y, int z, int c0) {
  if (x < 0 || y < 0 || z < 0 || x >= X || y >= Y || z >= Z) return nullptr;
  if (c0 < in.c1) {
    if (in.up1) {
      const int hx = X >> 1, hy = Y >> 1, hz = Z >> 1;
      const int64_t v = (((int64_t)b * hz + (z >> 1)) * hy + (y >> 1)) * hx + (x >> 1);
      return in.s1 + v * in.c1 + c0;
    }
    const int64_t v = (((int64_t)b * Z + z) * Y + y) * X + x;
    return in.s1 + v * in.c1 + c0;
  }
  const int c2 = cin - in.c1;
  const int64_t v = (((int64_t)b * Z + z) * Y + y) * X + x;
  return in.s2 + v * c2 + (c0 - in.c1);
}

}  // namespace

// Output epilogue modes.
enum { kOutBf16 = 0, kOutF32 = 1, kOutF32Add = 2 };

template <int CIN, int COUT>
__global__ void __launch_bounds__(kConvThreads) k_conv3(ConvIn in, const __nv_bfloat16* __restrict__ W,
                                                       const float* __restrict__ bias, int X, int Y, int Z,
                                                       int relu, int out_mode, void* out) {
  static_assert(CIN % 16 == 0 && COUT % 16 == 0, "channel counts");
  constexpr int CS = CIN + 8;           // smem channel stride (bf16)
  constexpr int K = 27 * CIN;
  constexpr int KS = K + 8;             // smem weight row stride (bf16)
  constexpr int NT = COUT / 8;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __nv_bfloat16* hs = reinterpret_cast<__nv_bfloat16*>(smem_raw);       // [kHalo][CS]
  __nv_bfloat16* ws = hs + kHalo * CS;                                   // [COUT][KS]
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int x0 = blockIdx.x * kTX, y0 = blockIdx.y * kTY;
  const int zt = blockIdx.z * kTZ;            // global stacked z of the tile
  const int b = zt / Z, z0 = zt - b * Z;

  // ---- stage weights and the input halo
  constexpr int WCH = K / 8;                  // 16-byte chunks per weight row
  for (int i = tid; i < COUT * WCH; i += kConvThreads) {
    const int n = i / WCH, k8 = i - n * WCH;
    cp_async16(ws + n * KS + k8 * 8, W + (int64_t)n * K + k8 * 8, true);
  }
  constexpr int HCH = CIN / 8;
  for (int i = tid; i < kHalo * HCH; i += kConvThreads) {
    const int v = i / HCH, c8 = i - v * HCH;
    const int hx = v % kHX, hy = (v / kHX) % kHY, hz = v / (kHX * kHY);
    const __nv_bfloat16* src = in_ptr(in, CIN, X, Y, Z, b, x0 + hx - 1, y0 + hy - 1, z0 + hz - 1, c8 * 8);
    cp_async16(hs + v * CS + c8 * 8, src ? src : W, src != nullptr);
  }
  cp_async_commit();
  cp_async_wait_all();
  __syncthreads();

  // ---- implicit GEMM: warp = output row y0 + warp, 16 voxels along x
  const int g = lane >> 2, t = lane & 3;
  const int mrow = (lane & 7) + ((lane >> 3) & 1) * 8;   // A: voxel row of this lane's address
  const int acol = (lane >> 4) * 8;                       // A: channel offset
  const int brow = (lane & 7) + (lane >> 4) * 8;          // B: output-channel row within 16
  const int bcol = ((lane >> 3) & 1) * 8;                 // B: k offset
  for (int tz = 0; tz < kTZ; ++tz) {
    float acc[NT][4];
#pragma unroll
    for (int j = 0; j < NT; ++j) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.f;
    for (int tap = 0; tap < 27; ++tap) {
      const int dx = tap % 3, dy = (tap / 3) % 3, dz = tap / 9;
      const __nv_bfloat16* arow = hs + (((tz + dz) * kHY + (warp + dy)) * kHX + (mrow + dx)) * CS + acol;
      const __nv_bfloat16* brow_p = ws + brow * KS + tap * CIN + bcol;
#pragma unroll
      for (int kc = 0; kc < CIN / 16; ++kc) {
        uint32_t a0, a1, a2, a3;
        ldsm_x4(a0, a1, a2, a3, arow + kc * 16);
#pragma unroll
        for (int j = 0; j < NT / 2; ++j) {
          uint32_t b0, b1, b2, b3;
          ldsm_x4(b0, b1, b2, b3, brow_p + j * 16 * KS + kc * 16);
          mma_bf16(acc[2 * j], a0, a1, a2, a3, b0, b1);
          mma_bf16(acc[2 * j + 1], a0, a1, a2, a3, b2, b3);
        }
      }
    }
    // ---- epilogue
    const int y = y0 + warp, z = z0 + tz;
    if (y >= Y || z >= Z) continue;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int x = x0 + g + h * 8;
      if (x >= X) continue;
      const int64_t v = (((int64_t)b * Z + z) * Y + y) * X + x;
#pragma unroll
      for (int j = 0; j < NT; ++j) {
        const int n = j * 8 + 2 * t;
        float o0 = acc[j][2 * h], o1 = acc[j][2 * h + 1];
        if (bias) { o0 += bias[n]; o1 += bias[n + 1]; }
        if (relu) { o0 = fmaxf(o0, 0.f); o1 = fmaxf(o1, 0.f); }
        if (out_mode == kOutBf16) {
          *reinterpret_cast<__nv_bfloat162*>(static_cast<__nv_bfloat16*>(out) + v * COUT + n) =
              __floats2bfloat162_rn(o0, o1);
        } else {
          float2* o = reinterpret_cast<float2*>(static_cast<float*>(out) + v * COUT + n);
          if (out_mode == kOutF32Add) { const float2 p = *o; o0 += p.x; o1 += p.y; }
          *o = make_float2(o0, o1);
        }
      }
    }
  }
}

// Weight gradient: dW[n][tap*CIN + c] = sum_v G[v][n] * In[v + tap][c], G the
// pre-activation gradient (bf16, COUT channels) and In the conv input (CIN
// channels through the same source mapping as the forward pass).  Grid
// (groups, 27): CTA (g, tap) sums over the chunks g, g + groups, ... of
// 16 x 8 voxels and writes part[(g*27 + tap)][COUT][CIN].
template <int CIN, int COUT>
__global__ void __launch_bounds__(kConvThreads) k_conv3_wgrad(ConvIn in, const __nv_bfloat16* __restrict__ G,
                                                             int X, int Y, int Z, int nb, float* __restrict__ part) {
  constexpr int CS = CIN + 8, GS = COUT + 8;
  constexpr int MT = COUT / 16, NT = CIN / 8;
  __shared__ __align__(16) __nv_bfloat16 xs[kTX * kTY][CS];
  __shared__ __align__(16) __nv_bfloat16 gs[kTX * kTY][GS];
  __shared__ float red[COUT * CIN];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int tap = blockIdx.y, dx = tap % 3 - 1, dy = (tap / 3) % 3 - 1, dz = tap / 9 - 1;
  const int ntx = (X + kTX - 1) / kTX, nty = (Y + kTY - 1) / kTY;
  const int64_t nchunks = (int64_t)ntx * nty * Z * nb;
  float acc[MT][NT][4];
#pragma unroll
  for (int i = 0; i < MT; ++i)
#pragma unroll
    for (int j = 0; j < NT; ++j) acc[i][j][0] = acc[i][j][1] = acc[i][j][2] = acc[i][j][3] = 0.f;
  for (int64_t ch = blockIdx.x; ch < nchunks; ch += gridDim.x) {
    const int tx = (int)(ch % ntx), ty = (int)((ch / ntx) % nty);
    const int zz = (int)(ch / ((int64_t)ntx * nty));  // stacked z
    const int b = zz / Z, z = zz - b * Z;
    __syncthreads();
    for (int i = tid; i < kTX * kTY * (CIN / 8); i += kConvThreads) {
      const int v = i / (CIN / 8), c8 = i - v * (CIN / 8);
      const int x = tx * kTX + (v % kTX) + dx, y = ty * kTY + (v / kTX) + dy;
      const bool inside_out = tx * kTX + (v % kTX) < X && ty * kTY + (v / kTX) < Y;
      const __nv_bfloat16* src = inside_out ? in_ptr(in, CIN, X, Y, Z, b, x, y, z + dz, c8 * 8) : nullptr;
      cp_async16(&xs[v][c8 * 8], src ? src : G, src != nullptr);
    }
    for (int i = tid; i < kTX * kTY * (COUT / 8); i += kConvThreads) {
      const int v = i / (COUT / 8), c8 = i - v * (COUT / 8);
      const int x = tx * kTX + (v % kTX), y = ty * kTY + (v / kTX);
      const bool ok = x < X && y < Y;
      const int64_t gv = (((int64_t)b * Z + z) * Y + y) * X + x;
      cp_async16(&gs[v][c8 * 8], ok ? G + gv * COUT + c8 * 8 : G, ok);
    }
    cp_async_commit();
    cp_async_wait_all();
    __syncthreads();
    // warp w: voxels [16w, 16w + 16) of the chunk are this k-step
    const int vb = warp * 16;
    // A = G^T (m = output channel, k = voxel): stored [voxel][channel] -> trans
    // B = In (k = voxel, n = input channel): stored [voxel][channel] -> trans
    const int lrow = (lane & 7) + ((lane >> 4) & 1) * 8;  // voxel row for the A/B matrices 2,3
    const int lsel = (lane >> 3) & 1;
#pragma unroll
    for (int i = 0; i < MT; ++i) {
      uint32_t a0, a1, a2, a3;
      // matrices: (m0-7,k0-7) (m8-15,k0-7) (m0-7,k8-15) (m8-15,k8-15)
      ldsm_x4_t(a0, a1, a2, a3, &gs[vb + lrow][i * 16 + lsel * 8]);
#pragma unroll
      for (int j = 0; j < NT / 2; ++j) {
        uint32_t b0, b1, b2, b3;
        // matrices: (k0-7,n0-7) (k8-15,n0-7) (k0-7,n8-15) (k8-15,n8-15)
        ldsm_x4_t(b0, b1, b2, b3, &xs[vb + (lane & 7) + lsel * 8][j * 16 + (lane >> 4) * 8]);
        mma_bf16(acc[i][2 * j], a0, a1, a2, a3, b0, b1);
        mma_bf16(acc[i][2 * j + 1], a0, a1, a2, a3, b2, b3);
      }
    }
  }
  // deterministic sum over warps
  const int g = lane >> 2, t = lane & 3;
  for (int w = 0; w < 8; ++w) {
    __syncthreads();
    if (warp == w) {
#pragma unroll
      for (int i = 0; i < MT; ++i)
#pragma unroll
        for (int j = 0; j < NT; ++j)
#pragma unroll
          for (int e = 0; e < 4; ++e) {
            const int m = i * 16 + g + (e >> 1) * 8, n = j * 8 + 2 * t + (e & 1);
            red[m * CIN + n] = (w == 0 ? 0.f : red[m * CIN + n]) + acc[i][j][e];
          }
    }
  }
  __syncthreads();
  float* dst = part + ((int64_t)blockIdx.x * 27 + tap) * COUT * CIN;
  for (int i = tid; i < COUT * CIN; i += kConvThreads) dst[i] = red[i];
}

// dW[n][tap*CIN + c] = sum_g part[g][tap][n][c] (fixed order).
__global__ void k_wgrad_reduce(const float* __restrict__ part, int groups, int cin, int cout, float* __restrict__ dW) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int per = 27 * cout * cin;
  if (i >= per) return;
  const int tap = i / (cout * cin), r = i - tap * cout * cin, n = r / cin, c = r - n * cin;
  float s = 0.f;
  for (int g = 0; g < groups; ++g) s += part[(int64_t)g * per + i];
  dW[(int64_t)n * 27 * cin + tap * cin + c] = s;
}

// Bias gradient partials: part[blk][c] = sum over the block's voxels of G[v][c].
__global__ void k_bias_grad_partial(const __nv_bfloat16* __restrict__ G, int64_t nvox, int C, float* __restrict__ part) {
  extern __shared__ float sh[];
  const int c = threadIdx.x % C, lanes = blockDim.x / C, l = threadIdx.x / C;
  float s = 0.f;
  for (int64_t v = (int64_t)blockIdx.x * lanes + l; v < nvox; v += (int64_t)gridDim.x * lanes)
    s += __bfloat162float(G[v * C + c]);
  sh[threadIdx.x] = s;
  __syncthreads();
  if (l == 0) {
    float t = 0.f;
    for (int k = 0; k < lanes; ++k) t += sh[k * C + c];
    part[blockIdx.x * C + c] = t;
  }
}

__global__ void k_bias_grad_reduce(const float* __restrict__ part, int nblk, int C, float* __restrict__ db) {
  const int c = threadIdx.x;
  if (c >= C) return;
  float s = 0.f;
  for (int b = 0; b < nblk; ++b) s += part[b * C + c];
  db[c] = s;
}

// Pre-activation gradient of a ReLU layer: G = dY * (Y > 0) (or dY if !relu), bf16.
__global__ void k_relu_grad(const float* __restrict__ dY, const __nv_bfloat16* __restrict__ Y, int64_t n, int relu,
                            __nv_bfloat16* __restrict__ G) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float d = dY[i];
  if (relu && !(__bfloat162float(Y[i]) > 0.f)) d = 0.f;
  G[i] = __float2bfloat16_rn(d);
}

// 2x2x2 average pooling of stacked volumes (X, Y, Z even).
__global__ void k_pool2(const __nv_bfloat16* __restrict__ in, int X, int Y, int Z, int nb, int C,
                        __nv_bfloat16* __restrict__ out) {
  const int hx = X / 2, hy = Y / 2, hz = Z / 2;
  const int64_t n = (int64_t)nb * hz * hy * hx * C;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int c = (int)(i % C);
  int64_t v = i / C;
  const int x = (int)(v % hx); v /= hx;
  const int y = (int)(v % hy); v /= hy;
  const int z = (int)(v % hz);
  const int b = (int)(v / hz);
  float s = 0.f;
  for (int k = 0; k < 8; ++k) {
    const int64_t u = (((int64_t)b * Z + 2 * z + (k >> 2)) * Y + 2 * y + ((k >> 1) & 1)) * X + 2 * x + (k & 1);
    s += __bfloat162float(in[u * C + c]);
  }
  out[i] = __float2bfloat16_rn(0.125f * s);
}

// Backward of k_pool2: dIn[child] (+)= dOut[parent] / 8 (fp32).
__global__ void k_pool2_bwd(const float* __restrict__ dout, int X, int Y, int Z, int nb, int C, int accumulate,
                            float* __restrict__ din) {
  const int64_t n = (int64_t)nb * Z * Y * X * C;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int c = (int)(i % C);
  int64_t v = i / C;
  const int x = (int)(v % X); v /= X;
  const int y = (int)(v % Y); v /= Y;
  const int z = (int)(v % Z);
  const int b = (int)(v / Z);
  const int64_t p = (((int64_t)b * (Z / 2) + z / 2) * (Y / 2) + y / 2) * (X / 2) + x / 2;
  const float g = 0.125f * dout[p * C + c];
  din[i] = accumulate ? din[i] + g : g;
}

// Backward of nearest upsampling: dHalf[p] = sum of the 8 children of dFull,
// where dFull holds `cfull` channels and the upsampled block is [0, c).
__global__ void k_up2_bwd(const float* __restrict__ dfull, int X, int Y, int Z, int nb, int cfull, int c,
                          float* __restrict__ dhalf) {
  const int hx = X / 2, hy = Y / 2, hz = Z / 2;
  const int64_t n = (int64_t)nb * hz * hy * hx * c;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int ch = (int)(i % c);
  int64_t v = i / c;
  const int x = (int)(v % hx); v /= hx;
  const int y = (int)(v % hy); v /= hy;
  const int z = (int)(v % hz);
  const int b = (int)(v / hz);
  float s = 0.f;
  for (int k = 0; k < 8; ++k) {
    const int64_t u = (((int64_t)b * Z + 2 * z + (k >> 2)) * Y + 2 * y + ((k >> 1) & 1)) * X + 2 * x + (k & 1);
    s += dfull[u * cfull + ch];
  }
  dhalf[i] = s;
}

// Copy channels [c0, c0 + c) of a cfull-channel fp32 tensor into a c-channel one.
__global__ void k_channel_slice(const float* __restrict__ src, int64_t nvox, int cfull, int c0, int c,
                                int accumulate, float* __restrict__ dst) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nvox * c) return;
  const int64_t v = i / c;
  const int k = (int)(i - v * c);
  const float s = src[v * cfull + c0 + k];
  dst[i] = accumulate ? dst[i] + s : s;
}

// W'[c][tap'*COUT + n] = W[n][tap*CIN + c], tap' = 26 - tap: the data-gradient
// convolution's weights (bf16).
__global__ void k_flip_weights(const __nv_bfloat16* __restrict__ W, int cin, int cout, __nv_bfloat16* __restrict__ Wt) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= 27 * cin * cout) return;
  const int n = i / (27 * cin), r = i - n * 27 * cin, tap = r / cin, c = r - tap * cin;
  Wt[(int64_t)c * 27 * cout + (26 - tap) * cout + n] = W[i];
}

// Adam on fp32 master weights, bf16 copy for the kernels (bias-corrected,
// Kingma & Ba 2015, Algorithm 1).
// Adam step; with gn2 (the gradient's squared norm) the gradient is scaled to
// a norm of at most clip.
__global__ void k_adam(int64_t n, const float* __restrict__ grad, float lr, float b1, float b2, float eps, float c1,
                       float c2, float* __restrict__ w, float* __restrict__ m, float* __restrict__ v,
                       __nv_bfloat16* __restrict__ wb, const double* __restrict__ gn2, float clip) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float sc = 1.f;
  if (gn2) {
    const double nrm = sqrt(*gn2);
    if (nrm > clip) sc = (float)(clip / nrm);
  }
  const float g = grad[i] * sc;
  const float mi = b1 * m[i] + (1.f - b1) * g;
  const float vi = b2 * v[i] + (1.f - b2) * g * g;
  m[i] = mi;
  v[i] = vi;
  const float wi = w[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  w[i] = wi;
  if (wb) wb[i] = __float2bfloat16_rn(wi);
}

__global__ void k_f32_to_bf16(const float* __restrict__ a, int64_t n, __nv_bfloat16* __restrict__ b) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) b[i] = __float2bfloat16_rn(a[i]);
}

// ---- host launchers --------------------------------------------------------

template <int CIN, int COUT>
static size_t conv_smem() {
  return (size_t)kHalo * (CIN + 8) * 2 + (size_t)COUT * (27 * CIN + 8) * 2;
}

template <int CIN, int COUT>
static cudaError_t conv_launch(cudaStream_t s, const ConvIn& in, const __nv_bfloat16* W, const float* bias, int X,
                               int Y, int Z, int nb, int relu, int out_mode, void* out) {
  static PerDeviceOnce once;
  const size_t smem = conv_smem<CIN, COUT>();
  const cudaError_t attr_err = once_per_device(once, [smem] {
    return cudaFuncSetAttribute(k_conv3<CIN, COUT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  });
  if (attr_err != cudaSuccess) return attr_err;
  dim3 grid((X + kTX - 1) / kTX, (Y + kTY - 1) / kTY, nb * Z / kTZ);
  k_conv3<CIN, COUT><<<grid, kConvThreads, smem, s>>>(in, W, bias, X, Y, Z, relu, out_mode, out);
  return cudaGetLastError();
}

template <int CIN, int COUT>
static cudaError_t wgrad_launch(cudaStream_t s, const ConvIn& in, const __nv_bfloat16* G, int X, int Y, int Z, int nb,
                                int groups, float* part, float* dW) {
  k_conv3_wgrad<CIN, COUT><<<dim3(groups, 27), kConvThreads, 0, s>>>(in, G, X, Y, Z, nb, part);
  const int per = 27 * CIN * COUT;
  k_wgrad_reduce<<<(per + 255) / 256, 256, 0, s>>>(part, groups, CIN, COUT, dW);
  return cudaGetLastError();
}

#define TOPO_CONV_CASES(M) M(16, 16) M(16, 32) M(32, 16) M(32, 32) M(32, 64) M(64, 32)

cudaError_t unet_conv(cudaStream_t s, int cin, int cout, const __nv_bfloat16* s1, const __nv_bfloat16* s2, int c1,
                      int up1, const __nv_bfloat16* W, const float* bias, int X, int Y, int Z, int nb, int relu,
                      int out_mode, void* out) {
  if (Z % kTZ) return cudaErrorInvalidValue;
  ConvIn in{s1, s2, c1, up1};
#define TOPO_CONV_CASE(a, b) \
  if (cin == a && cout == b) return conv_launch<a, b>(s, in, W, bias, X, Y, Z, nb, relu, out_mode, out);
  TOPO_CONV_CASES(TOPO_CONV_CASE)
#undef TOPO_CONV_CASE
  return cudaErrorInvalidValue;
}

cudaError_t unet_wgrad(cudaStream_t s, int cin, int cout, const __nv_bfloat16* s1, const __nv_bfloat16* s2, int c1,
                       int up1, const __nv_bfloat16* G, int X, int Y, int Z, int nb, int groups, float* part,
                       float* dW) {
  ConvIn in{s1, s2, c1, up1};
#define TOPO_WGRAD_CASE(a, b) \
  if (cin == a && cout == b) return wgrad_launch<a, b>(s, in, G, X, Y, Z, nb, groups, part, dW);
  TOPO_CONV_CASES(TOPO_WGRAD_CASE)
#undef TOPO_WGRAD_CASE
  return cudaErrorInvalidValue;
}

static inline unsigned nblk64(int64_t n, int b) { return (unsigned)((n + b - 1) / b); }

void unet_bias_grad(cudaStream_t s, const __nv_bfloat16* G, int64_t nvox, int C, float* part, int nblk, float* db) {
  const int threads = 256 - 256 % C;
  k_bias_grad_partial<<<nblk, threads, threads * sizeof(float), s>>>(G, nvox, C, part);
  k_bias_grad_reduce<<<1, 64, 0, s>>>(part, nblk, C, db);
}

void unet_relu_grad(cudaStream_t s, const float* dY, const __nv_bfloat16* Y, int64_t n, int relu, __nv_bfloat16* G) {
  k_relu_grad<<<nblk64(n, 256), 256, 0, s>>>(dY, Y, n, relu, G);
}

void unet_pool(cudaStream_t s, const __nv_bfloat16* in, int X, int Y, int Z, int nb, int C, __nv_bfloat16* out) {
  const int64_t n = (int64_t)nb * (Z / 2) * (Y / 2) * (X / 2) * C;
  k_pool2<<<nblk64(n, 256), 256, 0, s>>>(in, X, Y, Z, nb, C, out);
}

void unet_pool_bwd(cudaStream_t s, const float* dout, int X, int Y, int Z, int nb, int C, int accumulate, float* din) {
  const int64_t n = (int64_t)nb * Z * Y * X * C;
  k_pool2_bwd<<<nblk64(n, 256), 256, 0, s>>>(dout, X, Y, Z, nb, C, accumulate, din);
}

void unet_up_bwd(cudaStream_t s, const float* dfull, int X, int Y, int Z, int nb, int cfull, int c, float* dhalf) {
  const int64_t n = (int64_t)nb * (Z / 2) * (Y / 2) * (X / 2) * c;
  k_up2_bwd<<<nblk64(n, 256), 256, 0, s>>>(dfull, X, Y, Z, nb, cfull, c, dhalf);
}

void unet_slice(cudaStream_t s, const float* src, int64_t nvox, int cfull, int c0, int c, int accumulate, float* dst) {
  k_channel_slice<<<nblk64(nvox * c, 256), 256, 0, s>>>(src, nvox, cfull, c0, c, accumulate, dst);
}

void unet_flip(cudaStream_t s, const __nv_bfloat16* W, int cin, int cout, __nv_bfloat16* Wt) {
  k_flip_weights<<<nblk64(27 * cin * cout, 256), 256, 0, s>>>(W, cin, cout, Wt);
}

void unet_adam(cudaStream_t s, int64_t n, const float* grad, float lr, float b1, float b2, float eps, int step,
               float* w, float* m, float* v, __nv_bfloat16* wb, const double* gn2, float clip) {
  const float c1 = 1.f - powf(b1, (float)step), c2 = 1.f - powf(b2, (float)step);
  k_adam<<<nblk64(n, 256), 256, 0, s>>>(n, grad, lr, b1, b2, eps, c1, c2, w, m, v, wb, gn2, clip);
}

void unet_to_bf16(cudaStream_t s, const float* a, int64_t n, __nv_bfloat16* b) {
  k_f32_to_bf16<<<nblk64(n, 256), 256, 0, s>>>(a, n, b);
}

}  // namespace topo
