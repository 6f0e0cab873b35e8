// 3x3x3 convolution of the learned preconditioner on the 5th-generation tensor
// cores (tcgen05.mma, accumulators in tensor memory), fed by TMA.
//
// Same operation, tensor layout and epilogue modes as k_conv3 in k_unet.cu:
// channels-last bf16 input ("NDHWC", several volumes stacked along z, each with
// its own zero padding), bf16 weights [Cout][27*Cin], fp32 accumulation.
//
// Implicit GEMM per CTA: M = 128 output voxels (8 along x by 16 along y, one z
// plane), N = Cout, K = 27 taps x Cin; the CTA does TZ = 2 planes.
//
// Shared-memory operands, "no swizzle" K-major canonical layout (core matrices
// of 8 rows x 16 bytes, rows 16 bytes apart):
//   * input halo, one plane per group of 8 channels: [cg][HZ][HY][HX][8] bf16
//     (HX = 10, HY = 18, HZ = 4).  Row m = xo + 8 yo of the A operand of tap
//     (dx, dy, dz) is halo voxel (xo + dx, yo + dy, tz + dz): the 8 rows of a
//     core matrix are 8 consecutive x (16 bytes apart), consecutive core
//     matrices along M are consecutive y (HX * 16 bytes apart, the stride-
//     dimension offset) and the second 8 channels of a K = 16 step are the next
//     group plane (the leading-dimension offset).  So every tap's A operand is
//     the same halo at a different start address: no im2col copy.
//   * weights, [tap][cg][Cout][8] bf16: core matrices of 8 output channels x 8
//     input channels (stride-dimension offset 128 bytes, leading-dimension
//     offset Cout * 16 bytes).
// Full-resolution input channel groups arrive by TMA tensor loads
// (cp.async.bulk.tensor, one 5-D box {8 ch, 10, 18, 4, 1} per group; the
// coordinates outside the volume, the conv's zero padding, are zero-filled by
// the copy engine).  Channel groups read through nearest upsampling (the
// decoder's upsample + concat) and the weights are staged by the threads with
// cp.async.  One thread issues the 27 * Cin / 16 MMAs per plane (M = 128,
// N = Cout, K = 16) and commits them to an mbarrier; the 4 warps then read the
// accumulators back (tcgen05.ld, warp w owns TMEM lanes 32w..32w+31 = output
// rows) and apply bias, ReLU and the store.
//
// Waits on mbarriers are bounded: a wait that gives up sets a device error flag
// (read by conv_tc_error), skips the remaining work, frees its tensor memory
// and returns.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>

#include <cstdint>
#include <mutex>

#include "topo_internal.h"

namespace topo {

namespace {

constexpr int kTcTX = 8, kTcTY = 16, kTcTZ = 2;
constexpr int kTcHX = kTcTX + 2, kTcHY = kTcTY + 2, kTcHZ = kTcTZ + 2;
constexpr int kTcPlane = kTcHZ * kTcHY * kTcHX * 16;  // bytes of one 8-channel group plane
constexpr int kTcThreads = 128;
constexpr int kTcMaxGroups = 8;                       // Cin <= 64
constexpr long long kTcSpin = 1ll << 24;              // try_wait rounds before giving up

__device__ int g_conv_tc_err;

struct TcMaps {
  CUtensorMap m[kTcMaxGroups];
};

__device__ __forceinline__ uint32_t su32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// tcgen05 shared-memory matrix descriptor: start address, leading-dimension
// byte offset, stride-dimension byte offset (all >> 4), version bits 46-48 =
// 0b001, base offset 0, no swizzle.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((addr & 0x3FFFF) >> 4) | ((uint64_t)((lbo >> 4) & 0x3FFF) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFF) << 32) | (1ull << 46);
}

// Instruction descriptor of kind::f16: D fp32 (bits 4-5 = 1), A and B bf16
// (bits 7-9, 10-12 = 1), both K-major, N >> 3 at bit 17, M >> 4 at bit 24.
template <int M, int N>
__host__ __device__ constexpr uint32_t idesc_bf16() {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, int count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(su32(bar)), "r"(count));
}

__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
  uint32_t done = 0;
  for (long long it = 0; it < kTcSpin; ++it) {
    asm volatile(
        "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(su32(bar)), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

__device__ __forceinline__ void cp_async16_z(uint32_t dst, const void* src, bool valid) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(dst), "l"(src), "r"(valid ? 16 : 0));
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

template <int NCOLS>
constexpr int tmem_cols() {
  return NCOLS <= 32 ? 32 : NCOLS <= 64 ? 64 : NCOLS <= 128 ? 128 : NCOLS <= 256 ? 256 : 512;
}

}  // namespace

// Channel groups of one tile's input halo: the TMA boxes of the full-
// resolution groups (thread 0; completion on `bar`) and, by all threads, the
// groups read through nearest upsampling (cp.async).
template <int CIN>
__device__ __forceinline__ void conv_tc_stage_halo(const TcMaps& maps, unsigned tma_groups,
                                                   const __nv_bfloat16* __restrict__ s1, int c1,
                                                   const __nv_bfloat16* zsrc, uint32_t halo, uint64_t* bar, int x0,
                                                   int y0, int z0, int b, int X, int Y, int Z) {
  constexpr int CG = CIN / 8;
  const int tid = threadIdx.x;
  if (tid == 0 && tma_groups) {
    const uint32_t bytes = (uint32_t)__popc(tma_groups) * kTcPlane;
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(su32(bar)), "r"(bytes) : "memory");
#pragma unroll 1
    for (int cg = 0; cg < CG; ++cg) {
      if (!((tma_groups >> cg) & 1)) continue;
      asm volatile(
          "cp.async.bulk.tensor.5d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, "
          "%5, %6}], [%7];" ::"r"(halo + cg * kTcPlane),
          "l"(&maps.m[cg]), "r"(0), "r"(x0 - 1), "r"(y0 - 1), "r"(z0 - 1), "r"(b), "r"(su32(bar))
          : "memory");
    }
  }
  const unsigned up_groups = ((1u << CG) - 1) & ~tma_groups;
  if (up_groups) {
    const int hxd = X >> 1, hyd = Y >> 1, hzd = Z >> 1;
    constexpr int HV = kTcHZ * kTcHY * kTcHX;
    for (int i = tid; i < CG * HV; i += kTcThreads) {
      const int cg = i / HV;
      if (!((up_groups >> cg) & 1)) continue;
      const int v = i - cg * HV;
      const int hx = v % kTcHX, hy = (v / kTcHX) % kTcHY, hz = v / (kTcHX * kTcHY);
      const int x = x0 + hx - 1, y = y0 + hy - 1, z = z0 + hz - 1;
      const bool inside = x >= 0 && y >= 0 && z >= 0 && x < X && y < Y && z < Z;
      const __nv_bfloat16* src = zsrc;
      if (inside) {
        const int64_t p = (((int64_t)b * hzd + (z >> 1)) * hyd + (y >> 1)) * hxd + (x >> 1);
        src = s1 + p * c1 + cg * 8;
      }
      cp_async16_z(halo + cg * kTcPlane + v * 16, src, inside);
    }
  }
}

// One CTA per tile of 8 x 16 x 2 output voxels (blockIdx: x tile, y tile,
// stacked z block).  Thread 0 issues the tile's 2 x 27 x Cin/16 MMAs into two
// accumulators of Cout columns as soon as the halo has landed and commits them
// to an mbarrier; the 4 warps then read them back and store.  (A persistent
// form that stages the weights once per CTA and double-buffers the halo and
// the accumulators over several tiles measured slower on the network's
// layers: shared memory then allows fewer CTAs per SM, and each tile's MMA
// chain is latency-bound, so throughput comes from the CTAs that overlap.)
// tma_groups: bit cg set when channel group cg comes by TMA (maps.m[cg]); the
// other groups are read through nearest upsampling from s1 (c1 channels at
// half resolution).
template <int CIN, int COUT>
__global__ void __launch_bounds__(kTcThreads) k_conv3_tc(const __grid_constant__ TcMaps maps, unsigned tma_groups,
                                                         const __nv_bfloat16* __restrict__ s1, int c1,
                                                         const __nv_bfloat16* __restrict__ W,
                                                         const float* __restrict__ bias, int X, int Y, int Z, int relu,
                                                         int out_mode, void* out) {
  static_assert(CIN % 16 == 0 && CIN <= 8 * kTcMaxGroups, "input channels");
  static_assert(COUT % 16 == 0 && COUT <= 256, "output channels (M = 128 needs N % 16 == 0)");
  constexpr int CG = CIN / 8;
  constexpr int KSTEPS = CIN / 16;
  constexpr int W_BYTES = 27 * CG * COUT * 16;
  constexpr int NCOL = tmem_cols<kTcTZ * COUT>();
  constexpr uint32_t IDESC = idesc_bf16<128, COUT>();
  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ __align__(8) uint64_t bar_tma, bar_mma;
  __shared__ uint32_t tmem_slot;
  __shared__ int s_ok;

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t wsm = su32(smem), halo = wsm + W_BYTES;
  const int x0 = blockIdx.x * kTcTX, y0 = blockIdx.y * kTcTY;
  const int zt = blockIdx.z * kTcTZ, b = zt / Z, z0 = zt - b * Z;

  if (tid == 0) {
    mbar_init(&bar_tma, 1);
    mbar_init(&bar_mma, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(su32(&tmem_slot)),
                 "r"(NCOL));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = tmem_slot;

  // weights, [tap][cg][COUT][8]; the halo (TMA by thread 0, upsampled groups by all)
  for (int i = tid; i < COUT * 27 * CG; i += kTcThreads) {
    const int n = i / (27 * CG), r = i - n * (27 * CG);
    const int tap = r / CG, cg = r - tap * CG;
    cp_async16_z(wsm + ((tap * CG + cg) * COUT + n) * 16, W + (int64_t)n * 27 * CIN + tap * CIN + cg * 8, true);
  }
  conv_tc_stage_halo<CIN>(maps, tma_groups, s1, c1, W, halo, &bar_tma, x0, y0, z0, b, X, Y, Z);
  asm volatile("cp.async.commit_group;\ncp.async.wait_all;" ::: "memory");
  // generic-proxy writes (cp.async) -> visible to the tensor cores' async proxy
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  __syncthreads();

  if (tid == 0) {
    const bool landed = tma_groups == 0 || mbar_wait(&bar_tma, 0);
    if (landed) {
      asm volatile("tcgen05.fence::after_thread_sync;");
#pragma unroll 1
      for (int tz = 0; tz < kTcTZ; ++tz) {
        const uint32_t d = tmem + tz * COUT;
#pragma unroll 1
        for (int tap = 0; tap < 27; ++tap) {
          const int dx = tap % 3, dy = (tap / 3) % 3, dz = tap / 9;
          const uint32_t a0 = halo + (((tz + dz) * kTcHY + dy) * kTcHX + dx) * 16;
#pragma unroll
          for (int ks = 0; ks < KSTEPS; ++ks) {
            const uint64_t ad = smem_desc(a0 + 2 * ks * kTcPlane, kTcPlane, kTcHX * 16);
            const uint64_t bd = smem_desc(wsm + (tap * CG + 2 * ks) * COUT * 16, COUT * 16, 128);
            const uint32_t acc = (tap | ks) ? 1u : 0u;
            asm volatile(
                "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
                "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d),
                "l"(ad), "l"(bd), "r"(IDESC), "r"(acc));
          }
        }
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                       su32(&bar_mma))
                   : "memory");
    } else {
      atomicExch(&g_conv_tc_err, 1);
    }
    s_ok = landed;
  }
  __syncthreads();
  bool ok = s_ok != 0;
  if (ok) {
    ok = mbar_wait(&bar_mma, 0);
    if (!ok) atomicExch(&g_conv_tc_err, 2);
  }
  asm volatile("tcgen05.fence::after_thread_sync;");

  if (ok) {
    const int m = warp * 32 + lane;
    const int x = x0 + (m & 7), y = y0 + (m >> 3);
    const bool in_xy = x < X && y < Y;
#pragma unroll 1
    for (int tz = 0; tz < kTcTZ; ++tz) {
      const int64_t v = (((int64_t)b * Z + z0 + tz) * Y + y) * X + x;
#pragma unroll
      for (int c0 = 0; c0 < COUT; c0 += 16) {
        float o[16];
        tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + tz * COUT + c0, o);
        if (!in_xy) continue;
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          if (bias) o[j] += bias[c0 + j];
          if (relu) o[j] = fmaxf(o[j], 0.f);
        }
        if (out_mode == 0) {
          uint4 pk[2];
          uint32_t* w32 = reinterpret_cast<uint32_t*>(pk);
#pragma unroll
          for (int j = 0; j < 8; ++j) {
            const __nv_bfloat162 h2 = __floats2bfloat162_rn(o[2 * j], o[2 * j + 1]);
            w32[j] = *reinterpret_cast<const uint32_t*>(&h2);
          }
          uint4* dst = reinterpret_cast<uint4*>(static_cast<__nv_bfloat16*>(out) + v * COUT + c0);
          dst[0] = pk[0];
          dst[1] = pk[1];
        } else {
          float4* dst = reinterpret_cast<float4*>(static_cast<float*>(out) + v * COUT + c0);
#pragma unroll
          for (int j = 0; j < 4; ++j) {
            float4 q = make_float4(o[4 * j], o[4 * j + 1], o[4 * j + 2], o[4 * j + 3]);
            if (out_mode == 2) {
              const float4 p = dst[j];
              q.x += p.x; q.y += p.y; q.z += p.z; q.w += p.w;
            }
            dst[j] = q;
          }
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(NCOL));
}

// ---- host side ---------------------------------------------------------------

namespace {

PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q{};
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  });
  return fn;
}

// 5-D view (8 channels, X, Y, Z, volumes) of a channels-last tensor with C
// channels, starting at channel c0; box {8, HX, HY, HZ, 1}.
cudaError_t encode_group_map(CUtensorMap* m, const __nv_bfloat16* base, int C, int c0, int X, int Y, int Z, int nb) {
  auto enc = tensor_map_encoder();
  if (!enc) return cudaErrorNotSupported;
  const cuuint64_t dims[5] = {8, (cuuint64_t)X, (cuuint64_t)Y, (cuuint64_t)Z, (cuuint64_t)nb};
  const cuuint64_t row = (cuuint64_t)C * 2;
  const cuuint64_t strides[4] = {row, row * X, row * X * Y, row * X * Y * Z};
  const cuuint32_t box[5] = {8, kTcHX, kTcHY, kTcHZ, 1};
  const cuuint32_t estr[5] = {1, 1, 1, 1, 1};
  const CUresult r = enc(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 5, const_cast<__nv_bfloat16*>(base + c0), dims, strides,
                         box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                         CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

template <int CIN, int COUT>
constexpr size_t conv_tc_smem() {
  return (size_t)27 * CIN * COUT * 2 + (size_t)(CIN / 8) * kTcPlane;
}

template <int CIN, int COUT>
cudaError_t conv_tc_launch(cudaStream_t s, const __nv_bfloat16* s1, const __nv_bfloat16* s2, int c1, int up1,
                           const __nv_bfloat16* W, const float* bias, int X, int Y, int Z, int nb, int relu,
                           int out_mode, void* out) {
  constexpr size_t smem = conv_tc_smem<CIN, COUT>();
  static PerDeviceOnce once;
  cudaError_t e = once_per_device(once, [] {
    return cudaFuncSetAttribute(k_conv3_tc<CIN, COUT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  });
  if (e != cudaSuccess) return e;
  TcMaps maps{};
  unsigned tma = 0;
  for (int cg = 0; cg < CIN / 8; ++cg) {
    const int c = cg * 8;
    if (c < c1) {
      if (up1) continue;  // upsampled: staged by the threads
      e = encode_group_map(&maps.m[cg], s1, c1, c, X, Y, Z, nb);
    } else {
      e = encode_group_map(&maps.m[cg], s2, CIN - c1, c - c1, X, Y, Z, nb);
    }
    if (e != cudaSuccess) return e;
    tma |= 1u << cg;
  }
  const dim3 grid((X + kTcTX - 1) / kTcTX, (Y + kTcTY - 1) / kTcTY, nb * Z / kTcTZ);
  k_conv3_tc<CIN, COUT><<<grid, kTcThreads, smem, s>>>(maps, tma, s1, c1, W, bias, X, Y, Z, relu, out_mode, out);
  return cudaGetLastError();
}

}  // namespace

// The tensor-core convolution for the layer shapes of the network; false
// when (cin, cout) has no instantiation.
cudaError_t unet_conv_tc(cudaStream_t s, int cin, int cout, const __nv_bfloat16* s1, const __nv_bfloat16* s2, int c1,
                         int up1, const __nv_bfloat16* W, const float* bias, int X, int Y, int Z, int nb, int relu,
                         int out_mode, void* out) {
  if (Z % kTcTZ) return cudaErrorInvalidValue;
  if (c1 % 8 || (cin - c1) % 8) return cudaErrorInvalidValue;
  if (up1 && (X % 2 || Y % 2 || Z % 2)) return cudaErrorInvalidValue;
#define TOPO_CONV_TC_CASE(a, bb)                                                                          \
  if (cin == a && cout == bb)                                                                            \
    return conv_tc_launch<a, bb>(s, s1, s2, c1, up1, W, bias, X, Y, Z, nb, relu, out_mode, out);
  TOPO_CONV_TC_CASE(16, 16)
  TOPO_CONV_TC_CASE(16, 32)
  TOPO_CONV_TC_CASE(32, 16)
  TOPO_CONV_TC_CASE(32, 32)
  TOPO_CONV_TC_CASE(32, 64)
  TOPO_CONV_TC_CASE(64, 32)
#undef TOPO_CONV_TC_CASE
  return cudaErrorInvalidValue;
}

// Reads and clears the device flag of the tensor-core convolution's bounded
// waits (0: no wait gave up).
cudaError_t conv_tc_error(int* flag) {
  int zero = 0;
  cudaError_t e = cudaMemcpyFromSymbol(flag, g_conv_tc_err, sizeof(int));
  if (e != cudaSuccess) return e;
  return cudaMemcpyToSymbol(g_conv_tc_err, &zero, sizeof(int));
}

}  // namespace topo
