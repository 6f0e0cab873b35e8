// Internal declarations shared by the translation units of libtopo_gb300.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>
#include <string>
#include <vector>

#include "../../include/topo_gb300.h"

namespace topo {

// Process-wide count of kernel launches issued by this library, and the
// calling thread's own count (graph captures measure their kernels with the
// latter, so launches from other threads are not mixed in).
extern std::atomic<long long> g_launches;
extern thread_local long long t_launches;
inline void count_launch(int n = 1) {
  g_launches.fetch_add(n, std::memory_order_relaxed);
  t_launches += n;
}

// Makes device `dev` current for the scope of one API call and gives the
// calling thread its previous device back on exit.  Every entry point that
// takes a handle runs on the handle's device, whatever device the calling
// thread had selected (a handle on GPU 1 driven from a thread left on GPU 0,
// the worker threads of topo_design_batch).  dev < 0 does nothing.
struct DeviceScope {
  int prev = -1;
  explicit DeviceScope(int dev) {
    if (dev < 0) return;
    int cur = -1;
    if (cudaGetDevice(&cur) != cudaSuccess) { cudaGetLastError(); return; }
    if (cur == dev) return;
    if (cudaSetDevice(dev) != cudaSuccess) { cudaGetLastError(); return; }
    prev = cur;
  }
  ~DeviceScope() { if (prev >= 0) cudaSetDevice(prev); }
  DeviceScope(const DeviceScope&) = delete;
  DeviceScope& operator=(const DeviceScope&) = delete;
};

// Runs `fn` (returning cudaError_t) once per CUDA device, on the calling
// thread's current device: settings such as a kernel's dynamic shared-memory
// opt-in belong to one device, so a process with handles on several GPUs needs
// them on each.  A failed attempt is retried by the next call.
struct PerDeviceOnce {
  std::atomic<unsigned long long> done{0};
};
template <typename Fn>
inline cudaError_t once_per_device(PerDeviceOnce& o, Fn&& fn) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= 64) return fn();
  const unsigned long long bit = 1ull << dev;
  if (o.done.load(std::memory_order_acquire) & bit) return cudaSuccess;
  e = fn();
  if (e == cudaSuccess) o.done.fetch_or(bit, std::memory_order_acq_rel);
  return e;
}

// Added to the z-march depth of an FP32 fine-kernel launch: element products
// on the tensor cores (k_fine_tc32) on levels without void planes.
constexpr int TOPO_FINE_TC_FLAG = 1 << 16;
// Added to the z-march depth of an FP32 fine-kernel launch: CTA tiles of 4 or
// 16 element rows (warps) instead of 8, for the modal kernel on levels
// without void planes (the per-tile z ranges are laid out for 8 rows).
constexpr int TOPO_FINE_ROWS4_FLAG = 1 << 17, TOPO_FINE_ROWS16_FLAG = 1 << 18;
constexpr int TOPO_FINE_FLAGS = TOPO_FINE_TC_FLAG | TOPO_FINE_ROWS4_FLAG | TOPO_FINE_ROWS16_FLAG;
// the flag of a tile height (0 for the default 8 rows)
inline int fine_rows_flag(int rows) {
  return rows == 4 ? TOPO_FINE_ROWS4_FLAG : rows == 16 ? TOPO_FINE_ROWS16_FLAG : 0;
}

// z blocks of the fine z-marching kernels: blocks of tz vertex planes, the
// last one also taking the remainder (up to 2 tz - 1 planes) rather than a
// short block of its own, which would recompute a whole element layer below
// it for a few planes.  Block k covers planes [k tz, fine_zblock_end(k)).
__host__ __device__ inline int fine_zblocks(int vz, int tz) { return vz / tz > 1 ? vz / tz : 1; }
__host__ __device__ inline int fine_zblock_end(int vz, int tz, int k) {
  return k + 1 >= fine_zblocks(vz, tz) ? vz : (k + 1) * tz;
}

// Vertex tile of the fine z-marching kernels: a CTA owns FINE_TILE_X - 1 by
// FINE_TILE_Y - 1 vertex columns and computes the FINE_TILE_X x FINE_TILE_Y
// element columns around them (one halo column and row below).
constexpr int FINE_TILE_X = 32, FINE_TILE_Y = 8;

// Dense grid level.  Element/vertex numbering is lexicographic (x fastest).
struct LevelDims {
  int ex, ey, ez;
  int vx, vy, vz;
  int64_t ne, nv;
  int factor;  // coarsening factor from the previous used level (1 for level 0)
  // Level 0 only (else null): per fine tile (bx + tiles_x * by), the lowest
  // and highest z of an active element among the tile's element columns, or
  // (ez, -1) when none is active.  The fine kernels march only the vertex
  // planes next to that range; the others see zero forces.
  const int2* colz;
  int colz_void;  // some tile's active range leaves void planes: the fine kernels narrow their z march
};

// Active z range per fine tile of level 0 from the element mask (host).
void fine_tile_zrange(const LevelDims& d, const uint8_t* eactive, std::vector<int2>& out);

// Device buffers of one level.  Vertex vectors are SoA [3][nv].
struct DevLevel {
  LevelDims d{};
  uint8_t* eactive = nullptr;  // [ne]
  uint8_t* vmask = nullptr;    // [nv] bits0-2 DOF free, bit3 active
  double *U = nullptr, *F = nullptr, *R = nullptr;    // FP64 [3nv]
  float *U32 = nullptr, *F32 = nullptr, *R32 = nullptr;  // FP32 [3nv]
  double* kel = nullptr;        // coarse: FP64 element matrices [ne][576]
  float* kel32 = nullptr;       // coarse: FP32 element matrices [ne][576]
  double* stencil = nullptr;    // coarse: FP64 [243][nv]
  float* stencil32 = nullptr;   // coarse: FP32 [243][nv], tiled on levels of 32,768 vertices or more (StIdx)
  double* dinv = nullptr;       // FP64 inverse diagonal blocks [9][nv] (Chebyshev)
  float* dinv32 = nullptr;      // FP32 inverse diagonal blocks [9][nv]; level 0: packed symmetric (float4 d00 d01 d02 d11 [nv], float2 d12 d22 [nv])
  double* cd = nullptr;         // FP64 Chebyshev direction [3nv]
  float* cd32 = nullptr;        // FP32 Chebyshev direction [3nv]
  double* U2 = nullptr;         // FP64 second iterate buffer (Chebyshev ping-pong) [3nv]
  float* U2_32 = nullptr;       // FP32 second iterate buffer [3nv]
  double lmax = 0, lmax32 = 0;  // Chebyshev spectral bound estimates
  double* eig = nullptr;        // last power-iteration vector, FP64 [3nv] (warm start)
  float* eig32 = nullptr;       // same, FP32
  double lprev = 0, lprev32 = 0;  // last estimates (warm-start guard)
};

// Host-side hierarchy description (computed once from the active mask).
struct Hierarchy {
  std::vector<LevelDims> dims;
  std::vector<std::vector<uint8_t>> eactive;  // per used level
  std::vector<std::vector<uint8_t>> vactive;  // per used level (bit3 only)
};

// Host-side set-up helpers (host_setup.cpp).
void element_template(double E, double nu, double h, double* Ke576);
Hierarchy build_hierarchy(int nx, int ny, int nz, const uint8_t* eactive, int max_coarse);
void spline_knots(int order, int partition, double bmin, double bmax, std::vector<double>& knots,
                  double& kmin, double& kstep);
// Galerkin transfer tables: T_pos = Q_pos^T Ke Q_pos for the 64 (factor 4) or 8
// (factor 2) fine-element positions, and the interpolation weights Q[pos][a][C].
void interp_weights(int factor, int px, int py, int pz, double Q[8][8]);
void galerkin_tables(const double* Ke, int factor, std::vector<double>& T);
int64_t gs_padded_count(const LevelDims& d, const uint8_t* active, bool vertices);

// Kernel launch wrappers (the .cu files).
struct Stream {
  cudaStream_t s;
};

// fine level (k_fine.cu)
template <typename T>
void launch_fine_apply(cudaStream_t s, const LevelDims& d, const T* rhop, const uint8_t* vmask,
                       const T* u, const T* f, T* out, bool residual, int nb = 1, int tz = 0);
// out = K u (level 0, one right-hand side) with per-CTA partial sums of u.out
// in partial; with dot and ctr (a zeroed counter) the last CTA also writes
// their total to *dot.  Returns the number of partials, or 0, launching
// nothing, when the kernel would need more than cap partial slots.
template <typename T>
int launch_fine_apply_dot(cudaStream_t s, const LevelDims& d, const T* rhop, const uint8_t* vmask, const T* u,
                          T* out, int tz, double* partial, int cap, double* dot = nullptr, unsigned* ctr = nullptr);
// FP64 vectors, double-float arithmetic (k_fine_modal_df)
// energy (residual only, one right-hand side): per-element u_e . (rho^p Ke u_e)
void launch_fine_apply_df(cudaStream_t s, const LevelDims& d, const double* rhop, const uint8_t* vmask,
                          const double* u, const double* f, double* out, bool residual, int nb = 1, int tz = 0,
                          double* energy = nullptr);
template <typename T>
void launch_fine_gs(cudaStream_t s, const LevelDims& d, const T* rhop, const uint8_t* vmask, T* u,
                    const T* f, int colour, bool reverse);
template <typename T>
void launch_fine_diag_inv(cudaStream_t s, const LevelDims& d, const T* rhop, const uint8_t* vmask,
                          T* dinv);
// FP32, one right-hand side: with dot_fo the kernel also leaves per-CTA partial
// sums of f.uout in dot_fo, and with dot and ctr (a zeroed counter) the last
// CTA writes their total to *dot.  Returns the number of partials, or 0 when
// none were formed (FP64, a batch, or more CTAs than cap).
template <typename T>
int launch_fine_cheb(cudaStream_t s, const LevelDims& d, const T* rhop, const uint8_t* vmask, const T* u,
                     const T* f, T* uout, const T* dinv, T* dvec, const double* coef, bool first,
                     int nb = 1, int tz = 0, bool d_is_u = false, double* dot_fo = nullptr, int cap = 0,
                     double* dot = nullptr, unsigned* ctr = nullptr);
template <typename T>
void launch_stencil_cheb(cudaStream_t s, const LevelDims& d, const T* st, const T* u, const T* f, T* uout,
                         const T* dinv, T* dvec, const double* coef, bool first, int nb = 1);
// First Chebyshev step from a zero iterate (u = 0): d = c_new D^-1 f, uout = d,
// with c_new = coef[1] in device memory.
// FP32: dvec may be null, and the next step then takes d from u (d_is_u).
template <typename T>
void launch_fine_cheb_zero(cudaStream_t s, const LevelDims& d, const T* rhop, const uint8_t* vmask, const T* f,
                           T* uout, const T* dinv, T* dvec, const double* coef, int nb = 1);
template <typename T>
void launch_cheb_zero_stored(cudaStream_t s, int64_t nv, const uint8_t* vmask, const T* dinv, const T* f, T* dvec,
                             T* uout, const double* coef, int nb = 1);
template <typename T>
void launch_fine_apply_dense(cudaStream_t s, const LevelDims& d, const T* rhop, const uint8_t* vmask,
                             const T* u, const T* f, T* out, bool residual);
void upload_template(const double* Ke576, double lam, double mu, double h);

// coarse levels (k_coarse.cu)
template <typename T>
void launch_stencil_apply(cudaStream_t s, const LevelDims& d, const T* st, const T* u, const T* f,
                          T* out, bool residual, int nb = 1);
template <typename T>
void launch_stencil_gs(cudaStream_t s, const LevelDims& d, const T* st, const uint8_t* vmask, T* u,
                       const T* f, int colour, bool reverse);
template <typename T>
void launch_stencil_diag_inv(cudaStream_t s, const LevelDims& d, const T* st, const uint8_t* vmask,
                             T* dinv);
template <typename T>
void launch_restrict(cudaStream_t s, const LevelDims& fine, const LevelDims& coarse, const T* rf,
                     T* fc, int nb = 1);
template <typename T>
void launch_prolong(cudaStream_t s, const LevelDims& fine, const LevelDims& coarse, const T* uc,
                    T* uf, const uint8_t* vmask_fine, int nb = 1);
void launch_galerkin_first_impl(cudaStream_t s, const LevelDims& fd, const LevelDims& cd,
                                const double* rhop, const uint8_t* eactive_f, const uint8_t* vmask_f,
                                const double* Ttab64, const float* Ttab32, const double* Ke,
                                const int* fixed_list, int nfixed, double* kel, float* kel32);
template <typename T>
void launch_galerkin_dyadic_t(cudaStream_t s, const LevelDims& fd, const LevelDims& cd,
                              const uint8_t* eactive_f, const T* kel_f, T* kel_c);
template <typename T>
void launch_assemble_stencil_t(cudaStream_t s, const LevelDims& d, const uint8_t* eactive,
                               const uint8_t* vmask, const T* kel, T* st);
void launch_dense_from_stencil(cudaStream_t s, const LevelDims& d, const double* st, double* A);
// work: the blocked kernel's panels (GJB*GJB + 4*GJB*n doubles; null selects
// the unblocked kernel); df_update: rank-GJB updates in double-float arithmetic.
// max_per_sm caps the blocked form's CTAs per SM (it runs beside other work
// on a second stream with 1).
int coarsest_invert(cudaStream_t s, int n, double* A, double* work, int* status_dev, bool df_update = false,
                    int max_per_sm = 2);
void launch_to_float(cudaStream_t s, const double* a, float* b, int64_t n);
template <typename T>
void launch_dense_gemv(cudaStream_t s, int n, const T* Ainv, const T* f_soa, T* u_soa, int64_t nv, int nb = 1);

// vectors and reductions (k_vec.cu)
int reduce_blocks(int64_t n);
// *out = sum of partial[0 .. nb) in index order (one CTA)
void launch_sum_partials(cudaStream_t s, const double* partial, int nb, double* out);
// ctr (optional): a zeroed counter; the last block then writes out itself (one
// launch).  skip_if_zero (with ctr): no work while *skip_if_zero is 0.
template <typename T>
void launch_dot(cudaStream_t s, const T* a, const T* b, int64_t n, double* partial, double* out,
                unsigned* ctr = nullptr, const double* skip_if_zero = nullptr);
// b == nullptr sums a.
void launch_sum(cudaStream_t s, const double* a, int64_t n, double* partial, double* out);
void launch_axpby(cudaStream_t s, double a, const double* x, double b, double* y, int64_t n);
template <typename T>
void launch_fill(cudaStream_t s, T* a, T v, int64_t n);
template <typename T>
void launch_copy(cudaStream_t s, const T* a, T* b, int64_t n);
void launch_d2f(cudaStream_t s, const double* a, float* b, int64_t n);
void launch_f2d_add(cudaStream_t s, const float* a, double* b, int64_t n);
// PCG helpers with device-resident scalars (sc: double scalar slots)
void launch_scalar_ratio(cudaStream_t s, double* sc, int num, int sub, int den, int out);
template <typename T>
void launch_pcg_dir(cudaStream_t s, const T* z, T* d, const double* sc, int beta_slot, bool first, int64_t n,
                    const double* first_if_zero = nullptr);
// launch_pcg_update fused with rr = r.r of the updated residual (2 launches);
// rold may be null (not kept)
template <typename T>
void launch_pcg_update_rr(cudaStream_t s, T* x, T* r, T* rold, const T* d, const T* q, const double* sc,
                          int alpha_slot, int64_t n, double* partial, double* rr, unsigned* ctr = nullptr);
// out = sum of nb partials in a fixed order

// design chain (k_design.cu)
struct SplineDev {
  int order;
  int nb[3];
  const int* i0[3];      // device [n_axis]: first basis index of each element slice, -1 out of range
  const double* N[3];    // device [n_axis][order]: basis values at the element centres
  const float2* Ndf[3];  // device [n_axis][order]: the same values split into (hi, lo) floats
  const int* lo[3];      // device [nb]: first element slice in the support of basis i
  const int* hi[3];      // device [nb]: one past the last element slice
};
// Host-side basis tables (Cox-de Boor, grid/Grid.cu:384-466 at element centres).
struct SplineTables {
  int order = 0;
  int nb[3] = {0, 0, 0};
  std::vector<double> knots[3];
  double kmin[3] = {0, 0, 0}, kstep[3] = {0, 0, 0};
  std::vector<int> i0[3];
  std::vector<double> N[3];
  std::vector<int> lo[3], hi[3];
};
void spline_tables(int order, const int* partition, const double* bmin, const double* bmax,
                   const int* nelem, double h, SplineTables& t);
// Two-pass separable evaluation; Btmp holds nb[0]*ey*ez doubles.
// coeff_df (optional scratch of nc float2): the coefficients are split into
// (hi, lo) floats there and both passes run in double-float
void launch_coeff_to_density(cudaStream_t s, const LevelDims& d, const uint8_t* eactive,
                             const SplineDev& sp, const double* coeff, double rho_min, double penal,
                             double* rho, double* rhop, float* rhop32, double* Btmp, float2* coeff_df = nullptr);
// coeff_df: the trial coefficients split into (hi, lo) floats (from launch_oc_trial)
void launch_trial_volume(cudaStream_t s, const LevelDims& d, const uint8_t* eactive,
                         const SplineDev& sp, const float2* coeff_df, double rho_min, double* partial,
                         double* out, double* Btmp);
void launch_sensitivity(cudaStream_t s, const LevelDims& d, const uint8_t* eactive,
                        const double* rho, const double* u, double penal, double lam, double mu,
                        double h, double* sens);
// sens = -p E / rho in place, from element energies E = u_e . (rho^p Ke u_e)
void launch_sensitivity_from_energy(cudaStream_t s, int64_t ne, const uint8_t* eactive, const double* rho,
                                    double penal, double* sens);
// The same filter in double-float, in place on sens (sens_df: ne float2 scratch;
// wts: the weights split into (hi, lo) floats)
void launch_filter_df(cudaStream_t s, const LevelDims& d, const uint8_t* eactive, double* sens,
                      float2* sens_df, const int4* offs, const float2* wts, int noffs);
void filter_table(double R, std::vector<int4>& offs, std::vector<double>& w);
void launch_spline_adjoint(cudaStream_t s, const LevelDims& d, const uint8_t* eactive,
                           const SplineDev& sp, const double* sens, double* csens, double* tmp1,
                           double* tmp2);
void launch_penalise(cudaStream_t s, int64_t ne, const uint8_t* eactive, const double* rho,
                     double penal, double* rhop, float* rhop32);
void launch_penalise_ref32(cudaStream_t s, int64_t ne, const uint8_t* eactive, double* rho, double penal,
                           double* rhop, float* rhop32);
void launch_round_f32(cudaStream_t s, int64_t n, double* x);
// Handle state used by the allocation-free entry point (k_noalloc.cu).
struct SplineView {
  LevelDims d;
  const uint8_t* eactive;
  SplineDev sp;
  cudaStream_t stream;
  int device;
};
int handle_spline_view(topo_handle* h, SplineView* out);
int handle_fail(topo_handle* h, int code, const char* msg);
// Level-0 view of the handle for the worst-case compliance driver (worst.cu).
struct LevelView {
  LevelDims d;
  const uint8_t* vmask;
  cudaStream_t stream;
  int device;
};
int handle_level_view(topo_handle* h, LevelView* out);
int handle_filter_prepare(topo_handle* h, double radius);
struct WorstState;
void worst_free(WorstState* w);
struct SupportState;
void support_free(SupportState* s);
int support_array(SupportState* s, int which, void** ptr, size_t* count);
WorstState*& handle_worst_slot(topo_handle* h);
#define RET_IF(x)                   \
  do {                              \
    const int rc_ = (x);            \
    if (rc_ != TOPO_OK) return rc_; \
  } while (0)
// cnew_df (optional): cnew split into (hi, lo) floats as well; thres_p
// (optional): the threshold read from device memory instead of thres
void launch_oc_trial(cudaStream_t s, int64_t nc, const double* cold, const double* csens, double thres,
                     double damp, double step, double cmin, double cmax, double* cnew, float2* cnew_df = nullptr,
                     const double* thres_p = nullptr);
void launch_maxabs(cudaStream_t s, const double* a, int64_t n, double* partial, double* out);

// bc_regions.cpp: region-predicate boundary conditions (host).
int bc_from_regions(int nx, int ny, int nz, const uint8_t* eactive, const topo_bc_regions* s, uint8_t* fixed,
                    double* loads, int* nfixed, int* nloaded);

// unet.cu: learned preconditioner (U-Net) state, training and application.
struct UNetState;
size_t unet_param_count();
cudaError_t unet_create(UNetState** out, cudaStream_t s, uint64_t seed);
int unet_conv_kernel(const UNetState* u);
// Flags of the tcgen05 kernels' bounded waits (read and cleared; 0: none gave up).
cudaError_t fine_tc_error(int* flag);
cudaError_t conv_tc_error(int* flag);
void unet_set_conv_kernel(UNetState* u, int kind);
void unet_free(UNetState* u);
cudaError_t unet_set_params(UNetState* u, cudaStream_t s, const float* host);
cudaError_t unet_get_params(UNetState* u, cudaStream_t s, float* host);
cudaError_t unet_prepare(UNetState* u, cudaStream_t s, const LevelDims& d, const uint8_t* eactive, const double* rho,
                         double rho_min);
cudaError_t unet_apply(UNetState* u, cudaStream_t s, const LevelDims& d, const uint8_t* vmask, const float* rhop32,
                       int tz, const float* r, float* z,
                       double* partial);
cudaError_t unet_rejected(UNetState* u, cudaStream_t s, int* out);
cudaError_t unet_harvest_record(UNetState* u, cudaStream_t s, int64_t n3, const double* r, const float* z,
                                const double* x, int cap);
cudaError_t unet_harvest_finish(UNetState* u, cudaStream_t s, const LevelDims& d, const uint8_t* vmask,
                                const double* ustar, int crops_per_iterate, double* partial);
cudaError_t unet_dataset_reserve(UNetState* u, int cap, int S);
int unet_dataset_count(const UNetState* u);
int unet_crop_side(const UNetState* u);
cudaError_t unet_dataset_get(UNetState* u, cudaStream_t s, int slot, float* x, float* t, uint8_t* m);
cudaError_t unet_train(UNetState* u, cudaStream_t s, int steps, int batch, double lr, uint64_t seed, int lo, int hi,
                       bool update, double* loss_out);
cudaError_t unet_host_pass(UNetState* u, cudaStream_t s, int X, int Y, int Z, int nb, const float* x, const float* t,
                           const uint8_t* m, float* y, double* loss, float* grad);

// k_multi.cu: batched vectors of the multi-right-hand-side solver.
template <typename T>
void launch_bdot(cudaStream_t s, const T* a, const T* b, int64_t n, int nb, double* partial, double* out);
void launch_bbeta(cudaStream_t s, int nb, const double* rz, const double* zrold, const double* rzold, bool first,
                  double* beta);
void launch_balpha(cudaStream_t s, int nb, const double* rz, const double* dq, const double* rr, const double* ff,
                   double rtol2, double* alpha, double* rzold);
template <typename T>
void launch_bdir(cudaStream_t s, int64_t n, int nb, const T* z, T* d, const double* beta);
template <typename T>
void launch_bupdate(cudaStream_t s, int64_t n, int nb, T* x, T* r, T* rold, const T* d, const T* q,
                    const double* alpha);

// Batched buffers of the multi-right-hand-side solver (topo_multi_reserve).
struct MultiRhs {
  int cap = 0;
  std::vector<float*> U, F, R, U2, cd;  // per level, cap * 3 nv
  double *x = nullptr, *f = nullptr, *r = nullptr, *d = nullptr, *q = nullptr, *rold = nullptr, *z = nullptr;
  float *x32 = nullptr, *d32 = nullptr, *q32 = nullptr;  // inner FP32 CG, level 0, cap * 3 nv
  double* part = nullptr;  // reduction partials [cap][256]
  double* sc = nullptr;    // scalars [kSlots][cap]
  std::vector<void*> allocs;
};

}  // namespace topo
