// C ABI of libtopo_gb300: handle life cycle, array transfer and the host
// orchestration of the hot path (operator update, V-cycle, PCG, mixed-precision
// defect correction, sensitivity chain and OC bisection).
#include <algorithm>
#include <thread>
#include <mutex>
#include <chrono>
#include <atomic>
#include <array>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include <cuda_profiler_api.h>

#include "topo_internal.h"

namespace topo {
std::atomic<long long> g_launches{0};
thread_local long long t_launches = 0;
}

using namespace topo;


// The sums fused into the FP32 fine kernels finish in their last CTA (1) or
// in a one-CTA kernel after them (0).  Measured at 256x128x128: without the
// last-CTA ticket (a fence and an atomic per CTA while the CTA waits) the
// Chebyshev step with r.z ran 111.0 against 117.8 us and the operator with d.q
// 85.3 against 90.2 us, but the 38 one-CTA sums took 8 us each; the design
// iteration was the same (27.00 against 27.02 ms).
#ifndef TOPO_FUSED_DOT_TICKET
#define TOPO_FUSED_DOT_TICKET 1
#endif

// CTAs per SM of the coarsest inversion when it runs on the side stream next
// to the solve's set-up kernels: one up to TOPO_GJ_SIDE_LARGE_N unknowns
// (256x128x128: n = 675, where the set-up kernels need the SMs as much as the
// inversion: two CTAs per SM there ran the design iteration at 26.0-26.3
// against 25.7 ms), two above, where the inversion outlasts the set-up by far
// (n = 1617: about 6 against 1 ms)
#ifndef TOPO_GJ_SIDE_PER_SM
#define TOPO_GJ_SIDE_PER_SM 1
#endif
#ifndef TOPO_GJ_SIDE_LARGE_N
#define TOPO_GJ_SIDE_LARGE_N 1000
#endif

#include "handle.h"

// z-march depth argument of the handle's FP32 fine-kernel launches
static inline int tz32_arg(const topo_handle* h) {
  return h->tz32 | (h->fine_tc ? TOPO_FINE_TC_FLAG : 0) | fine_rows_flag(h->rows32);
}

namespace {

int fail(topo_handle* h, int code, const char* fmt, ...) {
  if (h) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    h->err = buf;
  }
  return code;
}

#define CK(call)                                                                          \
  do {                                                                                    \
    cudaError_t e_ = (call);                                                              \
    if (e_ != cudaSuccess)                                                                \
      return fail(h, TOPO_E_CUDA, "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), \
                  __FILE__, __LINE__);                                                    \
  } while (0)

#define CKL()                                                                              \
  do {                                                                                     \
    cudaError_t e_ = cudaGetLastError();                                                   \
    if (e_ != cudaSuccess)                                                                 \
      return fail(h, TOPO_E_CUDA, "kernel launch failed: %s (%s:%d)", cudaGetErrorString(e_), \
                  __FILE__, __LINE__);                                                     \
  } while (0)

// Runs the rest of an entry point on the handle's device (null handle: nothing).
#define DEVICE_SCOPE(h) topo::DeviceScope device_scope_((h) ? (h)->cfg.device : -1)

// CUDA event destroyed when it leaves scope, on every return path.
struct ScopedEvent {
  cudaEvent_t e = nullptr;
  cudaError_t create() { return cudaEventCreate(&e); }
  operator cudaEvent_t() const { return e; }
  ScopedEvent() = default;
  ScopedEvent(const ScopedEvent&) = delete;
  ScopedEvent& operator=(const ScopedEvent&) = delete;
  ~ScopedEvent() { if (e) cudaEventDestroy(e); }
};

#define RET(x)                   \
  do {                           \
    int rc_ = (x);               \
    if (rc_ != TOPO_OK) return rc_; \
  } while (0)

template <typename T>
int dalloc(topo_handle* h, T** p, int64_t n) {
  *p = nullptr;
  if (n <= 0) n = 1;
  cudaError_t e = cudaMalloc((void**)p, sizeof(T) * (size_t)n);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(h, TOPO_E_NOMEM, "cudaMalloc of %lld bytes failed: %s", (long long)(sizeof(T) * n),
                cudaGetErrorString(e));
  }
  h->allocs.push_back((void*)*p);
  cudaMemsetAsync(*p, 0, sizeof(T) * (size_t)n, h->stream);
  return TOPO_OK;
}

// ---- profiling brackets --------------------------------------------------
EventPair* prof_begin(topo_handle* h, int fam) {
  if (!h->prof) return nullptr;
  if (h->capturing) {
    EventPair g;
    cudaEventCreate(&g.a);
    cudaEventCreate(&g.b);
    cudaEventRecordWithFlags(g.a, h->stream, cudaEventRecordExternal);
    h->gprof.push_back({fam, g});
    return &h->gprof.back().second;
  }
  EventPair p;
  if (!h->evpool.empty()) {
    p = h->evpool.back();
    h->evpool.pop_back();
  } else {
    cudaEventCreate(&p.a);
    cudaEventCreate(&p.b);
  }
  cudaEventRecord(p.a, h->stream);
  h->evs[fam].push_back(p);
  return &h->evs[fam].back();
}
void prof_end(topo_handle* h, EventPair* p) {
  if (!p) return;
  if (h->capturing) cudaEventRecordWithFlags(p->b, h->stream, cudaEventRecordExternal);
  else cudaEventRecord(p->b, h->stream);
}

// Adds the timings of the last graph replay to the profile (the replay must be
// complete before its events are re-recorded by the next one).
void prof_collect(topo_handle* h) {
  if (!h->gprof_pending) return;
  cudaEventSynchronize(h->gprof.back().second.b);
  for (auto& fp : h->gprof) {
    float t = 0;
    if (cudaEventElapsedTime(&t, fp.second.a, fp.second.b) == cudaSuccess) {
      h->gprof_ms[fp.first] += t;
      h->gprof_n[fp.first] += 1;
    }
  }
  h->gprof_pending = false;
}

void prof_drop_graph_events(topo_handle* h) {
  for (auto& fp : h->gprof) { cudaEventDestroy(fp.second.a); cudaEventDestroy(fp.second.b); }
  h->gprof.clear();
  h->gprof_pending = false;
}

// ---- level operations (templated on precision) ---------------------------
template <typename T> struct P;
template <> struct P<double> {
  static double* U(DevLevel& L) { return L.U; }
  static double* U2(DevLevel& L) { return L.U2; }
  static double* F(DevLevel& L) { return L.F; }
  static double* R(DevLevel& L) { return L.R; }
  static double* st(DevLevel& L) { return L.stencil; }
  static double* dinv(DevLevel& L) { return L.dinv; }
  static double* cd(DevLevel& L) { return L.cd; }
  static double* rhop(topo_handle* h) { return h->rhop; }
  static double* Ainv(topo_handle* h) { return h->A; }
  static double& lmax(DevLevel& L) { return L.lmax; }
  static double*& eig(DevLevel& L) { return L.eig; }
  static double& lprev(DevLevel& L) { return L.lprev; }
  static const int fam_apply = TOPO_K_FINE_APPLY64, fam_smooth = TOPO_K_FINE_SMOOTH64;
  static const int table = 0;  // Chebyshev coefficient table block
};
template <> struct P<float> {
  static float* U(DevLevel& L) { return L.U32; }
  static float* U2(DevLevel& L) { return L.U2_32; }
  static float* F(DevLevel& L) { return L.F32; }
  static float* R(DevLevel& L) { return L.R32; }
  static float* st(DevLevel& L) { return L.stencil32; }
  static float* dinv(DevLevel& L) { return L.dinv32; }
  static float* cd(DevLevel& L) { return L.cd32; }
  static float* rhop(topo_handle* h) { return h->rhop32; }
  static float* Ainv(topo_handle* h) { return h->A32; }
  static double& lmax(DevLevel& L) { return L.lmax32; }
  static float*& eig(DevLevel& L) { return L.eig32; }
  static double& lprev(DevLevel& L) { return L.lprev32; }
  static const int fam_apply = TOPO_K_FINE_APPLY32, fam_smooth = TOPO_K_FINE_SMOOTH32;
  static const int table = 1;
};

// (c_old, c_new) of Chebyshev step k on level l in precision T
template <typename T>
const double* cheb_coef(const topo_handle* h, int l, int k) {
  return h->chebc + 2 * ((P<T>::table * S_MAXLEV + l) * CHEB_MAX_DEG + k);
}

// out = A_l u (residual: out = f - A_l u)
template <typename T>
void level_apply(topo_handle* h, int l, const T* u, const T* f, T* out, bool residual) {
  DevLevel& L = h->lv[l];
  if (l == 0) {
    EventPair* ev = prof_begin(h, P<T>::fam_apply);
    if (sizeof(T) == 8 && h->fine_df)
      launch_fine_apply_df(h->stream, L.d, reinterpret_cast<const double*>(P<T>::rhop(h)), L.vmask,
                           reinterpret_cast<const double*>(u), reinterpret_cast<const double*>(f),
                           reinterpret_cast<double*>(out), residual, h->nb, h->tz64);
    else
      launch_fine_apply<T>(h->stream, L.d, P<T>::rhop(h), L.vmask, u, f, out, residual, h->nb,
                           sizeof(T) == 4 ? tz32_arg(h) : h->tz64);
    prof_end(h, ev);
  } else {
    launch_stencil_apply<T>(h->stream, L.d, P<T>::st(L), u, f, out, residual, h->nb);
  }
  count_launch();
}

template <typename T>
void level_residual(topo_handle* h, int l) {
  DevLevel& L = h->lv[l];
  level_apply<T>(h, l, P<T>::U(L), P<T>::F(L), P<T>::R(L), true);
}

template <typename T>
void gs_level(topo_handle* h, int l, int sweeps, bool reverse) {
  DevLevel& L = h->lv[l];
  for (int s = 0; s < sweeps; ++s)
    for (int cc = 0; cc < 8; ++cc) {
      const int col = reverse ? 7 - cc : cc;
      if (l == 0) {
        EventPair* ev = prof_begin(h, P<T>::fam_smooth);
        launch_fine_gs<T>(h->stream, L.d, P<T>::rhop(h), L.vmask, P<T>::U(L), P<T>::F(L), col, reverse);
        prof_end(h, ev);
      } else {
        launch_stencil_gs<T>(h->stream, L.d, P<T>::st(L), L.vmask, P<T>::U(L), P<T>::F(L), col, reverse);
      }
      count_launch();
    }
}

template <typename T>
void diag_inv_level(topo_handle* h, int l) {
  DevLevel& L = h->lv[l];
  if (l == 0) launch_fine_diag_inv<T>(h->stream, L.d, P<T>::rhop(h), L.vmask, P<T>::dinv(L));
  else launch_stencil_diag_inv<T>(h->stream, L.d, P<T>::st(L), L.vmask, P<T>::dinv(L));
  count_launch();
}

struct ChebParams {
  int degree = 2;
  double lo = 0.3, hi = 1.1;
};

// Chebyshev polynomial smoother in point-block-Jacobi form (three-term
// recurrence, Saad, Iterative Methods for Sparse Linear Systems, Alg. 12.1).
// Each step is one fused kernel that reads the iterate from one buffer and
// writes the next into the other; the result ends in level U.  With
// zero_start the iterate is known to be zero on entry (level U is not read),
// and the first step is the operator-free d = c_new D^-1 f.  The step
// coefficients come from the device table (cheb_upload), so a captured cycle
// stays valid when the spectral bounds move.
template <typename T>
void cheb_level(topo_handle* h, int l, const ChebParams& cp, bool zero_start, bool last_dots = false) {
  DevLevel& L = h->lv[l];
  T* ua = P<T>::U(L);
  T* ub = P<T>::U2(L);
  for (int k = 0; k < cp.degree; ++k) {
    const double* coef = cheb_coef<T>(h, l, k);
    // FP32 level 0 after a zero start: d = u after the first step, so it is
    // not stored and the second step reads it from u
    const bool d_in_u = l == 0 && sizeof(T) == 4 && zero_start;
    if (k == 0 && zero_start) {
      // not in the smoother's profiling family: no operator is applied
      if (l == 0)
        launch_fine_cheb_zero<T>(h->stream, L.d, P<T>::rhop(h), L.vmask, P<T>::F(L), ub, P<T>::dinv(L),
                                 d_in_u ? nullptr : P<T>::cd(L), coef, h->nb);
      else
        launch_cheb_zero_stored<T>(h->stream, L.d.nv, nullptr, P<T>::dinv(L), P<T>::F(L), P<T>::cd(L), ub, coef,
                                   h->nb);
    } else if (l == 0) {
      const bool dots = last_dots && k == cp.degree - 1;
      EventPair* ev = prof_begin(h, P<T>::fam_smooth);
      const int np = launch_fine_cheb<T>(
          h->stream, L.d, P<T>::rhop(h), L.vmask, ua, P<T>::F(L), ub, P<T>::dinv(L), P<T>::cd(L), coef, k == 0,
          h->nb, sizeof(T) == 4 ? tz32_arg(h) : h->tz64, d_in_u && k == 1, dots ? h->vdot : nullptr, h->fdot_cap,
          h->vdot_out, TOPO_FUSED_DOT_TICKET ? h->ctr : nullptr);
      if (np > 0 && !TOPO_FUSED_DOT_TICKET) {
        launch_sum_partials(h->stream, h->vdot, np, h->vdot_out);
        count_launch();
      }
      prof_end(h, ev);
      if (dots && np == 0) {  // r.z of the cycle's result (F is r, the output is z), unfused
        launch_dot<T>(h->stream, P<T>::F(L), ub, 3 * L.d.nv, h->partial, h->vdot_out, h->ctr);
        count_launch();
      }
    } else {
      launch_stencil_cheb<T>(h->stream, L.d, P<T>::st(L), ua, P<T>::F(L), ub, P<T>::dinv(L), P<T>::cd(L), coef,
                             k == 0, h->nb);
    }
    count_launch();
    std::swap(ua, ub);
  }
  if (ua != P<T>::U(L)) {
    cudaMemcpyAsync(P<T>::U(L), ua, sizeof(T) * 3 * L.d.nv * h->nb, cudaMemcpyDeviceToDevice, h->stream);
  }
}

template <typename T>
void smooth_level(topo_handle* h, int l, int sweeps, bool reverse, int smoother, const ChebParams& cp,
                  bool zero_start = false, bool last_dots = false) {
  if (smoother == TOPO_SMOOTH_CHEBYSHEV) {
    for (int s = 0; s < sweeps; ++s) cheb_level<T>(h, l, cp, zero_start && s == 0, last_dots && s == sweeps - 1);
  } else {
    gs_level<T>(h, l, sweeps, reverse);
  }
}

template <typename T>
void coarsest_solve_T(topo_handle* h) {
  DevLevel& L = h->lv.back();
  launch_dense_gemv<T>(h->stream, h->ndense, P<T>::Ainv(h), P<T>::F(L), P<T>::U(L), L.d.nv, h->nb);
  count_launch();
}

template <typename T>
void restrict_T(topo_handle* h, int lc) {
  launch_restrict<T>(h->stream, h->lv[lc - 1].d, h->lv[lc].d, P<T>::R(h->lv[lc - 1]), P<T>::F(h->lv[lc]), h->nb);
  count_launch();
}

template <typename T>
void prolong_T(topo_handle* h, int lf) {
  launch_prolong<T>(h->stream, h->lv[lf].d, h->lv[lf + 1].d, P<T>::U(h->lv[lf + 1]), P<T>::U(h->lv[lf]),
                    h->lv[lf].vmask, h->nb);
  count_launch();
}

// True when a V-cycle from a zero guess never reads level U before writing it
// in full: Chebyshev pre-smoothing, whose first step from zero writes the
// iterate without reading it.
inline bool cheb_zero_start(int smoother, int pre, const ChebParams& cp) {
  return smoother == TOPO_SMOOTH_CHEBYSHEV && pre >= 1 && cp.degree >= 1;
}

// V-cycle in the reference order (grid/Grid.cpp:2399-2444).  `sym` runs the
// adjoint sweep after the coarse correction so the cycle is a symmetric
// preconditioner.  Level-0 U must hold the initial guess, F the right-hand side;
// zero0 declares that guess to be zero (a preconditioner application), which
// lets the first Chebyshev step on level 0 skip the operator.  Coarse levels
// always start from zero: with Chebyshev pre-smoothing their first step skips
// the operator and writes U in full, so U is not cleared first.
template <typename T>
void vcycle_core(topo_handle* h, int pre, int post, bool sym, int smoother, const ChebParams& cp,
                 bool zero0 = false) {
  const int nl = (int)h->lv.size();
  const bool cheb_pre = cheb_zero_start(smoother, pre, cp);
  if (nl == 1) {
    smooth_level<T>(h, 0, pre, false, smoother, cp, zero0);
    smooth_level<T>(h, 0, post, sym, smoother, cp, false, h->vdot_on && sizeof(T) == 4);
    return;
  }
  for (int l = 0; l < nl; ++l) {
    if (l > 0) {
      level_residual<T>(h, l - 1);
      restrict_T<T>(h, l);
      if (!(cheb_pre && l < nl - 1))
        cudaMemsetAsync(P<T>::U(h->lv[l]), 0, sizeof(T) * 3 * h->lv[l].d.nv * h->nb, h->stream);
    }
    if (l < nl - 1) smooth_level<T>(h, l, pre, false, smoother, cp, l > 0 || zero0);
    else coarsest_solve_T<T>(h);
  }
  for (int l = nl - 2; l >= 0; --l) {
    prolong_T<T>(h, l);
    smooth_level<T>(h, l, post, sym, smoother, cp, false, l == 0 && h->vdot_on && sizeof(T) == 4);
  }
}

// What a captured FP32 V-cycle depends on besides buffer contents.
static std::vector<double> vcycle_key(const topo_handle* h, int pre, int post, int smoother, const ChebParams& cp,
                                      bool zero0) {
  std::vector<double> key = {(double)pre, (double)post, (double)smoother, (double)cp.degree,
                             (double)tz32_arg(h), (double)h->nb, (double)h->prof, (double)zero0,
                             (double)h->vdot_on, (double)(uintptr_t)h->vdot_out};
  for (const DevLevel& L : h->lv) {
    key.push_back((double)(uintptr_t)L.U32);
    key.push_back((double)(uintptr_t)L.F32);
  }
  return key;
}

// The FP32 preconditioning V-cycle as one CUDA graph launch.  The cycle is a
// fixed sequence of kernels, memsets and device copies for a given schedule,
// tiles and buffers, so it is captured once and replayed; any change of that
// key re-captures it.  The Chebyshev coefficients are read from the device
// table, so new spectral bounds need no new capture.  Small grids and the coarse levels
// are launch-bound, and one graph launch replaces about forty.
static void vcycle32(topo_handle* h, int pre, int post, int smoother, const ChebParams& cp, bool zero0) {
  if (!h->graphs || h->in_capture) {  // (inside a capture the cycle's kernels join the captured graph)
    vcycle_core<float>(h, pre, post, true, smoother, cp, zero0);
    return;
  }
  prof_collect(h);
  const std::vector<double> key = vcycle_key(h, pre, post, smoother, cp, zero0);
  if (!h->vgraph || key != h->vkey) {
    if (h->vgraph) { cudaGraphExecDestroy(h->vgraph); h->vgraph = nullptr; }
    prof_drop_graph_events(h);
    const long long l0 = t_launches;
    cudaGraph_t g = nullptr;
    bool ok = cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal) == cudaSuccess;
    if (ok) {
      h->capturing = true;
      vcycle_core<float>(h, pre, post, true, smoother, cp, zero0);
      h->capturing = false;
      ok = cudaStreamEndCapture(h->stream, &g) == cudaSuccess && g;
    }
    h->vgraph_kernels = t_launches - l0;
    g_launches.fetch_sub(h->vgraph_kernels);
    t_launches = l0;
    if (ok) ok = cudaGraphInstantiate(&h->vgraph, g, 0) == cudaSuccess;
    if (g) cudaGraphDestroy(g);
    cudaGetLastError();
    if (!ok) {  // capture not available: launch directly from now on
      h->vgraph = nullptr;
      h->graphs = false;
      prof_drop_graph_events(h);
      vcycle_core<float>(h, pre, post, true, smoother, cp, zero0);
      return;
    }
    h->vkey = key;
  }
  cudaGraphLaunch(h->vgraph, h->stream);
  count_launch((int)h->vgraph_kernels);
  h->gprof_pending = h->prof && !h->gprof.empty();
}

// Power iteration for the largest eigenvalue of D^{-1} A on a level, from the
// same deterministic start vector as the oracle.
template <typename T>
__global__ void k_power_start(int64_t nv, const uint8_t* vmask, T* x) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= 3 * nv) return;
  uint64_t hsh = (uint64_t)i * 0x9E3779B97F4A7C15ull;
  hsh ^= hsh >> 29;
  double v = 0.5 + (double)(hsh % 1000) / 1000.0;
  const int64_t vv = i % nv;
  const int c = (int)(i / nv);
  if (!((vmask[vv] >> c) & 1) || !(vmask[vv] & 8)) v = 0.0;
  x[i] = (T)v;
}

// z = s D^-1 r with s = 1/sqrt(*nrm2) (the power iteration's normalisation of
// its vector, applied after the operator, which is linear).  D^-1 is [9][nv],
// or with sym the packed symmetric layout of level 0's FP32 inverse (float4
// d00 d01 d02 d11 per vertex, then float2 d12 d22).
template <typename T>
__global__ void k_dinv_apply(int64_t nv, const T* dinv, const T* r, T* z, const double* nrm2, bool sym) {
  const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= nv) return;
  const T sc = (T)rsqrt(*nrm2);
  const T r0 = r[v] * sc, r1 = r[nv + v] * sc, r2 = r[2 * nv + v] * sc;
  if constexpr (sizeof(T) == 4) {
    if (sym) {
      const float4 a = reinterpret_cast<const float4*>(dinv)[v];
      const float2 b = reinterpret_cast<const float2*>(dinv + 4 * nv)[v];
      z[v] = a.x * r0 + a.y * r1 + a.z * r2;
      z[nv + v] = a.y * r0 + a.w * r1 + b.x * r2;
      z[2 * nv + v] = a.z * r0 + b.x * r1 + b.y * r2;
      return;
    }
  }
  for (int i = 0; i < 3; ++i)
    z[i * nv + v] = dinv[(3 * i) * nv + v] * r0 + dinv[(3 * i + 1) * nv + v] * r1 + dinv[(3 * i + 2) * nv + v] * r2;
}

template <typename T>
__global__ void k_to_double(int64_t n, const T* a, double* b) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) b[i] = (double)a[i];
}

inline unsigned nb256(int64_t n) { return (unsigned)((n + 255) / 256); }

// Loop control of the device-side inner CG (slots loop[0..3]: iterations of
// this solve, ||b|| reference, first non-finite iteration (1-based, 0 none),
// iterations summed over the solve).  Start: zero the count, take ||b|| from
// the outer residual (1 if that is 0) and test ||r|| / ||b|| > rtol.
__global__ void k_loop_start(double* loop, const double* rr_outer, const double* rr, double rtol, int maxit,
                             cudaGraphConditionalHandle hc) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const double bo = sqrt(*rr_outer);
  const double bn = bo > 0 ? bo : 1.0;
  loop[0] = 0.0;
  loop[1] = bn;
  cudaGraphSetConditional(hc, (sqrt(*rr) / bn > rtol && 0 < maxit) ? 1u : 0u);
}

// End of one iteration: count it and test again; a non-finite ||r|| stops the
// loop and is recorded.
__global__ void k_loop_step(double* loop, const double* rr, double rtol, int maxit, cudaGraphConditionalHandle hc) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const double it = loop[0] + 1.0;
  loop[0] = it;
  loop[3] += 1.0;
  const double rn = sqrt(*rr);
  unsigned go = 0;
  if (!isfinite(rn)) {
    if (loop[2] == 0.0) loop[2] = it;
  } else {
    go = (rn / loop[1] > rtol && it < (double)maxit) ? 1u : 0u;
  }
  cudaGraphSetConditional(hc, go);
}

// OC bisection on the device (slots oc[0..5]: lo, hi, threshold of the
// current trial, its volume fraction, trials, repeats).  Start: lo = 0, hi =
// max |dc|, the first threshold; the loop body (a do-while) runs at least once.
__global__ void k_ocl_start(double* oc, const double* gmax, cudaGraphConditionalHandle hc) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  oc[0] = 0.0;
  oc[1] = *gmax;
  oc[2] = 0.5 * (oc[0] + oc[1]);
  oc[4] = 0.0;
  oc[5] = 0.0;
  cudaGraphSetConditional(hc, 1u);
}

// After a trial of volume *vol: the volume fraction, the new bracket and the
// loop test of the reference (repeat while |V - vgoal| > 1e-4 and itn++ < 30,
// at most 32 trials); the next threshold when it repeats.
__global__ void k_ocl_step(double* oc, const double* vol, double den, double vgoal, cudaGraphConditionalHandle hc) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const double thres = oc[2];
  const double V = *vol / den;
  oc[3] = V;
  oc[4] += 1.0;
  double lo = oc[0], hi = oc[1];
  if (V > vgoal) lo = thres;
  else if (V < vgoal) hi = thres;
  oc[0] = lo;
  oc[1] = hi;
  bool go = fabs(V - vgoal) > 1e-4;
  if (go) {
    go = oc[5] < 30.0;
    oc[5] += 1.0;
  }
  if (go) oc[2] = 0.5 * (lo + hi);
  cudaGraphSetConditional(hc, go ? 1u : 0u);
}

// beta = (r.z - z.rold) / rold.z after the first iteration (the host loop's
// scalar ratio, taken when the iteration counter is past 0).
__global__ void k_loop_beta(const double* loop, double* sc) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  if (loop[0] > 0.0) sc[S_BETA] = (sc[S_RZ] - sc[S_ZROLD]) / sc[S_RZOLD];
}

int read_scalars(topo_handle* h, int first, int count);

// Inside a capture on h->stream: a conditional node of `type` (IF or WHILE)
// with condition hc after the work captured so far, and the capture goes on
// after it.  body() is captured as the node's body graph on a helper stream,
// which stands in for h->stream meanwhile, so the enclosing capture stays open
// (streams forked from it, the side stream say, need not have joined).
// Kernels of one body pass come back in *per_body.  TOPO_E_STATE: the node
// could not be made (no helper stream left, or a conditional node nested in
// another one's body not available); the enclosing capture then fails.
template <typename Body>
int capture_cond_node(topo_handle* h, cudaGraphConditionalHandle hc, cudaGraphConditionalNodeType type,
                      Body&& body, long long* per_body) {
  const cudaStreamCaptureMode mode = cudaStreamCaptureModeThreadLocal;
  cudaStream_t s = h->stream;
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  cudaGraph_t g = nullptr;
  const cudaGraphNode_t* dp = nullptr;
  size_t nd = 0;
  if (h->cdepth >= TOPO_COND_DEPTH || !h->cstream[h->cdepth]) return TOPO_E_STATE;
  if (cudaStreamGetCaptureInfo(s, &cs, nullptr, &g, &dp, nullptr, &nd) != cudaSuccess ||
      cs != cudaStreamCaptureStatusActive || !g)
    return TOPO_E_STATE;
  cudaGraphNodeParams cp = {};
  cp.type = cudaGraphNodeTypeConditional;
  cp.conditional.handle = hc;
  cp.conditional.type = type;
  cp.conditional.size = 1;
  cudaGraphNode_t cnode = nullptr;
  if (cudaGraphAddNode(&cnode, g, dp, nullptr, nd, &cp) != cudaSuccess) return TOPO_E_STATE;
  if (cudaStreamUpdateCaptureDependencies(s, &cnode, nullptr, 1, cudaStreamSetCaptureDependencies) != cudaSuccess)
    return TOPO_E_STATE;
  cudaStream_t bs = h->cstream[h->cdepth];
  if (cudaStreamBeginCaptureToGraph(bs, cp.conditional.phGraph_out[0], nullptr, nullptr, 0, mode) != cudaSuccess)
    return TOPO_E_STATE;
  h->stream = bs;
  ++h->cdepth;
  const long long l1 = t_launches;
  const int rc = body();
  *per_body = t_launches - l1;
  --h->cdepth;
  h->stream = s;
  cudaGraph_t gs = nullptr;
  const bool ended = cudaStreamEndCapture(bs, &gs) == cudaSuccess;
  RET(rc);
  return ended ? TOPO_OK : TOPO_E_STATE;
}

// Helper streams for the bodies of nested conditional nodes, made before a
// capture begins.
int ensure_cond_streams(topo_handle* h) {
  for (int k = 0; k < TOPO_COND_DEPTH; ++k)
    if (!h->cstream[k]) CK(cudaStreamCreateWithFlags(&h->cstream[k], cudaStreamNonBlocking));
  return TOPO_OK;
}

// Conditions of the levels' restart nodes in a captured power iteration.
struct LevelConds {
  cudaGraphConditionalHandle c[S_MAXLEV];
};

// Spectral bounds on the device, slots of precision table tb: for each level
// in `mask`, lam = (x.z) / |x| (0 when x = 0) from its power-iteration sums
// in sc[S_PW + 2 l ..].  final = 0 (a captured estimate after its first pass):
// sets each warm level's condition to whether lam fell more than 5% below
// sc[S_LPREV] (8 more steps then run) and counts those levels in sc[S_DI + 2].
// final = 1: sc[S_LAM] = sc[S_LPREV] = lam, the values the host computes from
// the same sums when it runs the loop (IEEE division and square root).
__global__ void k_power_lam(double* sc, int tb, unsigned mask, unsigned warm, int final, LevelConds conds) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  int restarts = 0;
  for (int l = 0; l < S_MAXLEV; ++l) {
    if (!((mask >> l) & 1u)) continue;
    const double xx = sc[S_PW + 2 * l], xz = sc[S_PW + 2 * l + 1];
    const double lam = xx > 0 ? xz / sqrt(xx) : 0.0;
    double* lp = sc + S_LPREV + tb * S_MAXLEV + l;
    if (final) {
      sc[S_LAM + tb * S_MAXLEV + l] = lam;
      *lp = lam;
    } else {
      const bool again = ((warm >> l) & 1u) && lam < 0.95 * *lp;
      restarts += again ? 1 : 0;
      cudaGraphSetConditional(conds.c[l], again ? 1u : 0u);
    }
  }
  if (!final) sc[S_DI + 2] = (double)restarts;
}

// Chebyshev coefficients of levels 0 .. nl-1 from their bounds lam[l] and the
// interval [lo, hi] x lam (three-term recurrence, Saad, Iterative Methods for
// Sparse Linear Systems, Alg. 12.1): tab[2 (l CHEB_MAX_DEG + k) + {0, 1}] =
// (c_old, c_new) of step k.  One thread per level.
__global__ void k_cheb_table(const double* lam, int nl, double lo, double hi, int degree, double* tab) {
  const int l = threadIdx.x;
  if (l >= nl) return;
  const double lmax = lam[l] * hi, lmin = lam[l] * lo;
  const double theta = 0.5 * (lmax + lmin), delta = 0.5 * (lmax - lmin);
  const double sigma = theta / delta;
  double rho_old = 1.0 / sigma;
  for (int k = 0; k < degree; ++k) {
    double c_old = 0.0, c_new = 1.0 / theta;
    if (k > 0) {
      const double rho_new = 1.0 / (2.0 * sigma - rho_old);
      c_old = rho_new * rho_old;
      c_new = 2.0 * rho_new / delta;
      rho_old = rho_new;
    }
    tab[2 * (l * CHEB_MAX_DEG + k)] = c_old;
    tab[2 * (l * CHEB_MAX_DEG + k) + 1] = c_new;
  }
}

// Largest eigenvalue of D^-1 A of every level whose bound is stale, by power
// iteration.  First estimate of a level: 12 steps from the deterministic start
// (as the oracle).  After an operator update: 4 steps from the previous
// design's vector (the design moves a little per iteration, so the estimate
// keeps refining); if that estimate falls more than 5% below the previous one
// (an abrupt change of the operator), 8 more.  The levels' steps are launched
// back to back with their own scalar slots, so all levels cost one host read
// (two when a warm estimate dropped).
// One step: with s = 1/|x|, z = D^-1 A (s x) = s D^-1 (A x) and the Rayleigh
// estimate (s x).z = s (x.z); x <- z.  Work vectors: the level's R, U2 and
// Chebyshev direction buffers (all free outside a V-cycle).
template <typename T>
int estimate_bounds(topo_handle* h) {
  const int nl = (int)h->lv.size();
  if (nl > S_MAXLEV) return fail(h, TOPO_E_STATE, "%d levels exceed the %d of the spectral-bound slots", nl, S_MAXLEV);
  struct Run {
    int l;
    bool warm;
    T *x, *y, *z;
    double lam;
  };
  std::vector<Run> runs;
  for (int l = 0; l < nl; ++l) {
    DevLevel& L = h->lv[l];
    if (P<T>::lmax(L) != 0.0) continue;
    diag_inv_level<T>(h, l);
    Run r{l, P<T>::eig(L) != nullptr, P<T>::R(L), P<T>::cd(L), P<T>::U2(L), 0.0};
    const int64_t n3 = 3 * L.d.nv;
    if (r.warm) {
      CK(cudaMemcpyAsync(r.x, P<T>::eig(L), sizeof(T) * n3, cudaMemcpyDeviceToDevice, h->stream));
    } else {
      RET(dalloc(h, &P<T>::eig(L), n3));
      k_power_start<T><<<nb256(n3), 256, 0, h->stream>>>(L.d.nv, L.vmask, r.x);
      count_launch();
    }
    runs.push_back(r);
  }
  if (runs.empty()) return TOPO_OK;
  auto power_steps = [&](Run& r, int k) {
    DevLevel& L = h->lv[r.l];
    const int64_t n3 = 3 * L.d.nv;
    double* sl = h->sc + S_PW + 2 * r.l;
    for (int it = 0; it < k; ++it) {
      launch_dot<T>(h->stream, r.x, r.x, n3, h->partial, sl, h->ctr);
      if (r.l == 0) launch_fine_apply<T>(h->stream, L.d, P<T>::rhop(h), L.vmask, r.x, nullptr, r.y, false, 1,
                                         sizeof(T) == 4 ? tz32_arg(h) : h->tz64);
      else launch_stencil_apply<T>(h->stream, L.d, P<T>::st(L), r.x, nullptr, r.y, false);
      k_dinv_apply<T><<<nb256(L.d.nv), 256, 0, h->stream>>>(L.d.nv, P<T>::dinv(L), r.y, r.z, sl,
                                                           sizeof(T) == 4 && r.l == 0);
      launch_dot<T>(h->stream, r.x, r.z, n3, h->partial, sl + 1, h->ctr);
      std::swap(r.x, r.z);
      count_launch(4);
    }
  };
  auto read_all = [&]() -> int {
    RET(read_scalars(h, S_PW, 2 * nl));
    for (Run& r : runs) {
      const double xx = h->hsc[S_PW + 2 * r.l], xz = h->hsc[S_PW + 2 * r.l + 1];
      r.lam = xx > 0 ? xz / std::sqrt(xx) : 0.0;
    }
    return TOPO_OK;
  };
  unsigned mask = 0, warm = 0;
  for (Run& r : runs) {
    mask |= 1u << r.l;
    warm |= r.warm ? 1u << r.l : 0u;
  }
  for (Run& r : runs) power_steps(r, r.warm ? 4 : 12);
  if (h->iter_capture) {
    // inside a captured design iteration: the restart test on the device and
    // one conditional node per level for its 8 more steps (an even count, so
    // the iterate ends in the same buffer either way)
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    cudaGraph_t g = nullptr;
    if (cudaStreamGetCaptureInfo(h->stream, &cs, nullptr, &g, nullptr, nullptr, nullptr) != cudaSuccess || !g)
      return TOPO_E_STATE;
    LevelConds conds{};
    for (Run& r : runs)
      if (cudaGraphConditionalHandleCreate(&conds.c[r.l], g, 0, cudaGraphCondAssignDefault) != cudaSuccess)
        return TOPO_E_STATE;
    k_power_lam<<<1, 32, 0, h->stream>>>(h->sc, P<T>::table, mask, warm, 0, conds);
    count_launch();
    for (Run& r : runs) {
      long long per = 0;
      RET(capture_cond_node(h, conds.c[r.l], cudaGraphCondTypeIf, [&]() -> int {
        power_steps(r, 8);
        return TOPO_OK;
      }, &per));
      h->d_if_body = per;
    }
  } else {
    RET(read_all());
    bool more = false;
    for (Run& r : runs)
      if (r.warm && r.lam < 0.95 * P<T>::lprev(h->lv[r.l])) {
        power_steps(r, 8);
        more = true;
      }
    if (more) RET(read_all());
  }
  k_power_lam<<<1, 32, 0, h->stream>>>(h->sc, P<T>::table, mask, warm, 1, LevelConds{});
  count_launch();
  for (Run& r : runs) {
    DevLevel& L = h->lv[r.l];
    CK(cudaMemcpyAsync(P<T>::eig(L), r.x, sizeof(T) * 3 * L.d.nv, cudaMemcpyDeviceToDevice, h->stream));
    // (a captured estimate: the values are read after the graph ran; any
    // nonzero mark keeps the bound from being estimated twice in the capture)
    P<T>::lmax(L) = h->iter_capture ? -1.0 : r.lam;
    P<T>::lprev(L) = h->iter_capture ? -1.0 : r.lam;
  }
  return TOPO_OK;
}

// Chebyshev coefficients of every level in precision T from the spectral
// bounds in sc[S_LAM] (on the device, so a captured design iteration computes
// them from bounds it estimated itself, and a host-run one gets the same).
template <typename T>
int cheb_upload(topo_handle* h, const ChebParams& cp) {
  if (cp.degree > CHEB_MAX_DEG)
    return fail(h, TOPO_E_BAD_INPUT, "Chebyshev degree %d above %d", cp.degree, CHEB_MAX_DEG);
  const size_t off = (size_t)P<T>::table * 2 * S_MAXLEV * CHEB_MAX_DEG;
  k_cheb_table<<<1, 32, 0, h->stream>>>(h->sc + S_LAM + P<T>::table * S_MAXLEV, (int)h->lv.size(), cp.lo, cp.hi,
                                         cp.degree, h->chebc + off);
  count_launch();
  CKL();
  return TOPO_OK;
}

template <typename T>
int prepare_smoother(topo_handle* h, int smoother, const ChebParams& cp) {
  if (smoother != TOPO_SMOOTH_CHEBYSHEV) return TOPO_OK;
  RET(estimate_bounds<T>(h));
  return cheb_upload<T>(h, cp);
}

int read_scalars(topo_handle* h, int first, int count) {
  if (h->iter_capture)  // (a captured design iteration reads its results after the launch)
    return fail(h, TOPO_E_STATE, "host read of slots %d..%d inside a captured design iteration", first,
                first + count - 1);
  CK(cudaMemcpyAsync(h->hsc + first, h->sc + first, sizeof(double) * count, cudaMemcpyDeviceToHost,
                     h->stream));
  CK(cudaStreamSynchronize(h->stream));
  return TOPO_OK;
}

// One iteration of the flexible CG below: z = M r, the new direction d,
// q = A d with d.q, x += alpha d, r -= alpha q with the new r.r in sc[S_RR].
// `it` is the iteration number when the host runs the loop; it is -1 when the
// loop runs on the device (a graphed solve), where the iteration counter in
// the loop slots `loop` (the inner loop's by default) tells the first
// iteration from the others.
template <typename T, typename Prec>
int fcg_body(topo_handle* h, T* x, T* r, T* d, T* q, T* rold, T* z, double* sc, Prec&& prec, bool prec_dots,
             int it, double* loop = nullptr) {
  if (!loop) loop = h->sc + S_LOOP;
  DevLevel& L0 = h->lv[0];
  const int64_t n3 = 3 * L0.d.nv;
  RET(prec(r, z));
  if (!prec_dots) {  // else the preconditioner left r.z and z.rold in the scalar slots
    launch_dot<T>(h->stream, r, z, n3, h->partial, sc + S_RZ, h->ctr);
    count_launch();
    if (it != 0) {  // (on the device loop's first iteration the kernel returns at once)
      launch_dot<T>(h->stream, z, rold, n3, h->partial, sc + S_ZROLD, h->ctr, it < 0 ? loop : nullptr);
      count_launch();
    }
  }
  if (it < 0) {
    k_loop_beta<<<1, 32, 0, h->stream>>>(loop, sc);
    count_launch();
  } else if (it > 0) {
    launch_scalar_ratio(h->stream, sc, S_RZ, S_ZROLD, S_RZOLD, S_BETA);
  }
  launch_pcg_dir<T>(h->stream, z, d, sc, S_BETA, it == 0, n3, it < 0 ? loop : nullptr);
  // q = A d with d.q: fused into the FP32 operator's epilogue
  int nparts = 0;
  if (sizeof(T) == 4 && h->fdot && h->nb == 1) {
    EventPair* ev = prof_begin(h, P<T>::fam_apply);
    nparts = launch_fine_apply_dot<T>(h->stream, L0.d, P<T>::rhop(h), L0.vmask, d, q, tz32_arg(h), h->fdot,
                                      h->fdot_cap, sc + S_DQ, TOPO_FUSED_DOT_TICKET ? h->ctr : nullptr);
    if (nparts > 0 && !TOPO_FUSED_DOT_TICKET) {
      launch_sum_partials(h->stream, h->fdot, nparts, sc + S_DQ);
      count_launch();
    }
    prof_end(h, ev);
  }
  if (nparts > 0) {
    count_launch();
  } else {
    level_apply<T>(h, 0, d, nullptr, q, false);
    launch_dot<T>(h->stream, d, q, n3, h->partial, sc + S_DQ, h->ctr);
    count_launch();
  }
  launch_scalar_ratio(h->stream, sc, S_RZ, -1, S_DQ, S_ALPHA);
  // x += alpha d, rold = r, r -= alpha q with r.r of the new residual; rold
  // is not kept when the preconditioner runs the plain (Fletcher-Reeves) form
  launch_pcg_update_rr<T>(h->stream, x, r, (prec_dots && h->inner_fr) ? nullptr : rold, d, q, sc, S_ALPHA, n3,
                          h->partial, sc + S_RR, h->ctr);
  CK(cudaMemcpyAsync(sc + S_RZOLD, sc + S_RZ, sizeof(double), cudaMemcpyDeviceToDevice, h->stream));
  count_launch(it > 0 ? 4 : 3);
  CKL();
  return TOPO_OK;
}

// Flexible conjugate gradients (Polak-Ribiere beta, i.e. FCG with one stored
// direction) on level 0 in precision T.  Solves A x = b (warm start in x);
// prec(r, z) writes z = M r.  Scalars live in device slots sc[base .. base+6],
// so an FCG may run nested inside another one's preconditioner.
template <typename T, typename Prec>
int fcg_T(topo_handle* h, T* x, const T* b, T* r, T* d, T* q, T* rold, T* z, double rtol, int maxit,
          int base, Prec&& prec, int* iters, double* rel_out, double bnorm_ref, bool x_zero = false,
          bool prec_dots = false) {
  DevLevel& L0 = h->lv[0];
  const int64_t n3 = 3 * L0.d.nv;
  double* sc = h->sc + base;
  if (x_zero) {  // x = 0 on entry: r = b (r may be b itself)
    if (r != b) CK(cudaMemcpyAsync(r, b, sizeof(T) * n3, cudaMemcpyDeviceToDevice, h->stream));
  } else {
    level_apply<T>(h, 0, x, b, r, true);  // r = b - A x
  }
  launch_dot<T>(h->stream, r, r, n3, h->partial, sc + S_RR, h->ctr);
  count_launch();
  RET(read_scalars(h, base + S_RR, 1));
  double rn = std::sqrt(h->hsc[base + S_RR]);
  const double bn = bnorm_ref;
  int it = 0;
  while (rn / bn > rtol && it < maxit) {
    RET(fcg_body<T>(h, x, r, d, q, rold, z, sc, prec, prec_dots, it));
    RET(read_scalars(h, base + S_RR, 1));
    rn = std::sqrt(h->hsc[base + S_RR]);
    if (!std::isfinite(rn)) return fail(h, TOPO_E_NONFINITE, "CG residual became non-finite at iteration %d", it);
    ++it;
  }
  *iters = it;
  *rel_out = rn / bn;
  return TOPO_OK;
}

// Captures, on h->stream, one executable graph made of set-up kernels, a
// WHILE node and tail kernels.  setup(hc) ends with a kernel that sets the loop
// condition through hc; body(hc) is one pass of the loop and ends with a
// kernel that sets it again (the loop is bounded by that kernel).  Kernels
// counted while capturing come back split into the fixed part and one body
// pass.  TOPO_E_STATE: conditional graphs are not available here.
template <typename Setup, typename Body, typename Tail>
int capture_loop_graph(topo_handle* h, Setup&& setup, Body&& body, Tail&& tail, cudaGraphExec_t* exec,
                       long long* fixed, long long* per_body) {
  RET(ensure_cond_streams(h));
  cudaGraph_t g = nullptr;
  cudaGraphConditionalHandle hc = 0;
  cudaGraphNode_t cnode = nullptr;
  std::vector<cudaGraphNode_t> deps;
  const long long l0 = t_launches;
  long long l1 = l0, l2 = l0;
  int rc = TOPO_OK;
  const cudaStreamCaptureMode mode = cudaStreamCaptureModeThreadLocal;
  bool ok = cudaGraphCreate(&g, 0) == cudaSuccess &&
            cudaGraphConditionalHandleCreate(&hc, g, 0, cudaGraphCondAssignDefault) == cudaSuccess;
  h->in_capture = true;
  // set-up; its last nodes are the loop node's dependencies
  if (ok) ok = cudaStreamBeginCaptureToGraph(h->stream, g, nullptr, nullptr, 0, mode) == cudaSuccess;
  if (ok) {
    rc = setup(hc);
    cudaStreamCaptureStatus cs;
    const cudaGraphNode_t* dp = nullptr;
    size_t nd = 0;
    ok = cudaStreamGetCaptureInfo(h->stream, &cs, nullptr, nullptr, &dp, nullptr, &nd) == cudaSuccess;
    if (ok) deps.assign(dp, dp + nd);
    cudaGraph_t gs = nullptr;
    ok = cudaStreamEndCapture(h->stream, &gs) == cudaSuccess && ok && rc == TOPO_OK;
  }
  cudaGraph_t bg = nullptr;
  if (ok) {
    cudaGraphNodeParams cp = {};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = hc;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    ok = cudaGraphAddNode(&cnode, g, deps.data(), nullptr, deps.size(), &cp) == cudaSuccess;
    if (ok) bg = cp.conditional.phGraph_out[0];
  }
  if (ok) ok = cudaStreamBeginCaptureToGraph(h->stream, bg, nullptr, nullptr, 0, mode) == cudaSuccess;
  if (ok) {
    l1 = t_launches;
    rc = body(hc);
    l2 = t_launches;
    cudaGraph_t gs = nullptr;
    ok = cudaStreamEndCapture(h->stream, &gs) == cudaSuccess && rc == TOPO_OK;
  }
  if (ok) ok = cudaStreamBeginCaptureToGraph(h->stream, g, &cnode, nullptr, 1, mode) == cudaSuccess;
  if (ok) {
    rc = tail();
    cudaGraph_t gs = nullptr;
    ok = cudaStreamEndCapture(h->stream, &gs) == cudaSuccess && rc == TOPO_OK;
  }
  h->in_capture = false;
  *per_body = l2 - l1;
  *fixed = (t_launches - l0) - *per_body;
  g_launches.fetch_sub(t_launches - l0);
  t_launches = l0;
  *exec = nullptr;
  if (ok) ok = cudaGraphInstantiate(exec, g, 0) == cudaSuccess;
  if (g) cudaGraphDestroy(g);
  cudaGetLastError();
  if (!ok) {
    *exec = nullptr;
    return rc != TOPO_OK ? rc : TOPO_E_STATE;
  }
  return TOPO_OK;
}

// Inside a capture on h->stream: a WHILE node after the work captured so far.
// setup(hc) is captured before the node and ends with a kernel that sets the
// loop condition through hc; body(hc), one pass of the loop, is the node's
// body graph and ends with a kernel that sets it again (capture_cond_node).
template <typename Setup, typename Body>
int capture_nested_loop(topo_handle* h, Setup&& setup, Body&& body, long long* per_body) {
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  cudaGraph_t g = nullptr;
  if (cudaStreamGetCaptureInfo(h->stream, &cs, nullptr, &g, nullptr, nullptr, nullptr) != cudaSuccess ||
      cs != cudaStreamCaptureStatusActive || !g)
    return TOPO_E_STATE;
  cudaGraphConditionalHandle hc = 0;
  if (cudaGraphConditionalHandleCreate(&hc, g, 0, cudaGraphCondAssignDefault) != cudaSuccess) return TOPO_E_STATE;
  RET(setup(hc));
  return capture_cond_node(h, hc, cudaGraphCondTypeWhile, [&]() { return body(hc); }, per_body);
}

// The FP32 inner CG of the mixed solve, z = CG(r) from x = 0, as one CUDA
// graph: set-up (r in FP32, x = 0, r.r and the stopping test), a WHILE node
// whose body is one CG iteration (fcg_body) closed by a kernel that counts the
// iteration and sets the loop condition, and the copy of x to FP64 in z.  The
// iterations are the host loop's, kernel for kernel, with the same stopping
// rule (||r|| / ||b|| > rtol and fewer than maxit iterations; ||b|| is the
// outer residual's norm, 1 if that is 0) decided on the device, so the host
// does not wait for the GPU between inner iterations.  The graph is captured
// once per key (buffers, schedule, tiles) and replayed.  Iteration totals and
// a non-finite r.r are left in the loop slots for the caller.
template <typename Prec>
int inner_cg_graphed(topo_handle* h, const double* rin, double* zout, double rtol, int maxit, Prec&& prec,
                     std::vector<double> key) {
  DevLevel& L0 = h->lv[0];
  const int64_t n3 = 3 * L0.d.nv;
  double* sc = h->sc + 8;
  key.insert(key.end(), {rtol, (double)maxit, (double)(uintptr_t)rin, (double)(uintptr_t)zout,
                         (double)(uintptr_t)h->x32, (double)(uintptr_t)h->d32, (double)(uintptr_t)h->q32,
                         (double)tz32_arg(h), (double)(uintptr_t)h->fdot, (double)h->fdot_cap});
  auto setup = [&](cudaGraphConditionalHandle hc) -> int {
    launch_d2f(h->stream, rin, L0.F32, n3);
    CK(cudaMemsetAsync(h->x32, 0, sizeof(float) * n3, h->stream));
    launch_dot<float>(h->stream, L0.F32, L0.F32, n3, h->partial, sc + S_RR, h->ctr);
    k_loop_start<<<1, 32, 0, h->stream>>>(h->sc + S_LOOP, h->sc + S_RR, sc + S_RR, rtol, maxit, hc);
    count_launch(3);
    return TOPO_OK;
  };
  auto body = [&](cudaGraphConditionalHandle hc) -> int {
    RET(fcg_body<float>(h, h->x32, L0.F32, h->d32, h->q32, h->rold32, L0.U32, sc, prec, true, -1));
    k_loop_step<<<1, 32, 0, h->stream>>>(h->sc + S_LOOP, sc + S_RR, rtol, maxit, hc);
    count_launch();
    return TOPO_OK;
  };
  auto tail = [&]() -> int {  // z = x in FP64 after the loop
    k_to_double<float><<<nb256(n3), 256, 0, h->stream>>>(n3, h->x32, zout);
    count_launch();
    return TOPO_OK;
  };
  if (h->in_capture) {  // inside the outer solve's capture: a nested WHILE node
    RET(capture_nested_loop(h, setup, body, h->iter_capture ? &h->d_inner_body : &h->sgraph_inner));
    return tail();
  }
  if (!h->igraph || key != h->ikey) {
    if (h->igraph) { cudaGraphExecDestroy(h->igraph); h->igraph = nullptr; }
    const int rc = capture_loop_graph(h, setup, body, tail, &h->igraph, &h->igraph_fixed, &h->igraph_body);
    if (rc != TOPO_OK) {  // conditional graphs not available: the host runs the loop from now on
      if (rc == TOPO_E_STATE) h->igraph_ok = false;
      return rc;
    }
    h->ikey = key;
  }
  CK(cudaGraphLaunch(h->igraph, h->stream));
  count_launch((int)h->igraph_fixed);
  return TOPO_OK;
}

// The outer FP64 flexible CG of the mixed solve as one CUDA graph: a WHILE
// node whose body is one outer iteration (fcg_body: the FP32 preconditioner,
// one V-cycle or the inner CG as a nested WHILE node, then the FP64 matvec,
// step and update) closed by a kernel that counts the iteration and sets the
// loop condition on the outer loop slots.  The stopping rule is the host
// loop's (||r|| / ||F|| > rtol and fewer than maxit iterations) decided on
// the device, so the host waits for the GPU once per solve instead of once
// per outer iteration.  The set-up (r = f - A x and r.r in sc[S_RR], F.F in
// sc[S_FF]) is launched before, outside the graph, where it overlaps the
// coarsest inversion on the side stream.  Captured once per key and replayed.
template <typename Prec>
int outer_cg_graphed(topo_handle* h, double rtol, int maxit, Prec&& prec, std::vector<double> key) {
  DevLevel& L0 = h->lv[0];
  double* loop = h->sc + S_OLOOP;
  key.insert(key.end(), {rtol, (double)maxit, (double)h->tz64, (double)h->fine_df, (double)(uintptr_t)h->x,
                         (double)(uintptr_t)h->r, (double)(uintptr_t)h->d, (double)(uintptr_t)h->q,
                         (double)(uintptr_t)h->rold, (double)(uintptr_t)L0.U, (double)(uintptr_t)h->x32,
                         (double)(uintptr_t)h->d32, (double)(uintptr_t)h->q32, (double)(uintptr_t)h->rold32,
                         (double)tz32_arg(h), (double)(uintptr_t)h->fdot, (double)h->fdot_cap});
  auto setup = [&](cudaGraphConditionalHandle hc) -> int {
    CK(cudaMemsetAsync(loop + 2, 0, 2 * sizeof(double), h->stream));
    k_loop_start<<<1, 32, 0, h->stream>>>(loop, h->sc + S_FF, h->sc + S_RR, rtol, maxit, hc);
    count_launch();
    return TOPO_OK;
  };
  auto body = [&](cudaGraphConditionalHandle hc) -> int {
    RET(fcg_body<double>(h, h->x, h->r, h->d, h->q, h->rold, L0.U, h->sc, prec, false, -1, loop));
    k_loop_step<<<1, 32, 0, h->stream>>>(loop, h->sc + S_RR, rtol, maxit, hc);
    count_launch();
    return TOPO_OK;
  };
  if (h->iter_capture) {  // inside a captured design iteration: a nested WHILE node
    h->d_inner_body = 0;
    RET(capture_nested_loop(h, setup, body, &h->d_outer_body));
    h->d_outer_body -= h->d_inner_body;
    return TOPO_OK;
  }
  if (!h->sgraph || key != h->skey) {
    if (h->sgraph) { cudaGraphExecDestroy(h->sgraph); h->sgraph = nullptr; }
    auto tail = [&]() -> int { return TOPO_OK; };
    h->sgraph_inner = 0;
    const int rc = capture_loop_graph(h, setup, body, tail, &h->sgraph, &h->sgraph_fixed, &h->sgraph_body);
    if (rc != TOPO_OK) {  // (nested conditional graphs not available, say): the host runs the outer loop from now on
      h->sgraph_ok = false;
      return rc;
    }
    h->sgraph_body -= h->sgraph_inner;  // the inner loop's body is counted per inner iteration
    h->skey = key;
  }
  CK(cudaGraphLaunch(h->sgraph, h->stream));
  count_launch((int)h->sgraph_fixed);
  return TOPO_OK;
}

// V-cycle preconditioner in precision T: z = V(r) with a zero initial guess.
// z must be level-0 U of precision T (the V-cycle works in place there).
template <typename T>
int vcycle_prec(topo_handle* h, const T* r, int pre, int post, int smoother, const ChebParams& cp) {
  DevLevel& L0 = h->lv[0];
  const int64_t n3 = 3 * L0.d.nv;
  if (P<T>::F(L0) != r) CK(cudaMemcpyAsync(P<T>::F(L0), r, sizeof(T) * n3, cudaMemcpyDeviceToDevice, h->stream));
  if (!cheb_zero_start(smoother, pre, cp)) CK(cudaMemsetAsync(P<T>::U(L0), 0, sizeof(T) * n3, h->stream));
  if (sizeof(T) == 4) vcycle32(h, pre, post, smoother, cp, true);
  else vcycle_core<T>(h, pre, post, true, smoother, cp, true);
  return TOPO_OK;
}

int check_ready(topo_handle* h, bool need_ops) {
  if (!h) return TOPO_E_BAD_INPUT;
  if (!h->bc_set) return fail(h, TOPO_E_STATE, "boundary conditions not set (call topo_set_bc)");
  if (need_ops && !h->ops_ready) return fail(h, TOPO_E_STATE, "operators not built (call topo_update_operators)");
  return TOPO_OK;
}

int update_penalised_if_stale(topo_handle* h) {
  if (!h->rhop_stale) return TOPO_OK;
  if (h->ref_fp32)
    launch_penalise_ref32(h->stream, h->lv[0].d.ne, h->lv[0].eactive, h->rho, h->cfg.power_penalty, h->rhop,
                          h->rhop32);
  else
    launch_penalise(h->stream, h->lv[0].d.ne, h->lv[0].eactive, h->rho, h->cfg.power_penalty, h->rhop,
                    h->rhop32);
  count_launch();
  CKL();
  h->rhop_stale = false;
  return TOPO_OK;
}

}  // namespace

// ===========================================================================
// C ABI
// The element constants live in __constant__ memory, one copy per device: live
// handles on a device must share E, nu and h.
namespace {
std::mutex g_mat_mutex;
struct MatReg { int refs = 0; double E = 0, nu = 0, h = 0; };
MatReg g_mat[64];
}  // namespace

static bool material_acquire(const topo_config* c) {
  if (c->device < 0 || c->device >= 64) return false;
  std::lock_guard<std::mutex> lock(g_mat_mutex);
  MatReg& m = g_mat[c->device];
  if (m.refs > 0 && (m.E != c->youngs_modulus || m.nu != c->poisson_ratio || m.h != c->h)) return false;
  m.E = c->youngs_modulus; m.nu = c->poisson_ratio; m.h = c->h;
  ++m.refs;
  return true;
}
static void material_release(int device) {
  if (device < 0 || device >= 64) return;
  std::lock_guard<std::mutex> lock(g_mat_mutex);
  if (g_mat[device].refs > 0) --g_mat[device].refs;
}

// ===========================================================================
extern "C" {

int topo_create(const topo_config* cfg, const uint8_t* eactive, topo_handle** out) {
  if (!cfg || !out) return TOPO_E_BAD_INPUT;
  *out = nullptr;
  if (cfg->nx < 1 || cfg->ny < 1 || cfg->nz < 1 || !(cfg->h > 0) || !(cfg->youngs_modulus > 0) ||
      !(cfg->poisson_ratio > -1.0 && cfg->poisson_ratio < 0.5) || !(cfg->power_penalty >= 1.0) ||
      !(cfg->min_density > 0 && cfg->min_density <= 1.0))
    return TOPO_E_BAD_INPUT;
  if ((int64_t)(cfg->nx + 1) * (cfg->ny + 1) * (cfg->nz + 1) >= ((int64_t)1 << 31))
    return TOPO_E_BAD_INPUT;
  if (!material_acquire(cfg)) return TOPO_E_BAD_INPUT;  // other live handles on the device use other E, nu, h
  struct Release {
    int dev; bool keep = false;
    ~Release() { if (!keep) material_release(dev); }
  } release{cfg->device};
  topo::DeviceScope device_scope(cfg->device);
  auto h = std::make_unique<topo_handle>();
  h->cfg = *cfg;
  if (h->cfg.max_coarse_elements <= 0) h->cfg.max_coarse_elements = 400;
  topo_handle* hp = h.get();
  {
    topo_handle* h = hp;  // for CK
    CK(cudaSetDevice(cfg->device));
    CK(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
  }
  h->H = build_hierarchy(cfg->nx, cfg->ny, cfg->nz, eactive, h->cfg.max_coarse_elements);
  element_template(cfg->youngs_modulus, cfg->poisson_ratio, cfg->h, h->Ke);
  h->lam = cfg->youngs_modulus * cfg->poisson_ratio / ((1 + cfg->poisson_ratio) * (1 - 2 * cfg->poisson_ratio));
  h->mu = cfg->youngs_modulus / (2 * (1 + cfg->poisson_ratio));
  upload_template(h->Ke, h->lam, h->mu, cfg->h);
  const int nl = (int)h->H.dims.size();
  h->lv.resize(nl);
  int rc = TOPO_OK;
  auto A = [&](int r) { if (rc == TOPO_OK) rc = r; };
  for (int l = 0; l < nl; ++l) {
    DevLevel& L = h->lv[l];
    L.d = h->H.dims[l];
    const int64_t nv = L.d.nv, ne = L.d.ne;
    A(dalloc(hp, &L.eactive, ne));
    A(dalloc(hp, &L.vmask, nv));
    A(dalloc(hp, &L.U, 3 * nv)); A(dalloc(hp, &L.F, 3 * nv)); A(dalloc(hp, &L.R, 3 * nv));
    A(dalloc(hp, &L.U32, 3 * nv)); A(dalloc(hp, &L.F32, 3 * nv)); A(dalloc(hp, &L.R32, 3 * nv));
    A(dalloc(hp, &L.dinv, 9 * nv)); A(dalloc(hp, &L.dinv32, 9 * nv));
    A(dalloc(hp, &L.cd, 3 * nv)); A(dalloc(hp, &L.cd32, 3 * nv));
    A(dalloc(hp, &L.U2, 3 * nv)); A(dalloc(hp, &L.U2_32, 3 * nv));
    if (l > 0) {
      A(dalloc(hp, &L.kel, 576 * ne)); A(dalloc(hp, &L.kel32, 576 * ne));
      A(dalloc(hp, &L.stencil, 243 * nv));
      // FP32: room for the tiled layout (243 x 32 values per started group of 32 vertices)
      A(dalloc(hp, &L.stencil32, 243 * ((nv + 31) / 32 * 32)));
    }
    if (rc != TOPO_OK) break;
    std::vector<uint8_t> vm(h->H.vactive[l]);
    for (auto& m : vm) m = (m & 8) ? 0xF : 0;
    cudaMemcpyAsync(L.eactive, h->H.eactive[l].data(), ne, cudaMemcpyHostToDevice, h->stream);
    cudaMemcpyAsync(L.vmask, vm.data(), nv, cudaMemcpyHostToDevice, h->stream);
    std::vector<int2> colz;
    if (l == 0) {  // active z range per fine tile: the fine kernels skip the void
      fine_tile_zrange(L.d, h->H.eactive[0].data(), colz);
      int2* dcz = nullptr;
      A(dalloc(hp, &dcz, (int64_t)colz.size()));
      if (rc != TOPO_OK) break;
      cudaMemcpyAsync(dcz, colz.data(), sizeof(int2) * colz.size(), cudaMemcpyHostToDevice, h->stream);
      L.d.colz = dcz;
      L.d.colz_void = 0;
      for (const int2& r : colz) L.d.colz_void |= (r.x > 0 || r.y < L.d.ez - 1) ? 1 : 0;
    }
    cudaStreamSynchronize(h->stream);
  }
  const LevelDims& d0 = h->lv.empty() ? LevelDims{} : h->lv[0].d;
  if (rc == TOPO_OK) {
    A(dalloc(hp, &h->rho, d0.ne)); A(dalloc(hp, &h->rhop, d0.ne)); A(dalloc(hp, &h->rhop32, d0.ne));
    A(dalloc(hp, &h->sens, d0.ne)); A(dalloc(hp, &h->sens_tmp, d0.ne));
    A(dalloc(hp, &h->work, 3 * d0.nv)); A(dalloc(hp, &h->x, 3 * d0.nv)); A(dalloc(hp, &h->r, 3 * d0.nv));
    A(dalloc(hp, &h->d, 3 * d0.nv)); A(dalloc(hp, &h->q, 3 * d0.nv)); A(dalloc(hp, &h->rold, 3 * d0.nv));
    A(dalloc(hp, &h->f, 3 * d0.nv));
    A(dalloc(hp, &h->x32, 3 * d0.nv)); A(dalloc(hp, &h->r32, 3 * d0.nv)); A(dalloc(hp, &h->d32, 3 * d0.nv));
    A(dalloc(hp, &h->q32, 3 * d0.nv)); A(dalloc(hp, &h->rold32, 3 * d0.nv));
    A(dalloc(hp, &h->dKe, 576));
    A(dalloc(hp, &h->partial, 2048)); A(dalloc(hp, &h->sc, S_COUNT)); A(dalloc(hp, &h->status, 4));
    // partials of the fused fine-operator dot: one per CTA of 32 x 8 element
    // tiles (31 x 7 owned vertices) at z-march depths of 4 and more
    h->fdot_cap = (int)std::min<int64_t>(1 << 24, (int64_t)((d0.vx + 30) / 31) * ((d0.vy + 6) / 7) * ((d0.vz + 3) / 4));
    A(dalloc(hp, &h->fdot, h->fdot_cap));
    A(dalloc(hp, &h->vdot, h->fdot_cap));
    A(dalloc(hp, &h->ctr, 1));
    A(dalloc(hp, &h->chebc, CHEB_TABLE));
  }
  if (rc == TOPO_OK && nl > 1) {
    const LevelDims& dl = h->lv.back().d;
    h->ndense = (int)(3 * dl.nv);
    if (h->ndense > 20000) rc = fail(hp, TOPO_E_BAD_INPUT, "coarsest level too large (%d DOFs)", h->ndense);
    else {
      A(dalloc(hp, &h->A, (int64_t)h->ndense * h->ndense));
      A(dalloc(hp, &h->A32, (int64_t)h->ndense * h->ndense));
      A(dalloc(hp, &h->gjwork, 128 * (int64_t)h->ndense + 32 * 32));  // block, panels in FP64 and split
      A(dalloc(hp, &h->coarse64tmp, 243 * dl.nv));
    }
    std::vector<double> T;
    galerkin_tables(h->Ke, h->lv[1].d.factor, T);
    std::vector<float> T32(T.begin(), T.end());
    A(dalloc(hp, &h->dT64, (int64_t)T.size()));
    A(dalloc(hp, &h->dT32, (int64_t)T.size()));
    if (rc == TOPO_OK) {
      cudaMemcpyAsync(h->dT64, T.data(), sizeof(double) * T.size(), cudaMemcpyHostToDevice, h->stream);
      cudaMemcpyAsync(h->dT32, T32.data(), sizeof(float) * T32.size(), cudaMemcpyHostToDevice, h->stream);
      cudaStreamSynchronize(h->stream);
    }
  }
  if (rc == TOPO_OK) {
    cudaMemcpyAsync(h->dKe, h->Ke, sizeof(double) * 576, cudaMemcpyHostToDevice, h->stream);
    std::vector<double> tab(CHEB_TABLE, 0.0);
    tab[CHEB_TABLE - 1] = 1.0;
    cudaMemcpyAsync(h->chebc, tab.data(), sizeof(double) * CHEB_TABLE, cudaMemcpyHostToDevice, h->stream);
    cudaMemsetAsync(h->sc, 0, sizeof(double) * S_COUNT, h->stream);
    cudaHostAlloc((void**)&h->hsc, sizeof(double) * S_COUNT, cudaHostAllocDefault);
    // density starts at 1 on active elements
    std::vector<double> one(d0.ne);
    for (int64_t e = 0; e < d0.ne; ++e) one[e] = h->H.eactive[0][e] ? 1.0 : 0.0;
    cudaMemcpyAsync(h->rho, one.data(), sizeof(double) * d0.ne, cudaMemcpyHostToDevice, h->stream);
    cudaStreamSynchronize(h->stream);
    h->rhop_stale = true;
    for (auto a : h->H.eactive[0]) h->active_elements += a ? 1 : 0;
    h->gs_padded_elements = gs_padded_count(d0, h->H.eactive[0].data(), false);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) rc = fail(hp, TOPO_E_CUDA, "set-up failed: %s", cudaGetErrorString(e));
  }
  if (rc != TOPO_OK) {
    std::string msg = hp->err;
    topo_destroy(h.release());
    (void)msg;
    return rc;
  }
  h->mat_registered = true;
  release.keep = true;
  *out = h.release();
  return TOPO_OK;
}

void topo_destroy(topo_handle* h) {
  DEVICE_SCOPE(h);
  if (!h) return;
  if (h->stream) cudaStreamSynchronize(h->stream);
  if (h->unet) unet_free(h->unet);
  if (h->side) cudaStreamSynchronize(h->side);
  if (h->mat_registered) material_release(h->cfg.device);
  if (h->side) cudaStreamDestroy(h->side);
  if (h->ev_ops) cudaEventDestroy(h->ev_ops);
  if (h->ev_coarse) cudaEventDestroy(h->ev_coarse);
  if (h->hstat) cudaFreeHost(h->hstat);
  if (h->vgraph) cudaGraphExecDestroy(h->vgraph);
  if (h->igraph) cudaGraphExecDestroy(h->igraph);
  if (h->ograph) cudaGraphExecDestroy(h->ograph);
  if (h->sgraph) cudaGraphExecDestroy(h->sgraph);
  if (h->dgraph) cudaGraphExecDestroy(h->dgraph);
  for (int k = 0; k < TOPO_COND_DEPTH; ++k)
    if (h->cstream[k]) cudaStreamDestroy(h->cstream[k]);
  for (int k = 0; k < 2; ++k) {
    if (h->ev_solve[k]) cudaEventDestroy(h->ev_solve[k]);
    if (h->ev_iter[k]) cudaEventDestroy(h->ev_iter[k]);
  }
  prof_drop_graph_events(h);
  if (h->multi) {
    for (void* p : h->multi->allocs) cudaFree(p);
    delete h->multi;
  }
  if (h->worst) worst_free(h->worst);
  if (h->support) support_free(h->support);
  if (h->rho_init) cudaFree(h->rho_init);
  if (h->vsens) cudaFree(h->vsens);
  for (void* p : h->allocs) cudaFree(p);
  for (int f = 0; f < TOPO_K_COUNT; ++f)
    for (auto& e : h->evs[f]) { cudaEventDestroy(e.a); cudaEventDestroy(e.b); }
  for (auto& e : h->evpool) { cudaEventDestroy(e.a); cudaEventDestroy(e.b); }
  if (h->hsc) cudaFreeHost(h->hsc);
  if (h->gal_fixed) cudaFree(h->gal_fixed);
  if (h->filt_offs) cudaFree(h->filt_offs);
  if (h->timer_ev[0]) { cudaEventDestroy(h->timer_ev[0]); cudaEventDestroy(h->timer_ev[1]); }
  if (h->filt_w) cudaFree(h->filt_w);
  if (h->filt_wdf) cudaFree(h->filt_wdf);
  if (h->stream) cudaStreamDestroy(h->stream);
  delete h;
}

const char* topo_last_error(const topo_handle* h) { return h ? h->err.c_str() : "null handle"; }

int topo_num_levels(const topo_handle* h, int* n) {
  DEVICE_SCOPE(h);
  if (!h || !n) return TOPO_E_BAD_INPUT;
  *n = (int)h->lv.size();
  return TOPO_OK;
}

int topo_level_dims(const topo_handle* h, int level, int* dims3, int* factor) {
  DEVICE_SCOPE(h);
  if (!h || !dims3 || level < 0 || level >= (int)h->lv.size()) return TOPO_E_BAD_INPUT;
  const LevelDims& d = h->lv[level].d;
  dims3[0] = d.ex; dims3[1] = d.ey; dims3[2] = d.ez;
  if (factor) *factor = d.factor;
  return TOPO_OK;
}

int topo_sync(topo_handle* h) {
  DEVICE_SCOPE(h);
  if (!h) return TOPO_E_BAD_INPUT;
  CK(cudaStreamSynchronize(h->stream));
  return TOPO_OK;
}

int topo_set_bc_regions(topo_handle* h, const topo_bc_regions* spec, int* nfixed, int* nloaded) {
  DEVICE_SCOPE(h);
  if (!h || !spec) return TOPO_E_BAD_INPUT;
  if ((spec->nfixed > 0 && !spec->fixed) || (spec->nload > 0 && !spec->load) || (spec->nforce > 0 && !spec->force) ||
      spec->nfixed < 0 || spec->nload < 0 || spec->nforce < 0 || !(spec->spacing > 0))
    return fail(h, TOPO_E_BAD_INPUT, "bad region spec");
  const LevelDims& d = h->lv[0].d;
  std::vector<uint8_t> fixed(d.nv);
  std::vector<double> loads(3 * d.nv);
  bc_from_regions(d.ex, d.ey, d.ez, h->H.eactive[0].data(), spec, fixed.data(), loads.data(), nfixed, nloaded);
  return topo_set_bc(h, fixed.data(), loads.data());
}

int topo_plan_bc_regions(int nx, int ny, int nz, const uint8_t* eactive, const topo_bc_regions* spec,
                         uint8_t* fixed, double* loads, int* nfixed, int* nloaded) {
  if (nx <= 0 || ny <= 0 || nz <= 0 || !spec || !fixed || !loads || !(spec->spacing > 0) ||
      (spec->nfixed > 0 && !spec->fixed) || (spec->nload > 0 && !spec->load) || (spec->nforce > 0 && !spec->force))
    return TOPO_E_BAD_INPUT;
  return bc_from_regions(nx, ny, nz, eactive, spec, fixed, loads, nfixed, nloaded);
}

int topo_set_bc(topo_handle* h, const uint8_t* fixed, const double* loads) {
  DEVICE_SCOPE(h);
  if (!h || !fixed || !loads) return TOPO_E_BAD_INPUT;
  DevLevel& L = h->lv[0];
  const int64_t nv = L.d.nv;
  std::vector<uint8_t> vm(nv);
  std::vector<double> F(3 * nv);
  for (int64_t v = 0; v < nv; ++v) {
    uint8_t m = h->H.vactive[0][v] & 0x8;
    if (m) m |= (uint8_t)(~fixed[v] & 0x7);
    vm[v] = m;
    for (int c = 0; c < 3; ++c) {
      const double ld = loads[c * nv + v];
      if (!std::isfinite(ld)) return fail(h, TOPO_E_BAD_INPUT, "non-finite load at vertex %lld", (long long)v);
      F[c * nv + v] = ((m >> c) & 1) ? ld : 0.0;
    }
  }
  CK(cudaMemcpyAsync(L.vmask, vm.data(), nv, cudaMemcpyHostToDevice, h->stream));
  CK(cudaMemcpyAsync(L.F, F.data(), sizeof(double) * 3 * nv, cudaMemcpyHostToDevice, h->stream));
  ++h->fgen;
  if (h->lv.size() > 1) {
    // coarse elements of level 1 containing a fine element with a fixed DOF
    const LevelDims& c = h->lv[1].d;
    const LevelDims& fd = L.d;
    const int fct = c.factor;
    std::vector<int> list;
    for (int cz = 0; cz < c.ez; ++cz)
      for (int cy = 0; cy < c.ey; ++cy)
        for (int cx = 0; cx < c.ex; ++cx) {
          bool hit = false;
          for (int pz = 0; pz < fct && !hit; ++pz)
            for (int py = 0; py < fct && !hit; ++py)
              for (int px = 0; px < fct && !hit; ++px) {
                const int fx = cx * fct + px, fy = cy * fct + py, fz = cz * fct + pz;
                if (fx >= fd.ex || fy >= fd.ey || fz >= fd.ez) continue;
                if (!h->H.eactive[0][fx + (int64_t)fd.ex * (fy + (int64_t)fd.ey * fz)]) continue;
                for (int a = 0; a < 8 && !hit; ++a) {
                  const int64_t vv = (fx + (a & 1)) + (int64_t)fd.vx * ((fy + ((a >> 1) & 1)) + (int64_t)fd.vy * (fz + (a >> 2)));
                  if ((vm[vv] & 7) != 7) hit = true;
                }
              }
          if (hit) list.push_back((int)(cx + (int64_t)c.ex * (cy + (int64_t)c.ey * cz)));
        }
    if (h->gal_fixed) { cudaFree(h->gal_fixed); h->gal_fixed = nullptr; }
    h->n_gal_fixed = (int)list.size();
    if (!list.empty()) {
      CK(cudaMalloc((void**)&h->gal_fixed, sizeof(int) * list.size()));
      CK(cudaMemcpyAsync(h->gal_fixed, list.data(), sizeof(int) * list.size(), cudaMemcpyHostToDevice, h->stream));
    }
  }
  CK(cudaMemsetAsync(L.U, 0, sizeof(double) * 3 * nv, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  h->bc_set = true;
  h->ops_ready = false;
  h->coarse_valid = false;
  for (auto& l : h->lv) { l.lmax = 0; l.lmax32 = 0; }
  return TOPO_OK;
}

int topo_set_spline(topo_handle* h, int order, const int* partition3, const double* bmin3,
                    const double* bmax3) {
  DEVICE_SCOPE(h);
  if (!h || !partition3 || !bmin3 || !bmax3 || order < 2 || order > 4) return TOPO_E_BAD_INPUT;
  for (int a = 0; a < 3; ++a)
    if (partition3[a] < 0 || !(bmax3[a] > bmin3[a])) return TOPO_E_BAD_INPUT;
  const LevelDims& d0 = h->lv[0].d;
  int nelem[3] = {d0.ex, d0.ey, d0.ez};
  spline_tables(order, partition3, bmin3, bmax3, nelem, h->cfg.h, h->st);
  SplineDev& sd = h->sd;
  sd.order = order;
  for (int a = 0; a < 3; ++a) {
    sd.nb[a] = h->st.nb[a];
    int *i0 = nullptr, *lo = nullptr, *hi = nullptr;
    double* N = nullptr;
    RET(dalloc(h, &i0, nelem[a]));
    RET(dalloc(h, &N, (int64_t)nelem[a] * order));
    RET(dalloc(h, &lo, sd.nb[a]));
    RET(dalloc(h, &hi, sd.nb[a]));
    CK(cudaMemcpyAsync(i0, h->st.i0[a].data(), sizeof(int) * nelem[a], cudaMemcpyHostToDevice, h->stream));
    CK(cudaMemcpyAsync(N, h->st.N[a].data(), sizeof(double) * nelem[a] * order, cudaMemcpyHostToDevice, h->stream));
    CK(cudaMemcpyAsync(lo, h->st.lo[a].data(), sizeof(int) * sd.nb[a], cudaMemcpyHostToDevice, h->stream));
    CK(cudaMemcpyAsync(hi, h->st.hi[a].data(), sizeof(int) * sd.nb[a], cudaMemcpyHostToDevice, h->stream));
    sd.i0[a] = i0; sd.N[a] = N; sd.lo[a] = lo; sd.hi[a] = hi;
  }
  for (int a = 0; a < 3; ++a) {  // basis values split for the double-float spline passes
    std::vector<float2> ndf(h->st.N[a].size());
    for (size_t k = 0; k < ndf.size(); ++k) {
      const double v = h->st.N[a][k];
      const float hi = (float)v;
      ndf[k] = make_float2(hi, (float)(v - (double)hi));
    }
    float2* Nd = nullptr;
    RET(dalloc(h, &Nd, (int64_t)ndf.size()));
    CK(cudaMemcpyAsync(Nd, ndf.data(), sizeof(float2) * ndf.size(), cudaMemcpyHostToDevice, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    sd.Ndf[a] = Nd;
  }
  const int64_t nc = (int64_t)sd.nb[0] * sd.nb[1] * sd.nb[2];
  RET(dalloc(h, &h->coeff, nc));
  RET(dalloc(h, &h->csens, nc));
  RET(dalloc(h, &h->volcsens, nc));
  RET(dalloc(h, &h->coeff_old, nc));
  RET(dalloc(h, &h->coeff_tmp, nc));
  RET(dalloc(h, &h->coeff_df, nc));
  RET(dalloc(h, &h->adj1, (int64_t)sd.nb[0] * d0.ey * d0.ez));
  RET(dalloc(h, &h->adj2, (int64_t)sd.nb[0] * sd.nb[1] * d0.ez));
  CK(cudaStreamSynchronize(h->stream));
  h->spline_set = true;
  return TOPO_OK;
}

int topo_num_coeffs(const topo_handle* h, int* n) {
  DEVICE_SCOPE(h);
  if (!h || !n) return TOPO_E_BAD_INPUT;
  if (!h->spline_set) return TOPO_E_STATE;
  *n = h->sd.nb[0] * h->sd.nb[1] * h->sd.nb[2];
  return TOPO_OK;
}

int topo_get_knots(const topo_handle* h, int axis, double* out, size_t count) {
  DEVICE_SCOPE(h);
  if (!h || !out || axis < 0 || axis > 2) return TOPO_E_BAD_INPUT;
  if (!h->spline_set) return TOPO_E_STATE;
  if (count != h->st.knots[axis].size()) return TOPO_E_BAD_INPUT;
  std::copy(h->st.knots[axis].begin(), h->st.knots[axis].end(), out);
  return TOPO_OK;
}

static int array_info(topo_handle* h, int which, int level, void** dptr, size_t* count, size_t* esize) {
  if (level < 0 || level >= (int)h->lv.size()) return TOPO_E_BAD_INPUT;
  DevLevel& L = h->lv[level];
  const LevelDims& d0 = h->lv[0].d;
  const int64_t nc = h->spline_set ? (int64_t)h->sd.nb[0] * h->sd.nb[1] * h->sd.nb[2] : 0;
  *esize = sizeof(double);
  switch (which) {
    case TOPO_RHO: *dptr = h->rho; *count = d0.ne; break;
    case TOPO_RHOP: *dptr = h->rhop; *count = d0.ne; break;
    case TOPO_SENS: *dptr = h->sens; *count = d0.ne; break;
    case TOPO_COEFF: if (!h->spline_set) return TOPO_E_STATE; *dptr = h->coeff; *count = nc; break;
    case TOPO_CSENS: if (!h->spline_set) return TOPO_E_STATE; *dptr = h->csens; *count = nc; break;
    case TOPO_VOLCSENS: if (!h->spline_set) return TOPO_E_STATE; *dptr = h->volcsens; *count = nc; break;
    case TOPO_MULTI_F: if (!h->multi || level != 0) return TOPO_E_STATE; *dptr = h->multi->f; *count = (size_t)h->multi->cap * 3 * d0.nv; break;
    case TOPO_MULTI_U: if (!h->multi || level != 0) return TOPO_E_STATE; *dptr = h->multi->x; *count = (size_t)h->multi->cap * 3 * d0.nv; break;
    case TOPO_U: *dptr = L.U; *count = 3 * L.d.nv; break;
    case TOPO_F: *dptr = L.F; *count = 3 * L.d.nv; break;
    case TOPO_R: *dptr = L.R; *count = 3 * L.d.nv; break;
    case TOPO_STENCIL: if (level == 0) return TOPO_E_BAD_INPUT; *dptr = L.stencil; *count = 243 * L.d.nv; break;
    case TOPO_KELEM: if (level == 0) return TOPO_E_BAD_INPUT; *dptr = L.kel; *count = 576 * L.d.ne; break;
    case TOPO_VMASK: *dptr = L.vmask; *count = L.d.nv; *esize = 1; break;
    case TOPO_EACTIVE: *dptr = L.eactive; *count = L.d.ne; *esize = 1; break;
    case TOPO_KE: *dptr = h->dKe; *count = 576; break;
    case TOPO_WORK: if (level != 0) return TOPO_E_BAD_INPUT; *dptr = h->work; *count = 3 * d0.nv; break;
    case TOPO_RHO_INIT: if (!h->rho_init || level != 0) return TOPO_E_STATE; *dptr = h->rho_init; *count = d0.ne; break;
    case TOPO_SSCSENS: case TOPO_DRIPCSENS: case TOPO_SURF_POINTS: case TOPO_SURF_NORMALS:
      if (level != 0) return TOPO_E_BAD_INPUT;
      return support_array(h->support, which, dptr, count);
    default: return TOPO_E_BAD_INPUT;
  }
  return TOPO_OK;
}

int topo_array_size(const topo_handle* h, int which, int level, size_t* count) {
  DEVICE_SCOPE(h);
  if (!h || !count) return TOPO_E_BAD_INPUT;
  void* p; size_t es;
  return array_info(const_cast<topo_handle*>(h), which, level, &p, count, &es);
}

int topo_put_array(topo_handle* h, int which, int level, const void* src, size_t count) {
  DEVICE_SCOPE(h);
  if (!h || !src) return TOPO_E_BAD_INPUT;
  void* p; size_t n, es;
  int rc = array_info(h, which, level, &p, &n, &es);
  if (rc != TOPO_OK) return fail(h, rc, "bad array id/level %d/%d", which, level);
  if (count != n) return fail(h, TOPO_E_BAD_INPUT, "array %d expects %zu elements, got %zu", which, n, count);
  if (which == TOPO_VMASK || which == TOPO_EACTIVE || which == TOPO_KE || which == TOPO_STENCIL ||
      which == TOPO_KELEM || which == TOPO_RHOP)
    return fail(h, TOPO_E_BAD_INPUT, "array %d is read-only", which);
  CK(cudaMemcpyAsync(p, src, n * es, cudaMemcpyHostToDevice, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  if (which == TOPO_RHO) { h->rhop_stale = true; h->ops_ready = false; }
  if (which == TOPO_F && level == 0) ++h->fgen;
  return TOPO_OK;
}

int topo_get_array(topo_handle* h, int which, int level, void* dst, size_t count) {
  DEVICE_SCOPE(h);
  if (!h || !dst) return TOPO_E_BAD_INPUT;
  void* p; size_t n, es;
  int rc = array_info(h, which, level, &p, &n, &es);
  if (rc != TOPO_OK) return fail(h, rc, "bad array id/level %d/%d", which, level);
  if (count != n) return fail(h, TOPO_E_BAD_INPUT, "array %d has %zu elements, asked %zu", which, n, count);
  if (which == TOPO_RHOP) RET(update_penalised_if_stale(h));
  CK(cudaMemcpyAsync(dst, p, n * es, cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  return TOPO_OK;
}

int topo_device_ptr(topo_handle* h, int which, int level, void** dptr) {
  DEVICE_SCOPE(h);
  if (!h || !dptr) return TOPO_E_BAD_INPUT;
  size_t n, es;
  return array_info(h, which, level, dptr, &n, &es);
}

int topo_coeff_to_density(topo_handle* h) {
  DEVICE_SCOPE(h);
  if (!h) return TOPO_E_BAD_INPUT;
  if (!h->spline_set) return fail(h, TOPO_E_STATE, "spline not set (call topo_set_spline)");
  const DevLevel& L = h->lv[0];
  if (h->ref_fp32) launch_round_f32(h->stream, (int64_t)h->sd.nb[0] * h->sd.nb[1] * h->sd.nb[2], h->coeff);
  launch_coeff_to_density(h->stream, L.d, L.eactive, h->sd, h->coeff, h->cfg.min_density,
                          h->cfg.power_penalty, h->rho, h->rhop, h->rhop32, h->adj1, h->coeff_df);
  count_launch(3);
  if (h->ref_fp32) {  // rho stored in FP32, rho^p by powf
    launch_penalise_ref32(h->stream, L.d.ne, L.eactive, h->rho, h->cfg.power_penalty, h->rhop, h->rhop32);
    count_launch(2);
  }
  CKL();
  h->rhop_stale = false;
  h->ops_ready = false;
  return TOPO_OK;
}

int topo_set_reference_precision(topo_handle* h, int enable) {
  DEVICE_SCOPE(h);
  if (!h) return TOPO_E_BAD_INPUT;
  h->ref_fp32 = enable != 0;
  h->rhop_stale = true;
  h->ops_ready = false;
  h->coarse_valid = false;
  return TOPO_OK;
}

int topo_set_operator_precision(topo_handle* h, int mask) {
  DEVICE_SCOPE(h);
  if (!h || mask < 1 || mask > 3) return TOPO_E_BAD_INPUT;
  h->op_precision = mask;
  h->ops_ready = false;
  h->coarse_valid = false;
  return TOPO_OK;
}

int topo_update_operators(topo_handle* h) {
  DEVICE_SCOPE(h);
  RET(check_ready(h, false));
  RET(update_penalised_if_stale(h));
  const int nl = (int)h->lv.size();
  const bool b64 = (h->op_precision & 1) != 0, b32 = (h->op_precision & 2) != 0;
  for (int l = 1; l < nl; ++l) {
    DevLevel& C = h->lv[l];
    DevLevel& Fl = h->lv[l - 1];
    if (l == 1) {
      launch_galerkin_first_impl(h->stream, Fl.d, C.d, h->rhop, Fl.eactive, Fl.vmask, h->dT64, h->dT32,
                                 h->dKe, h->gal_fixed, h->n_gal_fixed, b64 ? C.kel : nullptr,
                                 b32 ? C.kel32 : nullptr);
      count_launch((b64 ? 2 : 0) + (b32 ? 2 : 0));
    } else {
      if (b64) launch_galerkin_dyadic_t<double>(h->stream, Fl.d, C.d, Fl.eactive, Fl.kel, C.kel);
      if (b32) launch_galerkin_dyadic_t<float>(h->stream, Fl.d, C.d, Fl.eactive, Fl.kel32, C.kel32);
      count_launch((b64 ? 1 : 0) + (b32 ? 1 : 0));
    }
    if (b64) launch_assemble_stencil_t<double>(h->stream, C.d, C.eactive, C.vmask, C.kel, C.stencil);
    if (b32) launch_assemble_stencil_t<float>(h->stream, C.d, C.eactive, C.vmask, C.kel32, C.stencil32);
    count_launch((b64 ? 1 : 0) + (b32 ? 1 : 0));
    CKL();
  }
  // a lagged coarsest inverse (topo_set_coarse_refresh): the coarse levels
  // are current, the coarsest solve keeps the inverse of an earlier update
  const bool keep_inverse = nl > 1 && h->coarse_valid && h->coarse_every > 1 && ++h->coarse_age < h->coarse_every;
  if (nl > 1 && !keep_inverse) {
    h->coarse_age = 0;
    h->coarse_valid = true;
    DevLevel& Lc = h->lv.back();
    const double* st = Lc.stencil;
    if (!b64) {  // FP64 copy of the FP32 coarsest stencil
      CK(cudaMemsetAsync(h->coarse64tmp, 0, sizeof(double) * 243 * Lc.d.nv, h->stream));
      launch_f2d_add(h->stream, Lc.stencil32, h->coarse64tmp, 243 * Lc.d.nv);
      count_launch();
      st = h->coarse64tmp;
    }
    launch_dense_from_stencil(h->stream, Lc.d, st, h->A);
    count_launch(2);
    CKL();
    // FP32-only operators: the matrix comes from FP32 stencils; the updates
    // in double-float keep twice their precision on the FP32 pipe
    if (h->defer_coarse) {  // on the side stream, one CTA per SM, joined later
      if (!h->side) {
        CK(cudaStreamCreateWithFlags(&h->side, cudaStreamNonBlocking));
        CK(cudaEventCreateWithFlags(&h->ev_ops, cudaEventDisableTiming));
        CK(cudaEventCreateWithFlags(&h->ev_coarse, cudaEventDisableTiming));
        CK(cudaHostAlloc((void**)&h->hstat, 2 * sizeof(int), cudaHostAllocDefault));
      }
      CK(cudaEventRecord(h->ev_ops, h->stream));
      CK(cudaStreamWaitEvent(h->side, h->ev_ops, 0));
      const int e = coarsest_invert(h->side, h->ndense, h->A, h->gjwork, h->status, !b64,
                                    h->ndense > TOPO_GJ_SIDE_LARGE_N ? 2 : TOPO_GJ_SIDE_PER_SM);
      count_launch();
      if (e != (int)cudaSuccess)
        return fail(h, TOPO_E_CUDA, "coarsest inversion launch failed: %s", cudaGetErrorString((cudaError_t)e));
      CK(cudaMemcpyAsync(h->hstat, h->status, 2 * sizeof(int), cudaMemcpyDeviceToHost, h->side));
      launch_to_float(h->side, h->A, h->A32, (int64_t)h->ndense * h->ndense);
      count_launch();
      CK(cudaEventRecord(h->ev_coarse, h->side));
      h->coarse_pending = h->coarse_unchecked = true;
      for (auto& l : h->lv) { l.lmax = 0; l.lmax32 = 0; }
      h->ops64 = b64;
      h->ops32 = b32;
      h->ops_ready = true;
      return TOPO_OK;
    }
    int e = coarsest_invert(h->stream, h->ndense, h->A, h->gjwork, h->status, !b64);
    count_launch();
    if (e != (int)cudaSuccess)
      return fail(h, TOPO_E_CUDA, "coarsest inversion launch failed: %s", cudaGetErrorString((cudaError_t)e));
    int hstat[2] = {0, 0};
    CK(cudaMemcpyAsync(hstat, h->status, 2 * sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    if (hstat[1] != 0) {
      h->coarse_valid = false;
      return fail(h, TOPO_E_SINGULAR, "coarsest matrix indefinite at pivot %d", hstat[1] - 1);
    }
    h->coarse_dropped = hstat[0];
    launch_to_float(h->stream, h->A, h->A32, (int64_t)h->ndense * h->ndense);
    count_launch();
    CKL();
  }
  for (auto& l : h->lv) { l.lmax = 0; l.lmax32 = 0; }
  h->ops64 = b64;
  h->ops32 = b32;
  h->ops_ready = true;
  return TOPO_OK;
}

int topo_apply_fine(topo_handle* h, int precision) {
  DEVICE_SCOPE(h);
  RET(check_ready(h, false));
  RET(update_penalised_if_stale(h));
  DevLevel& L = h->lv[0];
  const int64_t n3 = 3 * L.d.nv;
  if (precision == 0) {  // FP64 modal kernel in native FP64
    launch_fine_apply<double>(h->stream, L.d, h->rhop, L.vmask, h->work, nullptr, L.R, false);
    count_launch();
  } else if (precision == 3) {  // FP64 vectors, double-float modal kernel
    launch_fine_apply_df(h->stream, L.d, h->rhop, L.vmask, h->work, nullptr, L.R, false);
    count_launch();
  } else if (precision == 2) {  // dense-row FP64 kernel (cross-check of the modal kernel)
    launch_fine_apply_dense<double>(h->stream, L.d, h->rhop, L.vmask, h->work, nullptr, L.R, false);
    count_launch();
  } else {
    launch_d2f(h->stream, h->work, h->x32, n3);
    level_apply<float>(h, 0, h->x32, nullptr, h->r32, false);
    CK(cudaMemsetAsync(L.R, 0, sizeof(double) * n3, h->stream));
    launch_f2d_add(h->stream, h->r32, L.R, n3);
    count_launch(2);
  }
  CKL();
  return TOPO_OK;
}

int topo_residual(topo_handle* h, int level) {
  DEVICE_SCOPE(h);
  RET(check_ready(h, level > 0));
  if (level < 0 || level >= (int)h->lv.size()) return TOPO_E_BAD_INPUT;
  RET(update_penalised_if_stale(h));
  level_residual<double>(h, level);
  CKL();
  return TOPO_OK;
}

int topo_apply_level(topo_handle* h, int level, int precision) {
  DEVICE_SCOPE(h);
  RET(check_ready(h, true));
  if (level < 1 || level >= (int)h->lv.size() || precision < 0 || precision > 1)
    return fail(h, TOPO_E_BAD_INPUT, "topo_apply_level: level %d (1..%d), precision %d (0 or 1)", level,
                (int)h->lv.size() - 1, precision);
  DevLevel& L = h->lv[level];
  const int64_t n3 = 3 * L.d.nv;
  if (precision == 0) {
    if (!h->ops64) return fail(h, TOPO_E_STATE, "FP64 operators not built (topo_set_operator_precision)");
    launch_stencil_apply<double>(h->stream, L.d, L.stencil, L.U, nullptr, L.R, false, 1);
    count_launch();
  } else {
    if (!h->ops32) return fail(h, TOPO_E_STATE, "FP32 operators not built (topo_set_operator_precision)");
    launch_d2f(h->stream, L.U, L.U32, n3);
    launch_stencil_apply<float>(h->stream, L.d, L.stencil32, L.U32, nullptr, L.R32, false, 1);
    CK(cudaMemsetAsync(L.R, 0, sizeof(double) * n3, h->stream));
    launch_f2d_add(h->stream, L.R32, L.R, n3);
    count_launch(3);
  }
  CKL();
  return TOPO_OK;
}

int topo_smooth(topo_handle* h, int level, int sweeps, int reverse) {
  DEVICE_SCOPE(h);
  RET(check_ready(h, level > 0));
  if (level < 0 || level >= (int)h->lv.size() || sweeps < 0) return TOPO_E_BAD_INPUT;
  RET(update_penalised_if_stale(h));
  gs_level<double>(h, level, sweeps, reverse != 0);
  CKL();
  return TOPO_OK;
}

int topo_restrict(topo_handle* h, int coarse_level) {
  DEVICE_SCOPE(h);
  if (!h || coarse_level < 1 || coarse_level >= (int)h->lv.size()) return TOPO_E_BAD_INPUT;
  restrict_T<double>(h, coarse_level);
  CKL();
  return TOPO_OK;
}

int topo_prolong(topo_handle* h, int fine_level) {
  DEVICE_SCOPE(h);
  if (!h || fine_level < 0 || fine_level >= (int)h->lv.size() - 1) return TOPO_E_BAD_INPUT;
  prolong_T<double>(h, fine_level);
  CKL();
  return TOPO_OK;
}

int topo_coarsest_solve(topo_handle* h) {
  DEVICE_SCOPE(h);
  RET(check_ready(h, true));
  if (h->lv.size() < 2) return TOPO_E_STATE;
  coarsest_solve_T<double>(h);
  CKL();
  return TOPO_OK;
}

int topo_vcycle(topo_handle* h, int pre, int post, double* relres) {
  DEVICE_SCOPE(h);
  RET(check_ready(h, true));
  if (!h->ops64) return fail(h, TOPO_E_STATE, "FP64 operators not built");
  ChebParams cp;
  vcycle_core<double>(h, pre, post, false, TOPO_SMOOTH_GS, cp);
  level_residual<double>(h, 0);
  DevLevel& L = h->lv[0];
  const int64_t n3 = 3 * L.d.nv;
  launch_dot<double>(h->stream, L.R, L.R, n3, h->partial, h->sc + S_RR);
  launch_dot<double>(h->stream, L.F, L.F, n3, h->partial, h->sc + S_FF);
  count_launch(4);
  CKL();
  RET(read_scalars(h, S_RR, 2));
  if (relres) *relres = std::sqrt(h->hsc[S_RR]) / std::sqrt(h->hsc[S_FF]);
  return TOPO_OK;
}

// The main stream waits for a coarsest inversion running on the side stream.
static int coarse_join(topo_handle* h) {
  // (in a captured design iteration the inversion is launched before the
  // graph, so the graph holds one wait on the event's record at launch time,
  // also when the capture's own update kept a lagged inverse: replays may
  // refresh it)
  if (h->iter_capture) {
    if (h->iter_waited) return TOPO_OK;
    h->iter_waited = true;
    h->coarse_pending = false;
    CK(cudaStreamWaitEvent(h->stream, h->ev_coarse, cudaEventWaitExternal));
    return TOPO_OK;
  }
  if (!h->coarse_pending) return TOPO_OK;
  CK(cudaStreamWaitEvent(h->stream, h->ev_coarse, 0));
  h->coarse_pending = false;
  return TOPO_OK;
}

// Joins the side stream's inversion and reads its status.
static int coarse_finish(topo_handle* h) {
  RET(coarse_join(h));
  if (!h->coarse_unchecked || h->iter_capture) return TOPO_OK;  // (a captured iteration reads it afterwards)
  CK(cudaEventSynchronize(h->ev_coarse));
  h->coarse_unchecked = false;
  if (h->hstat[1] != 0) {
    h->coarse_valid = false;
    return fail(h, TOPO_E_SINGULAR, "coarsest matrix indefinite at pivot %d", h->hstat[1] - 1);
  }
  h->coarse_dropped = h->hstat[0];
  return TOPO_OK;
}

static int solve_impl(topo_handle* h, const topo_solve_opts* o, topo_solve_stats* stats);

int topo_solve(topo_handle* h, const topo_solve_opts* o, topo_solve_stats* stats) {
  DEVICE_SCOPE(h);
  const int rc = solve_impl(h, o, stats);
  if (h) RET(coarse_finish(h));
  return rc;
}

// After a synchronisation: whether a bounded wait of a tcgen05 kernel this
// handle may have run gave up (the kernel then skipped its work).
static int tc_wait_status(topo_handle* h) {
  int f = 0, g = 0;
  if (h->fine_tc) CK(fine_tc_error(&f));
  if (h->unet && unet_conv_kernel(h->unet) == 1) CK(conv_tc_error(&g));
  if (f || g) return fail(h, TOPO_E_TIMEOUT, "a tensor-core kernel's bounded wait gave up (flags %d, %d)", f, g);
  return TOPO_OK;
}

static int solve_impl(topo_handle* h, const topo_solve_opts* o, topo_solve_stats* stats) {
  RET(check_ready(h, true));
  h->energy_ready = false;
  if (!o || o->rtol <= 0 || o->max_iter < 0 || o->pre < 0 || o->post < 0) return TOPO_E_BAD_INPUT;
  DevLevel& L0 = h->lv[0];
  const int64_t n3 = 3 * L0.d.nv;
  ChebParams cp;
  if (o->cheb_degree > 0) cp.degree = o->cheb_degree;
  if (o->cheb_lo > 0) cp.lo = o->cheb_lo;
  if (o->cheb_hi > 0) cp.hi = o->cheb_hi;
  ScopedEvent e0, e1;
  topo_solve_stats st{};
  // (inside a captured design iteration the solve is timed by external
  // event-record nodes, ||F|| is the one read when it was captured, and the
  // results are read after the graph ran)
  const bool cap = h->iter_capture;
  if (cap) {
    CK(cudaEventRecordWithFlags(h->ev_solve[0], h->stream, cudaEventRecordExternal));
  } else {
    CK(e0.create());
    CK(e1.create());
    CK(cudaEventRecord(e0, h->stream));
  }
  // ||F||
  launch_dot<double>(h->stream, L0.F, L0.F, n3, h->partial, h->sc + S_FF);
  count_launch(2);
  if (!cap) RET(read_scalars(h, S_FF, 1));
  const double fn = cap ? h->iter_fn : std::sqrt(h->hsc[S_FF]);
  int rc = TOPO_OK;
  if (o->mode != TOPO_SOLVE_MIXED) RET(coarse_join(h));
  if (fn == 0.0) {
    CK(cudaMemsetAsync(L0.U, 0, sizeof(double) * n3, h->stream));
    st.relres = 0.0;
  } else if (o->mode == TOPO_SOLVE_VCYCLE) {
    if (!h->ops64) return fail(h, TOPO_E_STATE, "FP64 operators not built");
    RET(prepare_smoother<double>(h, o->smoother, cp));
    double rr = 1.0;
    int it = 0;
    while (rr > o->rtol && it < o->max_iter) {
      vcycle_core<double>(h, o->pre, o->post, false, o->smoother, cp);
      level_residual<double>(h, 0);
      launch_dot<double>(h->stream, L0.R, L0.R, n3, h->partial, h->sc + S_RR);
      count_launch(2);
      CKL();
      RET(read_scalars(h, S_RR, 1));
      rr = std::sqrt(h->hsc[S_RR]) / fn;
      if (!std::isfinite(rr)) return fail(h, TOPO_E_NONFINITE, "V-cycle residual non-finite");
      ++it;
    }
    st.iterations = it;
    st.vcycles = it;
    st.relres = rr;
  } else if (o->mode == TOPO_SOLVE_PCG64) {
    if (!h->ops64) return fail(h, TOPO_E_STATE, "FP64 operators not built");
    RET(prepare_smoother<double>(h, o->smoother, cp));
    CK(cudaMemcpyAsync(h->x, L0.U, sizeof(double) * n3, cudaMemcpyDeviceToDevice, h->stream));
    CK(cudaMemcpyAsync(h->f, L0.F, sizeof(double) * n3, cudaMemcpyDeviceToDevice, h->stream));
    int it = 0;
    double rel = 0;
    int nvc = 0;
    auto prec = [&](const double* r, double* z) -> int {
      (void)z;  // z is level-0 U, where the V-cycle works
      ++nvc;
      return vcycle_prec<double>(h, r, o->pre, o->post, o->smoother, cp);
    };
    rc = fcg_T<double>(h, h->x, h->f, h->r, h->d, h->q, h->rold, L0.U, o->rtol, o->max_iter, 0, prec,
                       &it, &rel, fn);
    // restore level-0 state: F = f, U = x
    CK(cudaMemcpyAsync(L0.F, h->f, sizeof(double) * n3, cudaMemcpyDeviceToDevice, h->stream));
    CK(cudaMemcpyAsync(L0.U, h->x, sizeof(double) * n3, cudaMemcpyDeviceToDevice, h->stream));
    if (rc != TOPO_OK) return rc;
    st.iterations = it;
    st.vcycles = nvc;
  } else if (o->mode == TOPO_SOLVE_MIXED) {
    // FP64 flexible CG (FP64 fine matvec, dot products and step lengths) whose
    // preconditioner is an FP32 multigrid solve: one FP32 V-cycle, or up to
    // inner_max FP32 FCG iterations to a relative reduction of inner_rtol.
    if (!h->ops32) return fail(h, TOPO_E_STATE, "FP32 operators not built");
    RET(prepare_smoother<float>(h, o->smoother, cp));
    CK(cudaMemcpyAsync(h->x, L0.U, sizeof(double) * n3, cudaMemcpyDeviceToDevice, h->stream));
    CK(cudaMemcpyAsync(h->f, L0.F, sizeof(double) * n3, cudaMemcpyDeviceToDevice, h->stream));
    const double inner_rtol = o->inner_rtol > 0 ? o->inner_rtol : 1e-1;
    const int inner_max = o->inner_max > 0 ? o->inner_max : 1;
    int it = 0, nvc = 0;
    double rel = 0;
    // learned correction (1) or harvesting (2)
    if (o->learned < 0 || o->learned > 2) return fail(h, TOPO_E_BAD_INPUT, "learned must be 0, 1 or 2");
    if (o->learned && !h->unet) return fail(h, TOPO_E_STATE, "learned preconditioner not enabled (topo_unet_enable)");
    if (o->learned == 2 && inner_max > 1) return fail(h, TOPO_E_BAD_INPUT, "harvesting needs inner_max <= 1");
    bool net_on = o->learned == 1;
    const bool harvest = o->learned == 2;
    const double stall = o->learned_stall > 0 ? o->learned_stall : 0.99;
    double rbest = -1;  // best outer residual norm so far
    int since_best = 0;  // outer steps without progress on rbest
    if (o->learned) {
      const cudaError_t e = unet_prepare(h->unet, h->stream, L0.d, L0.eactive, h->rho, h->cfg.min_density);
      if (e != cudaSuccess) return fail(h, TOPO_E_CUDA, "U-Net set-up: %s", cudaGetErrorString(e));
    }
    auto net = [&](const float* r32, float* z32) -> int {
      if (!net_on) return TOPO_OK;
      const cudaError_t e = unet_apply(h->unet, h->stream, L0.d, L0.vmask, h->rhop32, tz32_arg(h), r32, z32, h->partial);
      if (e != cudaSuccess) return fail(h, TOPO_E_CUDA, "U-Net apply: %s", cudaGetErrorString(e));
      ++st.learned_applied;
      return TOPO_OK;
    };
    // The inner CG's r.z: from the V-cycle's last Chebyshev step when it is a
    // fine FP32 Chebyshev step and no network correction follows.  The cycle
    // is then a fixed symmetric linear operator, and the inner CG takes the
    // plain Fletcher-Reeves form (z.rold = 0, rold not kept).  With the
    // network (a varying preconditioner) it stays flexible, with separate
    // r.z and z.rold after the cycle.
    const bool vdots = o->smoother == TOPO_SMOOTH_CHEBYSHEV && o->post >= 1 && cp.degree >= 1 && h->nb == 1;
    // the inner CG on the device (one graph per inner solve) where its
    // iteration is a fixed kernel sequence: fused r.z, no network, no profiler
    bool igraph = h->graphs && h->igraph_ok && !h->prof && vdots && !o->learned && inner_max > 1;
    bool igraph_used = false;
    if (igraph) CK(cudaMemsetAsync(h->sc + S_LOOP + 2, 0, 2 * sizeof(double), h->stream));
    auto prec32 = [&](const float* r, float* z) -> int {
      (void)z;
      ++nvc;
      double* s_rz = h->sc + 8 + S_RZ;
      double* s_zr = h->sc + 8 + S_ZROLD;
      h->vdot_on = vdots && !net_on;
      h->inner_fr = h->vdot_on;
      h->vdot_out = s_rz;
      if (h->inner_fr) CK(cudaMemsetAsync(s_zr, 0, sizeof(double), h->stream));
      const int rc = vcycle_prec<float>(h, r, o->pre, o->post, o->smoother, cp);
      const bool fused = h->vdot_on;
      h->vdot_on = false;
      RET(rc);
      RET(net(r, L0.U32));
      if (!fused) {
        launch_dot<float>(h->stream, r, L0.U32, n3, h->partial, s_rz, h->ctr);
        launch_dot<float>(h->stream, L0.U32, h->rold32, n3, h->partial, s_zr, h->ctr);
        count_launch(2);
      }
      return TOPO_OK;
    };
    auto prec = [&](const double* r, double* z) -> int {
      RET(coarse_join(h));  // the first V-cycle needs the coarsest inverse
      const double rn = std::sqrt(h->hsc[S_RR]);
      // Fall back to the plain V-cycle for the rest of the solve when the
      // positivity guard fired (r.z <= 0 with the correction), or after 10
      // outer steps in a row that do not bring the best residual down by the
      // factor `stall` (CG residual norms are not monotone).
      if (rbest < 0 || rn < stall * rbest) {
        rbest = rbest < 0 ? rn : std::min(rbest, rn);
        since_best = 0;
      } else {
        ++since_best;
      }
      if (net_on) {
        int rej = 0;
        if (st.learned_applied > 0) {
          const cudaError_t e = unet_rejected(h->unet, h->stream, &rej);
          if (e != cudaSuccess) return fail(h, TOPO_E_CUDA, "U-Net guard: %s", cudaGetErrorString(e));
        }
        if (rej || since_best >= 10) {
          net_on = false;
          st.learned_fallback = 1;
        }
      }
      if (inner_max <= 1) {
        launch_d2f(h->stream, r, L0.F32, n3);
        if (!cheb_zero_start(o->smoother, o->pre, cp)) CK(cudaMemsetAsync(L0.U32, 0, sizeof(float) * n3, h->stream));
        ++nvc;
        vcycle32(h, o->pre, o->post, o->smoother, cp, true);
        RET(net(L0.F32, L0.U32));
        if (harvest && rn > 1e-4 * fn) {
          const cudaError_t e = unet_harvest_record(h->unet, h->stream, n3, r, L0.U32, h->x, 8);
          if (e != cudaSuccess) return fail(h, TOPO_E_CUDA, "harvest: %s", cudaGetErrorString(e));
        }
        k_to_double<float><<<nb256(n3), 256, 0, h->stream>>>(n3, L0.U32, z);
        count_launch(2);
        return TOPO_OK;
      }
      if (igraph) {  // the whole inner solve as one graph launch, no host wait
        const int nvc0 = nvc;  // (a capture runs prec32 once on the host)
        h->vdot_on = true;
        h->vdot_out = h->sc + 8 + S_RZ;
        const int grc = inner_cg_graphed(h, r, z, inner_rtol, inner_max, prec32,
                                         vcycle_key(h, o->pre, o->post, o->smoother, cp, true));
        h->vdot_on = false;
        nvc = nvc0;
        if (grc == TOPO_OK) {
          igraph_used = true;
          return TOPO_OK;
        }
        if (h->igraph_ok || h->in_capture) return grc;
        igraph = false;  // capture failed: the host loop from here on
      }
      launch_d2f(h->stream, r, L0.F32, n3);
      CK(cudaMemsetAsync(h->x32, 0, sizeof(float) * n3, h->stream));
      count_launch();
      int iit = 0;
      double irel = 0;
      // relative to ||r||, the FP64 norm of the outer residual, which the
      // outer CG has just read into the host slots
      const double rnorm = std::sqrt(h->hsc[S_RR]);
      // the inner residual lives in level-0 F32, the V-cycle's right-hand side,
      // so the preconditioner needs no copy; x32 = 0 gives r = b without a matvec
      RET(fcg_T<float>(h, h->x32, L0.F32, L0.F32, h->d32, h->q32, h->rold32, L0.U32, inner_rtol, inner_max,
                       8, prec32, &iit, &irel, rnorm > 0 ? rnorm : 1.0, true, true));
      k_to_double<float><<<nb256(n3), 256, 0, h->stream>>>(n3, h->x32, z);
      count_launch();
      return TOPO_OK;
    };
    // the whole outer CG on the device (one graph launch per solve) where its
    // preconditioner is one V-cycle or the graphed inner CG
    const bool sgraph = h->graphs && h->sgraph_ok && !h->prof && !o->learned && h->nb == 1 &&
                        (inner_max <= 1 || igraph);
    if (cap && !sgraph) return TOPO_E_STATE;  // (a captured design iteration needs the device loop)
    bool sgraph_used = false;
    if (sgraph) {
      level_apply<double>(h, 0, h->x, h->f, h->r, true);  // r = f - A x
      launch_dot<double>(h->stream, h->r, h->r, n3, h->partial, h->sc + S_RR, h->ctr);
      count_launch();
      RET(coarse_join(h));  // the loop's first V-cycle needs the coarsest inverse
      std::vector<double> key = vcycle_key(h, o->pre, o->post, o->smoother, cp, true);
      key.insert(key.end(), {inner_rtol, (double)inner_max, (double)igraph});
      const int grc = outer_cg_graphed(h, o->rtol, o->max_iter, prec, key);
      if (grc == TOPO_OK) {
        sgraph_used = true;
      } else {  // the capture failed: the host loop, now and for the handle's later solves
        if (cap) return grc;
        igraph_used = false;
        CKL();
      }
    }
    if (!sgraph_used)
      rc = fcg_T<double>(h, h->x, h->f, h->r, h->d, h->q, h->rold, L0.U, o->rtol, o->max_iter, 0, prec,
                         &it, &rel, fn);
    CK(cudaMemcpyAsync(L0.F, h->f, sizeof(double) * n3, cudaMemcpyDeviceToDevice, h->stream));
    CK(cudaMemcpyAsync(L0.U, h->x, sizeof(double) * n3, cudaMemcpyDeviceToDevice, h->stream));
    if (sgraph_used && !cap) {  // outer (and inner) iterations the device ran, and non-finite residuals
      RET(read_scalars(h, S_LOOP, S_OLOOP + 4 - S_LOOP));
      const long long outer_its = (long long)h->hsc[S_OLOOP];
      const long long inner_its = igraph ? (long long)h->hsc[S_LOOP + 3] : 0;
      it = (int)outer_its;
      nvc = igraph ? (int)inner_its : (int)outer_its;
      count_launch((int)(outer_its * h->sgraph_body + inner_its * h->sgraph_inner));
      if (igraph && h->hsc[S_LOOP + 2] != 0.0)
        return fail(h, TOPO_E_NONFINITE, "inner CG residual became non-finite at iteration %d",
                    (int)h->hsc[S_LOOP + 2] - 1);
      if (h->hsc[S_OLOOP + 2] != 0.0)
        return fail(h, TOPO_E_NONFINITE, "CG residual became non-finite at iteration %d",
                    (int)h->hsc[S_OLOOP + 2] - 1);
    } else if (igraph_used && !sgraph_used) {  // inner iterations the device ran, and a non-finite inner residual
      RET(read_scalars(h, S_LOOP + 2, 2));
      const long long inner_its = (long long)h->hsc[S_LOOP + 3];
      nvc += (int)inner_its;
      count_launch((int)(inner_its * h->igraph_body));
      if (h->hsc[S_LOOP + 2] != 0.0)
        return fail(h, TOPO_E_NONFINITE, "inner CG residual became non-finite at iteration %d",
                    (int)h->hsc[S_LOOP + 2] - 1);
    }
    if (rc != TOPO_OK) return rc;
    if (harvest) {
      const cudaError_t e = unet_harvest_finish(h->unet, h->stream, L0.d, L0.vmask, h->x, h->unet_crops, h->partial);
      if (e != cudaSuccess) return fail(h, TOPO_E_CUDA, "harvest: %s", cudaGetErrorString(e));
    }
    st.iterations = it;
    st.vcycles = nvc;
  } else {
    return fail(h, TOPO_E_BAD_INPUT, "unknown solve mode %d", o->mode);
  }
  if (o->mode != TOPO_SOLVE_VCYCLE && fn != 0.0) {
    // true FP64 residual of the final iterate (with the element energies of
    // the sensitivity when a design iteration asks for them)
    if (h->want_energy && h->fine_df && h->nb == 1) {
      EventPair* ev = prof_begin(h, P<double>::fam_apply);
      launch_fine_apply_df(h->stream, L0.d, h->rhop, L0.vmask, L0.U, L0.F, L0.R, true, 1, h->tz64, h->sens);
      prof_end(h, ev);
      count_launch();
      h->energy_ready = true;
    } else {
      level_residual<double>(h, 0);
    }
    launch_dot<double>(h->stream, L0.R, L0.R, n3, h->partial, h->sc + S_RR, h->ctr);
    count_launch();
    if (cap) {
      CK(cudaEventRecordWithFlags(h->ev_solve[1], h->stream, cudaEventRecordExternal));
      return TOPO_OK;
    }
    RET(read_scalars(h, S_RR, 1));
    st.relres = std::sqrt(h->hsc[S_RR]) / fn;
  }
  RET(tc_wait_status(h));
  CK(cudaEventRecord(e1, h->stream));
  CK(cudaEventSynchronize(e1));
  float ms = 0;
  cudaEventElapsedTime(&ms, e0, e1);
  st.ms = ms;
  if (stats) *stats = st;
  CKL();
  if (!std::isfinite(st.relres)) return fail(h, TOPO_E_NONFINITE, "final residual is not finite");
  if (st.relres > o->rtol) return fail(h, TOPO_E_NOT_CONVERGED, "relative residual %.3e above %.3e after %d iterations", st.relres, o->rtol, st.iterations);
  return TOPO_OK;
}

int topo_compliance(topo_handle* h, double* c) {
  DEVICE_SCOPE(h);
  if (!h || !c) return TOPO_E_BAD_INPUT;
  DevLevel& L = h->lv[0];
  if (h->iter_capture) {  // read after the graph ran
    launch_dot<double>(h->stream, L.F, L.U, 3 * L.d.nv, h->partial, h->sc + S_DI);
    count_launch(2);
    *c = 0.0;
    return TOPO_OK;
  }
  launch_dot<double>(h->stream, L.F, L.U, 3 * L.d.nv, h->partial, h->sc + S_TMP);
  count_launch(2);
  CKL();
  RET(read_scalars(h, S_TMP, 1));
  *c = h->hsc[S_TMP];
  return TOPO_OK;
}

int topo_volume(topo_handle* h, int refden, double* v) {
  DEVICE_SCOPE(h);
  if (!h || !v) return TOPO_E_BAD_INPUT;
  launch_sum(h->stream, h->rho, h->lv[0].d.ne, h->partial, h->sc + S_TMP);
  count_launch(2);
  CKL();
  RET(read_scalars(h, S_TMP, 1));
  *v = h->hsc[S_TMP] / (double)(refden ? h->gs_padded_elements : h->active_elements);
  return TOPO_OK;
}

int topo_sensitivity(topo_handle* h) {
  DEVICE_SCOPE(h);
  if (!h) return TOPO_E_BAD_INPUT;
  const DevLevel& L = h->lv[0];
  launch_sensitivity(h->stream, L.d, L.eactive, h->rho, L.U, h->cfg.power_penalty, h->lam, h->mu,
                     h->cfg.h, h->sens);
  count_launch();
  if (h->ref_fp32) { launch_round_f32(h->stream, L.d.ne, h->sens); count_launch(); }
  CKL();
  return TOPO_OK;
}

}  // extern "C"

namespace topo {
// Neighbour offsets and weights of the sensitivity filter for `radius`
// (rebuilt when the radius changes).
int handle_filter_prepare(topo_handle* h, double radius) {
  if (!(radius > 0)) return TOPO_E_BAD_INPUT;
  if (radius > 16.0) return fail(h, TOPO_E_BAD_INPUT, "filter radius %.3g above 16 elements", radius);
  if (radius != h->filt_radius) {
    std::vector<int4> offs;
    std::vector<double> w;
    filter_table(radius, offs, w);
    if (h->filt_offs) { cudaFree(h->filt_offs); h->filt_offs = nullptr; }
    if (h->filt_w) { cudaFree(h->filt_w); h->filt_w = nullptr; }
    if (h->filt_wdf) { cudaFree(h->filt_wdf); h->filt_wdf = nullptr; }
    std::vector<float2> wdf(w.size());
    for (size_t k = 0; k < w.size(); ++k) {
      const float hi = (float)w[k];
      wdf[k] = make_float2(hi, (float)(w[k] - (double)hi));
    }
    CK(cudaMalloc((void**)&h->filt_offs, sizeof(int4) * offs.size()));
    CK(cudaMalloc((void**)&h->filt_w, sizeof(double) * w.size()));
    CK(cudaMalloc((void**)&h->filt_wdf, sizeof(float2) * w.size()));
    CK(cudaMemcpyAsync(h->filt_offs, offs.data(), sizeof(int4) * offs.size(), cudaMemcpyHostToDevice, h->stream));
    CK(cudaMemcpyAsync(h->filt_w, w.data(), sizeof(double) * w.size(), cudaMemcpyHostToDevice, h->stream));
    CK(cudaMemcpyAsync(h->filt_wdf, wdf.data(), sizeof(float2) * w.size(), cudaMemcpyHostToDevice, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    h->filt_n = (int)offs.size();
    h->filt_radius = radius;
  }
  return TOPO_OK;
}
}  // namespace topo

extern "C" {

int topo_filter(topo_handle* h, double radius) {
  DEVICE_SCOPE(h);
  if (!h || !(radius > 0)) return TOPO_E_BAD_INPUT;
  RET(handle_filter_prepare(h, radius));
  const DevLevel& L = h->lv[0];
  // double-float on the FP32 pipe, sens_tmp holding the split sensitivities
  launch_filter_df(h->stream, L.d, L.eactive, h->sens, reinterpret_cast<float2*>(h->sens_tmp), h->filt_offs,
                   h->filt_wdf, h->filt_n);
  count_launch(2);
  if (h->ref_fp32) { launch_round_f32(h->stream, L.d.ne, h->sens); count_launch(); }
  CKL();
  return TOPO_OK;
}

int topo_spline_adjoint(topo_handle* h) {
  DEVICE_SCOPE(h);
  if (!h) return TOPO_E_BAD_INPUT;
  if (!h->spline_set) return fail(h, TOPO_E_STATE, "spline not set");
  const DevLevel& L = h->lv[0];
  launch_spline_adjoint(h->stream, L.d, L.eactive, h->sd, h->sens, h->csens, h->adj1, h->adj2);
  count_launch(3);
  if (h->ref_fp32) {
    launch_round_f32(h->stream, (int64_t)h->sd.nb[0] * h->sd.nb[1] * h->sd.nb[2], h->csens);
    count_launch();
  }
  CKL();
  return TOPO_OK;
}

// FP64 fine operator on a batch of vectors, in the handle's fine arithmetic.
static void fine64(topo_handle* h, const LevelDims& d, const double* u, const double* f, double* out, bool residual,
                   int nb) {
  if (h->fine_df) launch_fine_apply_df(h->stream, d, h->rhop, h->lv[0].vmask, u, f, out, residual, nb, h->tz64);
  else launch_fine_apply<double>(h->stream, d, h->rhop, h->lv[0].vmask, u, f, out, residual, nb, h->tz64);
}

int topo_set_tiles(topo_handle* h, int tz32, int tz64) {
  DEVICE_SCOPE(h);
  if (!h || tz32 < 1 || tz32 > 256 || tz64 < 1 || tz64 > 256) return TOPO_E_BAD_INPUT;
  h->tz32 = tz32;
  h->tz64 = tz64;
  return TOPO_OK;
}

int topo_set_graphs(topo_handle* h, int enable) {
  DEVICE_SCOPE(h);
  if (!h) return TOPO_E_BAD_INPUT;
  if (enable < 0 || enable > 3) return TOPO_E_BAD_INPUT;
  h->graphs = enable != 0;
  if (h->vgraph) { cudaGraphExecDestroy(h->vgraph); h->vgraph = nullptr; }
  if (h->igraph) { cudaGraphExecDestroy(h->igraph); h->igraph = nullptr; }
  if (h->ograph) { cudaGraphExecDestroy(h->ograph); h->ograph = nullptr; }
  if (h->sgraph) { cudaGraphExecDestroy(h->sgraph); h->sgraph = nullptr; }
  if (h->dgraph) { cudaGraphExecDestroy(h->dgraph); h->dgraph = nullptr; }
  h->igraph_ok = h->ograph_ok = true;
  h->sgraph_ok = enable != 2;
  h->dgraph_ok = enable == 1;
  return TOPO_OK;
}

int topo_set_coarse_refresh(topo_handle* h, int every) {
  DEVICE_SCOPE(h);
  if (!h || every < 1) return TOPO_E_BAD_INPUT;
  h->coarse_every = every;
  h->coarse_age = 0;
  return TOPO_OK;
}

int topo_graph_state(const topo_handle* h, int* state) {
  if (!h || !state) return TOPO_E_BAD_INPUT;
  *state = (h->vgraph ? 1 : 0) | (h->igraph ? 2 : 0) | (h->sgraph ? 4 : 0) |
           (h->sgraph && h->sgraph_inner > 0 ? 8 : 0) | (h->ograph ? 16 : 0) | (h->dgraph ? 32 : 0);
  return TOPO_OK;
}

int topo_set_fine_tile_rows(topo_handle* h, int rows) {
  DEVICE_SCOPE(h);
  if (!h || (rows != 4 && rows != 8 && rows != 16)) return TOPO_E_BAD_INPUT;
  h->rows32 = rows;
  return TOPO_OK;
}

int topo_set_fine_tensor_cores(topo_handle* h, int on) {
  DEVICE_SCOPE(h);
  if (!h || on < 0 || on > 1) return TOPO_E_BAD_INPUT;
  h->fine_tc = on != 0;
  return TOPO_OK;
}

int topo_set_fine_arithmetic(topo_handle* h, int arith) {
  DEVICE_SCOPE(h);
  if (!h || arith < 0 || arith > 1) return TOPO_E_BAD_INPUT;
  h->fine_df = arith;
  return TOPO_OK;
}

int topo_profiler_range(int start) {
  const cudaError_t e = start ? cudaProfilerStart() : cudaProfilerStop();
  return e == cudaSuccess ? TOPO_OK : TOPO_E_CUDA;
}

int topo_design_batch(topo_handle** hs, int n, const topo_iter_opts* opts, int nopts, int iterations, int threads,
                      topo_iter_stats* last, topo_batch_stats* st) {
  if (!hs || n <= 0 || !opts || (nopts != 1 && nopts != n) || iterations < 0 || threads <= 0) return TOPO_E_BAD_INPUT;
  for (int i = 0; i < n; ++i)
    if (!hs[i]) return TOPO_E_BAD_INPUT;
  std::atomic<int> next{0}, failures{0}, first_rc{TOPO_OK};
  std::vector<double> busy(n, 0.0);
  const auto t0 = std::chrono::steady_clock::now();
  auto worker = [&]() {
    for (int k = next.fetch_add(1); k < n; k = next.fetch_add(1)) {
      const topo_iter_opts& o = opts[nopts == 1 ? 0 : k];
      const auto a = std::chrono::steady_clock::now();
      for (int it = 0; it < iterations; ++it) {
        topo_iter_stats s{};
        const int rc = topo_design_iteration(hs[k], &o, &s);
        if (rc != TOPO_OK && rc != TOPO_E_NOT_CONVERGED) {
          ++failures;
          int expect = TOPO_OK;
          first_rc.compare_exchange_strong(expect, rc);
          break;
        }
        if (last) last[k] = s;
      }
      busy[k] = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - a).count();
    }
  };
  const int nt = std::min(threads, n);
  std::vector<std::thread> pool;
  for (int t = 1; t < nt; ++t) pool.emplace_back(worker);
  worker();
  for (auto& t : pool) t.join();
  if (st) {
    st->wall_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    st->sum_ms = 0;
    st->max_ms = 0;
    for (double b : busy) { st->sum_ms += b; st->max_ms = std::max(st->max_ms, b); }
    st->failures = failures.load();
  }
  return first_rc.load();
}

int topo_autotune(topo_handle* h, const topo_solve_opts* base, topo_solve_opts* best, topo_tune_report* rep) {
  DEVICE_SCOPE(h);
  RET(check_ready(h, true));
  if (!base || !best || base->mode != TOPO_SOLVE_MIXED || base->smoother != TOPO_SMOOTH_CHEBYSHEV || base->learned)
    return fail(h, TOPO_E_BAD_INPUT, "autotune: base schedule must be MIXED with the Chebyshev smoother");
  if (!h->ops32) return fail(h, TOPO_E_STATE, "FP32 operators not built");
  topo_tune_report r{};
  DevLevel& L0 = h->lv[0];
  const int64_t n3 = 3 * L0.d.nv;
  ScopedEvent t0, t1, a, b;
  CK(t0.create()); CK(t1.create()); CK(a.create()); CK(b.create());
  CK(cudaEventRecord(t0, h->stream));
  ChebParams cp;
  if (base->cheb_degree > 0) cp.degree = base->cheb_degree;
  if (base->cheb_lo > 0) cp.lo = base->cheb_lo;
  if (base->cheb_hi > 0) cp.hi = base->cheb_hi;
  RET(prepare_smoother<float>(h, TOPO_SMOOTH_CHEBYSHEV, cp));
  const double* unit = h->chebc + CHEB_TABLE - 2;  // (c_old, c_new) = (0, 1)
  // ---- stage 1: z-march depth of the fine kernels
  const int tzs[4] = {4, 8, 16, 32};
  int best32 = h->tz32, best64 = h->tz64;
  double b32 = 1e30, b64 = 1e30;
  int best_tc = h->fine_tc ? 1 : 0, best_rows = h->rows32;
  for (int k = 0; k < 4; ++k) {
    // the FP32 Chebyshev step: modal element products with CTA tiles of 8, 4
    // and 16 element rows, and on the tensor cores
    for (int form = 0; form < 4; ++form) {
      const int flags = form == 1 ? TOPO_FINE_TC_FLAG : form == 2 ? TOPO_FINE_ROWS4_FLAG
                        : form == 3 ? TOPO_FINE_ROWS16_FLAG : 0;
      double* slot = form == 0 ? &r.cheb_ms[k] : form == 1 ? &r.cheb_tc_ms[k] : &r.cheb_rows_ms[form - 2][k];
      for (int rep = 0; rep < 2; ++rep) {  // warm-up, then timed
        CK(cudaEventRecord(a, h->stream));
        for (int i = 0; i < 5; ++i)
          launch_fine_cheb<float>(h->stream, L0.d, h->rhop32, L0.vmask, L0.U32, L0.F32, L0.U2_32, L0.dinv32,
                                  L0.cd32, unit, true, 1, tzs[k] | flags);
        CK(cudaEventRecord(b, h->stream));
        CK(cudaEventSynchronize(b));
        float ms = 0;
        cudaEventElapsedTime(&ms, a, b);
        *slot = ms / 5;
      }
    }
    for (int rep = 0; rep < 2; ++rep) {
      CK(cudaEventRecord(a, h->stream));
      for (int i = 0; i < 5; ++i) {
        if (h->fine_df) launch_fine_apply_df(h->stream, L0.d, h->rhop, L0.vmask, h->work, nullptr, L0.R, false, 1, tzs[k]);
        else launch_fine_apply<double>(h->stream, L0.d, h->rhop, L0.vmask, h->work, nullptr, L0.R, false, 1, tzs[k]);
      }
      CK(cudaEventRecord(b, h->stream));
      CK(cudaEventSynchronize(b));
      float ms = 0;
      cudaEventElapsedTime(&ms, a, b);
      r.apply_ms[k] = ms / 5;
    }
    count_launch(50);
    if (r.cheb_ms[k] < b32) { b32 = r.cheb_ms[k]; best32 = tzs[k]; best_tc = 0; best_rows = 8; }
    if (r.cheb_tc_ms[k] < b32) { b32 = r.cheb_tc_ms[k]; best32 = tzs[k]; best_tc = 1; best_rows = 8; }
    for (int q = 0; q < 2; ++q)
      if (r.cheb_rows_ms[q][k] < b32) { b32 = r.cheb_rows_ms[q][k]; best32 = tzs[k]; best_tc = 0; best_rows = q ? 16 : 4; }
    if (r.apply_ms[k] < b64) { b64 = r.apply_ms[k]; best64 = tzs[k]; }
  }
  CKL();
  h->tz32 = best32;
  h->tz64 = best64;
  h->fine_tc = best_tc != 0;
  h->rows32 = best_rows;
  r.tz32 = best32;
  r.tz64 = best64;
  r.tc = best_tc;
  r.rows32 = best_rows;
  // ---- stage 2: solver schedule, each candidate from the same initial U
  double* u0 = nullptr;
  CK(cudaMalloc((void**)&u0, sizeof(double) * n3));
  CK(cudaMemcpyAsync(u0, L0.U, sizeof(double) * n3, cudaMemcpyDeviceToDevice, h->stream));
  // each candidate is timed on its second run: the first captures its graphs
  // (V-cycle, solve loops), which the design iterations then replay
  auto run = [&](const topo_solve_opts& o, double* ms) -> int {
    topo_solve_stats st{};
    int rc = TOPO_OK;
    for (int rep = 0; rep < (h->graphs ? 2 : 1); ++rep) {
      cudaMemcpyAsync(L0.U, u0, sizeof(double) * n3, cudaMemcpyDeviceToDevice, h->stream);
      rc = topo_solve(h, &o, &st);
      if (rc != TOPO_OK) break;
    }
    *ms = st.ms;
    return rc;
  };
  *best = *base;
  double bt = 1e30;
  int rc0 = run(*base, &r.base_ms);
  if (rc0 == TOPO_OK) bt = r.base_ms;
  // FP32 inner iterations x V(s,s) x Chebyshev degree x lower end of the
  // Chebyshev interval (the base's, and 0.1 lambda_max) x inner tolerance (the
  // base's, and 0.03).  On the 256x128x128 half-MBB beam: lower end 0.3 took 23
  // V-cycles per solve, 0.1 took 19; degree 3 with 0.06 and inner tolerance
  // 0.03 took 3 outer iterations and 14 V-cycles.
  const int inners[4] = {1, 2, 4, 6};
  const double base_lo = base->cheb_lo > 0 ? base->cheb_lo : ChebParams{}.lo;
  const double base_irt = base->inner_rtol > 0 ? base->inner_rtol : 1e-1;
  const double los[2] = {base_lo, 0.1}, irts[2] = {base_irt, 0.03};
  const int nlo = base_lo == 0.1 ? 1 : 2, nirt = base_irt == 0.03 ? 1 : 2;
  for (int ii = 0; ii < 4; ++ii)
    for (int sm = 1; sm <= 2; ++sm)
      for (int deg = 2; deg <= 3; ++deg)
        for (int il = 0; il < nlo; ++il)
          for (int ir = 0; ir < nirt; ++ir) {
            topo_solve_opts o = *base;
            o.inner_max = inners[ii];
            o.pre = o.post = sm;
            o.cheb_degree = deg;
            o.cheb_lo = los[il];
            o.inner_rtol = irts[ir];
            double ms = 0;
            ++r.candidates;
            if (run(o, &ms) == TOPO_OK && ms < bt) { bt = ms; *best = o; }
          }
  // ---- stage 3: two passes of coordinate search from the best schedule over
  // the interval's lower end, the inner tolerance and the degree (each change
  // kept when it is faster).  On the 256x128x128 beam degree 3 with lower end
  // 0.06 and inner tolerance 0.03 beat the best grid point by 8%.
  std::vector<double> lo_alt = {0.05, 0.1, 0.2};
  if (std::find(lo_alt.begin(), lo_alt.end(), base_lo) == lo_alt.end()) lo_alt.push_back(base_lo);
  std::vector<double> irt_alt = {0.03};
  if (base_irt != 0.03) irt_alt.push_back(base_irt);
  for (int pass = 0; pass < 2; ++pass) {
    for (int param = 0; param < 3; ++param) {
      const topo_solve_opts cur = *best;
      std::vector<topo_solve_opts> cands;
      if (param == 0) {
        for (const double lo : lo_alt)
          if (lo != cur.cheb_lo) { topo_solve_opts o = cur; o.cheb_lo = lo; cands.push_back(o); }
      } else if (param == 1) {
        for (const double irt : irt_alt)
          if (irt != cur.inner_rtol) { topo_solve_opts o = cur; o.inner_rtol = irt; cands.push_back(o); }
      } else {
        topo_solve_opts o = cur;
        o.cheb_degree = cur.cheb_degree == 2 ? 3 : 2;
        cands.push_back(o);
      }
      for (const topo_solve_opts& o : cands) {
        double ms = 0;
        ++r.candidates;
        if (run(o, &ms) == TOPO_OK && ms < bt) { bt = ms; *best = o; }
      }
    }
  }
  // ---- stage 4: joint moves the coordinate search cannot make one at a time:
  // degrees 2, 3, 4 x lower ends 0.02, 0.04, 0.06 x inner tolerances 0.03, 0.05,
  // from the best schedule's inner iterations and smoothing steps.  On the
  // 256x128x128 beam degree 3 wants a lower interval end and a tighter inner
  // tolerance together (fewer outer iterations, each V-cycle stronger), while
  // either change alone is slower: 3 outer iterations and 14 V-cycles against
  // 5 and 19 (solve 21.1 against 22.9 ms); degree 4 takes 12 V-cycles (20.8 ms).
  {
    const topo_solve_opts cur = *best;
    const double lo4[3] = {0.02, 0.04, 0.06}, irt4[2] = {0.03, 0.05};
    for (int deg = 2; deg <= 4; ++deg)
      for (const double lo : lo4)
        for (const double irt : irt4) {
          topo_solve_opts o = cur;
          o.cheb_degree = deg;
          o.cheb_lo = lo;
          o.inner_rtol = irt;
          double ms = 0;
          ++r.candidates;
          if (run(o, &ms) == TOPO_OK && ms < bt) { bt = ms; *best = o; }
        }
  }
  // ---- stage 5: stronger inner solves around the best (more FP32 iterations
  // to a tighter tolerance, so fewer FP64 outer iterations, each with its
  // double-float matvec) and a degree above it
  {
    const topo_solve_opts cur = *best;
    const int im5[2] = {cur.inner_max + 2, cur.inner_max + 4};
    const double irt5[2] = {0.01, 0.02};
    for (const int im : im5)
      for (const double irt : irt5) {
        topo_solve_opts o = cur;
        o.inner_max = im;
        o.inner_rtol = irt;
        double ms = 0;
        ++r.candidates;
        if (run(o, &ms) == TOPO_OK && ms < bt) { bt = ms; *best = o; }
      }
    if (cur.cheb_degree + 1 <= CHEB_MAX_DEG) {
      topo_solve_opts o = *best;
      o.cheb_degree = best->cheb_degree + 1;
      double ms = 0;
      ++r.candidates;
      if (run(o, &ms) == TOPO_OK && ms < bt) { bt = ms; *best = o; }
    }
  }
  r.best_ms = bt;
  cudaMemcpyAsync(L0.U, u0, sizeof(double) * n3, cudaMemcpyDeviceToDevice, h->stream);
  CK(cudaEventRecord(t1, h->stream));
  CK(cudaEventSynchronize(t1));
  cudaFree(u0);
  float tms = 0;
  cudaEventElapsedTime(&tms, t0, t1);
  r.tune_ms = tms;
  h->err.clear();
  if (rep) *rep = r;
  if (bt >= 1e30) return fail(h, TOPO_E_NOT_CONVERGED, "autotune: no schedule converged");
  return TOPO_OK;
}

int topo_multi_reserve(topo_handle* h, int capacity) {
  DEVICE_SCOPE(h);
  if (!h || capacity <= 0 || capacity > 1024) return TOPO_E_BAD_INPUT;
  if (h->multi) {
    for (void* p : h->multi->allocs) cudaFree(p);
    delete h->multi;
    h->multi = nullptr;
  }
  std::unique_ptr<MultiRhs> m(new MultiRhs);
  m->cap = capacity;
  auto alloc = [&](void** p, size_t bytes) -> int {
    if (cudaMalloc(p, std::max<size_t>(bytes, 256)) != cudaSuccess) return TOPO_E_NOMEM;
    m->allocs.push_back(*p);
    return cudaMemsetAsync(*p, 0, bytes, h->stream) == cudaSuccess ? TOPO_OK : TOPO_E_CUDA;
  };
  int rc = TOPO_OK;
  for (size_t l = 0; l < h->lv.size() && rc == TOPO_OK; ++l) {
    const size_t n = (size_t)capacity * 3 * h->lv[l].d.nv * sizeof(float);
    float *a, *b, *c, *d, *e;
    rc |= alloc((void**)&a, n); rc |= alloc((void**)&b, n); rc |= alloc((void**)&c, n);
    rc |= alloc((void**)&d, n); rc |= alloc((void**)&e, n);
    m->U.push_back(a); m->F.push_back(b); m->R.push_back(c); m->U2.push_back(d); m->cd.push_back(e);
  }
  const size_t n64 = (size_t)capacity * 3 * h->lv[0].d.nv * sizeof(double);
  for (double** v : {&m->x, &m->f, &m->r, &m->d, &m->q, &m->rold, &m->z})
    if (rc == TOPO_OK) rc = alloc((void**)v, n64);
  for (float** v : {&m->x32, &m->d32, &m->q32})
    if (rc == TOPO_OK) rc = alloc((void**)v, n64 / 2);
  if (rc == TOPO_OK) rc = alloc((void**)&m->part, (size_t)capacity * 256 * sizeof(double));
  if (rc == TOPO_OK) rc = alloc((void**)&m->sc, (size_t)capacity * 16 * sizeof(double));
  if (rc != TOPO_OK) {
    for (void* p : m->allocs) cudaFree(p);
    return fail(h, rc, "multi-RHS buffers for %d right-hand sides", capacity);
  }
  CK(cudaStreamSynchronize(h->stream));
  h->multi = m.release();
  return TOPO_OK;
}

int topo_solve_multi(topo_handle* h, int nrhs, const topo_solve_opts* o, topo_multi_stats* stats, double* relres) {
  DEVICE_SCOPE(h);
  RET(check_ready(h, true));
  if (!o || o->rtol <= 0 || o->max_iter < 0 || o->pre < 0 || o->post < 0) return TOPO_E_BAD_INPUT;
  if (!h->multi) return fail(h, TOPO_E_STATE, "call topo_multi_reserve first");
  if (nrhs <= 0 || nrhs > h->multi->cap) return fail(h, TOPO_E_BAD_INPUT, "nrhs %d outside 1..%d", nrhs, h->multi->cap);
  if (o->mode != TOPO_SOLVE_MIXED || o->smoother != TOPO_SMOOTH_CHEBYSHEV || o->learned)
    return fail(h, TOPO_E_BAD_INPUT, "multi-RHS solve: mode MIXED, Chebyshev smoother, no learned part");
  if (!h->ops32) return fail(h, TOPO_E_STATE, "FP32 operators not built");
  ChebParams cp;
  if (o->cheb_degree > 0) cp.degree = o->cheb_degree;
  if (o->cheb_lo > 0) cp.lo = o->cheb_lo;
  if (o->cheb_hi > 0) cp.hi = o->cheb_hi;
  RET(prepare_smoother<float>(h, TOPO_SMOOTH_CHEBYSHEV, cp));
  MultiRhs& m = *h->multi;
  DevLevel& L0 = h->lv[0];
  const int nb = nrhs;
  const int64_t n3 = 3 * L0.d.nv;
  // the batched buffers stand in for the level vectors during the solve
  struct Swap {
    topo_handle* h;
    std::vector<std::array<float*, 5>> saved;
    Swap(topo_handle* hh, MultiRhs& mm, int nbb) : h(hh) {
      for (size_t l = 0; l < h->lv.size(); ++l) {
        DevLevel& L = h->lv[l];
        saved.push_back({L.U32, L.F32, L.R32, L.U2_32, L.cd32});
        L.U32 = mm.U[l]; L.F32 = mm.F[l]; L.R32 = mm.R[l]; L.U2_32 = mm.U2[l]; L.cd32 = mm.cd[l];
      }
      h->nb = nbb;
    }
    ~Swap() {
      for (size_t l = 0; l < h->lv.size(); ++l) {
        DevLevel& L = h->lv[l];
        L.U32 = saved[l][0]; L.F32 = saved[l][1]; L.R32 = saved[l][2]; L.U2_32 = saved[l][3]; L.cd32 = saved[l][4];
      }
      h->nb = 1;
    }
  } swap(h, m, nb);
  enum { B_RR, B_FF, B_RZ, B_ZROLD, B_RZOLD, B_DQ, B_ALPHA, B_BETA,
         I_RR, I_FF, I_RZ, I_RZOLD, I_DQ, I_ALPHA, I_BETA, I_ZERO };  // outer, inner (16 slots)
  const int inner_max = o->inner_max > 1 ? o->inner_max : 1;
  const double inner_rtol = o->inner_rtol > 0 ? o->inner_rtol : 1e-1;
  double* sb = m.sc;
  auto slot = [&](int k) { return sb + (size_t)k * m.cap; };
  ScopedEvent e0, e1;
  CK(e0.create());
  CK(e1.create());
  CK(cudaEventRecord(e0, h->stream));
  // r = f - A x, ||r||^2, ||f||^2 per right-hand side
  fine64(h, L0.d, m.x, m.f, m.r, true, nb);
  launch_bdot<double>(h->stream, m.r, m.r, n3, nb, m.part, slot(B_RR));
  launch_bdot<double>(h->stream, m.f, m.f, n3, nb, m.part, slot(B_FF));
  count_launch(5);
  std::vector<double> rr(nb), ff(nb);
  CK(cudaMemcpyAsync(rr.data(), slot(B_RR), sizeof(double) * nb, cudaMemcpyDeviceToHost, h->stream));
  CK(cudaMemcpyAsync(ff.data(), slot(B_FF), sizeof(double) * nb, cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  const double rtol2 = o->rtol * o->rtol;
  auto converged = [&]() {
    for (int k = 0; k < nb; ++k)
      if (rr[k] > rtol2 * ff[k]) return false;
    return true;
  };
  int it = 0, nvc = 0;
  if (inner_max > 1) CK(cudaMemsetAsync(slot(I_ZERO), 0, sizeof(double) * nb, h->stream));
  while (!converged() && it < o->max_iter) {
    launch_d2f(h->stream, m.r, L0.F32, n3 * nb);
    if (inner_max <= 1) {
      // z = V(r): one FP32 V-cycle for the whole batch
      if (!cheb_zero_start(TOPO_SMOOTH_CHEBYSHEV, o->pre, cp))
        CK(cudaMemsetAsync(L0.U32, 0, sizeof(float) * n3 * nb, h->stream));
      vcycle32(h, o->pre, o->post, TOPO_SMOOTH_CHEBYSHEV, cp, true);
      ++nvc;
      k_to_double<float><<<nb256(n3 * nb), 256, 0, h->stream>>>(n3 * nb, L0.U32, m.z);
    } else {
      // z = inner_max iterations of an FP32 CG per right-hand side on A z = r,
      // preconditioned by the batched V-cycle (a fixed symmetric operator, so
      // the Fletcher-Reeves form: zrold = 0, rold not kept).  Its residual is
      // level-0 F32, the V-cycle's right-hand side, x32 starts at 0; a
      // right-hand side whose inner residual fell by inner_rtol gets alpha = 0
      // and stops there, so the loop needs no host decision.
      float* r32 = L0.F32;
      float* z32 = L0.U32;
      CK(cudaMemsetAsync(m.x32, 0, sizeof(float) * n3 * nb, h->stream));
      launch_bdot<float>(h->stream, r32, r32, n3, nb, m.part, slot(I_FF));
      CK(cudaMemcpyAsync(slot(I_RR), slot(I_FF), sizeof(double) * nb, cudaMemcpyDeviceToDevice, h->stream));
      count_launch(2);
      for (int j = 0; j < inner_max; ++j) {
        if (!cheb_zero_start(TOPO_SMOOTH_CHEBYSHEV, o->pre, cp))
          CK(cudaMemsetAsync(z32, 0, sizeof(float) * n3 * nb, h->stream));
        vcycle32(h, o->pre, o->post, TOPO_SMOOTH_CHEBYSHEV, cp, true);
        ++nvc;
        launch_bdot<float>(h->stream, r32, z32, n3, nb, m.part, slot(I_RZ));
        launch_bbeta(h->stream, nb, slot(I_RZ), slot(I_ZERO), slot(I_RZOLD), j == 0, slot(I_BETA));
        launch_bdir<float>(h->stream, n3, nb, z32, m.d32, slot(I_BETA));
        launch_fine_apply<float>(h->stream, L0.d, h->rhop32, L0.vmask, m.d32, nullptr, m.q32, false, nb,
                                 tz32_arg(h));
        launch_bdot<float>(h->stream, m.d32, m.q32, n3, nb, m.part, slot(I_DQ));
        launch_balpha(h->stream, nb, slot(I_RZ), slot(I_DQ), slot(I_RR), slot(I_FF), inner_rtol * inner_rtol,
                      slot(I_ALPHA), slot(I_RZOLD));
        launch_bupdate<float>(h->stream, n3, nb, m.x32, r32, nullptr, m.d32, m.q32, slot(I_ALPHA));
        launch_bdot<float>(h->stream, r32, r32, n3, nb, m.part, slot(I_RR));
        count_launch(14);
      }
      k_to_double<float><<<nb256(n3 * nb), 256, 0, h->stream>>>(n3 * nb, m.x32, m.z);
    }
    launch_bdot<double>(h->stream, m.r, m.z, n3, nb, m.part, slot(B_RZ));
    if (it > 0) launch_bdot<double>(h->stream, m.z, m.rold, n3, nb, m.part, slot(B_ZROLD));
    launch_bbeta(h->stream, nb, slot(B_RZ), slot(B_ZROLD), slot(B_RZOLD), it == 0, slot(B_BETA));
    launch_bdir<double>(h->stream, n3, nb, m.z, m.d, slot(B_BETA));
    fine64(h, L0.d, m.d, nullptr, m.q, false, nb);
    launch_bdot<double>(h->stream, m.d, m.q, n3, nb, m.part, slot(B_DQ));
    launch_balpha(h->stream, nb, slot(B_RZ), slot(B_DQ), slot(B_RR), slot(B_FF), rtol2, slot(B_ALPHA),
                  slot(B_RZOLD));
    launch_bupdate<double>(h->stream, n3, nb, m.x, m.r, m.rold, m.d, m.q, slot(B_ALPHA));
    launch_bdot<double>(h->stream, m.r, m.r, n3, nb, m.part, slot(B_RR));
    count_launch(it > 0 ? 16 : 14);
    CKL();
    CK(cudaMemcpyAsync(rr.data(), slot(B_RR), sizeof(double) * nb, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    for (int k = 0; k < nb; ++k)
      if (!std::isfinite(rr[k])) return fail(h, TOPO_E_NONFINITE, "right-hand side %d became non-finite", k);
    ++it;
  }
  // true FP64 residuals of the final iterates
  fine64(h, L0.d, m.x, m.f, m.r, true, nb);
  launch_bdot<double>(h->stream, m.r, m.r, n3, nb, m.part, slot(B_RR));
  count_launch(3);
  CK(cudaMemcpyAsync(rr.data(), slot(B_RR), sizeof(double) * nb, cudaMemcpyDeviceToHost, h->stream));
  CK(cudaEventRecord(e1, h->stream));
  CK(cudaEventSynchronize(e1));
  float ms = 0;
  cudaEventElapsedTime(&ms, e0, e1);
  double worst = 0;
  for (int k = 0; k < nb; ++k) {
    const double rel = ff[k] > 0 ? std::sqrt(rr[k] / ff[k]) : 0.0;
    if (relres) relres[k] = rel;
    worst = std::max(worst, rel);
  }
  if (stats) {
    stats->iterations = it;
    stats->vcycles = nvc;
    stats->max_relres = worst;
    stats->ms = ms;
  }
  if (worst > o->rtol) return fail(h, TOPO_E_NOT_CONVERGED, "largest relative residual %.3e above %.3e", worst, o->rtol);
  return TOPO_OK;
}

int topo_unet_enable(topo_handle* h, unsigned long long seed) {
  DEVICE_SCOPE(h);
  if (!h) return TOPO_E_BAD_INPUT;
  if (h->unet) { unet_free(h->unet); h->unet = nullptr; }
  const cudaError_t e = unet_create(&h->unet, h->stream, seed);
  if (e != cudaSuccess) { h->unet = nullptr; return fail(h, e == cudaErrorMemoryAllocation ? TOPO_E_NOMEM : TOPO_E_CUDA, "U-Net: %s", cudaGetErrorString(e)); }
  return TOPO_OK;
}

int topo_unet_set_conv_kernel(topo_handle* h, int kind) {
  if (!h) return TOPO_E_BAD_INPUT;
  if (!h->unet) return fail(h, TOPO_E_STATE, "learned preconditioner not enabled (topo_unet_enable)");
  if (kind != TOPO_CONV_TCGEN05 && kind != TOPO_CONV_MMA_SYNC) return fail(h, TOPO_E_BAD_INPUT, "unknown convolution kernel %d", kind);
  unet_set_conv_kernel(h->unet, kind);
  return TOPO_OK;
}

int topo_unet_num_params(size_t* n) {
  if (!n) return TOPO_E_BAD_INPUT;
  *n = unet_param_count();
  return TOPO_OK;
}

static int unet_ready(topo_handle* h) {
  if (!h) return TOPO_E_BAD_INPUT;
  if (!h->unet) return fail(h, TOPO_E_STATE, "learned preconditioner not enabled (topo_unet_enable)");
  return TOPO_OK;
}

int topo_unet_get_params(topo_handle* h, float* dst, size_t n) {
  DEVICE_SCOPE(h);
  RET(unet_ready(h));
  if (!dst || n != unet_param_count()) return fail(h, TOPO_E_BAD_INPUT, "expected %zu parameters", unet_param_count());
  CK(unet_get_params(h->unet, h->stream, dst));
  return TOPO_OK;
}

int topo_unet_set_params(topo_handle* h, const float* src, size_t n) {
  DEVICE_SCOPE(h);
  RET(unet_ready(h));
  if (!src || n != unet_param_count()) return fail(h, TOPO_E_BAD_INPUT, "expected %zu parameters", unet_param_count());
  for (size_t i = 0; i < n; ++i)
    if (!std::isfinite(src[i])) return fail(h, TOPO_E_BAD_INPUT, "non-finite parameter %zu", i);
  CK(unet_set_params(h->unet, h->stream, src));
  return TOPO_OK;
}

static int unet_dims_ok(topo_handle* h, int X, int Y, int Z, int nb) {
  if (X <= 0 || Y <= 0 || Z <= 0 || nb <= 0 || X % 8 || Y % 8 || Z % 8 || (int64_t)nb * X * Y * Z > (1LL << 27))
    return fail(h, TOPO_E_BAD_INPUT, "U-Net tensor dims must be positive multiples of 8");
  return TOPO_OK;
}

int topo_unet_forward(topo_handle* h, int X, int Y, int Z, int nb, const float* x, float* y) {
  DEVICE_SCOPE(h);
  RET(unet_ready(h));
  RET(unet_dims_ok(h, X, Y, Z, nb));
  if (!x || !y) return TOPO_E_BAD_INPUT;
  CK(unet_host_pass(h->unet, h->stream, X, Y, Z, nb, x, nullptr, nullptr, y, nullptr, nullptr));
  return TOPO_OK;
}

int topo_unet_loss_grad(topo_handle* h, int X, int Y, int Z, int nb, const float* x, const float* t,
                        const uint8_t* mask, double* loss, float* grad) {
  DEVICE_SCOPE(h);
  RET(unet_ready(h));
  RET(unet_dims_ok(h, X, Y, Z, nb));
  if (!x || !t || !mask || !loss || !grad) return TOPO_E_BAD_INPUT;
  CK(unet_host_pass(h->unet, h->stream, X, Y, Z, nb, x, t, mask, nullptr, loss, grad));
  return TOPO_OK;
}

int topo_unet_dataset_reserve(topo_handle* h, int capacity, int crop, int crops_per_iterate) {
  DEVICE_SCOPE(h);
  RET(unet_ready(h));
  if (capacity <= 0 || crop <= 0 || crop % 8 || crop > 64 || crops_per_iterate <= 0 || crops_per_iterate > 4096)
    return fail(h, TOPO_E_BAD_INPUT, "dataset: capacity > 0, crop a multiple of 8 up to 64, 1..4096 crops per iterate");
  const cudaError_t e = unet_dataset_reserve(h->unet, capacity, crop);
  if (e == cudaErrorInvalidValue) return fail(h, TOPO_E_STATE, "dataset already reserved");
  if (e != cudaSuccess) return fail(h, TOPO_E_NOMEM, "dataset: %s", cudaGetErrorString(e));
  h->unet_crops = crops_per_iterate;
  return TOPO_OK;
}

int topo_unet_dataset_size(topo_handle* h, int* n) {
  DEVICE_SCOPE(h);
  RET(unet_ready(h));
  if (!n) return TOPO_E_BAD_INPUT;
  *n = unet_dataset_count(h->unet);
  return TOPO_OK;
}

int topo_unet_dataset_get(topo_handle* h, int slot, float* x, float* t, uint8_t* mask, int* crop) {
  DEVICE_SCOPE(h);
  RET(unet_ready(h));
  if (!x || !t || !mask || !crop) return TOPO_E_BAD_INPUT;
  *crop = unet_crop_side(h->unet);
  const cudaError_t e = unet_dataset_get(h->unet, h->stream, slot, x, t, mask);
  if (e == cudaErrorInvalidValue) return fail(h, TOPO_E_BAD_INPUT, "no crop %d", slot);
  if (e != cudaSuccess) return fail(h, TOPO_E_CUDA, "dataset: %s", cudaGetErrorString(e));
  return TOPO_OK;
}

int topo_unet_train(topo_handle* h, int steps, int batch, double lr, unsigned long long seed, int lo, int hi,
                    int update, double* loss) {
  DEVICE_SCOPE(h);
  RET(unet_ready(h));
  if (!loss || steps <= 0 || steps > 65536 || batch <= 0 || batch > 64 || !(lr > 0))
    return fail(h, TOPO_E_BAD_INPUT, "train: 1..65536 steps, batch 1..64, lr > 0");
  if (unet_dataset_count(h->unet) == 0) return fail(h, TOPO_E_STATE, "no harvested crops");
  const cudaError_t e = unet_train(h->unet, h->stream, steps, batch, lr, seed, lo, hi, update != 0, loss);
  if (e != cudaSuccess) return fail(h, TOPO_E_CUDA, "train: %s", cudaGetErrorString(e));
  return TOPO_OK;
}

int topo_volume_csens(topo_handle* h, int refden, double scale, double* out_dev) {
  DEVICE_SCOPE(h);
  if (!h) return TOPO_E_BAD_INPUT;
  if (!h->spline_set) return fail(h, TOPO_E_STATE, "spline not set");
  if (!out_dev) out_dev = h->volcsens;
  const DevLevel& L = h->lv[0];
  const double den = (double)(refden ? h->gs_padded_elements : h->active_elements);
  // d volume / d rho_e = 1/den on every active element; the adjoint skips the rest
  launch_fill<double>(h->stream, h->sens_tmp, scale / den, L.d.ne);
  launch_spline_adjoint(h->stream, L.d, L.eactive, h->sd, h->sens_tmp, out_dev, h->adj1, h->adj2);
  count_launch(4);
  CKL();
  return TOPO_OK;
}

}  // extern "C"

namespace topo {
// Read-only view of the handle state the allocation-free spline adjoint needs.
int handle_spline_view(topo_handle* h, SplineView* out) {
  if (!h || !out) return TOPO_E_BAD_INPUT;
  if (!h->spline_set) return fail(h, TOPO_E_STATE, "spline not set");
  out->d = h->lv[0].d;
  out->eactive = h->lv[0].eactive;
  out->sp = h->sd;
  out->stream = h->stream;
  out->device = h->cfg.device;
  return TOPO_OK;
}
int handle_fail(topo_handle* h, int code, const char* msg) { return fail(h, code, "%s", msg); }
int handle_level_view(topo_handle* h, LevelView* out) {
  if (!h || !out) return TOPO_E_BAD_INPUT;
  out->d = h->lv[0].d;
  out->vmask = h->lv[0].vmask;
  out->stream = h->stream;
  out->device = h->cfg.device;
  return TOPO_OK;
}
WorstState*& handle_worst_slot(topo_handle* h) { return h->worst; }
}  // namespace topo

// The OC bisection of topo_oc_update as one CUDA graph: start (bracket [0,
// max |dc|] from the device slot S_TMP), a WHILE node whose body is one trial
// (coefficients at the threshold, their volume) closed by the bracket update
// and loop test, and the second application when asked.  The trials, their
// thresholds and the stopping rule are the host loop's, decided on the
// device; the trial count and final threshold are left in the OC slots.
static int oc_bisection_graphed(topo_handle* h, const topo_oc_opts* o, int64_t nc, double den) {
  const DevLevel& L = h->lv[0];
  double* oc = h->sc + S_OC;
  const SplineDev& sp = h->sd;
  std::vector<double> key = {(double)nc, den, o->vgoal, o->damp, o->step, o->cmin, o->cmax,
                             (double)o->apply_twice, (double)sp.order, h->cfg.min_density};
  for (int a = 0; a < 3; ++a)
    key.insert(key.end(), {(double)sp.nb[a], (double)(uintptr_t)sp.i0[a], (double)(uintptr_t)sp.Ndf[a]});
  for (const void* p : {(const void*)h->coeff, (const void*)h->coeff_old, (const void*)h->csens,
                        (const void*)h->coeff_df, (const void*)h->coeff_tmp, (const void*)h->adj1,
                        (const void*)L.eactive})
    key.push_back((double)(uintptr_t)p);
  auto setup = [&](cudaGraphConditionalHandle hc) -> int {
    k_ocl_start<<<1, 32, 0, h->stream>>>(oc, h->sc + S_TMP, hc);
    count_launch();
    return TOPO_OK;
  };
  auto body = [&](cudaGraphConditionalHandle hc) -> int {
    launch_oc_trial(h->stream, nc, h->coeff_old, h->csens, 0.0, o->damp, o->step, o->cmin, o->cmax, h->coeff,
                    h->coeff_df, oc + 2);
    launch_trial_volume(h->stream, L.d, L.eactive, h->sd, h->coeff_df, h->cfg.min_density, h->partial,
                        h->sc + S_TMP, h->adj1);
    k_ocl_step<<<1, 32, 0, h->stream>>>(oc, h->sc + S_TMP, den, o->vgoal, hc);
    count_launch(5);
    return TOPO_OK;
  };
  auto tail = [&]() -> int {
    if (o->apply_twice) {
      launch_oc_trial(h->stream, nc, h->coeff, h->csens, 0.0, o->damp, o->step, o->cmin, o->cmax, h->coeff_tmp,
                      nullptr, oc + 2);
      CK(cudaMemcpyAsync(h->coeff, h->coeff_tmp, sizeof(double) * nc, cudaMemcpyDeviceToDevice, h->stream));
      count_launch();
    }
    return TOPO_OK;
  };
  if (h->iter_capture) {  // inside a captured design iteration: a nested WHILE node
    RET(capture_nested_loop(h, setup, body, &h->d_oc_body));
    return tail();
  }
  if (!h->ograph || key != h->okey) {
    if (h->ograph) { cudaGraphExecDestroy(h->ograph); h->ograph = nullptr; }
    const int rc = capture_loop_graph(h, setup, body, tail, &h->ograph, &h->ograph_fixed, &h->ograph_body);
    if (rc != TOPO_OK) {
      if (rc == TOPO_E_STATE) h->ograph_ok = false;
      return rc;
    }
    h->okey = key;
  }
  CK(cudaGraphLaunch(h->ograph, h->stream));
  count_launch((int)h->ograph_fixed);
  return TOPO_OK;
}

extern "C" {

int topo_oc_update(topo_handle* h, const topo_oc_opts* o, topo_oc_stats* stats) {
  DEVICE_SCOPE(h);
  if (!h || !o) return TOPO_E_BAD_INPUT;
  if (!h->spline_set) return fail(h, TOPO_E_STATE, "spline not set");
  const DevLevel& L = h->lv[0];
  const int64_t nc = (int64_t)h->sd.nb[0] * h->sd.nb[1] * h->sd.nb[2];
  const double den = (double)(o->reference_volume ? h->gs_padded_elements : h->active_elements);
  launch_maxabs(h->stream, h->csens, nc, h->partial, h->sc + S_TMP);
  count_launch(2);
  double gmax = 0.0;
  if (!(h->graphs && h->ograph_ok)) {  // the device-side bisection reads it in place
    RET(read_scalars(h, S_TMP, 1));
    gmax = h->hsc[S_TMP];
  }
  CK(cudaMemcpyAsync(h->coeff_old, h->coeff, sizeof(double) * nc, cudaMemcpyDeviceToDevice, h->stream));
  if (h->graphs && h->ograph_ok) {
    const int rc = oc_bisection_graphed(h, o, nc, den);
    if (rc == TOPO_OK) {
      RET(topo_coeff_to_density(h));
      if (h->iter_capture) {  // the density sum, read after the graph ran
        launch_sum(h->stream, h->rho, L.d.ne, h->partial, h->sc + S_DI + 1);
        count_launch(2);
        return TOPO_OK;
      }
      if (stats) {
        double v = 0;
        RET(topo_volume(h, o->reference_volume, &v));
        RET(read_scalars(h, S_OC, 6));
        count_launch((int)((long long)h->hsc[S_OC + 4] * h->ograph_body));
        stats->trials = (int)h->hsc[S_OC + 4];
        stats->lambda = h->hsc[S_OC + 2];
        stats->volume = v;
      }
      return TOPO_OK;
    }
    if (rc != TOPO_E_STATE || h->iter_capture) return rc;  // else the host loop below, from now on
  }
  double lo = 0.0, hi = gmax, thres = 0.5 * (lo + hi), V = 0.0;
  int itn = 0, trials = 0;
  do {
    thres = 0.5 * (lo + hi);
    launch_oc_trial(h->stream, nc, h->coeff_old, h->csens, thres, o->damp, o->step, o->cmin, o->cmax, h->coeff,
                    h->coeff_df);
    launch_trial_volume(h->stream, L.d, L.eactive, h->sd, h->coeff_df, h->cfg.min_density, h->partial,
                        h->sc + S_TMP, h->adj1);
    count_launch(4);
    CKL();
    RET(read_scalars(h, S_TMP, 1));
    V = h->hsc[S_TMP] / den;
    ++trials;
    if (V > o->vgoal) lo = thres;
    else if (V < o->vgoal) hi = thres;
  } while (std::fabs(V - o->vgoal) > 1e-4 && itn++ < 30);
  if (o->apply_twice) {
    launch_oc_trial(h->stream, nc, h->coeff, h->csens, thres, o->damp, o->step, o->cmin, o->cmax, h->coeff_tmp);
    CK(cudaMemcpyAsync(h->coeff, h->coeff_tmp, sizeof(double) * nc, cudaMemcpyDeviceToDevice, h->stream));
    count_launch();
  }
  RET(topo_coeff_to_density(h));
  if (stats) {
    stats->trials = trials;
    stats->lambda = thres;
    double v = 0;
    RET(topo_volume(h, o->reference_volume, &v));
    stats->volume = v;
  }
  return TOPO_OK;
}

static int gs_maps_impl(topo_handle* h, const LevelDims& d, const std::vector<uint8_t>& va,
                        const std::vector<uint8_t>& ea, int* vidmap, size_t nvid, int* eidmap,
                        size_t neid, int* gs_num8, int* n_gsvertices, int* n_gselements) {
  int64_t nvs[8] = {0}, nes[8] = {0}, nva = 0, nea = 0;
  for (int z = 0; z < d.vz; ++z)
    for (int y = 0; y < d.vy; ++y)
      for (int x = 0; x < d.vx; ++x)
        if (va[x + (int64_t)d.vx * (y + (int64_t)d.vy * z)] & 8) { nvs[(x & 1) + 2 * (y & 1) + 4 * (z & 1)]++; ++nva; }
  for (int z = 0; z < d.ez; ++z)
    for (int y = 0; y < d.ey; ++y)
      for (int x = 0; x < d.ex; ++x)
        if (ea[x + (int64_t)d.ex * (y + (int64_t)d.ey * z)]) { nes[(x & 1) + 2 * (y & 1) + 4 * (z & 1)]++; ++nea; }
  if ((vidmap && nvid != (size_t)nva) || (eidmap && neid != (size_t)nea))
    return fail(h, TOPO_E_BAD_INPUT, "gs map sizes: need %lld vertices, %lld elements", (long long)nva, (long long)nea);
  int64_t voff[8], eoff[8], vt = 0, et = 0;
  for (int c = 0; c < 8; ++c) {
    voff[c] = vt; eoff[c] = et;
    const int64_t pv = (nvs[c] + 31) / 32 * 32, pe = (nes[c] + 31) / 32 * 32;
    if (gs_num8) gs_num8[c] = (int)pv;
    vt += pv; et += pe;
  }
  int64_t cv[8] = {0}, ce[8] = {0}, k = 0;
  if (vidmap)
    for (int z = 0; z < d.vz; ++z)
      for (int y = 0; y < d.vy; ++y)
        for (int x = 0; x < d.vx; ++x)
          if (va[x + (int64_t)d.vx * (y + (int64_t)d.vy * z)] & 8) {
            const int c = (x & 1) + 2 * (y & 1) + 4 * (z & 1);
            vidmap[k++] = (int)(voff[c] + cv[c]++);
          }
  k = 0;
  if (eidmap)
    for (int z = 0; z < d.ez; ++z)
      for (int y = 0; y < d.ey; ++y)
        for (int x = 0; x < d.ex; ++x)
          if (ea[x + (int64_t)d.ex * (y + (int64_t)d.ey * z)]) {
            const int c = (x & 1) + 2 * (y & 1) + 4 * (z & 1);
            eidmap[k++] = (int)(eoff[c] + ce[c]++);
          }
  if (n_gsvertices) *n_gsvertices = (int)vt;
  if (n_gselements) *n_gselements = (int)et;
  return TOPO_OK;
}

int topo_gs_maps(topo_handle* h, int level, int* vidmap, size_t nvid, int* eidmap, size_t neid,
                 int* gs_num8, int* n_gsvertices, int* n_gselements) {
  DEVICE_SCOPE(h);
  if (!h || level < 0 || level >= (int)h->lv.size()) return TOPO_E_BAD_INPUT;
  return gs_maps_impl(h, h->lv[level].d, h->H.vactive[level], h->H.eactive[level], vidmap, nvid,
                      eidmap, neid, gs_num8, n_gsvertices, n_gselements);
}

int topo_plan_gs_maps(int nx, int ny, int nz, const uint8_t* eactive, int max_coarse, int level,
                      int* vidmap, size_t nvid, int* eidmap, size_t neid, int* gs_num8,
                      int* n_gsvertices, int* n_gselements) {
  if (nx < 1 || ny < 1 || nz < 1) return TOPO_E_BAD_INPUT;
  Hierarchy H = build_hierarchy(nx, ny, nz, eactive, max_coarse > 0 ? max_coarse : 400);
  if (level < 0 || level >= (int)H.dims.size()) return TOPO_E_BAD_INPUT;
  return gs_maps_impl(nullptr, H.dims[level], H.vactive[level], H.eactive[level], vidmap, nvid, eidmap,
                      neid, gs_num8, n_gsvertices, n_gselements);
}

int topo_element_template(double E, double nu, double h, double* Ke576) {
  if (!Ke576 || !(h > 0) || !(nu > -1.0 && nu < 0.5)) return TOPO_E_BAD_INPUT;
  element_template(E, nu, h, Ke576);
  return TOPO_OK;
}

int topo_plan_levels(int nx, int ny, int nz, const uint8_t* eactive, int max_coarse, int max_levels,
                     int* nlevels, int* dims, int* factors) {
  if (nx < 1 || ny < 1 || nz < 1 || !nlevels) return TOPO_E_BAD_INPUT;
  Hierarchy H = build_hierarchy(nx, ny, nz, eactive, max_coarse > 0 ? max_coarse : 400);
  *nlevels = (int)H.dims.size();
  for (int l = 0; l < (int)H.dims.size() && l < max_levels; ++l) {
    if (dims) { dims[3 * l] = H.dims[l].ex; dims[3 * l + 1] = H.dims[l].ey; dims[3 * l + 2] = H.dims[l].ez; }
    if (factors) factors[l] = H.dims[l].factor;
  }
  return TOPO_OK;
}

int topo_spline_axis(int order, int partition, double bmin, double bmax, int nelem, double h,
                     double* knots, int* i0, double* N) {
  if (order < 2 || order > 4 || partition < 0 || nelem < 1 || !(bmax > bmin) || !(h > 0)) return TOPO_E_BAD_INPUT;
  SplineTables t;
  int part3[3] = {partition, partition, partition};
  double a3[3] = {bmin, bmin, bmin}, b3[3] = {bmax, bmax, bmax};
  int ne3[3] = {nelem, 1, 1};
  spline_tables(order, part3, a3, b3, ne3, h, t);
  if (knots) std::copy(t.knots[0].begin(), t.knots[0].end(), knots);
  if (i0) std::copy(t.i0[0].begin(), t.i0[0].end(), i0);
  if (N) std::copy(t.N[0].begin(), t.N[0].end(), N);
  return TOPO_OK;
}

int topo_host_alloc(size_t bytes, void** ptr) {
  if (!ptr) return TOPO_E_BAD_INPUT;
  cudaError_t e = cudaHostAlloc(ptr, bytes, cudaHostAllocDefault);
  return e == cudaSuccess ? TOPO_OK : TOPO_E_NOMEM;
}

int topo_host_free(void* ptr) {
  return cudaFreeHost(ptr) == cudaSuccess ? TOPO_OK : TOPO_E_CUDA;
}

int topo_timer_start(topo_handle* h) {
  DEVICE_SCOPE(h);
  if (!h) return TOPO_E_BAD_INPUT;
  if (!h->timer_ev[0]) {
    CK(cudaEventCreate(&h->timer_ev[0]));
    CK(cudaEventCreate(&h->timer_ev[1]));
  }
  CK(cudaEventRecord(h->timer_ev[0], h->stream));
  return TOPO_OK;
}

int topo_timer_stop(topo_handle* h, double* ms) {
  DEVICE_SCOPE(h);
  if (!h || !ms || !h->timer_ev[0]) return TOPO_E_BAD_INPUT;
  CK(cudaEventRecord(h->timer_ev[1], h->stream));
  CK(cudaEventSynchronize(h->timer_ev[1]));
  float t = 0;
  CK(cudaEventElapsedTime(&t, h->timer_ev[0], h->timer_ev[1]));
  *ms = t;
  return TOPO_OK;
}

}  // extern "C"

namespace {

// Whether a design iteration with these options can run as one graph: the
// mixed solve with the Chebyshev multigrid and its device loops, on a handle
// that has run one design iteration already (side stream for the coarsest
// inversion, warm spectral-bound vectors, filter table of this radius).
bool iteration_graphable(const topo_handle* h, const topo_iter_opts* o) {
  const topo_solve_opts& so = o->solve;
  const bool vdots = so.post >= 1 && (so.cheb_degree > 0 ? so.cheb_degree : ChebParams{}.degree) >= 1;
  if (!(h->graphs && h->dgraph_ok && h->sgraph_ok && h->ograph_ok && !h->prof && h->nb == 1))
    return false;
  if (so.mode != TOPO_SOLVE_MIXED || so.smoother != TOPO_SMOOTH_CHEBYSHEV || so.learned != 0) return false;
  if (so.inner_max > 1 && !(h->igraph_ok && vdots)) return false;
  if (!h->side || !h->spline_set || !h->bc_set || h->lv.size() < 2) return false;
  if (h->filt_radius != (o->filter_radius > 0 ? o->filter_radius : 2.0)) return false;
  for (const DevLevel& L : h->lv)
    if (!L.eig32) return false;
  return true;
}

// Writes a design iteration's results from the slots read after its graph ran.
int iteration_graph_results(topo_handle* h, const topo_iter_opts* o, topo_iter_stats* st) {
  const topo_solve_opts& so = o->solve;
  // the coarsest inversion's status (copied to pinned memory inside the graph)
  const bool checked = h->coarse_unchecked;
  h->coarse_pending = false;
  h->coarse_unchecked = false;
  if (checked && h->hstat[1] != 0) {
    h->coarse_valid = false;
    return fail(h, TOPO_E_SINGULAR, "coarsest matrix indefinite at pivot %d", h->hstat[1] - 1);
  }
  h->coarse_dropped = h->hstat[0];
  for (size_t l = 0; l < h->lv.size(); ++l) {
    h->lv[l].lmax32 = h->hsc[S_LAM + S_MAXLEV + l];
    h->lv[l].lprev32 = h->hsc[S_LPREV + S_MAXLEV + l];
  }
  const bool inner = so.inner_max > 1;
  const long long outer_its = (long long)h->hsc[S_OLOOP];
  const long long inner_its = inner ? (long long)h->hsc[S_LOOP + 3] : 0;
  const long long trials = (long long)h->hsc[S_OC + 4];
  const long long restarts = (long long)h->hsc[S_DI + 2];
  count_launch((int)(outer_its * h->d_outer_body + inner_its * h->d_inner_body + trials * h->d_oc_body +
                     restarts * h->d_if_body));
  RET(tc_wait_status(h));
  if (inner && h->hsc[S_LOOP + 2] != 0.0)
    return fail(h, TOPO_E_NONFINITE, "inner CG residual became non-finite at iteration %d", (int)h->hsc[S_LOOP + 2] - 1);
  if (h->hsc[S_OLOOP + 2] != 0.0)
    return fail(h, TOPO_E_NONFINITE, "CG residual became non-finite at iteration %d", (int)h->hsc[S_OLOOP + 2] - 1);
  st->solve.iterations = (int)outer_its;
  st->solve.vcycles = inner ? (int)inner_its : (int)outer_its;
  st->solve.relres = std::sqrt(h->hsc[S_RR]) / h->iter_fn;
  float ms = 0;
  cudaEventElapsedTime(&ms, h->ev_solve[0], h->ev_solve[1]);
  st->solve.ms = ms;
  if (!std::isfinite(st->solve.relres)) return fail(h, TOPO_E_NONFINITE, "final residual is not finite");
  st->compliance = h->hsc[S_DI];
  if (!std::isfinite(st->compliance)) return fail(h, TOPO_E_NONFINITE, "compliance is not finite");
  st->oc_trials = (int)trials;
  st->volume = h->hsc[S_DI + 1] / (double)(o->oc.reference_volume ? h->gs_padded_elements : h->active_elements);
  if (st->solve.relres > so.rtol) {
    fail(h, TOPO_E_NOT_CONVERGED, "relative residual %.3e above %.3e after %d iterations", st->solve.relres,
         so.rtol, st->solve.iterations);
    return TOPO_E_NOT_CONVERGED;
  }
  return TOPO_OK;
}

// A design iteration as one CUDA graph after the operator update (whose
// coarsest inversion on the side stream the graph waits for before the first
// V-cycle): spectral bounds (a conditional node per level for the restart), the mixed
// solve (its outer CG a WHILE node with the inner CG nested in it), the final
// residual with the element energies, compliance, sensitivity, filter, spline
// adjoint, OC bisection (a WHILE node), density and its sum.  It is the host
// sequence of topo_design_iteration kernel for kernel, captured once per key
// (options, tiles, load vector) and replayed; the host reads the results once,
// after the launch (iteration_graph_finish).  A failure detected afterwards
// restores the coefficients and density the iteration started from, as the
// host sequence, which stops before the OC update, leaves them.  This part
// captures the graph when its key changed and launches it without waiting.
int iteration_graph_launch(topo_handle* h, const topo_iter_opts* o) {
  const topo_solve_opts& so = o->solve;
  const topo_oc_opts& oc = o->oc;
  std::vector<double> key = {(double)so.mode, (double)so.smoother, (double)so.pre, (double)so.post, so.rtol,
                             (double)so.max_iter, so.inner_rtol, (double)so.cheb_degree, so.cheb_lo, so.cheb_hi,
                             (double)so.inner_max, oc.vgoal, oc.damp, oc.step, oc.cmin, oc.cmax,
                             (double)oc.apply_twice, (double)oc.reference_volume, o->filter_radius,
                             (double)tz32_arg(h), (double)h->tz64, (double)h->fine_df, (double)h->op_precision,
                             (double)h->ref_fp32, (double)h->fgen, (double)h->sd.order};
  // buffers the captured kernels address (set_bc, set_spline or a multi-RHS
  // reservation may move some)
  for (int a = 0; a < 3; ++a)
    key.insert(key.end(), {(double)h->sd.nb[a], (double)(uintptr_t)h->sd.i0[a], (double)(uintptr_t)h->sd.Ndf[a]});
  for (const void* p : {(const void*)h->coeff, (const void*)h->coeff_old, (const void*)h->csens,
                        (const void*)h->coeff_df, (const void*)h->coeff_tmp, (const void*)h->adj1,
                        (const void*)h->rho, (const void*)h->rhop, (const void*)h->rhop32, (const void*)h->sens,
                        (const void*)h->sens_tmp, (const void*)h->gal_fixed, (const void*)h->A,
                        (const void*)h->A32, (const void*)h->x, (const void*)h->f, (const void*)h->x32})
    key.push_back((double)(uintptr_t)p);
  for (const DevLevel& L : h->lv)
    for (const void* p : {(const void*)L.U, (const void*)L.F, (const void*)L.R, (const void*)L.U32,
                          (const void*)L.F32, (const void*)L.R32, (const void*)L.eig32, (const void*)L.stencil32})
      key.push_back((double)(uintptr_t)p);
  DevLevel& L0 = h->lv[0];
  const int64_t n3 = 3 * L0.d.nv;
  // The operator update runs before the graph: its coarsest inversion is a
  // cooperative kernel on the side stream, which ran at half speed as a node
  // of the graph (20 against 9.5 ms at n = 1617); the graph waits for its
  // event before the first V-cycle, so it still overlaps the spectral bounds
  // and the first residual.
  for (int k = 0; k < 2; ++k)
    if (!h->ev_iter[k]) CK(cudaEventCreate(&h->ev_iter[k]));
  CK(cudaEventRecord(h->ev_iter[0], h->stream));
  h->defer_coarse = true;
  const int urc = topo_update_operators(h);
  h->defer_coarse = false;
  RET(urc);
  if (!h->dgraph || key != h->dkey) {
    if (h->dgraph) { cudaGraphExecDestroy(h->dgraph); h->dgraph = nullptr; }
    // ||F|| for the capture (the key holds the load vector's write count)
    launch_dot<double>(h->stream, L0.F, L0.F, n3, h->partial, h->sc + S_FF);
    count_launch(2);
    RET(read_scalars(h, S_FF, 1));
    h->iter_fn = std::sqrt(h->hsc[S_FF]);
    if (!(h->iter_fn > 0) || !std::isfinite(h->iter_fn)) return TOPO_E_STATE;
    for (int k = 0; k < 2; ++k)
      if (!h->ev_solve[k]) CK(cudaEventCreate(&h->ev_solve[k]));
    RET(ensure_cond_streams(h));
    const long long l0 = t_launches;
    cudaGraph_t g = nullptr;
    int rc = TOPO_OK;
    h->err.clear();
    bool ok = cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal) == cudaSuccess;
    if (ok) {
      h->in_capture = h->iter_capture = true;
      h->iter_waited = false;
      h->d_outer_body = h->d_inner_body = h->d_oc_body = h->d_if_body = 0;
      topo_solve_stats ss{};
      h->want_energy = true;
      rc = topo_solve(h, &so, &ss);
      h->want_energy = false;
      double c = 0;
      if (rc == TOPO_OK) rc = topo_compliance(h, &c);
      if (rc == TOPO_OK && h->energy_ready) {
        launch_sensitivity_from_energy(h->stream, L0.d.ne, L0.eactive, h->rho, h->cfg.power_penalty, h->sens);
        count_launch();
        if (h->ref_fp32) { launch_round_f32(h->stream, L0.d.ne, h->sens); count_launch(); }
        h->energy_ready = false;
      } else if (rc == TOPO_OK) {
        rc = TOPO_E_STATE;
      }
      if (rc == TOPO_OK) rc = topo_filter(h, o->filter_radius > 0 ? o->filter_radius : 2.0);
      if (rc == TOPO_OK) rc = topo_spline_adjoint(h);
      topo_oc_stats ocs{};
      if (rc == TOPO_OK) rc = topo_oc_update(h, &oc, &ocs);
      h->in_capture = h->iter_capture = false;
      ok = cudaStreamEndCapture(h->stream, &g) == cudaSuccess && g && rc == TOPO_OK;
    }
    const long long total = t_launches - l0;
    g_launches.fetch_sub(total);
    t_launches = l0;
    if (ok) ok = cudaGraphInstantiate(&h->dgraph, g, 0) == cudaSuccess;
    if (g) cudaGraphDestroy(g);
    if (!ok) {  // the host sequence from now on
      const cudaError_t ce = cudaGetLastError();
      const std::string why = h->err;
      fail(h, TOPO_E_STATE, "design iteration not captured as a graph (status %d, %s; %s): host sequence", rc,
           cudaGetErrorString(ce), why.c_str());
      h->dgraph = nullptr;
      h->dgraph_ok = false;
      // (the capture set host state as if it had run: the operator update
      // launched above stands, its inversion not yet joined; bounds stale)
      h->ops_ready = true;
      h->coarse_pending = h->coarse_unchecked = true;
      for (auto& l : h->lv) { l.lmax = 0; l.lmax32 = 0; }
      return TOPO_E_STATE;
    }
    h->dgraph_fixed = total - (h->d_outer_body + h->d_inner_body + h->d_oc_body) -
                      (long long)h->lv.size() * h->d_if_body;
    h->dkey = key;
  }
  CK(cudaGraphLaunch(h->dgraph, h->stream));
  count_launch((int)h->dgraph_fixed);
  CK(cudaEventRecord(h->ev_iter[1], h->stream));
  CK(cudaMemcpyAsync(h->hsc, h->sc, sizeof(double) * S_COUNT, cudaMemcpyDeviceToHost, h->stream));
  return TOPO_OK;
}

// Waits for a design iteration launched by iteration_graph_launch and writes
// its results.
int iteration_graph_finish(topo_handle* h, const topo_iter_opts* o, topo_iter_stats* st) {
  CK(cudaStreamSynchronize(h->stream));
  float ms = 0;
  cudaEventElapsedTime(&ms, h->ev_iter[0], h->ev_iter[1]);
  st->ms = ms;
  const int rc = iteration_graph_results(h, o, st);
  if (rc != TOPO_OK && rc != TOPO_E_NOT_CONVERGED) {
    // the graph ran the OC update on a failed solve: back to the start design
    const int64_t nc = (int64_t)h->sd.nb[0] * h->sd.nb[1] * h->sd.nb[2];
    CK(cudaMemcpyAsync(h->coeff, h->coeff_old, sizeof(double) * nc, cudaMemcpyDeviceToDevice, h->stream));
    RET(topo_coeff_to_density(h));
    CK(cudaStreamSynchronize(h->stream));
  }
  return rc;
}

int design_iteration_graphed(topo_handle* h, const topo_iter_opts* o, topo_iter_stats* st) {
  RET(iteration_graph_launch(h, o));
  return iteration_graph_finish(h, o, st);
}

}  // namespace

extern "C" {

int topo_design_iteration(topo_handle* h, const topo_iter_opts* o, topo_iter_stats* stats) {
  DEVICE_SCOPE(h);
  if (!h || !o) return TOPO_E_BAD_INPUT;
  if (iteration_graphable(h, o)) {
    topo_iter_stats st{};
    const int rc = design_iteration_graphed(h, o, &st);
    if (rc != TOPO_E_STATE) {
      if (stats) *stats = st;
      return rc;
    }
  }
  ScopedEvent e0, e1;
  CK(e0.create());
  CK(e1.create());
  CK(cudaEventRecord(e0, h->stream));
  topo_iter_stats st{};
  h->defer_coarse = true;  // the coarsest inversion overlaps the solve's set-up
  const int urc = topo_update_operators(h);
  h->defer_coarse = false;
  RET(urc);
  h->want_energy = true;
  int rc = topo_solve(h, &o->solve, &st.solve);
  h->want_energy = false;
  if (rc != TOPO_OK && rc != TOPO_E_NOT_CONVERGED) return rc;
  RET(topo_compliance(h, &st.compliance));
  if (!std::isfinite(st.compliance)) return fail(h, TOPO_E_NONFINITE, "compliance is not finite");
  if (h->energy_ready) {  // u is the solve's final iterate, rho unchanged since
    const DevLevel& L = h->lv[0];
    launch_sensitivity_from_energy(h->stream, L.d.ne, L.eactive, h->rho, h->cfg.power_penalty, h->sens);
    count_launch();
    if (h->ref_fp32) { launch_round_f32(h->stream, L.d.ne, h->sens); count_launch(); }
    h->energy_ready = false;
  } else {
    RET(topo_sensitivity(h));
  }
  RET(topo_filter(h, o->filter_radius > 0 ? o->filter_radius : 2.0));
  RET(topo_spline_adjoint(h));
  topo_oc_stats oc{};
  RET(topo_oc_update(h, &o->oc, &oc));
  st.oc_trials = oc.trials;
  st.volume = oc.volume;
  CK(cudaEventRecord(e1, h->stream));
  CK(cudaEventSynchronize(e1));
  float ms = 0;
  cudaEventElapsedTime(&ms, e0, e1);
  st.ms = ms;
  if (stats) *stats = st;
  return rc;
}

int topo_profile_enable(topo_handle* h, int enable) {
  DEVICE_SCOPE(h);
  if (!h) return TOPO_E_BAD_INPUT;
  h->prof = enable != 0;
  for (int f = 0; f < TOPO_K_COUNT; ++f) { h->gprof_ms[f] = 0; h->gprof_n[f] = 0; }
  return TOPO_OK;
}

int topo_profile_read(topo_handle* h, int family, int* launches, double* ms) {
  DEVICE_SCOPE(h);
  if (!h || family < 0 || family >= TOPO_K_COUNT) return TOPO_E_BAD_INPUT;
  CK(cudaStreamSynchronize(h->stream));
  prof_collect(h);
  double tot = h->gprof_ms[family];
  const int ng = h->gprof_n[family];
  h->gprof_ms[family] = 0;
  h->gprof_n[family] = 0;
  for (auto& p : h->evs[family]) {
    float t = 0;
    cudaEventElapsedTime(&t, p.a, p.b);
    tot += t;
    h->evpool.push_back(p);
  }
  if (launches) *launches = (int)h->evs[family].size() + ng;
  if (ms) *ms = tot;
  h->evs[family].clear();
  return TOPO_OK;
}

int topo_launch_count(const topo_handle* h, long long* n) {
  DEVICE_SCOPE(h);
  (void)h;
  if (!n) return TOPO_E_BAD_INPUT;
  *n = g_launches.load();
  return TOPO_OK;
}

}  // extern "C"
