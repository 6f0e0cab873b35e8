// The handle: everything one topology-optimisation problem owns on its GPU.
// Shared by the translation units that implement the C ABI (capi.cu and the
// entry points split out of it).
#pragma once

#include <string>
#include <utility>
#include <vector>

#include "topo_internal.h"

namespace topo {

// Nesting depth of conditional graph nodes in a captured design iteration
// (outer CG > inner CG > V-cycle; power-iteration restarts; OC bisection).
constexpr int TOPO_COND_DEPTH = 3;

// Scalar slots in device memory used by the PCG drivers.
// Slots 0-7 belong to one CG level; a nested CG uses base 8 (slots 8-15).
enum Slot {
  S_RZ = 0, S_ZROLD = 1, S_RZOLD = 2, S_DQ = 3, S_RR = 4, S_FF = 5, S_ALPHA = 6, S_BETA = 7,
  S_TMP = 16, S_PW = 24, S_MAXLEV = 16,
  // device-controlled inner CG loop: iterations of the current inner solve,
  // its ||b|| reference, the first iteration whose r.r was non-finite
  // (1-based, 0 = none), inner iterations summed over the solve
  S_LOOP = S_PW + 2 * S_MAXLEV,
  // device-side OC bisection: lo, hi, the current trial's threshold, its
  // volume fraction, trials, repeats (the reference loop's itn)
  S_OC = S_LOOP + 4,
  // device-controlled outer CG loop of the mixed solve (the same four slots
  // as S_LOOP)
  S_OLOOP = S_OC + 6,
  // spectral bounds per precision table (FP64 first) and level: the current
  // estimate of lambda_max(D^-1 A) and the previous one (warm-start guard)
  S_LAM = S_OLOOP + 4, S_LPREV = S_LAM + 2 * S_MAXLEV,
  // results of a graphed design iteration: compliance F.U, the density sum
  // after the OC update, levels whose power iteration restarted
  S_DI = S_LPREV + 2 * S_MAXLEV, S_COUNT = S_DI + 3
};

// Chebyshev step coefficients (c_old, c_new) in device memory: per precision
// (FP64 first), level and step, then the pair (0, 1).
constexpr int CHEB_MAX_DEG = 32;
constexpr int CHEB_TABLE = 2 * (2 * S_MAXLEV * CHEB_MAX_DEG + 1);

struct EventPair {
  cudaEvent_t a, b;
};

}  // namespace topo

struct topo_handle {
  topo_config cfg{};
  topo::UNetState* unet = nullptr;  // learned preconditioner (topo_unet_enable)
  bool mat_registered = false;      // holds a reference on the device's element constants
  int nb = 1;                       // right-hand sides the level vectors hold (multi-RHS solve)
  int fine_df = 1;                  // FP64 fine operator in double-float arithmetic (topo_set_fine_arithmetic)
  int tz32 = 16, tz64 = 16;         // z-march depth of the fine kernels, FP32 / FP64 (topo_autotune)
  bool fine_tc = false;             // FP32 fine element products on the tensor cores (topo_set_fine_tensor_cores)
  // the coarsest inverse is recomputed at every coarse_every-th operator
  // update (topo_set_coarse_refresh); coarse_age counts the updates since,
  // coarse_valid says whether the held inverse belongs to this hierarchy
  int coarse_every = 1;
  int coarse_age = 0;
  bool coarse_valid = false;
  int rows32 = 8;                   // element rows of the FP32 modal kernel's CTA tile: 4, 8, 16 (topo_set_fine_tile_rows)
  // FP32 V-cycle replayed as one CUDA graph (topo_set_graphs); re-captured when its key changes
  bool graphs = true;
  cudaGraphExec_t vgraph = nullptr;
  std::vector<double> vkey;
  long long vgraph_kernels = 0;
  // inner FP32 CG of the mixed solve as one graph with a device-side WHILE
  // loop (igraph); kernels of its fixed part and of one loop iteration
  bool in_capture = false;
  bool igraph_ok = true;
  cudaGraphExec_t igraph = nullptr;
  std::vector<double> ikey;
  long long igraph_fixed = 0, igraph_body = 0;
  // the mixed solve's outer CG as one graph with a device-side WHILE loop
  // (sgraph), the inner CG nested in it as a second WHILE loop; kernels of its
  // fixed part, of one outer iteration (without the inner loop's body) and of
  // one inner iteration
  bool sgraph_ok = true;
  cudaGraphExec_t sgraph = nullptr;
  std::vector<double> skey;
  long long sgraph_fixed = 0, sgraph_body = 0, sgraph_inner = 0;
  // a whole design iteration as one graph (dgraph, topo_design_iteration),
  // captured with iter_capture set: the functions it calls then leave their
  // results in device slots and emit their loops as conditional nodes.
  // Kernels of its fixed part and of one pass of each conditional body.
  bool iter_capture = false;
  bool iter_waited = false;           // the capture holds its wait for the coarsest inversion
  // helper streams that capture the bodies of nested conditional nodes
  cudaStream_t cstream[topo::TOPO_COND_DEPTH] = {};
  int cdepth = 0;
  bool dgraph_ok = true;
  cudaGraphExec_t dgraph = nullptr;
  std::vector<double> dkey;
  long long dgraph_fixed = 0, d_outer_body = 0, d_inner_body = 0, d_oc_body = 0, d_if_body = 0;
  double iter_fn = 0;                 // ||F|| when the design-iteration graph was captured
  unsigned long long fgen = 0;        // writes of the level-0 load vector (topo_set_bc, topo_put_array)
  cudaEvent_t ev_solve[2] = {nullptr, nullptr};  // recorded inside it around the solve
  cudaEvent_t ev_iter[2] = {nullptr, nullptr};   // around its launch
  // OC bisection as one graph with a device-side WHILE loop (ograph)
  bool ograph_ok = true;
  cudaGraphExec_t ograph = nullptr;
  std::vector<double> okey;
  long long ograph_fixed = 0, ograph_body = 0;
  // coarsest inversion of a design iteration on a second stream (side),
  // overlapped with the solve's set-up; the main stream waits for ev_coarse
  // before its first V-cycle (coarse_join) and the status is read at the end
  // of the solve (coarse_finish)
  cudaStream_t side = nullptr;
  cudaEvent_t ev_ops = nullptr, ev_coarse = nullptr;
  int* hstat = nullptr;           // pinned copy of the inversion status
  bool defer_coarse = false;      // topo_design_iteration's operator update
  bool coarse_pending = false;    // the main stream has not waited for it yet
  bool coarse_unchecked = false;  // its status has not been read yet
  // profiling inside the graph: event pairs captured as external event-record
  // nodes, collected after each replay has completed
  bool capturing = false;
  std::vector<std::pair<int, topo::EventPair>> gprof;
  bool gprof_pending = false;
  double gprof_ms[TOPO_K_COUNT] = {0};
  int gprof_n[TOPO_K_COUNT] = {0};
  topo::MultiRhs* multi = nullptr;  // batched buffers (topo_multi_reserve)
  topo::WorstState* worst = nullptr;  // load region and block buffers (topo_set_load_region)
  topo::SupportState* support = nullptr;  // surface points and constraint gradients (topo_support_constraints)
  // Heaviside projection: rho = H(rho_init) after topo_heaviside_project
  double* rho_init = nullptr;
  double* vsens = nullptr;          // projected volume sensitivity before its adjoint
  bool rho_projected = false;
  int unet_crops = 64;              // crops per harvested iterate
  cudaStream_t stream = nullptr;
  std::string err;
  topo::Hierarchy H;
  std::vector<topo::DevLevel> lv;
  double Ke[576];
  double lam = 0, mu = 0;
  std::vector<void*> allocs;
  // element template and Galerkin tables
  double* dKe = nullptr;
  double* dT64 = nullptr;
  float* dT32 = nullptr;
  // level-0 design arrays
  double *rho = nullptr, *rhop = nullptr, *sens = nullptr, *sens_tmp = nullptr;
  float* rhop32 = nullptr;
  bool rhop_stale = false;
  // spline
  bool spline_set = false;
  topo::SplineTables st;
  topo::SplineDev sd{};
  double *coeff = nullptr, *csens = nullptr, *coeff_old = nullptr, *coeff_tmp = nullptr;
  float2* coeff_df = nullptr;  // OC trial coefficients split into (hi, lo) floats
  double* volcsens = nullptr;  // scale * d volume / d coefficient (topo_volume_csens)
  double *adj1 = nullptr, *adj2 = nullptr;
  // level-0 work vectors
  double *work = nullptr, *x = nullptr, *r = nullptr, *d = nullptr, *q = nullptr, *rold = nullptr,
         *f = nullptr;
  float *x32 = nullptr, *r32 = nullptr, *d32 = nullptr, *q32 = nullptr, *rold32 = nullptr;
  // coarsest level
  int ndense = 0;
  double* A = nullptr;
  float* A32 = nullptr;
  double* gjwork = nullptr;  // panels of the blocked Gauss-Jordan inversion
  double* coarse64tmp = nullptr;  // FP64 copy of an FP32 coarsest stencil
  int* status = nullptr;
  // first coarse level: elements whose fine elements touch fixed DOFs
  int* gal_fixed = nullptr;
  int n_gal_fixed = 0;
  int coarse_dropped = 0;  // null directions dropped by the coarsest inverse
  cudaEvent_t timer_ev[2] = {nullptr, nullptr};
  // sensitivity filter ball (offsets and weights) for the last radius used
  double filt_radius = -1.0;
  int4* filt_offs = nullptr;
  double* filt_w = nullptr;
  float2* filt_wdf = nullptr;  // the weights split into (hi, lo) floats
  int filt_n = 0;
  // reductions
  double* partial = nullptr;
  double* fdot = nullptr;  // per-CTA partials of the fine operator's fused dot
  int fdot_cap = 0;
  // ticket counter of the reductions whose last block writes the total (the
  // handle's stream runs them one at a time; the last block resets it)
  unsigned* ctr = nullptr;
  // inner CG: the FP32 V-cycle's last Chebyshev step also forms r.z (partials
  // in vdot) when vdot_on; the sum lands in *vdot_out
  double* vdot = nullptr;
  bool vdot_on = false;
  double* vdot_out = nullptr;
  bool inner_fr = false;  // inner CG in Fletcher-Reeves form (z.rold taken as 0)
  double* chebc = nullptr;          // Chebyshev coefficient table (device)
  double* sc = nullptr;    // device scalar slots
  double* hsc = nullptr;   // pinned host mirror
  int64_t active_elements = 0, gs_padded_elements = 0;
  bool bc_set = false, ops_ready = false;
  // design iteration: the solve's final residual also writes element energies
  // into sens (want_energy), and says so (energy_ready)
  bool want_energy = false, energy_ready = false;
  int op_precision = 3;    // bit0 FP64 operators, bit1 FP32 operators
  bool ref_fp32 = false;   // reference precision: rho, coefficients, sensitivities kept in FP32, rho^p by powf
  bool ops64 = false, ops32 = false;
  // profiling
  bool prof = false;
  std::vector<topo::EventPair> evs[TOPO_K_COUNT];
  std::vector<topo::EventPair> evpool;
};
