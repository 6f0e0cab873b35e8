/*
 * topo_gb300.h -- C ABI of the GB300-native topology-optimisation hot path.
 *
 * One handle owns one design problem on one GPU: the voxel grid and its
 * multigrid hierarchy, boundary conditions, the B-spline design field, the
 * solver state and every device buffer.  All calls return a TOPO_* status and
 * never exit the process; topo_last_error() gives the message.  Arrays cross
 * the boundary as plain host pointers with explicit element counts.
 *
 * Layout shared by every array (dense grid, lexicographic, x fastest):
 *   element e = ex + nx*(ey + ny*ez);  vertex v = x + (nx+1)*(y + (ny+1)*z)
 *   vertex vectors are SoA [3][nv]; element matrices [ne][24*24] with local node
 *   a = ax + 2ay + 4az and DOF 3a+c; coarse stencils [27][9][nv] with neighbour
 *   d = (dx+1) + 3(dy+1) + 9(dz+1) and a row-major 3x3 block.
 * topo_gs_maps() converts to the reference's GS-coloured ordering.
 *
 * Each entry point names the reference interface it replaces
 * (NanXYZH/TopOptSpline3D, file:line).
 */
#ifndef TOPO_GB300_H
#define TOPO_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum topo_status {
  TOPO_OK = 0,
  TOPO_E_CUDA = 1,          /* a CUDA runtime call failed */
  TOPO_E_BAD_INPUT = 2,     /* invalid argument (sizes, pointers, ranges) */
  TOPO_E_STATE = 3,         /* call order violated (e.g. solve before set_bc) */
  TOPO_E_NOT_CONVERGED = 4, /* solver hit its iteration cap above tolerance */
  TOPO_E_SINGULAR = 5,      /* coarsest-level factorisation met a non-positive pivot */
  TOPO_E_NOMEM = 6,         /* device allocation failed */
  TOPO_E_NONFINITE = 7,     /* NaN/Inf detected in a result */
  TOPO_E_TIMEOUT = 8        /* a kernel's bounded device-side wait gave up (its work was skipped) */
};

/* Array ids for topo_put_array / topo_get_array / topo_device_ptr. */
enum topo_array {
  TOPO_RHO = 0,      /* double[ne]   element density */
  TOPO_RHOP = 1,     /* double[ne]   rho^p */
  TOPO_COEFF = 2,    /* double[nc]   spline coefficients, x fastest */
  TOPO_SENS = 3,     /* double[ne]   d compliance / d rho (filtered in place) */
  TOPO_CSENS = 4,    /* double[nc]   d compliance / d coefficient */
  TOPO_U = 5,        /* double[3*nv] displacement (per level) */
  TOPO_F = 6,        /* double[3*nv] force / right-hand side (per level) */
  TOPO_R = 7,        /* double[3*nv] residual (per level) */
  TOPO_STENCIL = 8,  /* double[243*nv] coarse-level stencil (level >= 1) */
  TOPO_KELEM = 9,    /* double[576*ne] coarse element matrices (level >= 1) */
  TOPO_VMASK = 10,   /* uint8[nv]    bits 0-2 DOF free, bit 3 vertex active */
  TOPO_EACTIVE = 11, /* uint8[ne]    element active mask (per level) */
  TOPO_KE = 12,      /* double[576]  element template */
  TOPO_WORK = 13,    /* double[3*nv] scratch vector (level 0): input of topo_apply_fine */
  TOPO_VOLCSENS = 14, /* double[nc]  scaled d volume / d coefficient (topo_volume_csens) */
  TOPO_MULTI_F = 15,  /* double[cap*3*nv] right-hand sides of topo_solve_multi (after topo_multi_reserve) */
  TOPO_MULTI_U = 16,  /* double[cap*3*nv] solutions / initial guesses of topo_solve_multi */
  TOPO_SSCSENS = 17,  /* double[nc]  d self-support constraint / d coefficient (topo_support_constraints) */
  TOPO_DRIPCSENS = 18, /* double[nc] d drip constraint / d coefficient */
  TOPO_RHO_INIT = 19, /* double[ne]  density before the Heaviside projection (topo_heaviside_project) */
  TOPO_SURF_POINTS = 20,  /* double[3*npts] surface points of the last topo_support_constraints, SoA xyz */
  TOPO_SURF_NORMALS = 21  /* double[3*npts] their spline gradients (the constraint's normals) */
};

typedef struct topo_config {
  int nx, ny, nz;               /* element grid (domain bounding box) */
  double h;                     /* element edge length */
  double youngs_modulus;        /* E   (reference flag youngs_modulus, default 1e6) */
  double poisson_ratio;         /* nu  (reference flag poisson_ratio, default 0.4) */
  double power_penalty;         /* SIMP p (default 3) */
  double min_density;           /* rho_min (default 1e-3) */
  int max_coarse_elements;      /* coarsen while active elements exceed this (reference: 400) */
  int device;                   /* CUDA device ordinal */
} topo_config;

typedef struct topo_handle topo_handle;

/* Solver modes for topo_solve. */
enum topo_solve_mode {
  TOPO_SOLVE_VCYCLE = 0,  /* reference: repeated V-cycles (utils/test_utils.cpp:937-941) */
  TOPO_SOLVE_PCG64 = 1,   /* FP64 MG-PCG, symmetric V-cycle preconditioner */
  TOPO_SOLVE_MIXED = 2    /* FP64 flexible CG preconditioned by FP32 multigrid */
};

enum topo_smoother {
  TOPO_SMOOTH_GS = 0,        /* 8-colour point-block Gauss-Seidel (reference) */
  TOPO_SMOOTH_CHEBYSHEV = 1  /* point-block-Jacobi Chebyshev */
};

typedef struct topo_solve_opts {
  int mode;           /* topo_solve_mode */
  int smoother;       /* topo_smoother */
  int pre, post;      /* smoothing steps per level */
  double rtol;        /* relative residual target ||f - K u|| / ||f|| (FP64) */
  int max_iter;       /* V-cycles (mode 0) or outer CG iterations (modes 1, 2) */
  double inner_rtol;  /* mode 2: relative reduction of each inner FP32 solve */
  int cheb_degree;    /* Chebyshev polynomial degree per smoothing step */
  double cheb_lo, cheb_hi; /* Chebyshev interval [lo*lmax, hi*lmax] */
  int inner_max;      /* mode 2: FP32 iterations per preconditioner application (1 = one V-cycle) */
  int learned;        /* mode 2: 0 off, 1 add the U-Net correction to every FP32 V-cycle
                         (topo_unet_enable first), 2 harvest training crops (needs inner_max <= 1) */
  double learned_stall; /* mode 2, learned = 1: drop the network for the rest of the solve after 10
                           outer steps in a row that do not bring the best residual below
                           learned_stall times itself (0 = 0.99), or as soon as a corrected
                           preconditioner output fails r.z > 0 (that step keeps the plain V-cycle) */
} topo_solve_opts;

typedef struct topo_solve_stats {
  int iterations;     /* V-cycles (mode 0) or outer CG iterations = FP64 fine matvecs (modes 1, 2) */
  int vcycles;        /* V-cycles applied (FP32 ones in mode 2) */
  double relres;      /* final FP64 relative residual */
  double ms;          /* device time of the solve */
  int learned_applied;  /* U-Net corrections applied */
  int learned_fallback; /* 1 if the stall rule switched back to the plain V-cycle */
} topo_solve_stats;

typedef struct topo_oc_opts {
  double vgoal;       /* target volume ratio */
  double damp;        /* OC exponent (reference damp_ratio 0.5) */
  double step;        /* move limit (reference design_step 0.03) */
  double cmin, cmax;  /* coefficient bounds (reference min_coeff 0, max_coeff 1) */
  int apply_twice;    /* reproduce the reference's double application of the final step */
  int reference_volume; /* volume denominator with the reference's GS padding */
} topo_oc_opts;

typedef struct topo_oc_stats {
  int trials;
  double lambda;
  double volume;
} topo_oc_stats;

/* --- lifetime ------------------------------------------------------------ */
/* Replaces HierarchyGrid::genFromMesh(const std::vector<unsigned>&, int[3]) (grid/Grid.cpp:977)
 * plus setParameters (optimization/optimization.cpp:35-65) and buildGrids (15-22).
 * eactive: uint8[nx*ny*nz] or NULL (all active).  The element constants are per device:
 * TOPO_E_BAD_INPUT if another live handle on the device has a different E, nu or h. */
int topo_create(const topo_config* cfg, const uint8_t* eactive, topo_handle** out);
/* Replaces HierarchyGrid::~HierarchyGrid (grid/Grid.h:1027-1033) and gpu_manager_t teardown. */
void topo_destroy(topo_handle* h);
/* Replaces the printf-only cuda_error_check (culib/cudaCommon.cuh:6-11). */
const char* topo_last_error(const topo_handle* h);
/* Replaces HierarchyGrid::n_grid (grid/Grid.h:1017) and Grid::_layer / elementLength. */
int topo_num_levels(const topo_handle* h, int* nlevels);
int topo_level_dims(const topo_handle* h, int level, int* dims3, int* factor);
/* Waits for all work queued on the handle's stream. */
int topo_sync(topo_handle* h);

/* --- set-up -------------------------------------------------------------- */
/* Replaces setBoundaryCondition + setForceSupport(getPreloadForce(), F)
 * (optimization/optimization.cpp:1023-1028, optimization/projection.cu:344-368).
 * fixed: uint8[nv], bit c set = DOF c fixed; loads: double[3*nv]. */
int topo_set_bc(topo_handle* h, const uint8_t* fixed, const double* loads);
/* Replaces HierarchyGrid::set_spline_partition (grid/Grid.cu:3134-3203) and
 * Grid::set_spline_knot_series / set_spline_knot_infoSymbol (grid/Grid.cpp:3253-3377,
 * grid/Grid.cu:3205-3216).  bmin/bmax: spline box before the 2*delta/(p+1) enlargement. */
int topo_set_spline(topo_handle* h, int order, const int* partition3, const double* bmin3,
                    const double* bmax3);
int topo_num_coeffs(const topo_handle* h, int* ncoeff);

/* Boundary conditions from region predicates: the reference's JSON "fixedarea",
 * "loadarea" and "force" sections (config_parser.cpp:389-455,
 * boundary/BoundaryCondition.h) evaluated on the surface vertices of the active
 * domain as Grid::computeProjectionMatrix does (grid/Grid.cpp:2660-2726): a
 * surface vertex in the fixed union has all three DOFs fixed; otherwise, in the
 * load union, its nodal force is the sum of the force fields whose region holds it. */
enum topo_region_type {
  TOPO_REGION_BOX = 0,        /* corners a, b */
  TOPO_REGION_SPHERE = 1,     /* center a, radius r */
  TOPO_REGION_HALFSPACE = 2,  /* plane through a, b, c; positive side of (b-a) x (c-a) */
  TOPO_REGION_CYLINDER = 3    /* bottom center a, height vector b, radius r */
};
typedef struct topo_region {
  int type;                   /* topo_region_type */
  int closed;                 /* include the boundary */
  int complement;             /* negate */
  double a[3], b[3], c[3];
  double r;
} topo_region;
enum topo_field_type {
  TOPO_FIELD_CONST = 0,                  /* norm * direction */
  TOPO_FIELD_RADIAL_NORM_CONST_DIR = 1,  /* amplifier*exp(-|center-p|^(2 damp)) * direction */
  TOPO_FIELD_CONST_NORM_RADIAL_DIR = 2,  /* norm * unit(center - p) */
  TOPO_FIELD_RADIAL_NORM_RADIAL_DIR = 3, /* amplifier*exp(-|center-p|^(2 damp)) * unit(center2 - p) */
  TOPO_FIELD_TWIST = 4                   /* axis center -> center2, amplifier */
};
typedef struct topo_force_field {
  int type;                   /* topo_field_type */
  topo_region region;         /* where the field acts */
  double norm, amplifier, damp_ratio;
  double direction[3], center[3], center2[3];
} topo_force_field;
typedef struct topo_bc_regions {
  double origin[3];           /* position of vertex (0,0,0) */
  double spacing;             /* vertex spacing */
  const topo_region* fixed; int nfixed;        /* "fixedarea" union */
  const topo_region* load; int nload;          /* "loadarea" union */
  const topo_force_field* force; int nforce;   /* "force" fields (summed) */
} topo_bc_regions;
/* Computes the per-DOF fixed mask and loads and applies them as topo_set_bc does;
 * nfixed / nloaded (may be NULL) receive the support and load vertex counts. */
int topo_set_bc_regions(topo_handle* h, const topo_bc_regions* spec, int* nfixed, int* nloaded);
int topo_get_knots(const topo_handle* h, int axis, double* out, size_t count);

/* --- arrays -------------------------------------------------------------- */
/* Replace Grid::getRho/getCoeff/getSens/getCSens/getForce/getDisplacement
 * (grid/Grid.h:420-450), init_coefflist/init_rholist, and the *2matlab dumps. */
int topo_array_size(const topo_handle* h, int which, int level, size_t* count);
int topo_put_array(topo_handle* h, int which, int level, const void* src, size_t count);
int topo_get_array(topo_handle* h, int which, int level, void* dst, size_t count);
/* Borrowed device pointer, valid until topo_destroy. */
int topo_device_ptr(topo_handle* h, int which, int level, void** dptr);

/* --- hot path ------------------------------------------------------------ */
/* Replaces Grid::coeff2density (grid/Grid.cu:3361-3456): rho = clamp(spline(coeff)). */
int topo_coeff_to_density(topo_handle* h);
/* Which coarse operators topo_update_operators builds: bit 0 FP64 (V-cycle and FP64
 * PCG modes), bit 1 FP32 (mixed mode).  Default 3.  The reference builds FP64 only
 * (grid/Grid.cu:839-1265). */
int topo_set_operator_precision(topo_handle* h, int mask);
/* Reference precision (enable = 1; default 0): the arrays the reference stores
 * in FP32 are kept at FP32 values, and rho^p is taken with powf in FP32
 * (grid/Grid.cu:1739).  Coefficients are rounded to FP32 before each density
 * evaluation (so also after every OC update), rho after it; sensitivities after
 * the element sensitivity and after the filter, coefficient sensitivities after
 * the spline adjoint.  The solve stays as configured.  It quantifies how far
 * the FP64 path's design trajectory lies from the reference's FP32 storage. */
int topo_set_reference_precision(topo_handle* h, int enable);
/* Replaces HierarchyGrid::update_stencil (grid/Grid.cpp:4167-4178): rho^p, Galerkin
 * coarse operators (grid/Grid.cu:839-1265) and the coarsest factorisation
 * (grid/Grid.cpp:3614-3669). */
int topo_update_operators(topo_handle* h);
/* Replaces Grid::applyK (grid/Grid.cu:4278-4356): TOPO_R(level 0) <- K(rho) TOPO_WORK,
 * fixed rows zero.  precision: 0 = FP64 modal kernel, 1 = FP32 kernel, 2 = FP64 dense-row
 * kernel, 3 = FP64 vectors with the double-float modal kernel. */
int topo_apply_fine(topo_handle* h, int precision);
/* Coarse-level operator, the assembled 27-point block stencil of the residual
 * update on coarse levels (grid/Grid.cu:2126-2224): TOPO_R(level) <-
 * A_level TOPO_U(level) for level >= 1 with the FP64 (precision 0) or FP32
 * (precision 1; U rounded to FP32, the result widened) operators, which
 * topo_set_operator_precision must have built. */
int topo_apply_level(topo_handle* h, int level, int precision);
/* Arithmetic of the FP64 fine operator used by the solvers (residuals and the
 * outer CG matvec): 0 = native FP64, 1 = double-float (pairs of floats with
 * error-free transformations, ~48-bit significands, on the FP32 pipe; default).
 * Vectors, dot products and step lengths stay FP64 either way. */
int topo_set_fine_arithmetic(topo_handle* h, int arith);
/* Element products of the FP32 fine kernels (the multigrid smoother, residual
 * and operator on level 0, the preconditioner's side of the mixed solve): 0 =
 * the modal form on the FP32 pipe, 1 = on the tensor cores (tcgen05.mma in
 * three-term TF32, u_hi K_hi + u_hi K_lo + u_lo K_hi with fp32 accumulators in
 * tensor memory: FP32-level accuracy).  Levels with void planes keep the modal
 * form.  Grid::gs_relax / update_residual on the finest level
 * (grid/Grid.cu:1698-1842, 2277-2333) have no tensor-core counterpart. */
int topo_set_fine_tensor_cores(topo_handle* h, int on);
/* Element rows (4, 8 or 16) of the CTA tile (32 element columns by that many
 * rows, marched in z) of the FP32 modal fine kernels on levels without void
 * planes; each vertex's sum is formed the same way in every tile height, so
 * the outputs are identical.  The autotuner times the three heights. */
int topo_set_fine_tile_rows(topo_handle* h, int rows);
/* CUDA graphs per handle, captured on first use and re-captured when the
 * schedule, tiles or buffers change: the FP32 V-cycle of the mixed solver; the
 * mixed solve's outer FP64 CG as one graph with a device-side loop (one
 * V-cycle per outer iteration, or the inner FP32 CG nested in it as a second
 * device-side loop), so the host waits once per solve; the inner CG alone
 * where the outer loop runs on the host; the OC bisection; a whole design
 * iteration of topo_design_iteration with the mixed solve and the Chebyshev
 * multigrid, from its second iteration on a handle (after the operator update,
 * whose coarsest inversion it waits for: spectral bounds, solve, compliance,
 * sensitivity, filter, adjoint, OC update as one launch; its loops decided on
 * the device; the results read once after it; the load vector must then
 * change through topo_set_bc or topo_put_array, not through a device pointer).
 * 1 = on (default), 2 = on but the outer solve loop on the host, 3 = on but no
 * whole-iteration graph, 0 = direct launches and host loops (the same kernels
 * in the same order: the same results bit for bit).  Graphs are not used while
 * topo_profile_enable is on. */
int topo_set_graphs(topo_handle* h, int enable);
/* Recompute the coarsest level's dense inverse at every `every`-th operator
 * update only (1, the default, is every update, as the reference does); in
 * between, the coarse levels are current and the coarsest solve applies the
 * inverse of the last refresh.  The mixed solve's flexible CG takes the
 * slightly older coarse solve; it still converges to the requested residual.
 * Boundary conditions, operator precision and a checkpoint load force a
 * refresh at the next update (a resumed run therefore equals an uninterrupted
 * one bit for bit only from a refresh on). */
int topo_set_coarse_refresh(topo_handle* h, int every);
/* Which graphs the handle holds now (bits): 1 FP32 V-cycle, 2 inner CG on its
 * own, 4 outer solve loop, 8 inner CG nested in the outer loop's graph, 16 OC
 * bisection, 32 a whole design iteration (topo_design_iteration).  A form whose
 * capture failed (a driver without conditional graph nodes, say) is left to
 * the host from then on and not set. */
int topo_graph_state(const topo_handle* h, int* state);
/* Replaces Grid::update_residual (grid/Grid.cu:2420-2454). */
int topo_residual(topo_handle* h, int level);
/* Replaces Grid::gs_relax (grid/Grid.cu:1844-1887); reverse = adjoint sweep order. */
int topo_smooth(topo_handle* h, int level, int sweeps, int reverse);
/* Replace Grid::restrict_residual / prolongate_correction (grid/Grid.cu:2572-2691). */
int topo_restrict(topo_handle* h, int coarse_level);
int topo_prolong(topo_handle* h, int fine_level);
/* Replaces Grid::solve_fem_host (grid/Grid.cpp:4040-4102), on the GPU. */
int topo_coarsest_solve(topo_handle* h);
/* Replaces HierarchyGrid::v_cycle (grid/Grid.cpp:2399-2444); returns ||R||/||F||. */
int topo_vcycle(topo_handle* h, int pre, int post, double* relres);
/* Replaces the driver's solve loop (utils/test_utils.cpp:937-941); warm-starts from U. */
int topo_solve(topo_handle* h, const topo_solve_opts* opts, topo_solve_stats* stats);
/* Replaces Grid::compliance (grid/Grid.cpp:4035-4038): F . U. */
int topo_compliance(topo_handle* h, double* c);
/* Replaces Grid::volumeRatio (grid/Grid.cu:5462-5470). */
int topo_volume(topo_handle* h, int reference_denominator, double* v);
/* Replaces computeSensitivity_kernel (optimization/optimization.cu:96-159). */
int topo_sensitivity(topo_handle* h);
/* Replaces Grid::filterSensitivity (grid/Grid.cu:4218-4246). */
int topo_filter(topo_handle* h, double radius);
/* Replaces Grid::ddensity2dcoeff_update (grid/Grid.cu:3643-3748). */
int topo_spline_adjoint(topo_handle* h);
/* Allocation-free spline adjoint; it has no counterpart in the reference.
 * It does the same work as topo_spline_adjoint for callers that must not
 * allocate device memory when they call it: a fixed memory budget, a loop that
 * must stay out of the CUDA allocator, or memory owned by another component.
 * sens_dev (double[ne]) and csens_dev (double[nc]) are device pointers the caller
 * owns; work is queued on the handle's stream.  The intermediate planes
 * (nb_x*ny*nz + nb_x*nb_y*nz doubles) live in one fixed 2097152-double (16 MiB)
 * device array per GPU, kept until the process exits; larger problems get
 * TOPO_E_BAD_INPUT.  No cudaMalloc/cudaFree is called.  The first call on a
 * device looks up the array's device address (cudaGetSymbolAddress), so make
 * it before any stream capture.  All calls share the array: calls that overlap
 * on the GPU (several streams or handles at once) race. */
int topo_spline_adjoint_noalloc(topo_handle* h, const double* sens_dev, double* csens_dev);
/* Replaces updateCoeff (optimization/optimization.cu:589-695). */
int topo_oc_update(topo_handle* h, const topo_oc_opts* opts, topo_oc_stats* stats);
/* Replaces Grid::dvol2dcoeff (grid/Grid.cu:3750-3859): out_dev[nc] (device; NULL =
 * the handle's TOPO_VOLCSENS array, reference getVolCSens) = scale * d volume /
 * d coefficient, volume = sum(rho) / den with den the padded GS element count
 * (refden = 1, reference volumeRatio) or the active count.  The reference reads an
 * uninitialised d volume / d rho on this path; here it is 1/den on every active
 * element.  Uses the SENS scratch, not SENS itself. */
int topo_volume_csens(topo_handle* h, int refden, double scale, double* out_dev);

/* --- MMA: Method of Moving Asymptotes -------------------------------------- */
/* Replaces MMA::mma_t (optimization/mma_t.h:159-266, mma_t.cpp, mma_t.cu): Svanberg's
 * MMA with the primal-dual interior-point subproblem, parameters a0 = 1, a = 0,
 * c = 10, d = 1, m <= 4 constraints g_i(x) <= 0.  One cooperative kernel runs the
 * whole subproblem per update, in FP64. */
typedef struct topo_mma topo_mma;

typedef struct topo_mma_stats {
  int subiterations;          /* Newton steps of the subproblem (reference caps at 81) */
  double kkt_err;             /* inf-norm of the KKT residual at the last step */
  double step;                /* last line-search step */
  double dx_norm;             /* |x_new - x_old|_2 */
  int overflow;               /* 1 if the Newton-step cap was hit */
  int converged;              /* mma_t::update's return: change < 1e-3 for more than 10 calls */
} topo_mma_stats;

/* mma_t(n, m): own CUDA stream on `device`. */
int topo_mma_create(int n, int m, int device, topo_mma** out);
/* MMA over the spline coefficients of h (n = coefficient count), on h's stream. */
int topo_mma_create_for(topo_handle* h, int m, topo_mma** out);
void topo_mma_destroy(topo_mma* mma);
const char* topo_mma_last_error(const topo_mma* mma);
int topo_mma_size(const topo_mma* mma, int* n, int* m);
/* mma_t::set_constrain_amplifier (optimization/mma_t.cpp:468-472). */
int topo_mma_set_constraint_amplifier(topo_mma* mma, double c, double d);
/* mma_t::init(lower, upper) with per-variable host arrays or uniform bounds
 * (optimization/mma_t.h:221-230); x starts at the midpoint of the move limits. */
int topo_mma_init(topo_mma* mma, const double* lb, const double* ub);
int topo_mma_init_uniform(topo_mma* mma, double lb, double ub);
/* mma_t::update(df, dg, g) (optimization/mma_t.cpp:18-51): df_dev[n] and dg_dev[i][n]
 * are device pointers, g[m] host values.  Blocks until the step is done. */
int topo_mma_update(topo_mma* mma, const double* df_dev, const double* const* dg_dev, const double* g,
                    topo_mma_stats* stats);
/* mma_t::get_x(dst) (optimization/mma_t.cu:150-153): device-to-device copy, queued. */
int topo_mma_get_x(topo_mma* mma, double* dst_dev);
/* Host copies of x (blocking). */
int topo_mma_read_x(topo_mma* mma, double* dst_host);
int topo_mma_write_x(topo_mma* mma, const double* src_host);

/* --- reference ordering -------------------------------------------------- */
/* Reproduces Grid::enumerate_gs_subset (grid/Grid.cpp:4104-4165) with the colour of
 * grid/Grid.cu:1286-1328: vidmap[active vertex rank] = GS id, eidmap likewise,
 * gs_num[8] padded colour sizes.  Arrays sized by the active counts. */
int topo_gs_maps(topo_handle* h, int level, int* vidmap, size_t nvid, int* eidmap, size_t neid,
                 int* gs_num8, int* n_gsvertices, int* n_gselements);

/* --- measurement --------------------------------------------------------- */
/* When enabled, CUDA events bracket every launch of a kernel family on the
 * handle's stream; topo_profile_read returns launches and summed milliseconds. */
int topo_profile_enable(topo_handle* h, int enable);
int topo_profile_read(topo_handle* h, int family, int* launches, double* ms);

enum topo_kernel_family {
  TOPO_K_FINE_APPLY64 = 0,
  TOPO_K_FINE_APPLY32 = 1,
  TOPO_K_FINE_SMOOTH64 = 2,
  TOPO_K_FINE_SMOOTH32 = 3,
  TOPO_K_COUNT = 8
};

/* Number of kernel launches the library has issued in this process. */
int topo_launch_count(const topo_handle* h, long long* launches);

/* Pinned host staging memory for topo_put_array / topo_get_array. */
int topo_host_alloc(size_t bytes, void** ptr);
int topo_host_free(void* ptr);
/* CUDA events on the handle's stream: topo_timer_stop returns the device time
 * since the matching topo_timer_start, after waiting for it. */
int topo_timer_start(topo_handle* h);
int topo_timer_stop(topo_handle* h, double* ms);

/* --- one design iteration ------------------------------------------------- */
typedef struct topo_iter_opts {
  topo_solve_opts solve;
  topo_oc_opts oc;
  double filter_radius;       /* reference filter_radius (default 2) */
} topo_iter_opts;

typedef struct topo_iter_stats {
  double compliance;          /* F . U after the solve */
  double volume;              /* volume ratio after the OC update */
  topo_solve_stats solve;
  int oc_trials;
  double ms;                  /* device time of the whole iteration */
} topo_iter_stats;

/* Replaces one pass of the loop body of TestSuit::testOrdinarySplineTopopt
 * (utils/test_utils.cpp:928-958): update_stencil, solve (warm start), compliance,
 * computeSensitivity (sensitivity, filter, spline adjoint) and updateCoeff. */
int topo_design_iteration(topo_handle* h, const topo_iter_opts* opts, topo_iter_stats* stats);

/* --- many designs at once ------------------------------------------------- */
/* Independent designs (no reference counterpart): `iterations` design
 * iterations on each of n handles, run from `threads` host threads so the
 * handles' streams execute concurrently on the GPU (each handle's FP32 V-cycles
 * replay as CUDA graphs).  opts: one set for all (nopts = 1) or one per handle.
 * last[n] (may be NULL) receives each handle's last iteration statistics.
 * Handles on one device must share E, nu and h (topo_create enforces it). */
typedef struct topo_batch_stats {
  double wall_ms;     /* host wall time of the whole batch */
  double sum_ms;      /* sum over handles of their own wall time */
  double max_ms;      /* slowest handle */
  int failures;       /* handles that stopped on an error */
} topo_batch_stats;
int topo_design_batch(topo_handle** handles, int n, const topo_iter_opts* opts, int nopts, int iterations,
                      int threads, topo_iter_stats* last, topo_batch_stats* stats);

/* --- autotuner ------------------------------------------------------------ */
/* Tile and schedule choice for the current problem state (no reference
 * counterpart).  Stage 1 times the fine-level kernels at z-march depths
 * 4, 8, 16 and 32 (the FP32 Chebyshev step with the modal and with the
 * tensor-core element products, and the FP64 operator; CUDA events, 5 launches
 * each; the modal form also with CTA tiles of 4 and 16 element rows) and keeps
 * the fastest for the handle (depths, topo_set_fine_tensor_cores and
 * topo_set_fine_tile_rows).  Stage 2 solves from the
 * current U with each candidate schedule of the mixed solver (FP32 inner
 * iterations 1, 2, 4, 6 x smoothing steps 1, 2 x Chebyshev degree 2, 3 x lower
 * end of the Chebyshev interval base->cheb_lo, 0.1 x inner tolerance
 * base->inner_rtol, 0.03), stage 3 runs two passes of coordinate search from
 * the best schedule over the lower end (0.05, 0.1, 0.2, base), the inner
 * tolerance (0.03, base) and the degree, stage 4 tries degrees 2, 3 and 4 jointly
 * with lower ends 0.02, 0.04, 0.06 and inner tolerances 0.03, 0.05, stage 5 two
 * and four more inner iterations with inner tolerances 0.01, 0.02 and the next
 * degree, and the fastest that converges is written into *best (other fields from *base, which must be TOPO_SOLVE_MIXED
 * with the Chebyshev smoother).  With graphs on, each candidate is solved twice and timed on the second
 * solve (the first captures its graphs, which design iterations replay).  U is restored. */
typedef struct topo_tune_report {
  int tz32, tz64;           /* chosen z-march depths */
  double cheb_ms[4];        /* FP32 Chebyshev step at depths 4, 8, 16, 32 */
  double apply_ms[4];       /* FP64 operator at depths 4, 8, 16, 32 */
  int candidates;           /* schedules tried */
  double base_ms, best_ms;  /* solve time of *base and of *best */
  double tune_ms;           /* device time spent tuning */
  int tc;                   /* FP32 fine element products chosen: 1 tensor cores, 0 modal */
  double cheb_tc_ms[4];     /* FP32 Chebyshev step on the tensor cores at depths 4, 8, 16, 32 */
  int rows32;               /* element rows of the FP32 modal kernel's CTA tile chosen: 4, 8 or 16 */
  double cheb_rows_ms[2][4];/* modal FP32 Chebyshev step with tiles of 4 and of 16 rows, depths 4..32 */
} topo_tune_report;
int topo_autotune(topo_handle* h, const topo_solve_opts* base, topo_solve_opts* best, topo_tune_report* report);
/* Sets the fine kernels' z-march depths (FP32 kernels, FP64 operator) directly,
 * e.g. to replay an earlier autotune result. */
int topo_set_tiles(topo_handle* h, int tz32, int tz64);
/* Opens (start = 1) or closes (start = 0) the profiler's capture range
 * (cudaProfilerStart / cudaProfilerStop), so a profiler started with capture
 * off records only warm work, e.g. one design iteration after the warm-up. */
int topo_profiler_range(int start);

/* --- many load cases in one solve ------------------------------------------ */
/* Multi-right-hand-side solve (config "batched": many load cases as right-hand
 * sides of one V-cycle; no reference counterpart).  Every FP32 V-cycle launch
 * and every FP64 operator application processes all right-hand sides at once:
 * the operator data (rho^p, masks, stencils, coarsest inverse) is read once per
 * launch for the whole batch, and each right-hand side has its own flexible-CG
 * scalars (a converged one is frozen).  Right-hand sides live in TOPO_MULTI_F,
 * solutions (and initial guesses) in TOPO_MULTI_U, each [cap][3][nv]. */
typedef struct topo_multi_stats {
  int iterations;     /* outer FP64 flexible-CG iterations (the slowest right-hand side) */
  int vcycles;        /* batched FP32 V-cycles */
  double max_relres;  /* largest final FP64 relative residual */
  double ms;          /* device time */
} topo_multi_stats;
/* Allocates the batched buffers for up to `capacity` right-hand sides. */
int topo_multi_reserve(topo_handle* h, int capacity);
/* Solves the first nrhs right-hand sides with TOPO_SOLVE_MIXED and the Chebyshev
 * smoother (opts->mode / smoother / inner_max must be MIXED / CHEBYSHEV / <= 1);
 * relres (may be NULL) receives nrhs final FP64 relative residuals. */
int topo_solve_multi(topo_handle* h, int nrhs, const topo_solve_opts* opts, topo_multi_stats* stats,
                     double* relres);

/* --- worst-case (robust) compliance ---------------------------------------- */
/* The reference's default optimisation (optimization/optimization.cpp:673-767)
 * designs against the worst unit load on a load region: the largest
 * compliance f.K^-1 f over loads f of unit norm on the region's vertices
 * (modifiedPM, optimization/optimization.cpp:213-351).  With supports, a load
 * either acts along each load vertex's normal (the reference's
 * with_support_constrain_force_direction: forceProject removes the tangential
 * parts, optimization/projection.cpp:289-360) or in any direction
 * (with_support_free_force).  The worst load is the leading eigenvector of
 * M = S^T K^-1 S, S the scatter from load coordinates to nodal forces. */

/* Replaces setLoadNodes (optimization/projection.cpp:129-269) and
 * uploadLoadNodes (optimization/projection.cu:71-118): n load vertices
 * (level-0 vertex ids) with unit outward normals normals[3*n] (xyz per
 * vertex; ignored with free_direction).  Fixed DOFs carry no load. */
int topo_set_load_region(topo_handle* h, int n, const int* vertices, const double* normals);

typedef struct topo_worst_opts {
  topo_solve_opts solve;      /* multi-RHS solve per block iteration: MIXED, CHEBYSHEV, inner_max <= 1;
                                 solve.rtol is the FP64 tolerance of the final solve */
  int free_direction;         /* 0: force along each vertex normal; 1: any direction */
  int block;                  /* load vectors iterated together (1 = the reference's single vector) */
  int max_iter;               /* block iterations (reference 500) */
  double tol;                 /* stop when the worst load changes by less than this (reference fch 1e-4) */
  unsigned long long seed;    /* start vectors (the reference seeds cuRAND by time, Q10) */
} topo_worst_opts;

typedef struct topo_worst_stats {
  double compliance;          /* worst-case compliance f.U of the unit worst load */
  double second;              /* next Ritz value (the leading one's gap) */
  double change;              /* last change of the worst load, |f_new - f_old| */
  double relres;              /* FP64 relative residual of the final solve */
  int iterations;             /* block iterations */
  int solve_iterations;       /* outer FP64 CG iterations summed over the block solves */
  double ms;                  /* device time */
} topo_worst_stats;

/* Replaces modifiedPM (optimization/optimization.cpp:213-351) with a block
 * (subspace) iteration of Rayleigh-Ritz steps over `block` load vectors, each
 * step one multi-right-hand-side solve warm-started from the previous step's
 * displacements rotated into the new basis.  Leaves the unit worst load in
 * TOPO_F and its displacement in TOPO_U (level 0), so topo_sensitivity and the
 * rest of the design chain act on the worst case as the reference's
 * optimization() does.  Needs topo_update_operators with FP32 operators and
 * reserves multi-RHS buffers for `block` right-hand sides. */
int topo_worst_compliance(topo_handle* h, const topo_worst_opts* opts, topo_worst_stats* stats);

/* --- Heaviside projection and manufacturing constraints ------------------- */
/* Replaces projectDensities (optimization/optimization.cu:313-353):
 * TOPO_RHO_INIT <- rho, rho <- clamp(H_beta(rho_init), rho_min, 1) with
 * H_beta(s) = (tanh(beta/2) + tanh(beta (s - 1/2))) / (2 tanh(beta/2)). */
int topo_heaviside_project(topo_handle* h, double beta);
/* Chain rule of the projection on TOPO_SENS (before topo_filter):
 * sens *= dH/drho(rho_init) (computeProjectionSensitivity_kernel,
 * optimization/optimization.cu:161-183). */
int topo_heaviside_sensitivity(topo_handle* h, double beta);
/* The projected volume's coefficient gradient of computeSensitivity2
 * (optimization/optimization.cu:243-311): scale / den * dH/drho on active
 * elements, filtered with filter_radius (> 0) and taken through the spline
 * adjoint into out_dev[nc] (NULL = TOPO_VOLCSENS); den as topo_volume_csens. */
int topo_heaviside_volume_csens(topo_handle* h, double beta, int refden, double filter_radius, double scale,
                                double* out_dev);

/* Self-support and drip constraints of the spline design
 * (deal_surface_points, optimization/optimization.cpp:1103-1127;
 * grid/Grid.cu:5529-7156).  Surface points: the crossings of the spline's 1/2
 * level set with the edges of a (lattice + 2)^3 lattice of cell centres over
 * the domain box padded by one cell (spline - 1/2 inside the box, -1/2
 * outside; compute_background_mcPoints_value, grid/Grid.cu:3986-4095), kept in
 * lattice order when they lie in an active element, thinned to max_points by
 * the reference's equidistant pick.  Normal = spline gradient; when most
 * points see solid a small step along it (Heaviside with `beta` at 1/2), all
 * normals are flipped.  Per point inner = n_z / |n| / cos(print_angle pi);
 * the self-support value by ss_mode (0 p-norm, 1 p-norm all, 2 h, 3 h all,
 * 4 overhang sigmoid, 5 overhang all; "down only" modes count points with
 * n_z < 0), the drip value by drip_mode (6 exp, 7 exp all; 0-5 contribute
 * zero, as in the reference's compute_spline_drip_constraint_test), each
 * averaged over its count (p-norm modes: mean^(1/p) - 1).  Their coefficient
 * gradients (points held fixed, each point's terms summed in point order per
 * coefficient, divided by the count) go to TOPO_SSCSENS / TOPO_DRIPCSENS. */
typedef struct topo_support_opts {
  int lattice;            /* lattice cells per axis (reference 64) */
  int max_points;         /* surface points kept (reference 200000) */
  double print_angle;     /* in units of pi (reference opt_print_angle; its flag default 3/4 parses as 0) */
  int ss_mode;            /* 0..5 as above (reference default "oh" = 4) */
  int drip_mode;          /* 0..7 (reference default "oh" = 4, which contributes zero) */
  double beta;            /* Heaviside sharpness of the normal-direction test */
  double p_norm, hfunction_c, sigmoid_c;   /* 0 = the reference's 8, 10, 0.09 */
  double drip_beta, drip_mu, drip_angle, drip_alpha, drip_beta_scale; /* 0 = 128, 32, 160 deg (radians), 4, 10 */
  int drip_version;       /* 1: Gaussian of the gradient slope; else the sigmoid of the angle */
  int reference_quirks;   /* drip gradient as the reference computes it (Hessian derivatives summed over the
                             taps already visited, the y slope derivative written over the x one) */
} topo_support_opts;
typedef struct topo_support_stats {
  int candidates;         /* level-set crossings in active elements */
  int points;             /* points used */
  int overhang_points;    /* points with n_z < 0 */
  int flipped;            /* normals flipped by the direction test */
  double ss_value;        /* global self-support value (the MMA constraint is scale * (ss - 1)) */
  double drip_value;      /* global drip value (the constraint is scale * drip) */
} topo_support_stats;
int topo_support_constraints(topo_handle* h, const topo_support_opts* opts, topo_support_stats* stats);

/* --- learned preconditioner (U-Net) --------------------------------------- */
/* A 3-level 3D convolutional U-Net (16/32/64 channels, 3x3x3 kernels, 246,931
 * effective parameters, bf16 weights, fp32 accumulation) corrects the FP32
 * multigrid preconditioner of TOPO_SOLVE_MIXED: with z = V(r),
 * z' = z + beta lz N(s(r/lr), s(z/lz), log rho), lr and lz the local rms of r
 * and z (blocks of 8^3 vertices, floored at 1e-2 of the global rms),
 * s(x) = x/(1+|x|/8), and beta the energy-optimal amount of the correction
 * c = lz N, beta = c.(r - A z) / c.(A c) (beta = 0 keeps z).  It is trained with
 * the library's own forward, backward and Adam kernels (clipped gradients,
 * warm-up and cosine step size) on crops harvested from the solver's iterates
 * (target (e_k - z_k)/lz_k, e_k = u* - u_k).  The last layer starts at zero
 * (N = 0: the plain V-cycle).  No reference counterpart. */
/* Creates the network of h with He-normal weights from `seed`. */
int topo_unet_enable(topo_handle* h, unsigned long long seed);
/* Kernel of the network's 3x3x3 convolutions (forward and data gradient):
 * TOPO_CONV_TCGEN05 runs them on the 5th-generation tensor cores (tcgen05.mma,
 * fp32 accumulators in tensor memory, input halo by TMA tensor loads),
 * TOPO_CONV_MMA_SYNC (default: 1.19x faster on the network's 16-64-channel
 * layers, measured on GB300) on the warp-level mma.sync path.  Both compute
 * bf16 x bf16 -> fp32 in the same layouts; they differ only in the fp32
 * summation order. */
enum { TOPO_CONV_MMA_SYNC = 0, TOPO_CONV_TCGEN05 = 1 };
int topo_unet_set_conv_kernel(topo_handle* h, int kind);
/* Parameter count of the flat fp32 layout: per layer W[cout][27][cin] then b[cout],
 * layers L0a L0b L1a L1b L2a L2b D1a D1b D0a D0b (cin of L0a padded to 16 with
 * channels 0-7 used, cout of D0b 16 with channels 0-2 used). */
int topo_unet_num_params(size_t* n);
int topo_unet_get_params(topo_handle* h, float* dst, size_t n);
int topo_unet_set_params(topo_handle* h, const float* src, size_t n);
/* Host-tensor passes: x [nb][Z][Y][X][8] (residual xyz, V-cycle output xyz,
 * log-density, 0; residual and output in local units), X, Y, Z
 * multiples of 8; y [..][3] network output; loss = sum m (y - t)^2 / sum m t^2
 * over DOFs with mask bit c set; grad [n] its parameter gradient. */
int topo_unet_forward(topo_handle* h, int X, int Y, int Z, int nb, const float* x, float* y);
int topo_unet_loss_grad(topo_handle* h, int X, int Y, int Z, int nb, const float* x, const float* t,
                        const uint8_t* mask, double* loss, float* grad);
/* Crop dataset: `capacity` crops of crop^3 vertices (crop a multiple of 8);
 * each harvesting solve adds crops_per_iterate crops per recorded iterate. */
int topo_unet_dataset_reserve(topo_handle* h, int capacity, int crop, int crops_per_iterate);
int topo_unet_dataset_size(topo_handle* h, int* n);
/* Host copy of crop `slot`: x [crop^3][8], t [crop^3][3], mask [crop^3] (crop
 * side returned in *crop; size the arrays for the reserved side). */
int topo_unet_dataset_get(topo_handle* h, int slot, float* x, float* t, uint8_t* mask, int* crop);
/* `steps` Adam steps (update = 1) or evaluations (update = 0) on random batches
 * drawn from crops [lo, hi) (hi <= 0: all); loss = mean relative loss. */
int topo_unet_train(topo_handle* h, int steps, int batch, double lr, unsigned long long seed, int lo, int hi,
                    int update, double* loss);

/* --- domains, files and checkpoints -------------------------------------- */
/* The reference's domain input: an LSB-first uint32 bit mask over a
 * reso[0] x reso[1] x reso[2] frame, bit b of word w = element 32w + b with x
 * fastest (HierarchyGrid::genFromMesh(const std::vector<unsigned>&, int[3]),
 * grid/Grid.cpp:977; the frame is the next power of two above the part,
 * voxelizer/voxelize_main.cpp:312-340).  The handle's grid is the nx x ny x nz
 * box at the frame's origin; a set bit outside it is TOPO_E_BAD_INPUT. */
int topo_bitmask_to_eactive(const int* reso3, const uint32_t* words, int nx, int ny, int nz, uint8_t* eactive);
/* The inverse: words[ceil(reso0*reso1*reso2 / 32)] from eactive (NULL = all active). */
int topo_eactive_to_bitmask(int nx, int ny, int nz, const uint8_t* eactive, const int* reso3, uint32_t* words);
/* Replaces HierarchyGrid::genFromMesh(const std::vector<unsigned>&, int[3])
 * (grid/Grid.cpp:977-1040): topo_create on the bit mask's domain. */
int topo_create_bitmask(const topo_config* cfg, const int* reso3, const uint32_t* words, topo_handle** out);

/* Mesh -> domain bit mask (voxelizer/voxelize_main.cpp:344-406 with the solid
 * rule of voxelizer/voxelize_solid.cu:78-166): a closed triangle mesh
 * (verts[3*nverts] xyz, tris[3*ntris] vertex ids) in a cube frame around its
 * bounding box, padded to the next power of two above preferred_resolution
 * (reso_out; box6_out = min xyz, max xyz).  A voxel is solid when an odd
 * number of triangles lie beyond its centre along x.  words (may be NULL for
 * a size query) receives reso^3 / 32 LSB-first words, the input of
 * topo_create_bitmask.  topo_voxel_frame computes only the frame (host). */
int topo_voxel_frame(const float* verts, int nverts, int preferred_resolution, int* reso_out, float* box6_out);
int topo_voxelize_mesh(int device, const float* verts, int nverts, const int* tris, int ntris, int preferred_resolution,
                       int* reso_out, float* box6_out, uint32_t* words, size_t nwords_cap);

/* Raw binary records, the reference's bio::write_vector / read_vector
 * (utils/binaryIO.h:70-108): the array as count values, FP64 or (fp32 = 1)
 * FP32, no header.  topo_write_array(h, TOPO_COEFF, 0, path, 1) is
 * HierarchyGrid::writeCoeff (grid/Grid.cpp:2139-2156); reading checks that
 * the file holds exactly the array. */
int topo_write_array(topo_handle* h, int which, int level, const char* path, int fp32);
int topo_read_array(topo_handle* h, int which, int level, const char* path, int fp32);
/* The active elements' (x, y, z, value) as FP32 records, 4 per element in
 * lexicographic order: what HierarchyGrid::writeDensity / writeSensitivity
 * (grid/Grid.cpp:1266-1310, 2062-2098) pass to OpenVDB.  which = TOPO_RHO or
 * TOPO_SENS; count (may be NULL) receives the number of records. */
int topo_write_active_records(topo_handle* h, int which, const char* path, int64_t* count);

/* Checkpoint of a design run (no reference counterpart: the reference
 * restarts from a coefficient file).  Holds the coefficients, the density,
 * the warm-start displacement, the spectral-bound warm starts of every level,
 * the z-march depths and `user_bytes` of caller data (iteration counters,
 * solver options).  A run resumed from it on a handle with the same grid,
 * boundary conditions, spline and settings repeats the uninterrupted run bit
 * for bit.  Loading fails with TOPO_E_BAD_INPUT on another grid or spline;
 * user (may be NULL) receives at most user_cap bytes, *user_bytes the size. */
int topo_checkpoint_save(topo_handle* h, const char* path, const void* user, size_t user_bytes);
int topo_checkpoint_load(topo_handle* h, const char* path, void* user, size_t user_cap, size_t* user_bytes);
/* The MMA state (iterate and history, bounds, asymptotes, amplifiers, stop
 * counter) of the same size. */
int topo_mma_checkpoint_save(topo_mma* mma, const char* path);
int topo_mma_checkpoint_load(topo_mma* mma, const char* path);

/* --- host-only set-up helpers (no GPU needed) ----------------------------- */
/* Element template (element/templateMatrix.cpp:31-99), row-major 24x24. */
int topo_element_template(double E, double nu, double h, double* Ke576);
/* Level plan (grid/Grid.cpp:747-769, 909-911): writes up to max_levels element dims
 * (3 ints each) and coarsening factors. */
int topo_plan_levels(int nx, int ny, int nz, const uint8_t* eactive, int max_coarse_elements,
                     int max_levels, int* nlevels, int* dims, int* factors);
/* Knot vector (2*order+partition) and basis tables at element centres along one axis
 * (grid/Grid.cpp:3253-3337, grid/Grid.cu:384-466): i0[nelem] first basis index or -1,
 * N[nelem*order] basis values. */
int topo_spline_axis(int order, int partition, double bmin, double bmax, int nelem, double h,
                     double* knots, int* i0, double* N);
/* topo_set_bc_regions on the host: fixed[nv] and loads[3*nv] for an element box with
 * mask eactive (NULL = all active). */
int topo_plan_bc_regions(int nx, int ny, int nz, const uint8_t* eactive, const topo_bc_regions* spec,
                         uint8_t* fixed, double* loads, int* nfixed, int* nloaded);
/* Reference GS ordering of one level of the plan (see topo_gs_maps). */
int topo_plan_gs_maps(int nx, int ny, int nz, const uint8_t* eactive, int max_coarse_elements,
                      int level, int* vidmap, size_t nvid, int* eidmap, size_t neid, int* gs_num8,
                      int* n_gsvertices, int* n_gselements);

#ifdef __cplusplus
}
#endif
#endif /* TOPO_GB300_H */
