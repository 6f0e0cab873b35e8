/*
 * topo_oracle.h -- CPU FP64 restatement of the reference's per-design-iteration
 * topology-optimisation path (NanXYZH/TopOptSpline3D).
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the parity checker for the CUDA
 * product (libtopo_gb300.so) and the timed CPU baseline.  Only tests/, the
 * smoke entry point and bench.py's CPU-baseline leg may load it; the product
 * never links or calls it.
 *
 * Parity status: the reference cannot be built here (Eigen, gflags, CGAL,
 * OpenVDB and a forced-on MATLAB engine are absent) and ships no golden
 * vectors, so this restatement is pinned by known-answer tests derived from
 * the mathematics (element-matrix null space, partition of unity, filter
 * weights, Galerkin products against explicit sparse products) rather than by
 * reference outputs: parity is "unpinned" in the strict sense.
 *
 * Layout (shared with the CUDA product so arrays compare element-wise):
 *   element e = ex + nx*(ey + ny*ez); vertex v = x + (nx+1)*(y + (ny+1)*z)
 *   vertex vectors: SoA [3][nv]; element matrices: [ne][24*24] row-major with
 *   local node a = ax + 2ay + 4az and DOF 3a+c (reference element/templateMatrix.cpp:15-27);
 *   coarse stencils: [27][9][nv] (reference GraftArray<double,27,9>, culib/lib.cuh:163-188),
 *   neighbour d = (dx+1) + 3(dy+1) + 9(dz+1), 3x3 block row-major.
 */
#pragma once
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_problem orc_problem;

/* 24x24 trilinear-hex stiffness from 2x2x2 Gauss (element/templateMatrix.cpp:31-99). */
void orc_ke_template(double E, double nu, double h, double* Ke576);

/* Problem set-up: element grid nx*ny*nz of size h, active element mask (NULL = all active). */
orc_problem* orc_create(int nx, int ny, int nz, double h, double E, double nu,
                        double penal, double rho_min, const uint8_t* eactive);
void orc_destroy(orc_problem* p);

/* Number of multigrid levels actually used and the element dims of each level. */
int orc_num_levels(const orc_problem* p);
void orc_level_dims(const orc_problem* p, int level, int* dims3);
int orc_level_factor(const orc_problem* p, int level);  /* coarsening factor from level-1 (4 or 2) */

/* Boundary conditions: fixed[v] bit c set = DOF c of vertex v is fixed; loads [3][nv]. */
void orc_set_bc(orc_problem* p, const uint8_t* fixed, const double* loads);

/* Spline set-up: order (3 = quadratic, reference default), partitions per axis,
 * bound box [min3, max3] before enlargement; knots follow grid/Grid.cpp:3253-3337
 * (float arithmetic, stored as double). */
void orc_set_spline(orc_problem* p, int order, const int* partition3, const double* bmin3,
                    const double* bmax3);
int orc_num_coeffs(const orc_problem* p);
void orc_get_knots(const orc_problem* p, int axis, double* out); /* 2*order+partition */

/* Arrays by name id (see ORC_* below). */
void orc_put(orc_problem* p, int which, int level, const void* src);
void orc_get(const orc_problem* p, int which, int level, void* dst);
int64_t orc_size(const orc_problem* p, int which, int level); /* element count */

/* Pipeline pieces. */
void orc_coeff_to_density(orc_problem* p);           /* rho <- clamp(spline(coeff)) */
void orc_update_penalised(orc_problem* p);           /* rhop <- rho^p */
void orc_update_operators(orc_problem* p);           /* Galerkin levels + coarsest factor */
void orc_apply_fine(orc_problem* p, const double* u, double* y); /* y = A u (masked) */
void orc_residual(orc_problem* p, int level);        /* R = F - A U on a level */
void orc_smooth(orc_problem* p, int level, int sweeps, int reverse);
void orc_restrict(orc_problem* p, int coarse_level);  /* F_c = P^T R_f */
void orc_prolong(orc_problem* p, int fine_level);     /* U_f += P U_c */
void orc_coarsest_solve(orc_problem* p);
double orc_vcycle(orc_problem* p, int pre, int post); /* reference order, returns rel. residual */
/* Preconditioned CG on level 0 with a symmetric V-cycle (forward pre-smoothing,
 * backward post-smoothing); warm start from U; returns iterations, writes relres. */
int orc_pcg(orc_problem* p, int pre, int post, double rtol, int maxit, int smoother, double* relres);
double orc_compliance(const orc_problem* p);          /* F . U */
double orc_volume(const orc_problem* p, int reference_denominator);
void orc_sensitivity(orc_problem* p);                 /* SENS <- -p rho^(p-1) u^T Ke u */
void orc_filter(orc_problem* p, double radius);       /* SENS <- filtered SENS */
void orc_spline_adjoint(orc_problem* p);              /* CSENS <- d/dc of SENS chain */
/* OC on coefficients (optimization/optimization.cu:559-695); returns trials. */
int orc_oc_update(orc_problem* p, double vgoal, double damp, double step, double cmin,
                  double cmax, int apply_twice, int reference_denominator, double* lambda_out);

/* Reference GS ordering (grid/Grid.cpp:4104-4165): vertex/element lexicographic
 * active index -> GS id with colours padded to 32.  Returns n_gsvertices. */
int orc_gs_maps(const orc_problem* p, int level, int* vidmap, int* eidmap, int* gs_num8,
                int* n_gselements);

/* Chebyshev smoother bounds for the point-block-Jacobi-preconditioned operator. */
void orc_set_chebyshev(orc_problem* p, int degree, double lo_frac, double hi_scale);

/* MMA optimiser (mma_oracle.cpp; reference optimization/mma_t.*): n design
 * variables, m <= ORC_MMA_MAX_M constraints g_i(x) <= 0. */
#define ORC_MMA_MAX_M 8
typedef struct orc_mma orc_mma;
orc_mma* orc_mma_create(int n, int m);
void orc_mma_destroy(orc_mma* o);
void orc_mma_set_constraint_amplifier(orc_mma* o, double c, double d);
void orc_mma_init(orc_mma* o, const double* lb, const double* ub);
int orc_mma_update(orc_mma* o, const double* df, const double* dg, const double* g);
void orc_mma_get_x(const orc_mma* o, double* x);
void orc_mma_set_x(orc_mma* o, const double* x);
/* sub-iterations, final KKT inf-norm, last step, |x - x_prev|_2, overflowed */
void orc_mma_get_stats(const orc_mma* o, double* s5);

enum {
  ORC_RHO = 0,     /* double[ne] */
  ORC_RHOP = 1,    /* double[ne] */
  ORC_COEFF = 2,   /* double[nc] */
  ORC_SENS = 3,    /* double[ne] */
  ORC_CSENS = 4,   /* double[nc] */
  ORC_U = 5,       /* double[3*nv] per level */
  ORC_F = 6,       /* double[3*nv] per level */
  ORC_R = 7,       /* double[3*nv] per level */
  ORC_STENCIL = 8, /* double[243*nv] per coarse level */
  ORC_KELEM = 9,   /* double[576*ne] per coarse level */
  ORC_VMASK = 10,  /* uint8[nv] per level: bits0-2 DOF free, bit3 vertex active */
  ORC_EACTIVE = 11,/* uint8[ne] per level */
  ORC_KE = 12,     /* double[576] */
  ORC_DIAG = 13    /* double[9*nv] per level: diagonal 3x3 blocks */
};

#ifdef __cplusplus
}
#endif
