/* CPU ORACLE -- TEST INFRASTRUCTURE ONLY.
 * C interface of the plain C++ restatement of the reference PDDSparse hot path
 * (see oracle_internal.h for the parity status).  Loaded by the tests, by
 * __graft_entry__.smoke() and by bench.py's CPU-baseline leg; never by the
 * product library. */
#pragma once
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Problem ids shared with the product's problem descriptor. */
enum {
  ORC_POISSON_SINCOS = 0, /* u = sin(pi x)cos(pi y) + xy, sigma = sqrt2 I        */
  ORC_MONEGROS = 1,       /* BVPs/EDPs/Monegros_Poisson_CPP.hpp (libm only)      */
  ORC_HELMHOLTZ = 2,      /* u = sin(a x)cos(b y), c const; p = {a, b, c}       */
  ORC_VARCOEF = 3,        /* sigma = diag(1+x^2/2, 1+y^2/2), b = (y,-x), ...    */
  ORC_LUT = 4             /* coefficients and g from tables (orc_set_lut)       */
};

typedef struct {
  int kind;
  double p[8];
} orc_problem;

typedef struct {
  int N;               /* paths per knot                                        */
  double h;            /* Euler-Maruyama step                                   */
  uint64_t seed;       /* Philox key                                            */
  uint32_t instance;   /* Philox counter word 3                                 */
  int portable;        /* 1: portable FP64 math (replay parity), 0: libm        */
  int sublinear;       /* 1: run the reference's sublinear continuation         */
  int dup_sum;         /* 0: reference G_return_withrep overwrite, 1: sum       */
  int threads;         /* OpenMP threads for the path loop                      */
  double fac[4];       /* RBF shape c per side kind (c2[kind] in the reference) */
  int64_t max_steps;   /* per path, per leg; exceeded -> status 3               */
  int adaptive_h;      /* 1: per-knot h of PDDSparseGM.cpp:4026-4028             */
  int fast_reduce;     /* 1: not the reference's reduction but its linearity form
                          (n_s exponentials per exit, G = -ipsi^T S / N), exits
                          reduced in parallel; G_var is not computed.  A faster
                          CPU form for comparison only, never a parity check. */
} orc_params;

/* ---- layout ---------------------------------------------------------------*/
void* orc_layout_new(double swx, double swy, double nex, double ney, int nsub, int nnode);
void orc_layout_free(void* L);
int orc_layout_nknots(const void* L);
int orc_layout_nwork(const void* L);
void orc_layout_work(const void* L, int* idx, double* x, double* y);
int orc_layout_ninterfaces(const void* L);
int orc_layout_interface(const void* L, int i, int* label, int* idx, double* x, double* y);
/* Stencil of a knot; side data packed as [4][maxn] in N,S,E,W order.
 * Returns 0, or -1 when a side holds more than maxn knots. */
int orc_stencil(const void* L, int knot, double* params, int* kinds, int* sizes,
                int* idx, double* x, double* y, int maxn);

/* ---- RBF interpolation matrix ---------------------------------------------*/
/* Psi_ij = exp(-|p_i - p_j|^2 / c^2); ipsi = full-pivot LU inverse, row-major.
 * cond = ||Psi||_F ||ipsi||_F (Meshes/stencil.cpp:171).  Returns rank. */
int orc_ipsi(int n, const double* x, const double* y, double c, double* ipsi, double* cond);
/* Same with the exponentials of the portable math (portable = 1), i.e. the
 * inverse the portable-mode estimation computes internally. */
int orc_ipsi_ex(int n, const double* x, const double* y, double c, int portable, double* ipsi,
                double* cond);

/* ---- estimation -----------------------------------------------------------*/
/* stats[0] linear steps, [1] sublinear steps, [2] global exits, [3] stencil exits */
int orc_knot(const void* L, const orc_problem* P, const orc_params* prm, int knot,
             double x0, double y0, const double* ipsi_in, int* gj, double* g, double* gvar,
             int maxnnz, int* nnz, double* B, double* BB, int64_t* stats);
/* Per-path linear exit records of one knot (replay comparisons). */
int orc_knot_paths(const void* L, const orc_problem* P, const orc_params* prm, int knot,
                   double x0, double y0, double* xl, double* yl, double* Yl, double* Zl,
                   double* xil, int32_t* steps_l, int32_t* steps_s);
/* Diagnostic sums of Reduce_Analytic per knot of a list (Solvers/
 * EMFKACSolver.hpp:542-558): sums[k * ORC_DIAG_N + q], q in the order
 * phi, phi^2, xi, xi^2, phi+xi, (phi+xi)^2, xi phi, tau of the linear leg,
 * the same 8 of the sublinear leg, normals drawn, paths (zeros for a knot
 * on the domain boundary). */
enum { ORC_DIAG_N = 18 };
int orc_run_diag(const void* L, const orc_problem* P, const orc_params* prm, const int* knots,
                 const double* x0, const double* y0, int nk, double* sums);
/* All knots of a list, in order.  Row k of G occupies [row_ptr[k], row_ptr[k+1]). */
int orc_run(const void* L, const orc_problem* P, const orc_params* prm, const int* knots,
            const double* x0, const double* y0, int nk, int* row_ptr, int* gj, double* g,
            double* gvar, int64_t maxnnz, double* B, double* BB, int64_t* stats);

/* ---- interface solve ------------------------------------------------------*/
/* (I + G) u = B from COO triplets (duplicates summed), Jacobi-preconditioned
 * BiCGSTAB with zero start (PDDSparseGM.cpp:3168-3246). */
int orc_bicgstab(int K, int64_t nnz, const int* ri, const int* ci, const double* v,
                 const double* b, double* x, int maxit, double tol, int* iters, double* err);

/* Tables of ORC_LUT: coef [ny][nx][8] = (sigma11, sigma22, b1, b2, c, f,
 * du/dx, du/dy), g [ny][nx]; bounds {x0, y0, x1, y1}.  Copied. */
void orc_set_lut(const float* coef, const float* g, int nx, int ny, const double* bounds);

/* ---- problem functions (for analytic checks) ------------------------------*/
double orc_problem_u(const orc_problem* P, double x, double y);

#ifdef __cplusplus
}
#endif
