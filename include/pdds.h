/* pdds_gb300 -- C ABI of the GB300-native PDDSparse hot path.
 *
 * The library estimates, on one GPU, the sparse interface system of the
 * probabilistic domain decomposition method PDDSparse: for every collocation
 * knot it runs Euler-Maruyama paths of the Feynman-Kac diffusion until they
 * leave the knot's stencil rectangle (Gobet-Menozzi shifted exit), turns the
 * exits into one row of G (Gaussian-RBF interpolation weights of the stencil
 * knots) and one entry of B, and solves (I + G) u = B.
 *
 * Reference interfaces replaced (paths inside the PDDS repository):
 *   struct bvp                          BVPs/BVP.hpp:89-137
 *   Fullfill_interfaces/Compute_Stencil PDDAlgorithms/PDDSparseGM.cpp:346-689, 1845-2041
 *   Stencil::Compute_ipsi               Meshes/stencil.cpp:115-243
 *   EMFKACSolver::Solve_OMP_Analytic    Solvers/EMFKACSolver.hpp:711-729
 *     (Simulate_OMP :108-216, Reduce_Analytic :514-575, G_update stencil.cpp:244-307,
 *      G_return_withrep stencil.cpp:343-406)
 *   PDDSparseGM::Solve worker loop      PDDAlgorithms/PDDSparseGM.cpp:795-848
 *   PDDSparseGM::Compute_Solution       PDDAlgorithms/PDDSparseGM.cpp:3168-3246
 *   MCinCUDA (the reference's unused GPU entry) Solvers/MCinCUDA.cu:441-480
 *
 * Conventions: every call returns a pdds_status; nothing aborts.  All work is
 * ordered on the context's CUDA stream; one context per host thread.  Output
 * buffers are caller-owned host memory; device scratch is context-owned.
 */
#ifndef PDDS_H
#define PDDS_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  PDDS_OK = 0,
  PDDS_ERR_INVALID = 1,         /* bad argument or call order            */
  PDDS_ERR_CUDA = 2,            /* CUDA runtime error (see last_error)   */
  PDDS_ERR_STEP_LIMIT = 3,      /* a path exceeded max_steps             */
  PDDS_ERR_TIMEOUT = 4,         /* a bounded device wait gave up         */
  PDDS_ERR_ILL_CONDITIONED = 5, /* an RBF matrix is numerically singular */
  PDDS_ERR_NOT_CONVERGED = 6,   /* interface solve missed its tolerance  */
  PDDS_ERR_NO_MEMORY = 7,
  PDDS_ERR_EXIT_SIDE = 8,       /* an exit matched no stencil side       */
  PDDS_ERR_BOUNDS = 9           /* a device index check failed (only the
                                   checked build, -DPDDS_CHECKED, checks) */
} pdds_status;

typedef struct pdds_ctx pdds_ctx;

/* ---------------------------------------------------------------- context */
pdds_status pdds_create(pdds_ctx** ctx, int device, uint32_t flags);
/* Frees the context.  Its device buffers are kept by the library (up to
 * 8 GB per device, blocks up to 2 GB) for the next context on the same
 * device, which then allocates no device memory for buffers of the same
 * sizes; pdds_release_cached_blocks returns them to the device. */
pdds_status pdds_destroy(pdds_ctx* ctx);
/* Frees the device buffers kept from destroyed contexts (device -1: on every
 * device).  The library also does so by itself when an allocation fails.
 * Call it before a cudaDeviceReset of the device: the reset frees them
 * behind the library's back. */
pdds_status pdds_release_cached_blocks(int32_t device);
const char* pdds_last_error(const pdds_ctx* ctx);
const char* pdds_version(void);

/* ---------------------------------------------------------------- problem
 * Replaces the function-pointer struct bvp (BVPs/BVP.hpp:89-137) on the GPU:
 * problems are compiled device functors selected by kind. */
typedef enum {
  PDDS_POISSON_SINCOS = 0, /* u = sin(pi x)cos(pi y) + x y, sigma = sqrt2 I, f = -Lap u  */
  PDDS_MONEGROS = 1,       /* the reference's Monegros Poisson test problem            */
  PDDS_HELMHOLTZ = 2,      /* u = sin(a x)cos(b y); p = {a, b, c}, c <= 0               */
  PDDS_VARCOEF = 3,        /* sigma = diag(1+x^2/2, 1+y^2/2), b = (y,-x),
                              c = -(1+x^2+y^2), u = e^x cos 2y + 1                      */
  PDDS_LUT = 4,            /* diagonal sigma, b, c, f, grad u and g served from tables  */
  PDDS_CIRCLE_POISSON = 5, /* u = r^2 sin(3 theta) + cos x, sigma = sqrt2 I, f = -Lap u  */
  PDDS_ROBIN_POISSON = 6   /* BVPs/EDPs/poisson_3.hpp: Lap u + f = 0 with
                              u = sin(pi(0.23x + 0.49y)) + cos(pi(0.331x + 0.667y)),
                              Dirichlet g = u except on the Robin side p[0] (one of
                              N 1, S 2, E 4, W 8, or 0 for none; the reference's
                              Stopping_mix takes W), where du/dn - varphi u = psi with
                              varphi = -2 + sin(pi y): paths reflect there with
                              Lepingle's step and carry the local-time terms.
                              Knots on the Robin side keep B = g as in the
                              reference's boundary shortcut.  MIXED and FP64
                              modes, rectangular layouts.                        */
} pdds_problem_kind;

typedef struct {
  int32_t kind;       /* pdds_problem_kind                                   */
  int32_t use_cv;     /* 1: control variate xi with the exact gradient       */
  double p[8];        /* kind parameters                                     */
} pdds_problem_desc;

pdds_status pdds_problem_set(pdds_ctx* ctx, const pdds_problem_desc* desc);

/* Tables of the PDDS_LUT problem (replaces the reference's LUT coefficient
 * sources: GSL splines, BVPs/EDPs/Monegros_Helmhotz.hpp:50-61, and the CUDA
 * LUT texture, BVPs/LUT2.cuh:11-92).  coef is host memory [ny][nx][8] FP32,
 * fields (sigma11, sigma22, b1, b2, c, f, du/dx, du/dy) on the grid
 * x_i = bounds[0] + i (bounds[2]-bounds[0])/(nx-1), y_j likewise; g is
 * [ny][nx] FP32 boundary values.  Copied to the device.  The FP64 and
 * replay forms sample the tables with bicubic Catmull-Rom interpolation,
 * clamped at the table edges.  The MIXED (FP32) form samples by problem
 * p[0]: 0 the cubic B-spline through the nodes (coefficients prefiltered
 * here, in FP64, held as two float4 textures; four linearly filtered fetches
 * per texture and sample), 1 the Catmull-Rom nodes (16 node loads), 2
 * bilinear interpolation of the nodes (one filtered fetch per texture).
 * All pass through the nodes; between them they differ by interpolation
 * error, O(node spacing^3) for the cubics and O(node spacing^2) for the
 * bilinear one, and the texture filter's 8-bit blend fractions add at most
 * 1/512 of the difference of neighbouring values. */
pdds_status pdds_problem_set_lut(pdds_ctx* ctx, const float* coef, const float* g, int32_t nx, int32_t ny,
                                 const double bounds[4]);

/* ---------------------------------------------------------------- layout
 * Rectangular domain [SW, NE] split into nsub x nsub subdomains with nnode
 * knots per interface segment (INTERSECTIONS_YES numbering) and the
 * reference's stencils (STEN_ELONG = 0.5).  fac[kind] is the RBF shape c of a
 * stencil side of that kind (c2[kind] in Stencil::Compute_ipsi). */
typedef struct {
  double sw[2], ne[2];
  int32_t nsub;
  int32_t nnode;
  double fac[4];
} pdds_layout_desc;

typedef struct {
  int32_t nknots;        /* K                                              */
  int32_t nboundary;     /* knots on the domain boundary (B = g, no paths) */
  int32_t nstencils;     /* distinct stencils                              */
  int32_t nsides;        /* distinct stencil sides                         */
  int32_t nshapes;       /* distinct side shapes (translates share one)    */
  int32_t max_side;      /* largest side                                   */
  int64_t nnz;           /* entries of G (rows of all knots)               */
  int64_t h2d_bytes;     /* bytes this call copied from host to device      */
} pdds_layout_info;

pdds_status pdds_layout_build(pdds_ctx* ctx, const pdds_layout_desc* desc, pdds_layout_info* info);

/* Disk of the given radius centred at the origin, split into nrings x
 * nsectors annular sectors (a CircleMesh; the reference's Circle* meshes are
 * empty stubs, its layouts are rectangular).  Knots on the arcs between
 * rings and the rays between sectors, nnode per segment, none at the centre;
 * stencils are the polar rectangles of the subdomains next to a knot's
 * interfaces, sides elongated by half a segment as on rectangles; the RBF
 * shape of a side is kappa[kind] times its knot spacing (chord).  The central
 * ring is one disk subdomain (no rays): the stencil of a knot on its boundary
 * is the disk of radius 2R/nrings with one periodic side.  A knot shared by
 * two sides of a stencil gets both sides' weights (dup_sum is implied: the
 * overwrite of the rectangular reference leaves cond(I + G) ~100 here but
 * biases G).  MIXED and FP64 modes (no replay form); problems with
 * sigma = sqrt2 I (PDDS_POISSON_SINCOS,
 * PDDS_CIRCLE_POISSON).  pdds_layout_stencil reports rect = {rho0, phi0,
 * rho1, phi1} with sides N = outer arc, S = inner arc, E = ray at phi1,
 * W = ray at phi0. */
typedef struct {
  double radius;
  int32_t nrings;
  int32_t nsectors;
  int32_t nnode;
  double kappa[4];
  /* ring widths: ring i (i = 0 the central disk) is ring_ratio^i times as
   * wide as the central disk's radius (0 or 1: equal widths R / nrings).  A
   * ratio below 1 gives a boundary-layer mesh whose thin outer rings hold
   * knots that leave their stencils in a step while knots of the wide inner
   * rings need thousands at the same h. */
  double ring_ratio;
} pdds_circle_desc;

pdds_status pdds_layout_build_circle(pdds_ctx* ctx, const pdds_circle_desc* desc, pdds_layout_info* info);
/* Knot i's position (the one the reference hands to its worker) and the
 * hand-out order of the reference's server loop. */
pdds_status pdds_layout_knots(pdds_ctx* ctx, double* x, double* y, int32_t* order);
/* CSR structure of G: row_ptr[K+1], col[nnz] (columns sorted per row). */
pdds_status pdds_layout_csr(pdds_ctx* ctx, int64_t* row_ptr, int32_t* col);
/* Stencil of knot k as the reference builds it: rect {x0,y0,x1,y1}, side kinds
 * and sizes (N,S,E,W), side knot indices packed [4][maxn]. */
pdds_status pdds_layout_stencil(pdds_ctx* ctx, int32_t knot, double* rect, int32_t* kinds,
                                int32_t* sizes, int32_t* idx, int32_t maxn);

/* A stencil built by the caller, as the reference's Stencil::Init and
 * Compute_ipsi receive it (Meshes/stencil.hpp:57-98, Meshes/stencil.cpp:11-85,
 * 115-243): the rectangle stencil_parameters = {x0, y0, x1, y1} and, per side
 * N, S, E, W, the knot indices and positions in the caller's order (a
 * repeated index keeps its last position and consecutive repeats are
 * dropped, as Init does) and the side's RBF shape c2.  n[d] = 0: no side.
 * A side's knots lie on that side of the rectangle, in increasing order
 * along it (the reference's interfaces list them so); at most 160 per side. */
typedef struct {
  double rect[4];
  int32_t n[4];
  const int32_t* index[4];
  const double* x[4];
  const double* y[4];
  double c2[4];
} pdds_stencil_desc;

/* Replaces the context's layout with caller-built knots and stencils (the
 * reference's worker receives a knot and builds its stencil itself,
 * PDDAlgorithms/PDDSparseGM.cpp:795-848, Compute_Stencil :1845-2041): knot i
 * sits at (x[i], y[i]) with stencil st[i] and draws the Philox knot word
 * knot_id[i] (NULL: i), so a knot of a built layout can be re-run alone on
 * its own random stream.  domain = {x0, y0, x1, y1} is the problem's
 * rectangle (the stencil's global_parameters): exits on it score g, and a
 * knot on it takes B = g.  G's columns are the caller's knot indices;
 * pdds_solve_interface needs them in [0, nknots), and subdomain solves need a
 * layout from pdds_layout_build.  Estimation then runs in every mode; the
 * replay mode's ipsi_override lists the knots in index order. */
pdds_status pdds_stencils_set(pdds_ctx* ctx, const double domain[4], int32_t nknots, const double* x,
                              const double* y, const int32_t* knot_id, const pdds_stencil_desc* st,
                              pdds_layout_info* info);

/* ---------------------------------------------------------------- estimate */
typedef enum {
  PDDS_MODE_REPLAY_FP64 = 0, /* bit-exact replay of the CPU restatement          */
  PDDS_MODE_FP64 = 1,        /* plain FP64 GPU form                               */
  PDDS_MODE_MIXED = 2        /* FP32 paths, FP64 accumulation and factorisation   */
} pdds_mode;

typedef struct {
  int32_t mode;          /* pdds_mode                                           */
  int32_t npaths;        /* paths per knot (N)                                  */
  double h;              /* Euler-Maruyama step                                 */
  uint64_t seed;         /* Philox key                                          */
  uint32_t instance;     /* Philox counter word 3 (independent replicas)        */
  int32_t dup_sum;       /* 0: G_return_withrep overwrite (reference), 1: sum   */
  int32_t want_var;      /* 1: compute G_var                                    */
  int32_t bins_per_gap;  /* MIXED: exit bins per knot spacing (0 = default 16)  */
  int64_t max_steps;     /* per path (0 = 1e6); exceeded -> PDDS_ERR_STEP_LIMIT */
  /* REPLAY only, optional: RBF inverse matrices per knot, packed knot by knot
   * in hand-out order, sides N,S,E,W, each n x n row-major with element
   * (j,i) = ipsi(j,i) of the reference; NULL = factorise on the device. */
  const double* ipsi_override;
  int64_t ipsi_override_len;
  /* 1: per-knot step h_k = min(h, (d_k / (2 * 0.5826 * |N^T sigma(x_k)|))^2) for
   * knots at distance d_k <= -1e-4 inside their stencil, the adaptive step of
   * the reference's iterative solvers (PDDSparseGM.cpp:4026-4028) */
  int32_t adaptive_h;
  /* MIXED and FP64 only, 1: Richardson extrapolation in the step.  Every path
   * is a pair driven by one Brownian motion, a fine level of step h/2 and a
   * coarse level of step h; G and B estimate 2 E[fine] - E[coarse], which
   * cancels the O(h) bias of the Gobet-shifted scheme.  Both levels' steps
   * count as path steps.  G_var then omits the fine/coarse covariance. */
  int32_t richardson;
  /* 1: keep the RBF factorisation and tables of the previous call on this
   * layout (they depend only on the layout and bins_per_gap); 0: recompute */
  int32_t reuse_tables;
  /* MIXED only, 1: variance-adaptive paths per knot, the rule of the
   * reference's Compute_h_N (PDDSparseGM.cpp:4338-4395): a pilot of npaths
   * paths per knot estimates the variance V_k of the knot's score, then
   * N_k = 4 V_k / (0.66666 target_stderr)^2 rounded up to a multiple of 256
   * and clamped to [npaths, npaths_max]; knots continue with paths
   * npaths .. N_k-1 of the same Philox streams (pdds_estimate_knot_paths). */
  int32_t adaptive_n;
  int32_t npaths_max;
  double target_stderr;
  /* MIXED only: threads per CTA of the path kernel, 128 or 256; 0 = by
   * layout size (128 from 8192 Monte Carlo knots).  Results do not depend
   * on it beyond FP32 summation order. */
  int32_t cta_threads;
  /* MIXED only, 1: the launch the persistent refill replaces, for
   * comparison -- one CTA per work item (not a CTA per SM slot pulling
   * items) and the knots in layout order (not heaviest first).  Same
   * results up to FP32 summation order. */
  int32_t plain_launch;
  /* MIXED only, 1: count the paths by their exit step counts for
   * pdds_estimate_step_histogram (two shared-memory atomics per finished
   * path pair; 0 leaves the histogram empty) */
  int32_t step_histogram;
  /* 1: per-knot diagnostic sums of the reduction for
   * pdds_estimate_diagnostics (all modes; MIXED on rectangular stencils) */
  int32_t diagnostics;
  /* Only the knots with paths at hand-out positions [knot_first,
   * knot_first + knot_count) (knot_count 0: to the last); the others' rows
   * and B are left zero (boundary knots always take B = g).  A knot's
   * results depend only on its own Philox streams, so a run split into
   * ranges gives every knot the values of one whole run: bit for bit in the
   * replay mode, up to summation order in FP64 and MIXED (a knot's paths
   * may be split into other chunks).  The unit of checkpoint/resume.  Not
   * with adaptive_n, batches or the autotuner. */
  int32_t knot_first;
  int32_t knot_count;
} pdds_estimate_desc;

typedef struct {
  int64_t path_steps;    /* Euler-Maruyama steps to the shifted exit     */
  int64_t paths;         /* simulated paths                              */
  int64_t exits_global;  /* exits on the domain boundary                 */
  int64_t exits_stencil; /* exits on interior stencil sides              */
  double ms_setup;       /* factorisation and tables                     */
  double ms_paths;       /* path kernels and reduction                   */
  int32_t kernel_launches;
  int32_t cta_threads;   /* MIXED: threads per CTA of the path kernel    */
  int64_t h2d_bytes;     /* bytes this call copied host -> device        */
  int64_t d2h_bytes;     /* bytes this call copied device -> host        */
} pdds_estimate_info;

/* Runs the estimation for all knots and keeps G and B on the device.  Any of
 * the host output pointers may be NULL: val[nnz], var[nnz] (needs want_var),
 * B[K], BB[K] (mean of the squared score, as Reduce_Analytic's BB).  val and
 * var may be fresh, never-touched host memory: the call touches their pages
 * while the device runs the paths, before the copies fill them. */
pdds_status pdds_estimate(pdds_ctx* ctx, const pdds_estimate_desc* desc, double* val, double* var,
                          double* B, double* BB, pdds_estimate_info* info);
/* Paths per knot of the last pdds_estimate (npaths[K]; 0 for boundary knots
 * and for knots outside its knot range). */
pdds_status pdds_estimate_knot_paths(pdds_ctx* ctx, int32_t* npaths);
/* Euler-Maruyama steps per knot of the last MIXED pdds_estimate, summed
 * over its paths (both levels of a Richardson pair): steps[K]. */
pdds_status pdds_estimate_knot_steps(pdds_ctx* ctx, int64_t* steps);
/* Exit step counts of the last MIXED pdds_estimate run with step_histogram:
 * hist[b] paths (each level of a Richardson pair counts) took between 2^b
 * and 2^(b+1) - 1 steps, b = 0 .. 31. */
pdds_status pdds_estimate_step_histogram(pdds_ctx* ctx, int64_t* hist);

/* Per-knot diagnostic sums of Reduce_Analytic (the sums[] of
 * Solvers/EMFKACSolver.hpp:14-47, accumulated at :542-558 and turned into
 * moments by Update, :656-685), over the knot's paths, with
 * phi = Z + Y g(X_tau) the score without the control variate and xi the
 * control variate, at the end of the linear leg (exit by the Gobet-shifted
 * rule) and of the sublinear leg (the reference's continuation to the first
 * step outside the stencil; the replay mode runs it, the FP64 and MIXED
 * modes do not, and their sublinear sums repeat the linear ones).  tau is
 * the elapsed time, steps x h (the reference starts its clock at +infinity
 * and counts down, so its tau sums are infinite).  The reference's enum
 * gives xi and xi^2 one slot (XiLinear2 = XiLinear); here they have two.
 * With Richardson pairs each pair adds 2 x fine - coarse of phi and xi (the
 * pair's estimate) and the fine level's tau.  MIXED sums FP32 values in
 * FP64 shared-memory atomics; the replay mode sums in path order, in FP64,
 * like the reference's serial loop. */
enum {
  PDDS_DIAG_SCORE = 0,        /* sum phi                       (ScoreLinear)     */
  PDDS_DIAG_SCORE2 = 1,       /* sum phi^2                     (ScoreLinear2)    */
  PDDS_DIAG_XI = 2,           /* sum xi                        (XiLinear)        */
  PDDS_DIAG_XI2 = 3,          /* sum xi^2                      (XiLinear2)       */
  PDDS_DIAG_SCORE_VR = 4,     /* sum (phi + xi)                (ScoreLinearVR)   */
  PDDS_DIAG_SCORE_VR2 = 5,    /* sum (phi + xi)^2              (ScoreLinearVR2)  */
  PDDS_DIAG_XI_SCORE = 6,     /* sum xi phi                    (XiScoreLinear)   */
  PDDS_DIAG_TAU = 7,          /* sum tau                       (tauLinear)       */
  PDDS_DIAG_SUB = 8,          /* + 0..7: the same sums of the sublinear leg      */
  PDDS_DIAG_RNG = 16,         /* normal variates drawn, 2 per step (RNGCalls)    */
  PDDS_DIAG_PATHS = 17,       /* paths summed (a Richardson pair counts once)    */
  PDDS_DIAG_N = 18
};
/* The diagnostic sums of the last pdds_estimate (or pdds_estimate_knot) run
 * with diagnostics = 1: sums[K * PDDS_DIAG_N], knot k's at k * PDDS_DIAG_N
 * (zeros for knots without paths). */
pdds_status pdds_estimate_diagnostics(pdds_ctx* ctx, double* sums);

/* One knot as EMFKACSolver::Solve_OMP_Analytic computes it
 * (Solvers/EMFKACSolver.hpp:711-729): from X0 = (x0, y0) inside the stencil
 * st of the problem's rectangle domain, with the paths, step and weight rule
 * of desc, the knot's G row -- G_j (sorted knot indices, the order of
 * G_return_withrep), G, G_var (want_var, or the replay mode) -- and B, BB.
 * A knot on the domain boundary takes B = g(X0), BB = B^2 and an empty row,
 * as the reference does.  knot_id is the Philox knot word (the knot's index
 * in its layout gives the stream pdds_estimate draws for it).  The arrays
 * hold max_nnz entries; *nnz receives the row length (PDDS_ERR_INVALID when
 * it exceeds max_nnz).  Replaces the context's layout by this one knot
 * (pdds_stencils_set). */
pdds_status pdds_estimate_knot(pdds_ctx* ctx, const double domain[4], double x0, double y0, int32_t knot_id,
                               const pdds_stencil_desc* st, const pdds_estimate_desc* desc, int32_t* G_j,
                               double* G, double* G_var, int32_t max_nnz, int32_t* nnz, double* B, double* BB,
                               pdds_estimate_info* info);

/* Autotuner of the MIXED path kernel (no counterpart in the reference):
 * times the kernel on a sample of knots of the current layout and problem
 * for candidate launch shapes -- persistent CTAs per SM (1 .. the occupancy
 * limit) and paths per work item (256 .. npaths) -- and keeps the fastest
 * for later pdds_estimate calls with the same problem kind and Richardson
 * setting.  Lanes refill from the work item's path counter the moment their
 * path exits (a refill threshold of one lane), so the refill needs no knob.
 * sample_knots <= 0 times the whole layout; a smaller sample runs on a grid
 * scaled by the sampled fraction of knots, so each CTA sees as many work
 * items as in the full run.  desc->cta_threads = 128 or 256 keeps that
 * block size and searches only the other shape parameters; 0 searches both
 * block sizes.  With desc->adaptive_n set and a variance-adaptive estimate
 * of the same problem kind run before on this layout, it also times that
 * estimate's continuation
 * (its work items after the pilot, each knot's paths N0 .. N_k) at both
 * block sizes, then at 2048 .. 16384 paths per item (4096 untuned), and
 * keeps the fastest for the continuation of later adaptive estimates: those
 * items hold the long paths, and a uniform sample does not show their tail.  The tuned shape is forgotten when a new layout or batch
 * is built.  Overwrites the device results of the last estimate. */
typedef struct {
  int32_t blocks_per_sm;     /* chosen persistent CTAs per SM            */
  int32_t paths_per_item;    /* chosen paths per work item (knot, chunk) */
  int32_t candidates;        /* launch shapes timed                      */
  int32_t sample_knots;      /* knots in the timing sample               */
  double best_ms;            /* sample time with the chosen shape        */
  double default_ms;         /* sample time with the default shape       */
  int32_t cta_threads;       /* chosen threads per CTA (128 or 256)      */
  int32_t continuation_threads; /* adaptive continuation's threads per CTA
                                   (0: not timed)                        */
  double continuation_ms[2]; /* its time at 128 and 256 threads (4096
                                paths per item)                          */
  int32_t continuation_paths_per_item; /* its chosen paths per item      */
} pdds_tune_info;

pdds_status pdds_autotune(pdds_ctx* ctx, const pdds_estimate_desc* desc, int32_t sample_knots,
                          pdds_tune_info* info);

/* ---------------------------------------------------------------- solve */
typedef enum {
  PDDS_SOLVE_BICGSTAB_FP64 = 0, /* Jacobi-preconditioned BiCGSTAB, FP64 (reference) */
  PDDS_SOLVE_GMRES_FP32_IR = 1  /* FP32 GMRES(m) inside FP64 iterative refinement   */
} pdds_solve_method;

typedef struct {
  int32_t method;
  int32_t restart;       /* GMRES(m), 2 <= m <= 40 (0 = 20) */
  int32_t max_iter;      /* inner iterations per call / refinement step */
  int32_t max_refine;    /* FP64 refinement steps */
  double tol;            /* relative residual in FP64 */
  /* GMRES over the whole GPU (systems of 4096 knots and more): polls of a
   * grid-barrier wait before it gives up and the solve returns
   * PDDS_ERR_TIMEOUT (0 = 2^24, about a second; >= 0) */
  int32_t barrier_poll_limit;
  /* PDDS_SOLVE_GMRES_FP32_IR: PDDS_GMRES_PIPELINED (0, the default) keeps
   * G V beside the basis and applies each step's product to the not yet
   * orthogonalised vector, one group barrier per Arnoldi step;
   * PDDS_GMRES_CLASSICAL forms the basis vector first (two barriers) */
  int32_t gmres_form;
  /* GMRES over the whole GPU: its CTAs (0 = one per SM).  Each Arnoldi step
   * is a chain of latency-bound phases over a few dozen rows per CTA; fewer
   * CTAs make the barrier and the reductions over the CTAs' partials shorter */
  int32_t grid_ctas;
} pdds_solve_desc;

#define PDDS_GMRES_PIPELINED 0
#define PDDS_GMRES_CLASSICAL 1

typedef struct {
  int32_t iterations;
  int32_t refinements;
  double rel_residual;
  double ms;
  int32_t kernel_launches;
  int64_t h2d_bytes;     /* bytes this call copied host -> device */
  int64_t d2h_bytes;     /* bytes this call copied device -> host */
} pdds_solve_info;

/* Solves (I + G) u = B with the G and B of the last pdds_estimate. */
pdds_status pdds_solve_interface(pdds_ctx* ctx, const pdds_solve_desc* desc, double* u,
                                 pdds_solve_info* info);

/* ---------------------------------------------------------------- batch
 * No counterpart in the reference, whose driver solves one problem per run
 * (PDDSparseGM::Solve, PDDAlgorithms/PDDSparseGM.cpp:691-851).  Many
 * independent instances of one problem kind (the kind and use_cv of
 * pdds_problem_set) with their own layouts and parameters run as one
 * sequence: one RBF factorisation launch, one path-kernel launch over the
 * knots of all instances, and one launch of the cluster GMRES that solves
 * every instance's (I + G) u = B with its own convergence test.  The layout
 * of the context becomes the block-diagonal union of the instances (instance
 * i's knots follow instance i-1's).  Instance i draws from Philox instance
 * word estimate.instance + i with its own knot numbering, so its random
 * stream is the one of a single-layout run of that instance. */
typedef struct {
  pdds_layout_desc layout; /* the instance's domain, grid and RBF shapes */
  double p[8];             /* the instance's problem parameters            */
  /* the instance's Euler-Maruyama step (0: the run's estimate.h).  The
   * step's bias scales with sqrt(h) over the subdomain size, so instances
   * with finer grids need smaller steps for the same accuracy; the steps per
   * path stay the same when h scales with the square of the subdomain size. */
  double h;
} pdds_instance_desc;

typedef struct {
  int32_t ninstances;
  int32_t max_knots;     /* knots of the largest instance */
  int64_t nknots;        /* knots of all instances        */
  int64_t nnz;           /* G entries of all instances    */
} pdds_batch_info;

pdds_status pdds_batch_build(pdds_ctx* ctx, const pdds_instance_desc* inst, int32_t n, pdds_batch_info* info);

typedef struct {
  pdds_estimate_desc estimate; /* mode must be PDDS_MODE_MIXED                */
  pdds_solve_desc solve;       /* method must be PDDS_SOLVE_GMRES_FP32_IR    */
  int32_t use_graph;           /* 1: capture the sequence in a CUDA graph on
                                  the first run and replay it while the batch
                                  and the descriptor stay the same          */
  /* the instances run in this many consecutive groups of the order given to
   * pdds_batch_build (0 = 16, at most the instance count): one path-kernel
   * launch per group, and the solves of a group, on a second stream of
   * higher priority, overlap the next group's paths, so an instance
   * completes when its group does; instances given smallest first complete
   * soonest on average */
  int32_t waves;
} pdds_batch_run_desc;

typedef struct {
  double ms;                   /* device time of the whole sequence          */
  int64_t path_steps;
  int64_t paths;
  int64_t exits_global;
  int64_t exits_stencil;
  int32_t kernel_launches;     /* kernels in the sequence                    */
  int32_t graph_replayed;      /* 1: this run replayed a captured graph      */
  int32_t max_iterations;      /* over instances                             */
  int32_t unconverged;         /* instances that missed the tolerance        */
  double max_rel_residual;
} pdds_batch_run_info;

pdds_status pdds_batch_run(pdds_ctx* ctx, const pdds_batch_run_desc* desc, pdds_batch_run_info* info);

/* Results of instance i after pdds_batch_run, in the instance's own knot
 * numbering (the one pdds_layout_build of its layout gives).  Any pointer
 * may be NULL; x, y, u, B hold nknots values.  latency_ms: time from the
 * start of the sequence until the instance's solution was complete. */
pdds_status pdds_batch_instance(pdds_ctx* ctx, int32_t i, int32_t* nknots, double* x, double* y, double* u,
                                double* B, int32_t* iterations, double* rel_residual, double* latency_ms);

/* ---------------------------------------------------------------- subdomain solve
 * Interior solution of every subdomain of a rectangular layout from the
 * interface solution (the reference hands each subdomain's four interfaces
 * to an Octave spectral solver, Subdomain::Solve, Meshes/subdomain.cpp:80-122).
 * For problems whose operator is Lap + c with constant c (PDDS_POISSON_SINCOS,
 * PDDS_MONEGROS, PDDS_HELMHOLTZ): one CTA per subdomain solves the 5-point
 * finite-difference problem on an m x m interior grid (2 <= m <= 64) by the
 * sine transform, in FP64, with Dirichlet data = the interface solution
 * interpolated along each edge (cubic Lagrange through its knots) and g on
 * the domain boundary.  Table-served problems (PDDS_LUT, including the
 * tables of pdds_semilinear_tables) have variable coefficients
 * sigma11^2/2 v_xx + sigma22^2/2 v_yy + b.grad v + c v + f = 0 sampled at the
 * grid nodes, central differences, solved by BiCGSTAB preconditioned with the
 * sine-transform solve of the subdomain-mean operator (relative residual
 * 1e-12, at most 200 iterations, else PDDS_ERR_NOT_CONVERGED).  u: interface
 * values u[K] (host), or NULL for those of the last pdds_solve_interface.
 * out[nsub*nsub][m][m]: subdomain s = column + nsub * row, value [j][i] at
 * x = x0 + (i+1) lx/(m+1), y = y0 + (j+1) ly/(m+1) of its rectangle
 * [x0, x0+lx] x [y0, y0+ly].  The solution with its edge values is also kept
 * on the device as one grid of nsub (m+1) + 1 nodes per side for
 * pdds_semilinear_tables. */
pdds_status pdds_subdomain_solve(pdds_ctx* ctx, int32_t m, const double* u, double* out);

/* Semilinear outer loop, one Newton step (Solve_SemiLin_numVR,
 * PDDSparseGM.cpp:3833-4080, with the equation of
 * BVPs/EDPs/Semilinear_u3_VR.hpp): Lap u - u^3 + F = 0 on the unit square,
 * u = a + sin(pi x) sin(pi y) (a = 1.1 in the reference), g = a on the
 * boundary, F = 2 pi^2 sin(pi x) sin(pi y) + u^3.  Builds, on the device, the
 * tables of the problem linearised around the iterate u_k -- sigma = sqrt2 I,
 * b = 0, c = -3 u_k^2, f = F + 2 u_k^3 and grad u_k for the control variate
 * (EquationSM_c_LUT, EquationSM_f_LUT, EquationSM_grad_LUT) -- on the grid of
 * nsub (m+1) + 1 nodes per side, and makes that table-served problem the
 * context's problem.  u_k is the last pdds_subdomain_solve (from_solution = 1,
 * same m) or the constant u0 (the reference's first iteration: c = -3.63,
 * f = F + 2.662 at u0 = 1.1).  A Newton iteration is then pdds_estimate,
 * pdds_solve_interface and pdds_subdomain_solve (Solve_Subdomains_SemiLin).
 *
 * equation = PDDS_OUTER_LINEAR_SHIFT gives instead one step of the
 * reference's fixed-point loop for a linear problem (Solve_Iterative_numVR,
 * PDDSparseGM.cpp:4081-4336, with BVPs/EDPs/Salou_Iterative.hpp, main_LinLoop.cpp):
 * Lap u + c2 u + F = 0 on any rectangle of the layout, u = sin(2 pi x + 1/2)
 * cos(pi^2 (x + y)), g = u, F = -Lap u - c2 u, split with the shift alpha
 * and rescaled by k (c2 = 20, alpha = 22, k = 9 in the reference):
 * sigma = sqrt(2/k) I, b = 0, c = (c2 - alpha)/k, f = (F + alpha u_k)/k and
 * grad u_k for the control variate (EquationLI_sigma, EquationLI_c_LUT,
 * EquationLI_f_LUT, EquationLI_grad_LUT).  The reference's first iteration
 * (Solve with the analytic EquationLI_f) is u0 = 0.  The error's component on
 * a Dirichlet eigenfunction of -Lap with eigenvalue lambda is multiplied by
 * alpha / (lambda + alpha - c2) per step, so the loop converges only when the
 * domain's lowest eigenvalue exceeds c2 (2 pi^2 / L^2 on a square of side L:
 * L < 0.9935 for c2 = 20). */
#define PDDS_OUTER_NEWTON_U3 0
#define PDDS_OUTER_LINEAR_SHIFT 1
typedef struct {
  int32_t m;              /* interior grid points per subdomain side (2..64)   */
  int32_t from_solution;  /* 1: around the last subdomain solve; 0: around u0 */
  int32_t use_cv;         /* control variate with grad u_k                     */
  int32_t equation;       /* PDDS_OUTER_NEWTON_U3 or PDDS_OUTER_LINEAR_SHIFT   */
  double u0;              /* constant first iterate                            */
  double a;               /* NEWTON_U3: u = a + sin(pi x) sin(pi y)            */
  double c2, alpha, k;    /* LINEAR_SHIFT: reaction, shift, time rescale (> 0) */
} pdds_semilinear_desc;
pdds_status pdds_semilinear_tables(pdds_ctx* ctx, const pdds_semilinear_desc* desc);

/* ---------------------------------------------------------------- self-checks
 * No counterpart in the reference (its increments come from Boost's
 * mt19937 + normal_distribution, Integrators/FKACIntegrator.hpp:15-19, and
 * its exponentials from libm, BVPs/BVP.hpp:84-87).  The library's own
 * generator and FP64 functions, evaluated on given inputs so that they can be
 * held against published known answers and libm: on the device (device >= 0,
 * compiled exactly as the path kernels use them) or on the host (device < 0,
 * the code the CPU restatement shares).  err, if given, receives a message of
 * at most err_len bytes.
 *
 * pdds_check_philox: out[4i..4i+3] = Philox-4x32-10 (Salmon et al., SC'11) of
 * the counter ctr[4i..4i+3] under the key (key[2i], key[2i+1]).  The path
 * kernels put (step pair, path, knot, instance) in the counter and the seed's
 * low and high words in the key.  form PDDS_PHILOX_PORTABLE is the generator of
 * the replay and FP64 kernels (host and device), PDDS_PHILOX_ROUND_KEYS the
 * MIXED kernel's form with the key schedule passed as kernel parameters
 * (device only). */
#define PDDS_PHILOX_PORTABLE 0
#define PDDS_PHILOX_ROUND_KEYS 1
pdds_status pdds_check_philox(int device, int32_t form, const uint32_t* ctr, const uint32_t* key, int32_t n,
                              uint32_t* out, char* err, int32_t err_len);
/* pdds_check_portable_math: out[i] = fn(x[i]) with the portable FP64
 * functions of the replay kernels (no FMA contraction); for the Box-Muller
 * pair, the bits of x[i] hold the two Philox words (low word = the radius
 * word) and out[i] is the first or second normal. */
#define PDDS_FN_EXP 0
#define PDDS_FN_LOG 1
#define PDDS_FN_SIN 2
#define PDDS_FN_COS 3
#define PDDS_FN_BOX_MULLER_Z0 4
#define PDDS_FN_BOX_MULLER_Z1 5
pdds_status pdds_check_portable_math(int device, int32_t fn, const double* x, int32_t n, double* out, char* err,
                                     int32_t err_len);

/* ---------------------------------------------------------------- allocation-free solve
 * No counterpart in the reference.  For callers that cannot let a library
 * allocate GPU memory (memory owned by another allocator, serving loops where
 * cudaMalloc/cudaFree would synchronise or stall, foreign-language hosts that
 * only lend device buffers): solves (I + G) u = B with the FP64 BiCGSTAB of
 * pdds_solve_interface on caller-owned DEVICE buffers -- G in CSR without the
 * unit diagonal (row_ptr[K+1], col[nnz], val[nnz]), B[K], u[K] -- and takes
 * its work vectors from a static device array instead of allocating.
 * K must not exceed PDDS_STATIC_SOLVE_MAX_K.  The array (6.3 MB) is held on
 * every GPU that loads the library until the process exits; all calls share
 * it, so calls that overlap on the GPU race.  The first call on a device
 * looks up the array's address; make it before any stream capture on that
 * device.  The address is kept for the life of the process: after a
 * cudaDeviceReset of a device, neither this entry point nor any other of the
 * library may be used on it.  stream may be NULL (legacy default stream);
 * err, if given, receives a message of at most err_len bytes. */
#define PDDS_STATIC_SOLVE_MAX_K 131072
pdds_status pdds_solve_bicgstab_static(int device, int32_t K, int64_t nnz, const int64_t* row_ptr,
                                       const int32_t* col, const double* val, const double* B,
                                       double* u, double tol, int32_t max_iter, void* stream,
                                       int32_t* iterations, double* rel_residual, char* err,
                                       int32_t err_len);

#ifdef __cplusplus
}
#endif
#endif /* PDDS_H */
