/*
 * helmholtz_gb300.h -- C ABI of the GB300 (sm_103a) implicit-boundary-integral
 * Helmholtz hot path.
 *
 * Everything here is plain C: pointers, sizes and status codes, no exits.
 * Every call returns HZ_OK (0) or a negative HZ_ERR_* code; hz_last_error()
 * gives the message of the last failure on the calling thread.
 *
 * Memory.  Arrays marked "where" are host pointers when where == HZ_HOST and
 * device pointers (on the operator's device) when where == HZ_DEVICE.  The
 * operator owns all device memory it allocates; host buffers stay owned by
 * the caller, as in the reference, whose routines take caller-allocated
 * arrays.  Calls on one operator are stream-ordered on its stream and must
 * not be made concurrently from several threads.
 *
 * Layout.  Grids are contiguous (N+1)^3 FP64 arrays, node (i,j,k) at
 * ((i*(N+1))+j)*(N+1)+k with coordinates (x,y,z) = (int_l + j*H,
 * int_l + i*H, int_l + k*H): the flattening of the reference's ragged
 * double*** grids (large3Dexample2.c:378-403,428-437).  Tube points are in
 * the reference's lexicographic (i,j,k) order (large3Dexample2.c:548-597).
 * Interleaved xyz arrays hold 3 doubles per point.  Complex vectors are
 * passed as separate real and imaginary arrays, as the reference does
 * (density / densityimg).
 */
#ifndef HELMHOLTZ_GB300_H
#define HELMHOLTZ_GB300_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define HZ_API __attribute__((visibility("default")))
#else
#define HZ_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

#define HZ_OK 0
#define HZ_ERR_ARG (-1)          /* invalid argument or size                    */
#define HZ_ERR_CUDA (-2)         /* CUDA runtime error (no device, OOM, ...)    */
#define HZ_ERR_STATE (-3)        /* call out of order (e.g. no tube built yet)  */
#define HZ_ERR_GRID (-4)         /* projected point outside the grid; the
                                    reference exits at interpolate3D.c:35       */
#define HZ_ERR_NONFINITE (-5)    /* NaN/Inf in an input or result               */
#define HZ_ERR_BREAKDOWN (-6)    /* Krylov breakdown (zero denominator)         */
#define HZ_ERR_DEVICE_WAIT (-7)  /* a bounded device-side wait gave up          */

#define HZ_HOST 0
#define HZ_DEVICE 1

/* Arithmetic of a matvec or solve. */
#define HZ_PREC_F64 0         /* plain FP64 everywhere                                  */
#define HZ_PREC_F32 1         /* FP32 pair sweep (tile-local origins; phase k rho reduced
                                 with a split k/(2 pi), or passed straight to the SFU
                                 sin/cos: hz_set_phase_mode), FP64 inner products        */
#define HZ_PREC_F32_REFINED 2 /* FP32 inner solves inside FP64 iterative refinement whose
                                 residual b - A x uses the FP64 sweep                   */

/* Krylov method. */
#define HZ_BICG 0     /* complex BiCG with A and A^H: BICGSTAB.c:5-339 (CompBiCG)  */
#define HZ_BICGSTAB 1 /* complex BiCGSTAB (the reference's real BiCGSTAB,
                         large3Dexample2.c:2265-2477, in complex arithmetic)      */
#define HZ_GMRES 2    /* restarted GMRES(restart), FP64 vectors, classical Gram-
                         Schmidt applied twice; A products only (no A^H)        */

/* Evaluation layers. */
#define HZ_SINGLE_LAYER 0 /* NeumannTest, large3Dexample2.c:1810-1824 */
#define HZ_DOUBLE_LAYER 1 /* the Dirichlet matrix's kernel off the surface */
#define HZ_COMBO_LAYER 2  /* Combo formulation: dG/dn_y - i eta G, Combo_NeumannTest
                             (large3Dexample2.c:1907-2059); needs hz_set_combo */

/* Boundary data kinds for hz_rhs_point_source. */
#define HZ_RHS_POINT_DIRICHLET 0 /* g = e^{ik|x-s|}/(4 pi |x-s|)                        */
#define HZ_RHS_POINT_NEUMANN 1   /* dg/dn along the outward normal -n                   */
#define HZ_RHS_MONOPOLE_NEUMANN 2 /* cal_partialu/img, large3Dexample2.c:4778,4840      */
#define HZ_RHS_MONOPOLE_DIRICHLET 3 /* cal_u/cal_uimg, large3Dexample2.c:4642,4724     */

/* Problem parameters: the reference's compile-time switches as runtime
 * values (frame.h INT_L/INT_U, PDE.h FACTOR/TAU_FACTOR/DIRICHLET/
 * INTERIOR_MODE, the driver's WAVE and N, weno_mode of main). */
typedef struct hz_params {
    int N;             /* cells per axis; the grid has (N+1)^3 nodes        */
    double int_l;      /* domain lower bound (reference: -2.0)              */
    double int_u;      /* domain upper bound (reference: 2.0)               */
    double wave;       /* wave number k                                     */
    double factor;     /* tube half-width eps = factor * H (reference: 2.0)  */
    double tau_factor; /* regularisation radius tau = tau_factor * H (2.0)  */
    int dirichlet;     /* 0: Neumann (single layer), 1: Dirichlet (double)  */
    int interior;      /* 0: exterior problem, 1: interior                  */
    int weno_order;    /* 5 (reference main) or 3                           */
} hz_params;

typedef struct hz_operator hz_operator;

typedef struct hz_solve_opts {
    int method;        /* HZ_BICG, HZ_BICGSTAB or HZ_GMRES                              */
    int precision;     /* HZ_PREC_*                                                     */
    double tol;        /* stop at ||b - A x|| / ||b|| < tol (reference DEFAULTACC 1e-7) */
    int maxit;         /* Krylov iteration cap (reference: 2000)                        */
    double inner_tol;  /* HZ_PREC_F32_REFINED: the tightest relative tolerance of an
                          inner solve (FP32 densities bound it near 1e-7).  Step k
                          solves to max(inner_tol, min(0.5, tol / (4 res_{k-1}))),
                          res_0 = 1: only as far as the FP64 residual still has
                          to fall.  An inner solve also stops once it has run
                          max(30, iterations to its last new minimum) iterations
                          without a new minimum, and returns its best iterate    */
    int max_outer;     /* HZ_PREC_F32_REFINED: refinement step cap.  A step that does
                          not lower the FP64 residual is undone and repeated once
                          with an inner GMRES(restart); a second such step ends
                          the refinement with the best iterate                     */
    int stagnation;    /* 1: also stop when |delta(||r||/||b||)| < 1e-3 tol (reference) */
    int restart;       /* HZ_GMRES: Krylov basis size before a restart (2..127)         */
} hz_solve_opts;

#define HZ_MAX_STEPS 8

typedef struct hz_solve_info {
    int iterations;       /* Krylov iterations in total (inner ones when refined) */
    int outer;            /* refinement steps (0 when not refined)                */
    double resid;         /* final ||b - A x|| / ||b|| in the solve's own arithmetic */
    double resid_f64;     /* final relative residual from an FP64 sweep (refined) */
    double seconds;       /* wall time of the solve                               */
    int64_t pair_evals;   /* kernel pair evaluations performed                    */
    int status;           /* HZ_OK, or why it stopped early                       */
    int converged;        /* 1 when the final residual (resid_f64 for refined
                             solves) is below tol, 0 when the solve stopped at
                             its iteration or refinement cap, on stagnation, or
                             (refined) when a refinement step stopped reducing
                             the FP64 residual; the call still returns HZ_OK and
                             its best iterate, as the reference's CompBiCG
                             returns after its last iteration                     */
    /* refined solves: the first HZ_MAX_STEPS refinement steps, one entry each */
    int steps;                           /* entries filled (min(outer, HZ_MAX_STEPS)) */
    int step_iters[HZ_MAX_STEPS];        /* inner Krylov iterations of the step
                                            (negative: the step ran GMRES)            */
    double step_inner_tol[HZ_MAX_STEPS]; /* inner tolerance the step solved to        */
    double step_resid[HZ_MAX_STEPS];     /* FP64 relative residual after the step     */
} hz_solve_info;

HZ_API const char *hz_last_error(void);

/* Reference defaults: [-2,2]^3, FACTOR 2, TAU_FACTOR 2, Neumann, exterior,
 * WENO5, N and wave as given. */
HZ_API void hz_params_default(hz_params *p, int N, double wave);

/* Operator lifetime.  hz_create selects the current CUDA device. */
HZ_API int hz_create(const hz_params *p, hz_operator **out);
HZ_API void hz_destroy(hz_operator *op);
/* Run subsequent work on this cudaStream_t (NULL: the operator's own). */
HZ_API int hz_set_stream(hz_operator *op, void *cuda_stream);
HZ_API void *hz_get_stream(hz_operator *op);

/* Upload the signed distance grid ((N+1)^3 doubles, d > 0 inside): the
 * reference reads it from distance<N>.txt (large3Dexample2.c:405-424). */
HZ_API int hz_set_distance(hz_operator *op, const double *d, int where);

/* Level-set preprocessing on the device: WENO gradient
 * (distance_application3D.c:56-140), curvatures (:35-53 over every node),
 * tube (large3Dexample2.c:548-597) and per-point arrays (:4340-4452).
 * Returns the tube size in *n. */
HZ_API int hz_build(hz_operator *op, int64_t *n);
HZ_API int64_t hz_tube_size(const hz_operator *op);

/* Autotuner: times every compiled variant of the FP32 pair sweep (block
 * shape x targets per thread) on this operator's tube, once as the fused
 * A p + A^H pt pass (BiCG) and once as a single product (GMRES, BiCGSTAB),
 * and keeps the fastest of each for all later FP32 sweeps.  Returns the
 * fused pass's variant and time.  hz_set_sweep_config forces one variant
 * for both. */
HZ_API int hz_autotune(hz_operator *op, int *chosen, double *ms_per_sweep);
HZ_API int hz_set_sweep_config(hz_operator *op, int cfg);

/* Phase of the FP32 pair sweep (hz_matvec, hz_matvec_pair and the FP32
 * products of hz_solve).  HZ_PHASE_SPLIT (default): the phase is first
 * reduced in revolutions with k/(2 pi) split into an FP32 head and tail,
 * which about halves the FP32-vs-FP64 product error (4.6e-8 -> 2.9e-8 on the
 * 256^3 torus at k = 20) at about 6 % of the sweep's throughput; there a
 * refined solve to 1e-6 then needs one FP64 residual instead of two (55 s
 * instead of 84 s).  HZ_PHASE_DIRECT: k rho goes to the SFU's sin/cos as one
 * FP32 product.  The multi right-hand-side, batch and Combo FP32 sweeps use
 * the direct phase. */
#define HZ_PHASE_DIRECT 0
#define HZ_PHASE_SPLIT 1
HZ_API int hz_set_phase_mode(hz_operator *op, int mode);

/* Per-kernel timing of the pair sweeps: CUDA events recorded on the launch
 * stream around every sweep kernel (also inside the solver's iteration
 * graphs).  enable = 1 / 0 switches it on / off and clears the totals,
 * enable = -1 only reads them: total device milliseconds and launches. */
HZ_API int hz_sweep_timing(hz_operator *op, int enable, double *total_ms, int64_t *launches);

/* Copy out grids (any pointer may be NULL). */
HZ_API int hz_get_grids(hz_operator *op, double *gx, double *gy, double *gz, double *mcurv, double *gcurv,
                 int where);
/* Copy out tube arrays (any pointer may be NULL); xs/nrm are 3n interleaved. */
HZ_API int hz_get_tube(hz_operator *op, int64_t *idx, double *xs, double *nrm, double *delta, double *jac,
                double *reg, double *w, int where);

/* q = A p (adjoint = 0) or q = A^H p (adjoint = 1): the matrix-free form of
 * the dense products of large3Dexample2.c:3262-3309 with entries
 * omp_get_Ccomp (:4463-4564). */
HZ_API int hz_matvec(hz_operator *op, int precision, int adjoint, const double *p_re, const double *p_im,
              double *q_re, double *q_im, int where);
/* Fused q = A p and qt = A^H pt in one pass over the pairs (the two products
 * of every BiCG iteration, :3262-3309). */
HZ_API int hz_matvec_pair(hz_operator *op, int precision, const double *p_re, const double *p_im,
                   const double *pt_re, const double *pt_im, double *q_re, double *q_im,
                   double *qt_re, double *qt_im, int where);
/* Multi right-hand side: Q = A P for nrhs column vectors stored one after
 * the other (vector r at offset r*n), one kernel evaluation per pair and
 * kernel pass; a pass takes a block of 8, 16 or 32 right-hand sides (FP64:
 * 8 or 16), the smallest block that holds the remaining columns. */
HZ_API int hz_matvec_multi(hz_operator *op, int precision, int nrhs, const double *p_re,
                    const double *p_im, double *q_re, double *q_im, int where);

/* Solve A X = B for nrhs right-hand sides ([nrhs][n] each) in lockstep over
 * the columns, every product a multi right-hand-side sweep over the columns
 * still iterating: opts->method HZ_GMRES runs one GMRES(restart) per column
 * (basis of (restart + 3) x nrhs x n complex FP64 vectors), any other method
 * BiCGSTAB.  HZ_PREC_F32_REFINED refines every column with FP64 residuals.
 * resid (may be NULL) receives each column's final relative residual. */
HZ_API int hz_solve_multi(hz_operator *op, const hz_solve_opts *opts, int nrhs, const double *b_re,
                          const double *b_im, double *x_re, double *x_im, int where,
                          hz_solve_info *info, double *resid);

/* Incident plane waves e^{ik d.x} for ndir unit directions (3 doubles each,
 * host memory): kind HZ_RHS_POINT_DIRICHLET gives the values at the
 * projected points, HZ_RHS_POINT_NEUMANN the outward normal derivative.
 * Output [ndir][n]. */
HZ_API int hz_rhs_plane_waves(hz_operator *op, int ndir, const double *dirs, int kind, double *b_re,
                              double *b_im, int where);

/* Solve A x = b (x0 = 0).  opts may be NULL: BiCG, FP64, tol 1e-7, 2000 its. */
HZ_API int hz_solve(hz_operator *op, const hz_solve_opts *opts, const double *b_re, const double *b_im,
             double *x_re, double *x_im, int where, hz_solve_info *info);
HZ_API void hz_solve_opts_default(hz_solve_opts *o);

/* Relative residual after each Krylov iteration of the operator's last
 * hz_solve with BiCG or BiCGSTAB (the FP32 inner solves one after another
 * for refined solves, each relative to its own right-hand side; empty after
 * GMRES).  Copies min(cap, count) values into out and sets *count.  No
 * counterpart in the reference, which prints only the final residual
 * (BICGSTAB.c:310). */
HZ_API int hz_residual_history(hz_operator *op, double *out, int cap, int *count);

/* Receiver misfit and its gradients by the adjoint method.
 * J = sum_m |u(x_m) - t_m|^2 with u = E sigma (layer as in hz_eval) and
 * A sigma = b.  One forward solve, one adjoint solve A^H lambda = E^H r
 * (r = u - t), and recomputed kernel derivatives give
 *   g = dJ/d(Re b) + i dJ/d(Im b) = 2 lambda                    (n values),
 *   dJ/dk at fixed b = 2 Re(r^H dE/dk sigma) - 2 Re(lambda^H dA/dk sigma),
 *   dJ/dw_s = Re(conj(lambda_s) sigma_s) / w_s   (tube-point weights, n).
 * Any output pointer may be NULL.  opts as for hz_solve (both solves). */
HZ_API int hz_misfit_gradient(hz_operator *op, const hz_solve_opts *opts, const double *b_re,
                              const double *b_im, int layer, int64_t m, const double *rx,
                              const double *t_re, const double *t_im, double *J, double *g_re,
                              double *g_im, double *dJ_dk, double *dJ_dw, int where, hz_solve_info *info);

/* Misfit gradient with respect to the distance-grid values (the shape):
 * J = sum_m |u(x_m) - t_m|^2 for the Dirichlet formulation with double-layer
 * receivers and point-source data g = e^{ik|x*-src|}/(4 pi |x*-src|) at the
 * projected points (src: 3 doubles, host memory), and dJ/dphi at every grid
 * node ((N+1)^3 doubles).  One forward and one adjoint solve (opts as in
 * hz_solve) give the sensitivities to every tube point's projection,
 * normal, weight and regularisation factor (an FP64 pair sweep); they are
 * pulled back through the projection, the trilinear interpolations, the
 * normalisations, delta_eps and the Jacobian exactly, and through the
 * WENO-gradient and curvature stencils by local central differences
 * (step 1e-7).  Tube membership changes (|phi| crossing eps) are not
 * differentiated.  Needs p.dirichlet = 1. */
HZ_API int hz_shape_gradient(hz_operator *op, const hz_solve_opts *opts, const double *src, int64_t m,
                             const double *rx, const double *t_re, const double *t_im, double *J, double *dJ_dphi,
                             int where, hz_solve_info *info);

/* Boundary data at the projected points (see HZ_RHS_*). src: 3 doubles. */
HZ_API int hz_rhs_point_source(hz_operator *op, const double *src, int kind, double *b_re, double *b_im,
                        int where);

/* Field at m receivers (xyz interleaved, host or device per where) from the
 * density sigma: single layer as NeumannTest (large3Dexample2.c:1810-1824)
 * or the double layer of the Dirichlet formulation. */
HZ_API int hz_eval(hz_operator *op, int layer, int64_t m, const double *rx, const double *s_re,
            const double *s_im, double *u_re, double *u_im, int where);

/* Whole-grid stencils without an operator.  d, outputs: (N+1)^3 doubles.
 * hz_assign_gradient replaces ASSIGN_GRADIENT (distance_application3D.c:56);
 * hz_assign_curvatures replaces the BothCurvs loop (large3Dexample2.c:446). */
HZ_API int hz_assign_gradient(int N, double H, const double *d, double *gx, double *gy, double *gz,
                       int weno_order, int where);
HZ_API int hz_assign_curvatures(int N, double H, const double *d, double *mcurv, double *gcurv, int where);

/* Reinitialise a level set toward the signed distance, in place: iters TVD
 * Runge-Kutta-2 pseudo-time steps (dt = cfl*H, cfl <= 1) of
 * phi_t + S(phi0)(|grad phi| - 1) = 0 with S(phi0) = phi0/sqrt(phi0^2+H^2),
 * |grad phi| from the Godunov Hamiltonian of finite_difference3D.c:5-27 on
 * WENO one-sided derivatives (weno.c:259-345, mirror boundaries).  The
 * reference itself has no reinitialisation (its Godunov() is unused). */
HZ_API int hz_reinitialize(int N, double H, double *phi, int iters, double cfl, int weno_order, int where);

/* Dense complex BiCG on a caller-provided row-major n x n matrix (real and
 * imaginary parts): the device form of CompBiCG (BICGSTAB.c:5-339). */
HZ_API int hz_dense_bicg(int64_t n, const double *a_re, const double *a_im, const double *b_re,
                  const double *b_im, double *x_re, double *x_im, double tol, int maxit,
                  int where, hz_solve_info *info);

/* ---- Dense assemblers of HelmholtzKernel.c (small-n parity API) ----------
 * The reference's dense n x n matrices, assembled on the device:
 *   HZ_DENSE_DOUBLE_LAYER  DoubleLayerKernel        (HelmholtzKernel.c:613-761)
 *   HZ_DENSE_COMBO         new_HelmholtzKernelCombo (HelmholtzKernel.c:173-610)
 *   HZ_DENSE_SPHERE        new_HelmholtzKernel      (HelmholtzKernel.c:3-169),
 *                          on the analytic sphere of hz_dense_opts
 * Memory: two n x n FP64 matrices per assembled operator (3.2 GB each at
 * n = 20,000); the matrix-free operator (hz_matvec) is the path at scale. */
#define HZ_DENSE_DOUBLE_LAYER 0
#define HZ_DENSE_COMBO 1
#define HZ_DENSE_SPHERE 2

/* Rows of the per-point array pts[HZ_DENSE_ROWS][n]; an assembler writes
 * the rows its reference counterpart fills (the rest are left as they are). */
enum {
    HZ_DP_ZX, HZ_DP_ZY, HZ_DP_ZZ,    /* grid node                                 */
    HZ_DP_XS, HZ_DP_YS, HZ_DP_ZS,    /* projection x*                              */
    HZ_DP_DIST,                      /* signed distance at the node                */
    HZ_DP_GX, HZ_DP_GY, HZ_DP_GZ,    /* unit normal at x*                          */
    HZ_DP_DELTA,                     /* delta_eps (double layer)                   */
    HZ_DP_JAC,                       /* Jacobian                                   */
    HZ_DP_CURV,                      /* 1/(radius - d) (sphere kernel)             */
    HZ_DP_REG, HZ_DP_REGIMG,         /* regularisation factor (double layer, Combo)*/
    HZ_DP_POLYW, HZ_DP_SINEW,        /* annulus weights PolyWeight/SineWeight      */
    HZ_DP_POLYRES, HZ_DP_SINERES,    /* H^3 J weight                               */
    HZ_DP_RESULT,                    /* H^3 delta J (double layer)                 */
    HZ_DENSE_ROWS
};

/* The reference's compile-time switches and call arguments of the dense
 * assemblers (PDE.h, frame.h, functions.h).  hz_dense_opts_default gives the
 * reference's values: POLY_TEST 0, SINE_TEST 1, one-sided switches 0, the
 * frame.h sphere (radius 1 at the origin), eta = DEFAULT_ETA = -1, the
 * driver's annulus [0.1 H, sqrt(H)] (large3Dexample2.c:61-63,298-305) and
 * epsilon = FACTOR H for the double layer. */
typedef struct hz_dense_opts {
    double delta0;      /* inner radius of the annulus (Combo, sphere kernel)        */
    double epsilon;     /* outer radius: |d| <= epsilon                               */
    double wavenum;     /* Combo: wave number of the double-layer part (the single-
                           layer part and the other assemblers use hz_params.wave)    */
    double eta;         /* Combo: weight of the -i eta single-layer part              */
    int poly, sine;     /* assemble the PolyWeight / SineWeight matrices              */
    int onesided;       /* TRAD_ONESIDED (double layer) or COMBO_ONESIDED             */
    int combo_interior; /* COMBO_INTERIOR                                              */
    double radius;      /* analytic sphere of new_HelmholtzKernel (frame.h)           */
    double center[3];
} hz_dense_opts;

HZ_API void hz_dense_opts_default(hz_dense_opts *o, int kind, const hz_params *p);

/* Number of points the assembler selects from the distance grid d
 * ((N+1)^3, ignored by HZ_DENSE_SPHERE, may then be NULL). */
HZ_API int hz_dense_count(int kind, const hz_params *p, const hz_dense_opts *o, const double *d, int where,
                          int64_t *n);

/* Assemble.  d and the grids gx, gy, gz (WENO gradient), mc, gc (mean and
 * Gaussian curvature) are (N+1)^3; pass NULL grids to have them computed
 * from d on the device (hz_assign_gradient / hz_assign_curvatures).  n must
 * equal hz_dense_count (HZ_ERR_ARG otherwise, where the reference exits).
 * Outputs (any may be NULL): pts [HZ_DENSE_ROWS][n]; k1 = the double-layer
 * matrix, or the PolyWeight matrix of Combo / sphere kernel; k2 = their
 * SineWeight matrix; row-major n x n, real and imaginary parts.  regcount
 * (may be NULL) receives the Combo's count of regularised pairs. */
HZ_API int hz_dense_assemble(int kind, const hz_params *p, const hz_dense_opts *o, const double *d,
                             const double *gx, const double *gy, const double *gz, const double *mc,
                             const double *gc, int64_t n, double *pts, double *k1_re, double *k1_im,
                             double *k2_re, double *k2_im, int64_t *regcount, int where);

/* ---- Batches of operators ------------------------------------------------
 * Independent surfaces (each its own built operator: grid, tube, k may
 * differ) solved together: every FP32 product of the batch is ONE
 * persistent launch whose CTAs share the (operator, target block, source
 * tile) work of all operators, so small and large tubes fill the GPU
 * together; the lockstep BiCGSTAB iteration around it runs as one CUDA
 * graph.  Vectors are passed per operator: arrays of `count` pointers, the
 * r-th of length hz_tube_size(ops[r]).  The operators must be built, use
 * the classic formulation and live on the same device; the batch keeps
 * pointers to them (destroy the batch first). */
typedef struct hz_batch hz_batch;
HZ_API int hz_batch_create(hz_operator *const *ops, int count, hz_batch **out);
HZ_API void hz_batch_destroy(hz_batch *b);
/* Time the FP32 batch sweep shapes and keep the fastest (variant, ms). */
HZ_API int hz_batch_autotune(hz_batch *b, int *chosen, double *ms_per_sweep);
/* Use batch sweep shape v (0..3) instead of the autotuner's choice. */
HZ_API int hz_batch_set_variant(hz_batch *b, int v);
/* q_r = A_r p_r for every operator: HZ_PREC_F32 (one persistent launch) or
 * HZ_PREC_F64 (one FP64 sweep per operator). */
HZ_API int hz_batch_matvec(hz_batch *b, int precision, const double *const *p_re, const double *const *p_im,
                           double *const *q_re, double *const *q_im, int where);
/* Solve A_r x_r = b_r for all r with lockstep BiCGSTAB (opts->method is
 * ignored); HZ_PREC_F32_REFINED refines every system with its FP64
 * residual.  resid (may be NULL): count final relative residuals. */
HZ_API int hz_batch_solve(hz_batch *b, const hz_solve_opts *opts, const double *const *b_re,
                          const double *const *b_im, double *const *x_re, double *const *x_im, int where,
                          hz_solve_info *info, double *resid);

/* Switch the operator to the Combo formulation (new_HelmholtzKernelCombo,
 * HelmholtzKernel.c:173-610) before hz_build: points on the annulus
 * o->delta0 <= |d| <= o->epsilon (hz_dense_opts_default(HZ_DENSE_COMBO) gives
 * the driver's [0.1 H, sqrt(H)]), weights SineWeight (o->sine) or PolyWeight,
 * operator A = -i eta (dG/dn_x - 1/2) + d^2G/dn_x dn_y at offset points,
 * applied matrix free in FP64 or FP32 (hz_matvec, hz_matvec_pair, hz_solve
 * with any precision: HZ_PREC_F32_REFINED runs FP32 products inside FP64
 * iterative refinement; hz_autotune, the multi right-hand-side, batch and
 * gradient entries are not available for it).  hz_eval with HZ_COMBO_LAYER
 * evaluates the field.  o = NULL switches back. */
HZ_API int hz_set_combo(hz_operator *op, const hz_dense_opts *o);

/* Number of kernel launches made by this library in this process (graph
 * launches count their kernels), for launch accounting. */
HZ_API int64_t hz_kernel_launches(void);

/* Poll limit of the pair sweeps' data waits (a CTA waiting for the bulk
 * copy of its next source tile) on the current device; polls < 0 restores
 * the default (2^24 polls, far above any real wait).  A wait that runs out
 * sets the device error word, the CTA lets its copies in flight land
 * (those waits keep the full bound) and exits, and the call returns
 * HZ_ERR_DEVICE_WAIT with the context still usable.  A short limit (0 gives
 * up at once) exercises that error path in tests. */
HZ_API int hz_set_wait_limit(long long polls);

/* Allocation-free FP64 product, for callers that cannot allocate device
 * memory when they need it (applications that hand out all device memory
 * from their own pools, plugin hosts that forbid allocation after start-up,
 * loops that cannot afford cudaMalloc's implicit synchronisation).  It has
 * no counterpart in the reference.  Computes q = A p (adjoint = 0) or
 * q = A^H p (adjoint = 1) for the tube described by p (N, int_l, int_u,
 * wave, tau_factor, dirichlet, interior are used) and the caller's device
 * arrays xs, nrm (3n interleaved), reg, w, p, q (n each), as hz_get_tube
 * returns them.  It calls no cudaMalloc, cudaFree or allocating library
 * routine: its scratch is one fixed __device__ array of about 3 MiB that
 * every GPU loading this library holds until the process exits; n above
 * HZ_NOALLOC_MAX_POINTS is rejected with HZ_ERR_ARG.  The array's device
 * address belongs to the current CUDA context; each call looks it up again
 * in the context current at the call (a host-side lookup, no allocation),
 * so a context switch or cudaDeviceReset between calls is safe; the first
 * call in a context must come before any stream capture.  All calls share the array:
 * calls that overlap on the GPU (other streams, other threads) race.  Work
 * is ordered on `stream` (NULL: the legacy default stream) and the call
 * waits for it to finish before returning its status. */
#define HZ_NOALLOC_MAX_POINTS 32768
HZ_API int hz_matvec_f64_noalloc(const hz_params *p, int64_t n, int adjoint, const double *xs,
                                 const double *nrm, const double *reg, const double *w,
                                 const double *p_re, const double *p_im, double *q_re, double *q_im,
                                 void *stream);

/* The reference driver's text files (host only, no device work):
 * distance<N>.txt ((N+1)^3 values, (i,j,k) order, large3Dexample2.c:405-424),
 * the boundary-data pair Rel_bN<N>k<k>.txt / Rel_bimgN<N>k<k>.txt (size line
 * then "%.15lf" per line, :1236-1252,1333), the density pair
 * Rel_DensityN<N>k<k>.txt / ...imgN... ("%.15lf " values, :3446-3474) and the
 * NeumannTest log Rel_Result_N<N>k<k>.txt (:1885-1896).  Readers check the
 * size line and report short or NaN data as errors. */
HZ_API int hz_reference_file_names(int N, double wave, char *b, char *bimg, char *dens, char *densimg,
                                   char *result, char *distance, size_t cap);
HZ_API int hz_read_distance_file(const char *path, int N, double *d);
HZ_API int hz_write_distance_file(const char *path, int N, const double *d);
HZ_API int hz_write_rhs_files(const char *path_re, const char *path_im, int64_t n, const double *b_re,
                              const double *b_im);
HZ_API int hz_read_rhs_files(const char *path_re, const char *path_im, int64_t n, double *b_re,
                             double *b_im);
HZ_API int hz_write_density_files(const char *path_re, const char *path_im, int64_t n, const double *x_re,
                                  const double *x_im);
HZ_API int hz_read_density_files(const char *path_re, const char *path_im, int64_t n, double *x_re,
                                 double *x_im);
HZ_API int hz_write_result_file(const char *path, double exact_re, double exact_im, double approx_re,
                                double approx_im);

/* Field on a plane (the reference's slice printer, printslice.c:5-746, as a
 * headless buffer): u at the n2 x n2 points lo + (a*h2, b*h2) of the plane
 * axis = c (axis 0: x = c, points (c, y, z); 1: y = c, points (x, c, z);
 * 2: z = c, points (x, y, c)), row a, column b, u[a*n2 + b].  Points whose
 * interpolated distance exceeds -mask (inside the body or near it) are set
 * to 0, as the reference prints 0 where distance() > -0.06. */
HZ_API int hz_eval_slice(hz_operator *op, int layer, int axis, double c, int n2, double lo, double h2,
                         double mask, const double *s_re, const double *s_im, double *u_re, double *u_im,
                         int where);

/* Measure the FP32 and FP64 FMA throughput of the current device (TFLOP/s,
 * one FMA = 2 FLOP), the roofline denominators of the pair sweeps. */
HZ_API int hz_measure_fma_peaks(double *fp32_tflops, double *fp64_tflops);

#ifdef __cplusplus
}
#endif
#endif
