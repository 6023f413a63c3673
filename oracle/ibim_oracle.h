/*
 * ibim_oracle.h -- CPU restatement of the reference IBIM Helmholtz hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the GPU
 * implementation: only tests/, __graft_entry__.smoke() and the cpu_baseline /
 * --impl reference legs of bench.py may load it.  The product path never
 * calls it and never falls back to it.
 *
 * Every function restates one reference routine (moorhsum/Helmholtz-3D-torrone)
 * with the same floating-point operation order, so that, built with
 * -ffp-contract=off, it reproduces the reference bit for bit on the same
 * machine.  Citations are file:line in the reference project.
 *
 * Grids are contiguous (N+1)^3 FP64 arrays in the reference's i-major order:
 *   node (i,j,k) at offset ((i*S)+j)*S+k, S = N+1,
 *   coordinates (x,y,z) = (int_l + j*H, int_l + i*H, int_l + k*H)
 * (large3Dexample2.c:428-437), so i is y, j is x and k is z.  d > 0 inside.
 */
#ifndef IBIM_ORACLE_H
#define IBIM_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    int N;              /* grid cells per axis; S = N+1 nodes            */
    double int_l;       /* lower domain bound (frame.h INT_L)            */
    double int_u;       /* upper domain bound (frame.h INT_U)            */
    double wave;        /* wave number k (WAVE)                          */
    double factor;      /* tube half width / H (PDE.h FACTOR)            */
    double tau_factor;  /* regularisation radius / H (PDE.h TAU_FACTOR)  */
    int dirichlet;      /* 1: double layer with n_j (PDE.h DIRICHLET)    */
    int interior;       /* 1: interior problem (PDE.h INTERIOR_MODE)     */
} or_params;

/* H = (int_u - int_l)/N, exactly as large3Dexample2.c:174. */
double or_h(const or_params *p);

/* weno.c:259-345: one-sided WENO3/WENO5 derivatives from a 5/7-point line. */
void or_weno(double *dfp, double *dfn, const double fi[], double dx, int order);

/* distance_application3D.c:56-140 with WENO_DX/DY/DZ (weno.c:117-254):
 * Godunov-upwinded, unnormalised WENO gradient at every node. */
void or_gradient(int N, double H, const double *d, double *gx, double *gy, double *gz, int order);

/* finite_difference3D.c:220-390 and :393-721: limited second differences. */
double or_xder2(const double *d, int N, double H, int i, int j, int k);
double or_yder2(const double *d, int N, double H, int i, int j, int k);
double or_zder2(const double *d, int N, double H, int i, int j, int k);
double or_dxy(const double *d, int N, double H, int i, int j, int k);
double or_dxz(const double *d, int N, double H, int i, int j, int k);
double or_dyz(const double *d, int N, double H, int i, int j, int k);

/* distance_application3D.c:35-53 over every node (loop large3Dexample2.c:446-455). */
void or_curvatures(int N, double H, const double *d, double *mcurv, double *gcurv);

/* Level-set reinitialisation (absent from the reference; scheme from its
 * unused Godunov(), finite_difference3D.c:5-27): iters TVD-RK2 steps of
 * phi_t + S(phi0)(|grad phi| - 1) = 0, S = phi0/sqrt(phi0^2+H^2), WENO
 * one-sided derivatives, dt = cfl*H.  In place. */
/* Godunov upwind |grad phi| of one node from its six one-sided
 * derivatives (finite_difference3D.c:5-27). */
double or_godunov(double signage, double a, double b, double c, double d, double e, double f);
void or_reinit(int N, double H, double *phi, int iters, double cfl, int order);

/* Tube {|d| <= eps} in lexicographic (i,j,k) order, large3Dexample2.c:548-597.
 * Writes linear node indices into idx (may be NULL); returns the count. */
int64_t or_tube(int N, const double *d, double eps, int64_t *idx);

/* Per-tube-point quantities, large3Dexample2.c:4298-4459 (omp_get_Ccomp init):
 * projection x* = z - d grad d, unit normal by trilinear interpolation of the
 * gradient grids at x* (interpolate3D.c:5-102, normalised a second time as in
 * the driver), delta_eps (functions.c:366-374), Jacobian, regularisation
 * factor (curvatures interpolated at x*, interpolate3D.c:569-605), weight
 * w = H^3 delta J.  Arrays are length n; xs/nrm are interleaved xyz (3n).
 * Returns 0, or the 1-based position of the first point whose interpolation
 * cell falls outside the grid (the reference exits there). */
int or_tube_init(const or_params *p, const double *d, const double *gx, const double *gy,
                 const double *gz, const double *mcurv, const double *gcurv, int64_t n,
                 const int64_t *idx, double *xs, double *nrm, double *delta, double *jac,
                 double *reg, double *w);

/* One complex matrix entry A[pi][pj], large3Dexample2.c:4463-4564
 * (regfactor indexed by the target for Neumann, by the source for Dirichlet). */
void or_entry(const or_params *p, const double *xs, const double *nrm, const double *reg,
              const double *w, int64_t pi, int64_t pj, double *re, double *im);

/* Dense row-block of A: rows [r0, r1), all n columns, row-major (r1-r0) x n. */
void or_dense_rows(const or_params *p, int64_t n, const double *xs, const double *nrm,
                   const double *reg, const double *w, int64_t r0, int64_t r1,
                   double *are, double *aim);

/* q = A p (adjoint = 0) or q = A^H p (adjoint = 1) for rows [r0, r1), with the
 * inner sum taken in ascending column order like the reference's dense loops
 * (large3Dexample2.c:3262-3309).  Rows run in parallel when nthreads > 1. */
void or_matvec(const or_params *p, int64_t n, const double *xs, const double *nrm,
               const double *reg, const double *w, const double *pre, const double *pim,
               double *qre, double *qim, int adjoint, int64_t r0, int64_t r1, int nthreads);

/* Complex BiCG of BICGSTAB.c:104-308 / large3Dexample2.c:3131-3433, matrix
 * free, x0 = 0.  Stops at ||r||/||b|| < acc, NaN, or stagnation.  Returns the
 * number of iterations; *resid gets the final relative residual. */
int or_bicg(const or_params *p, int64_t n, const double *xs, const double *nrm,
            const double *reg, const double *w, const double *bre, const double *bim,
            double *xre, double *xim, double acc, int maxit, int nthreads, double *resid);

/* Dense complex BiCG on a row-major n x n matrix: BICGSTAB.c:5-339 (CompBiCG). */
int or_bicg_dense(int64_t n, const double *are, const double *aim, const double *bre,
                  const double *bim, double *xre, double *xim, double acc, int maxit,
                  double *resid);

/* Off-surface evaluation at m receivers (xyz interleaved).  Single layer
 * (Neumann formulation) as NeumannTest, large3Dexample2.c:1752-1824:
 *   u(x) = sum_p [rho>tau] (-Phi(x,x*_p)) sigma_p w_p.
 * Double layer (Dirichlet formulation) with the matrix's own kernel:
 *   u(x) = sum_p [rho>tau] w_p sigma_p (x - x*_p).n_p Phi'(rho)/rho. */
void or_eval(const or_params *p, int64_t n, const double *xs, const double *nrm,
             const double *w, const double *sre, const double *sim, int64_t m,
             const double *rx, double *ure, double *uim, int double_layer, int nthreads);

/* Boundary data b_p at the projected points.  kind 0: point source
 * e^{ik|x-s|}/(4 pi |x-s|) at s (Dirichlet data); kind 1: its normal
 * derivative along the stored unit normal (Neumann data). */
void or_point_source_rhs(const or_params *p, int64_t n, const double *xs, const double *nrm,
                         const double *src, int kind, double *bre, double *bim);

/* ------------------------------------------------------------------ */
/* Dense assemblers of HelmholtzKernel.c (small-n parity API)          */
/* ------------------------------------------------------------------ */
/* Options of the dense assemblers: the reference's compile-time switches
 * (PDE.h POLY_TEST, SINE_TEST, TRAD_/COMBO_ONESIDED, COMBO_INTERIOR; the
 * sphere of frame.h) and the arguments of the calls. */
typedef struct {
    double delta0;      /* inner radius of the annulus delta0 <= |d|        */
    double epsilon;     /* outer radius |d| <= epsilon                       */
    double wavenum;     /* Combo: wave number of the double-layer part       */
    double eta;         /* Combo: coupling of the -i eta single-layer part   */
    int poly, sine;     /* POLY_TEST / SINE_TEST                             */
    int onesided;       /* TRAD_ONESIDED (double layer) / COMBO_ONESIDED     */
    int combo_interior; /* COMBO_INTERIOR                                    */
    double radius, cx, cy, cz; /* analytic sphere of new_HelmholtzKernel     */
} or_dense_opts;

/* Rows of the per-point output array pts[OR_DP_ROWS][n]. */
enum {
    OR_DP_ZX, OR_DP_ZY, OR_DP_ZZ, OR_DP_XS, OR_DP_YS, OR_DP_ZS, OR_DP_DIST, OR_DP_GX, OR_DP_GY, OR_DP_GZ,
    OR_DP_DELTA, OR_DP_JAC, OR_DP_CURV, OR_DP_REG, OR_DP_REGIMG, OR_DP_POLYW, OR_DP_SINEW, OR_DP_POLYRES,
    OR_DP_SINERES, OR_DP_RESULT, OR_DP_ROWS
};

/* Kinds: DoubleLayerKernel (HelmholtzKernel.c:613-761), new_HelmholtzKernelCombo
 * (:173-610), new_HelmholtzKernel (:3-169). */
enum { OR_DENSE_DOUBLE_LAYER = 0, OR_DENSE_COMBO = 1, OR_DENSE_SPHERE = 2 };

/* Per-point arrays of one assembler, in the reference's lexicographic
 * order.  pts (may be NULL) receives them when its point count equals
 * n_alloc.  Returns the point count, or -(1 + position) of the first point
 * whose interpolation cell falls outside the grid.  Grids are unused by
 * the sphere kernel (may be NULL there). */
int64_t or_dense_points(int kind, const or_params *p, const or_dense_opts *o, const double *d,
                        const double *gx, const double *gy, const double *gz, const double *mcurv,
                        const double *gcurv, int64_t n_alloc, double *pts);

/* Dense n x n matrices (row-major) from the per-point arrays.  Double
 * layer: K1 (re, im).  Combo and sphere kernel: K1 = the PolyWeight matrix
 * (if o->poly), K2 = the SineWeight matrix (if o->sine); unused pointers
 * may be NULL.  Returns the Combo's regcount (0 otherwise). */
int64_t or_dense_matrix(int kind, const or_params *p, const or_dense_opts *o, int64_t n, const double *pts,
                        double *k1re, double *k1im, double *k2re, double *k2im);

/* PolyWeight / SineWeight of functions.c:793-866 (MOMENT_ORDER 1). */
double or_poly_weight(double t, double tau);
double or_sine_weight(double t, double tau);

#ifdef __cplusplus
}
#endif
#endif
