/*
 * helmholtz_ref_api.h -- drop-in replacements for the reference's library
 * entry points (moorhsum/Helmholtz-3D-torrone), with the reference's own
 * signatures and C++ linkage, so a driver compiled with g++ against the
 * reference headers links against libhzgb300.so unchanged.
 *
 * The reference compiles its C sources as C++ (Makefile:1-3) and its
 * headers carry no extern "C", so these names are C++-mangled exactly like
 * the reference's objects.  Buffers are host memory owned by the caller,
 * as in the reference; the work runs on the current CUDA device.  Unlike
 * the reference, failures return a negative HZ_ERR_* status (message from
 * hz_last_error()) instead of calling exit(0).
 */
#ifndef HELMHOLTZ_REF_API_H
#define HELMHOLTZ_REF_API_H

#include "helmholtz_gb300.h"

/* distance_application3D.h:12 -- WENO (weno_mode 3 or 5) Godunov-upwinded
 * gradient of the distance grid at every node, distance_application3D.c:56-140.
 * Grids are the reference's ragged [SIZE][SIZE][SIZE] arrays, SIZE = N+1. */
HZ_API int ASSIGN_GRADIENT(int N, double H, double ***dist, double ***graddx, double ***graddy,
                           double ***graddz, int weno_mode);

/* Whole-grid form of the BothCurvs loop of large3Dexample2.c:446-455
 * (BothCurvs: distance_application3D.c:35-53, distance_application3D.h:11):
 * mean and Gaussian curvature at every node.  New entry point; the
 * reference calls BothCurvs once per node. */
HZ_API int ASSIGN_CURVATURES(int N, double H, double ***dist, double ***mcurv, double ***gcurv);

/* ---- Per-node functions, on the host -------------------------------------
 * The reference's per-node entry points, for drivers that loop over nodes
 * themselves (large3Dexample2.c:446-455 calls BothCurvs once per node).  A
 * GPU cannot speed up one node per call, so these run on the host in FP64
 * with the arithmetic of the whole-grid kernels (unfused, in the
 * reference's operation order: results bit-identical to the reference's).
 * Grids are the reference's ragged [N+1][N+1][N+1] arrays. */

/* weno.h:31, weno.c:259-345: WENO3 (order 3, fi[0..4]) or WENO5 (any other
 * order, fi[0..6]) one-sided derivatives at the centre of fi, spacing dx. */
HZ_API void weno(double *dfp, double *dfn, double fi[], const double dx, const int order);

/* weno.h:26-28, weno.c:117-254: WENO one-sided derivatives of uvalue at node
 * (i, j, k) along x (index j), y (index i), z (index k), mirrored across the
 * grid's faces; order 5 or 3 (other orders leave the outputs unchanged). */
HZ_API void WENO_DX(double ***uvalue, const int i, const int j, const int k, const int N, const double H,
                    double *ux_p, double *ux_n, const int order);
HZ_API void WENO_DY(double ***uvalue, const int i, const int j, const int k, const int N, const double H,
                    double *ux_p, double *ux_n, const int order);
HZ_API void WENO_DZ(double ***uvalue, const int i, const int j, const int k, const int N, const double H,
                    double *ux_p, double *ux_n, const int order);

/* distance_application3D.h:9-11, distance_application3D.c:4-53: Gaussian and
 * mean curvature of the distance grid at node (i, j, k) from the limited
 * second differences (finite_difference3D.c:220-721); BothCurvs returns 0. */
HZ_API double GaussianCurv(double ***dist, int i, int j, int k, int N, double H);
HZ_API double MeanCurv(double ***dist, int i, int j, int k, int N, double H);
HZ_API int BothCurvs(double ***dist, int i, int j, int k, int N, double H, double *meancurv, double *gausscurv);

/* BICGSTAB.h:15 -- complex BiCG on a dense caller-owned matrix
 * (BICGSTAB.c:5-339): tolerance DEFAULTACC (hz_ref_config.bicg_acc, 1e-7),
 * at most 1000 iterations. */
HZ_API int CompBiCG(int size, double *density, double *densityimg, double **Kernel, double **Kernelimg,
                    double *b, double *bimg);

/* BICGSTAB.h:16-17 -- the OpenMP variant (BICGSTAB.c:344-765), at most 2000
 * iterations; chunk is accepted and ignored. */
HZ_API int omp_CompBiCG(int size, double *density, double *densityimg, double **Kernel, double **Kernelimg,
                        double *b, double *bimg, int chunk);

/* ---- Dense assemblers (HelmholtzKernel.h:20-40) ------------------------
 * Same arguments and outputs as the reference: per-point lists of length
 * size and caller-owned ragged size x size matrices.  Like the reference
 * they read the driver's globals N, SIZE, H, HCUBED, WAVE
 * (HelmholtzKernel.h:16-18; defined by the driver, large3Dexample2.c:46-51)
 * and its compile-time switches, which here are the runtime values of
 * hz_ref_config (defaults: the reference headers' values).  size must equal
 * the number of points the assembler selects (HZ_ERR_ARG otherwise; the
 * reference exits).  The matrices are built on the device and copied row by
 * row into the caller's arrays. */

/* HelmholtzKernel.c:613-761: tube |d| <= epsilon, finite-difference double
 * layer, regularised within TAU_FACTOR H; returns 0. */
HZ_API int DoubleLayerKernel(int size, double epsilon, double ***level, double ***leveldx, double ***leveldy,
                             double ***leveldz, double ***levelmcurv, double ***levelgcurv, double *zxlist,
                             double *zylist, double *zzlist, double *zxstarlist, double *zystarlist,
                             double *zzstarlist, double *dist, double *gradx, double *grady, double *gradz,
                             double *delta, double *Jacobian, double *regfactor, double *regfactorimg,
                             double *result, double **Kernel, double **Kernelimg, double wavenum);

/* HelmholtzKernel.c:173-610: annulus delta <= |d| <= epsilon, -i eta single
 * layer plus the hypersingular double layer at x*_i + |d_j| n_i; the
 * PolyWeight / SineWeight matrices of the switches; returns regcount. */
HZ_API int new_HelmholtzKernelCombo(int size, double delta, double epsilon, double ***level, double ***leveldx,
                                    double ***leveldy, double ***leveldz, double ***levelmcurv,
                                    double ***levelgcurv, double *zxlist, double *zylist, double *zzlist,
                                    double *zxstarlist, double *zystarlist, double *zzstarlist, double *dist,
                                    double *gradx, double *grady, double *gradz, double *Jacobian,
                                    double *regfactor, double *regfactorimg, double *PolyW, double *SineW,
                                    double *PolyResult, double *SineResult, double **PolyKernelH,
                                    double **PolyKernelHimg, double **SineKernelH, double **SineKernelHimg,
                                    double wavenum, double eta);

/* HelmholtzKernel.c:3-169: the analytic sphere of the configuration
 * (frame.h radius, Cx, Cy, Cz); returns 0. */
HZ_API int new_HelmholtzKernel(int size, double delta, double epsilon, double *zxlist, double *zylist,
                               double *zzlist, double *zxstarlist, double *zystarlist, double *zzstarlist,
                               double *dist, double *gradx, double *grady, double *gradz, double *curv,
                               double *Jacobian, double *PolyW, double *SineW, double *PolyResult,
                               double *SineResult, double **PolyKernelH, double **PolyKernelHimg,
                               double **SineKernelH, double **SineKernelHimg);

/* The reference's compile-time switches read by the drop-ins above. */
typedef struct hz_ref_config {
    double int_l, int_u;     /* frame.h INT_L, INT_U            (-2, 2) */
    double tau_factor;       /* PDE.h TAU_FACTOR                    (2) */
    int interior;            /* PDE.h INTERIOR_MODE                 (0) */
    int poly, sine;          /* PDE.h POLY_TEST, SINE_TEST       (0, 1) */
    int trad_onesided;       /* PDE.h TRAD_ONESIDED                 (0) */
    int combo_onesided;      /* PDE.h COMBO_ONESIDED                (0) */
    int combo_interior;      /* PDE.h COMBO_INTERIOR                (0) */
    double radius;           /* frame.h radius                      (1) */
    double center[3];        /* frame.h Cx, Cy, Cz            (0, 0, 0) */
    double bicg_acc;         /* BICGSTAB.h DEFAULTACC: CompBiCG and
                                omp_CompBiCG stop at ||r||/||b|| below it (1e-7) */
} hz_ref_config;

#ifdef __cplusplus
extern "C" {
#endif
HZ_API void hz_ref_get_config(hz_ref_config *c);
HZ_API void hz_ref_set_config(const hz_ref_config *c);
#ifdef __cplusplus
}
#endif

#endif
