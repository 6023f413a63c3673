/*
 * ref_harness.cpp -- extern "C" entry points into the reference build.
 *
 * TEST INFRASTRUCTURE ONLY.  Linked by oracle/build_ref.py together with a
 * patched copy of the reference sources (moorhsum/Helmholtz-3D-torrone) into
 * oracle/_ref/libref_<variant>.so.  It drives the reference's own functions
 * in the order large3Dexample2.c:main does (grid allocation :378-403,
 * ASSIGN_GRADIENT :443, BothCurvs loop :446-455, tube count :548-597,
 * omp_get_Ccomp :3225-3246, CompBiCG BICGSTAB.c:5) so that golden vectors
 * and the CPU baseline come from the reference itself.
 *
 * omp_get_Ccomp keeps its tube arrays in function statics that cannot be
 * reset, so one process serves one (N, k, distance grid) configuration.
 */
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <cmath>
#include <omp.h>

#include "PDE.h"
#include "frame.h"
#include "constants.h"

/* Reference symbols (C++ linkage, as the reference is compiled by g++). */
extern int N, SIZE;
extern double H, HCUBED, WAVE, G_DELTA;
extern double ***DIST, ***DIST_DX, ***DIST_DY, ***DIST_DZ, ***MCURV, ***GCURV;
int ASSIGN_GRADIENT(int N, double H, double ***dist, double ***graddx, double ***graddy,
                    double ***graddz, int weno_mode);
int BothCurvs(double ***dist, int i, int j, int k, int N, double H, double *meancurv,
              double *gausscurv);
void weno(double *dfp, double *dfn, double fi[], const double dx, const int order);
double Godunov(double signage, double a, double b, double c, double d, double e, double f);
int cal_interpgrad(int N, double H, double xj, double yj, double zj, double ***gradx,
                   double ***grady, double ***gradz, double *interpolatex, double *interpolatey,
                   double *interpolatez);
int cal_BothCurvs(double x, double y, double z, double H, double ***mcurv, double ***gcurv,
                  double *calmcurv, double *calgcurv);
double cal_delta(double epsilon, double x);
double omp_get_Ccomp(int size, int pi, int pj, double epsilon, double tempC[]);
int CompBiCG(int size, double *density, double *densityimg, double **Kernel, double **Kernelimg,
             double *b, double *bimg);
int omp_CompBiCG(int size, double *density, double *densityimg, double **Kernel, double **Kernelimg,
                 double *b, double *bimg, int chunk);
int DoubleLayerKernel(int size, double epsilon, double ***level, double ***leveldx, double ***leveldy,
                      double ***leveldz, double ***levelmcurv, double ***levelgcurv, double *zxlist, double *zylist,
                      double *zzlist, double *zxstarlist, double *zystarlist, double *zzstarlist, double *dist,
                      double *gradx, double *grady, double *gradz, double *delta, double *Jacobian, double *regfactor,
                      double *regfactorimg, double *result, double **Kernel, double **Kernelimg, double wavenum);

int new_HelmholtzKernel(int size, double delta, double epsilon, double *zxlist, double *zylist, double *zzlist,
                        double *zxstarlist, double *zystarlist, double *zzstarlist, double *dist, double *gradx,
                        double *grady, double *gradz, double *curv, double *Jacobian, double *PolyW, double *SineW,
                        double *PolyResult, double *SineResult, double **PolyKernelH, double **PolyKernelHimg,
                        double **SineKernelH, double **SineKernelHimg);
int new_HelmholtzKernelCombo(int size, double delta, double epsilon, double ***level, double ***leveldx,
                             double ***leveldy, double ***leveldz, double ***levelmcurv, double ***levelgcurv,
                             double *zxlist, double *zylist, double *zzlist, double *zxstarlist, double *zystarlist,
                             double *zzstarlist, double *dist, double *gradx, double *grady, double *gradz,
                             double *Jacobian, double *regfactor, double *regfactorimg, double *PolyW, double *SineW,
                             double *PolyResult, double *SineResult, double **PolyKernelH, double **PolyKernelHimg,
                             double **SineKernelH, double **SineKernelHimg, double wavenum, double eta);

static double ***alloc_grid(int S)
{
    double ***g = (double ***)malloc(S * sizeof(double **));
    for (int i = 0; i < S; i++) {
        g[i] = (double **)malloc(S * sizeof(double *));
        for (int j = 0; j < S; j++) g[i][j] = (double *)malloc(S * sizeof(double));
    }
    return g;
}

static void copy_out(double ***g, int S, double *out)
{
    for (int i = 0; i < S; i++)
        for (int j = 0; j < S; j++) memcpy(out + ((size_t)i * S + j) * S, g[i][j], S * sizeof(double));
}

extern "C" {

/* INT_L, INT_U, FACTOR, TAU_FACTOR, DIRICHLET, INTERIOR_MODE this library was compiled with. */
void ref_config(double *out)
{
    out[0] = INT_L;
    out[1] = INT_U;
    out[2] = FACTOR;
    out[3] = TAU_FACTOR;
    out[4] = DIRICHLET;
    out[5] = INTERIOR_MODE;
}

/* main :170-176 globals, :378-424 grid fill (from memory instead of the
 * distance file), :443 gradient and :446-455 curvature loop. */
int ref_setup(int n_cells, double wave, const double *dist)
{
    N = n_cells;
    SIZE = N + 1;
    H = (INT_U - INT_L) / N;
    HCUBED = H * H * H;
    G_DELTA = 1.0 * pow(H, 1.0);
    WAVE = wave;
    DIST = alloc_grid(SIZE);
    DIST_DX = alloc_grid(SIZE);
    DIST_DY = alloc_grid(SIZE);
    DIST_DZ = alloc_grid(SIZE);
    MCURV = alloc_grid(SIZE);
    GCURV = alloc_grid(SIZE);
    for (int i = 0; i < SIZE; i++)
        for (int j = 0; j < SIZE; j++)
            memcpy(DIST[i][j], dist + ((size_t)i * SIZE + j) * SIZE, SIZE * sizeof(double));
    ASSIGN_GRADIENT(N, H, DIST, DIST_DX, DIST_DY, DIST_DZ, 5);
    for (int i = 0; i < SIZE; i++)
        for (int j = 0; j < SIZE; j++)
            for (int k = 0; k < SIZE; k++) BothCurvs(DIST, i, j, k, N, H, &MCURV[i][j][k], &GCURV[i][j][k]);
    return 0;
}

void ref_grids(double *gx, double *gy, double *gz, double *mc, double *gc)
{
    copy_out(DIST_DX, SIZE, gx);
    copy_out(DIST_DY, SIZE, gy);
    copy_out(DIST_DZ, SIZE, gz);
    copy_out(MCURV, SIZE, mc);
    copy_out(GCURV, SIZE, gc);
}

double ref_h(void) { return H; }
double ref_eps(void) { return FACTOR * H; } /* main :350 */

void ref_weno(double *dfp, double *dfn, const double *fi, double dx, int order)
{
    double f[7];
    memcpy(f, fi, (order == 5 ? 7 : 5) * sizeof(double));
    weno(dfp, dfn, f, dx, order);
}

/* finite_difference3D.c:5-27, as compiled here. */
double ref_godunov(double signage, double a, double b, double c, double d, double e, double f)
{
    return Godunov(signage, a, b, c, d, e, f);
}

/* main :548-597: members |d| <= eps in (i,j,k) order, as linear indices. */
int64_t ref_tube(double eps, int64_t *idx)
{
    int64_t c = 0;
    for (int i = 0; i < SIZE; i++)
        for (int j = 0; j < SIZE; j++)
            for (int k = 0; k < SIZE; k++)
                if (fabs(DIST[i][j][k]) <= eps) {
                    if (idx) idx[c] = ((int64_t)i * SIZE + j) * SIZE + k;
                    c++;
                }
    return c;
}

/* Per-point arrays computed with the reference's own routines in the order
 * of omp_get_Ccomp's initialisation (large3Dexample2.c:4340-4452). */
int ref_tube_points(double eps, int64_t n, double *xs, double *nrm, double *delta, double *jac,
                    double *reg, double *w)
{
    const double tau = H * TAU_FACTOR;
    int64_t c = 0;
    int flagged = 0;
    for (int i = 0; i < SIZE; i++) {
        double zy = INT_L + H * (double)(i);
        for (int j = 0; j < SIZE; j++) {
            double zx = INT_L + H * (double)(j);
            for (int k = 0; k < SIZE; k++) {
                double zz = INT_L + H * (double)(k);
                double d = DIST[i][j][k];
                if (fabs(d) > eps) continue;
                if (c >= n) return -1;
                double tx = zx - d * DIST_DX[i][j][k];
                double ty = zy - d * DIST_DY[i][j][k];
                double tz = zz - d * DIST_DZ[i][j][k];
                xs[3 * c] = tx;
                xs[3 * c + 1] = ty;
                xs[3 * c + 2] = tz;
                delta[c] = cal_delta(eps, d);
                jac[c] = 1 + 2. * d * MCURV[i][j][k] + d * d * GCURV[i][j][k];
                double gx, gy, gz;
                if (cal_interpgrad(N, H, tx, ty, tz, DIST_DX, DIST_DY, DIST_DZ, &gx, &gy, &gz) == 1) flagged++;
                double gn = sqrt(gx * gx + gy * gy + gz * gz);
                nrm[3 * c] = gx / gn;
                nrm[3 * c + 1] = gy / gn;
                nrm[3 * c + 2] = gz / gn;
                double cm, cg;
                cal_BothCurvs(tx, ty, tz, H, MCURV, GCURV, &cm, &cg);
                double r1 = cm / (4. * PI * tau);
                double r2 = -5. * tau * (2. * cm) * (4. * cm * cm - cg) / (512. * PI);
                double r3 = -25. * tau * (2. * cm) * cg / (1536. * PI);
                double r4 = WAVE * WAVE * tau * 2. * cm / (48. * PI);
                reg[c] = (INTERIOR_MODE == 1) ? (r1 + r2 + r3 + r4) : -1. * (r1 + r2 + r3 + r4);
                w[c] = HCUBED * delta[c] * jac[c];
                c++;
            }
        }
    }
    return flagged;
}

/* Entries straight from the reference operator omp_get_Ccomp. */
void ref_entries(int n, int64_t m, const int *pi, const int *pj, double *re, double *im)
{
    double eps = FACTOR * H, t[2];
    for (int64_t q = 0; q < m; q++) {
        omp_get_Ccomp(n, pi[q], pj[q], eps, t);
        re[q] = t[0];
        im[q] = t[1];
    }
}

/* Dense rows [r0, r1) of the operator, row-major (r1-r0) x n.  The pair
 * routine's per-call path only reads its arrays once they are built, so
 * after a serial first call the rows are spread over nthreads threads
 * (the reference itself calls it serially, :3225-3246). */
void ref_dense_rows(int n, int r0, int r1, double *are, double *aim, int nthreads)
{
    double eps = FACTOR * H, t[2];
    omp_get_Ccomp(n, r0, 0, eps, t);
#pragma omp parallel for schedule(dynamic, 4) num_threads(nthreads)
    for (int i = r0; i < r1; i++) {
        double tt[2];
        for (int j = 0; j < n; j++) {
            omp_get_Ccomp(n, i, j, eps, tt);
            are[(size_t)(i - r0) * n + j] = tt[0];
            aim[(size_t)(i - r0) * n + j] = tt[1];
        }
    }
}

/* q = A p for rows [r0, r1): every entry from omp_get_Ccomp followed by the
 * complex multiply-add of the reference's product loops (large3Dexample2.c:
 * 3243-3244), i.e. one pair evaluation per (row, column).  Rows are spread
 * over nthreads threads after the serial first call has built the arrays. */
void ref_rows_matvec(int n, int r0, int r1, const double *pre, const double *pim, double *qre, double *qim,
                     int nthreads)
{
    double eps = FACTOR * H, t[2];
    omp_get_Ccomp(n, r0, 0, eps, t);
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads)
    for (int i = r0; i < r1; i++) {
        double tt[2], sr = 0.0, si = 0.0;
        for (int k = 0; k < n; k++) {
            omp_get_Ccomp(n, i, k, eps, tt);
            sr += (tt[0] * pre[k] - tt[1] * pim[k]);
            si += (tt[0] * pim[k] + tt[1] * pre[k]);
        }
        qre[i - r0] = sr;
        qim[i - r0] = si;
    }
}

/* DoubleLayerKernel (HelmholtzKernel.c:613-761): per-point arrays (20 x n,
 * rows as below; curv and the weight rows stay untouched) and the dense
 * matrix, row-major. */
int ref_double_layer(int n, double epsilon, double *pts, double *are, double *aim)
{
    double eps = epsilon;
    double *a[20];
    for (int r = 0; r < 20; r++) a[r] = pts + (size_t)r * n;
    double **K = (double **)malloc(n * sizeof(double *));
    double **Ki = (double **)malloc(n * sizeof(double *));
    for (int i = 0; i < n; i++) {
        K[i] = are + (size_t)i * n;
        Ki[i] = aim + (size_t)i * n;
    }
    int rc = DoubleLayerKernel(n, eps, DIST, DIST_DX, DIST_DY, DIST_DZ, MCURV, GCURV, a[0], a[1], a[2], a[3], a[4],
                               a[5], a[6], a[7], a[8], a[9], a[10], a[11], a[13], a[14], a[19], K, Ki, WAVE);
    free(K);
    free(Ki);
    return rc;
}

static double **rows_of(double *a, int n)
{
    double **r = (double **)malloc((size_t)(n > 0 ? n : 1) * sizeof(double *));
    for (int i = 0; i < n; i++) r[i] = a + (size_t)i * n;
    return r;
}

/* Row order of pts (20 x n) for the dense assemblers: zx zy zz xs ys zs
 * dist gx gy gz delta jac curv reg regimg polyw sinew polyres sineres result. */

/* new_HelmholtzKernelCombo (HelmholtzKernel.c:173-610) on the set-up grids:
 * returns regcount.  k1 = the PolyWeight matrices, k2 = the SineWeight ones
 * (only those of the build's POLY_TEST / SINE_TEST are written). */
int ref_combo(int n, double delta0, double epsilon, double wavenum, double eta, double *pts, double *k1re,
              double *k1im, double *k2re, double *k2im)
{
    double *a[20];
    for (int r = 0; r < 20; r++) a[r] = pts + (size_t)r * n;
    double **P = rows_of(k1re, n), **Pi = rows_of(k1im, n), **Sm = rows_of(k2re, n), **Si = rows_of(k2im, n);
    int rc = new_HelmholtzKernelCombo(n, delta0, epsilon, DIST, DIST_DX, DIST_DY, DIST_DZ, MCURV, GCURV, a[0], a[1],
                                      a[2], a[3], a[4], a[5], a[6], a[7], a[8], a[9], a[11], a[13], a[14], a[15], a[16],
                                      a[17], a[18], P, Pi, Sm, Si, wavenum, eta);
    free(P);
    free(Pi);
    free(Sm);
    free(Si);
    return rc;
}

/* new_HelmholtzKernel (HelmholtzKernel.c:3-169), the analytic sphere of frame.h. */
int ref_sphere_kernel(int n, double delta0, double epsilon, double *pts, double *k1re, double *k1im, double *k2re,
                      double *k2im)
{
    double *a[20];
    for (int r = 0; r < 20; r++) a[r] = pts + (size_t)r * n;
    double **P = rows_of(k1re, n), **Pi = rows_of(k1im, n), **Sm = rows_of(k2re, n), **Si = rows_of(k2im, n);
    int rc = new_HelmholtzKernel(n, delta0, epsilon, a[0], a[1], a[2], a[3], a[4], a[5], a[6], a[7], a[8], a[9],
                                 a[12], a[11], a[15], a[16], a[17], a[18], P, Pi, Sm, Si);
    free(P);
    free(Pi);
    free(Sm);
    free(Si);
    return rc;
}

/* The reference build's switches of the dense assemblers. */
void ref_dense_flags(int *out)
{
    out[0] = POLY_TEST;
    out[1] = SINE_TEST;
    out[2] = TRAD_ONESIDED;
    out[3] = COMBO_ONESIDED;
    out[4] = COMBO_INTERIOR;
    out[5] = INTERIOR_MODE;
}

void ref_sphere(double *out)
{
    out[0] = radius;
    out[1] = Cx;
    out[2] = Cy;
    out[3] = Cz;
}

/* CompBiCG (BICGSTAB.c:5-339) on a row-major dense matrix. */
// chunk <= 0: the serial CompBiCG (BICGSTAB.c:5); chunk > 0: the OpenMP
// omp_CompBiCG (BICGSTAB.c:344) with that schedule chunk (the driver's
// DEFAULT_OMP_CACHE_CHUNKSIZE is 16, large3Dexample2.c:38).
int ref_compbicg(int n, const double *are, const double *aim, const double *b, const double *bimg,
                 double *x, double *ximg, int chunk)
{
    double **K = (double **)malloc(n * sizeof(double *));
    double **Ki = (double **)malloc(n * sizeof(double *));
    for (int i = 0; i < n; i++) {
        K[i] = (double *)malloc(n * sizeof(double));
        Ki[i] = (double *)malloc(n * sizeof(double));
        memcpy(K[i], are + (size_t)i * n, n * sizeof(double));
        memcpy(Ki[i], aim + (size_t)i * n, n * sizeof(double));
    }
    double *bb = (double *)malloc(n * sizeof(double)), *bi = (double *)malloc(n * sizeof(double));
    memcpy(bb, b, n * sizeof(double));
    memcpy(bi, bimg, n * sizeof(double));
    int rc = (chunk > 0) ? omp_CompBiCG(n, x, ximg, K, Ki, bb, bi, chunk) : CompBiCG(n, x, ximg, K, Ki, bb, bi);
    for (int i = 0; i < n; i++) {
        free(K[i]);
        free(Ki[i]);
    }
    free(K);
    free(Ki);
    free(bb);
    free(bi);
    return rc;
}

} /* extern "C" */
