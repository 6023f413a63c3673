/*
 * ibim_oracle.c -- CPU restatement of the reference IBIM Helmholtz hot path.
 *
 * TEST INFRASTRUCTURE ONLY (the checker, never the product).  See
 * ibim_oracle.h for the layout conventions.  Each routine follows the cited
 * reference code's arithmetic in the same operation order; build with
 * -ffp-contract=off so no fused multiply-adds are introduced.
 *
 * Defects of the reference (moorhsum/Helmholtz-3D-torrone) are restated in
 * their patched form:
 *   - large3Dexample2.c:4528/4530 read regfactor[j]/regfactor[i] with an
 *     uninitialised loop variable; the intent, used here, is regfactor[pj]
 *     (Dirichlet) and regfactor[pi] (Neumann);
 *   - BICGSTAB.c:289 and large3Dexample2.c:3417 read errornorm before the
 *     first assignment; it starts at 1.0 here.
 */
#include "ibim_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

/* constants.h:5-7 */
#define OR_PI 3.14159265358979323846264338328
#define OR_LARGENUM 1000000

#define IDX(i, j, k) ((((size_t)(i)) * (size_t)S + (size_t)(j)) * (size_t)S + (size_t)(k))

double or_h(const or_params *p) { return (p->int_u - p->int_l) / p->N; }

/* tools.c:296-344 */
static double t_max(double a, double b) { return (a >= b) ? a : b; }
static double t_min(double a, double b) { return (a <= b) ? a : b; }
static double t_old_minmod(double x, double y) { return (fabs(x) < fabs(y)) ? x : y; }
static double t_min_abs(double a, double b, double c)
{
    double q = (fabs(a) < fabs(b)) ? a : b;
    return (fabs(q) < fabs(c)) ? q : c;
}

/* ------------------------------------------------------------------ */
/* WENO (weno.c:259-345)                                               */
/* ------------------------------------------------------------------ */
void or_weno(double *dfp, double *dfn, const double fi[], double dx, int order)
{
    double aa, bb, cc, dd, ee, ff, df, ih;
    double IS0, IS1, IS2, a0, a1, a2, w0, w1, w2;
    const double eps = 1e-12; /* pow(10.0,-12) is exactly this double */
    ih = 1. / dx;
    if (order == 3) {
        const int c = 2;
        aa = fi[c - 1] - fi[c - 2];
        bb = fi[c] - fi[c - 1];
        cc = fi[c + 1] - fi[c];
        dd = fi[c + 2] - fi[c + 1];
        df = bb + cc;
        a0 = bb - aa;
        a1 = cc - bb;
        a2 = dd - cc;
        IS0 = (eps + a2 * a2) / (eps + a1 * a1);
        w0 = 1. / (1. + 2. * IS0 * IS0);
        *dfp = .5 * ih * (df - w0 * (dd - 2. * cc + bb));
        IS0 = (eps + a0 * a0) / (eps + a1 * a1);
        w0 = 1 / (1 + 2. * IS0 * IS0);
        *dfn = .5 * ih * (df - w0 * (aa - 2. * bb + cc));
        return;
    }
    {
        const int c = 3;
        aa = (fi[c - 2] - fi[c - 3]) * ih;
        bb = (fi[c - 1] - fi[c - 2]) * ih;
        cc = (fi[c] - fi[c - 1]) * ih;
        dd = (fi[c + 1] - fi[c]) * ih;
        ee = (fi[c + 2] - fi[c + 1]) * ih;
        ff = (fi[c + 3] - fi[c + 2]) * ih;
        df = (-bb + 7. * (cc + dd) - ee) / 12.;
        aa = bb - aa;
        bb = cc - bb;
        cc = dd - cc;
        dd = ee - dd;
        ee = ff - ee;
        IS0 = 13. * (ee - dd) * (ee - dd) + 3. * (ee - 3. * dd) * (ee - 3. * dd);
        IS1 = 13. * (dd - cc) * (dd - cc) + 3. * (dd + cc) * (dd + cc);
        IS2 = 13. * (cc - bb) * (cc - bb) + 3. * (3. * cc - bb) * (3. * cc - bb);
        a0 = 1. / ((eps + IS0) * (eps + IS0));
        a1 = 6. / ((eps + IS1) * (eps + IS1));
        a2 = 3. / ((eps + IS2) * (eps + IS2));
        w1 = 1. / (a0 + a1 + a2);
        w0 = a0 * w1;
        w2 = a2 * w1;
        *dfp = df + w0 * (ee - 2. * dd + cc) / 3. + (w2 - .5) * (dd - 2. * cc + bb) / 6.;
        IS0 = 13. * (aa - bb) * (aa - bb) + 3. * (aa - 3. * bb) * (aa - 3. * bb);
        IS1 = 13. * (bb - cc) * (bb - cc) + 3. * (bb + cc) * (bb + cc);
        IS2 = 13. * (cc - dd) * (cc - dd) + 3. * (3. * cc - dd) * (3. * cc - dd);
        a0 = 1. / ((eps + IS0) * (eps + IS0));
        a1 = 6. / ((eps + IS1) * (eps + IS1));
        a2 = 3. / ((eps + IS2) * (eps + IS2));
        w1 = 1. / (a0 + a1 + a2);
        w0 = a0 * w1;
        w2 = a2 * w1;
        *dfn = df - w0 * (aa - 2. * bb + cc) / 3. - (w2 - .5) * (bb - 2. * cc + dd) / 6.;
    }
}

/* Mirror reflection of weno.c:131-139: u[-m] -> u[m], u[N+m] -> u[N-m]. */
static int mirror(int x, int N)
{
    if (x < 0) return -x;
    if (x > N) return 2 * N - x;
    return x;
}

/* Gather the (2*half+1)-point line through node (i,j,k) along one axis
 * (axis 0 = j / x, 1 = i / y, 2 = k / z) and apply weno(). */
static void weno_axis(const double *d, int N, double H, int i, int j, int k, int axis, int order,
                      double *up, double *un)
{
    const int S = N + 1;
    const int half = (order == 5) ? 3 : 2;
    double f[7];
    int c = 0;
    int center = (axis == 0) ? j : (axis == 1) ? i : k;
    for (int x = center - half; x <= center + half; x++) {
        int m = mirror(x, N);
        if (axis == 0) f[c] = d[IDX(i, m, k)];
        else if (axis == 1) f[c] = d[IDX(m, j, k)];
        else f[c] = d[IDX(i, j, m)];
        c++;
    }
    or_weno(up, un, f, H, order);
}

/* distance_application3D.c:56-140 (weno_mode >= 3 branch). */
void or_gradient(int N, double H, const double *d, double *gx, double *gy, double *gz, int order)
{
    const int S = N + 1;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < S; i++)
        for (int j = 0; j < S; j++)
            for (int k = 0; k < S; k++) {
                double Dxp, Dxn, Dyp, Dyn, Dzp, Dzn;
                weno_axis(d, N, H, i, j, k, 0, order, &Dxp, &Dxn);
                weno_axis(d, N, H, i, j, k, 1, order, &Dyp, &Dyn);
                weno_axis(d, N, H, i, j, k, 2, order, &Dzp, &Dzn);
                double aplus = t_max(0.0, Dxp), aminus = t_min(0.0, Dxp);
                double bplus = t_max(0.0, Dxn), bminus = t_min(0.0, Dxn);
                double cplus = t_max(0.0, Dyp), cminus = t_min(0.0, Dyp);
                double dplus = t_max(0.0, Dyn), dminus = t_min(0.0, Dyn);
                double eplus = t_max(0.0, Dzp), eminus = t_min(0.0, Dzp);
                double fplus = t_max(0.0, Dzn), fminus = t_min(0.0, Dzn);
                size_t o = IDX(i, j, k);
                if (d[o] > 0.0) {
                    gx[o] = (fabs(aminus) > fabs(bplus)) ? aminus : bplus;
                    gy[o] = (fabs(cminus) > fabs(dplus)) ? cminus : dplus;
                    gz[o] = (fabs(eminus) > fabs(fplus)) ? eminus : fplus;
                } else {
                    gx[o] = (fabs(aplus) > fabs(bminus)) ? aplus : bminus;
                    gy[o] = (fabs(cplus) > fabs(dminus)) ? cplus : dminus;
                    gz[o] = (fabs(eplus) > fabs(fminus)) ? eplus : fminus;
                }
            }
}

/* finite_difference3D.c:5-27 (Godunov upwind |grad phi|). */
static double godunov(double signage, double a, double b, double c, double d, double e, double f)
{
    double aplus = t_max(a, 0.0) * t_max(a, 0.0), aminus = t_min(a, 0.0) * t_min(a, 0.0);
    double bplus = t_max(b, 0.0) * t_max(b, 0.0), bminus = t_min(b, 0.0) * t_min(b, 0.0);
    double cplus = t_max(c, 0.0) * t_max(c, 0.0), cminus = t_min(c, 0.0) * t_min(c, 0.0);
    double dplus = t_max(d, 0.0) * t_max(d, 0.0), dminus = t_min(d, 0.0) * t_min(d, 0.0);
    double eplus = t_max(e, 0.0) * t_max(e, 0.0), eminus = t_min(e, 0.0) * t_min(e, 0.0);
    double fplus = t_max(f, 0.0) * t_max(f, 0.0), fminus = t_min(f, 0.0) * t_min(f, 0.0);
    if (signage > 0) return sqrt(t_max(aminus, bplus) + t_max(cminus, dplus) + t_max(eminus, fplus));
    if (signage < 0) return sqrt(t_max(aplus, bminus) + t_max(cplus, dminus) + t_max(eplus, fminus));
    return 0.0;
}

double or_godunov(double signage, double a, double b, double c, double d, double e, double f)
{
    return godunov(signage, a, b, c, d, e, f);
}

/* One stage of phi_t + S(phi0)(|grad phi| - 1) = 0 (see or_reinit). */
static void reinit_stage(int N, double H, double dt, const double *phi0, const double *phi, const double *base,
                         double w0, double w1, double *out, int order)
{
    const int S = N + 1;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < S; i++)
        for (int j = 0; j < S; j++)
            for (int k = 0; k < S; k++) {
                double Dxp, Dxn, Dyp, Dyn, Dzp, Dzn;
                weno_axis(phi, N, H, i, j, k, 0, order, &Dxp, &Dxn);
                weno_axis(phi, N, H, i, j, k, 1, order, &Dyp, &Dyn);
                weno_axis(phi, N, H, i, j, k, 2, order, &Dzp, &Dzn);
                size_t o = IDX(i, j, k);
                double p0 = phi0[o];
                double sgn = p0 / sqrt(p0 * p0 + H * H);
                double g = godunov(p0, Dxp, Dxn, Dyp, Dyn, Dzp, Dzn);
                double stage = phi[o] - dt * sgn * (g - 1.0);
                out[o] = (w0 != 0.0) ? (w0 * base[o] + w1 * stage) : stage;
            }
}

void or_reinit(int N, double H, double *phi, int iters, double cfl, int order)
{
    const size_t S = (size_t)N + 1, total = S * S * S;
    double *phi0 = malloc(total * sizeof(double)), *t1 = malloc(total * sizeof(double));
    double *t2 = malloc(total * sizeof(double));
    memcpy(phi0, phi, total * sizeof(double));
    const double dt = cfl * H;
    for (int it = 0; it < iters; it++) {
        reinit_stage(N, H, dt, phi0, phi, phi, 0.0, 1.0, t1, order);
        reinit_stage(N, H, dt, phi0, t1, phi, 0.5, 0.5, t2, order);
        memcpy(phi, t2, total * sizeof(double));
    }
    free(phi0);
    free(t1);
    free(t2);
}

/* ------------------------------------------------------------------ */
/* Second differences (finite_difference3D.c:220-390)                  */
/* ------------------------------------------------------------------ */
/* One axis of the limited second difference.  v(m) is the grid value m
 * steps from the node along the axis, c the node's coordinate on that axis.
 * xorder selects the reference's min_abs argument order, which differs
 * between XDER2 (p,c,n) and YDER2/ZDER2 (p,n,c). */
typedef struct {
    const double *d;
    size_t base;
    ptrdiff_t stride;
} line_t;
#define LV(L, m) ((L).d[(size_t)((ptrdiff_t)(L).base + (ptrdiff_t)(m) * (L).stride)])

static double der2_axis(line_t L, int c, int N, double H, int xorder)
{
    double DDp, DDc, DDn, Dpp, Dp, Dn, Dnn;
    if (c == 0) return 2.0 * (LV(L, 1) - LV(L, 0)) / (H * H);
    if (c == N) return 2.0 * (LV(L, -1) - LV(L, 0)) / (H * H);
    if (c < 3) {
        DDp = (2.0 * LV(L, 0) - 5.0 * LV(L, 1) + 4.0 * LV(L, 2) - LV(L, 3)) / (H * H);
        DDc = (LV(L, 1) - 2.0 * LV(L, 0) + LV(L, -1)) / (H * H);
        return (fabs(DDp) < fabs(DDc)) ? DDp : DDc;
    }
    if (c > N - 3) {
        DDn = (2.0 * LV(L, 0) - 5.0 * LV(L, -1) + 4.0 * LV(L, -2) - LV(L, -3)) / (H * H);
        DDc = (LV(L, 1) - 2.0 * LV(L, 0) + LV(L, -1)) / (H * H);
        return (fabs(DDn) < fabs(DDc)) ? DDn : DDc;
    }
    Dpp = LV(L, 2) - LV(L, 1);
    Dp = LV(L, 1) - LV(L, 0);
    Dn = LV(L, 0) - LV(L, -1);
    Dnn = LV(L, -1) - LV(L, -2);
    DDp = (2.0 * LV(L, 0) - 5.0 * LV(L, 1) + 4.0 * LV(L, 2) - LV(L, 3)) / (H * H);
    DDc = (LV(L, 1) - 2.0 * LV(L, 0) + LV(L, -1)) / (H * H);
    DDn = (2.0 * LV(L, 0) - 5.0 * LV(L, -1) + 4.0 * LV(L, -2) - LV(L, -3)) / (H * H);
    if ((Dp * Dnn <= 0.0) && (Dpp * Dn <= 0.0))
        return xorder ? t_min_abs(DDp, DDc, DDn) : t_min_abs(DDp, DDn, DDc);
    else if (Dp * Dnn <= 0.0)
        return t_old_minmod(DDp, DDc);
    else if (Dpp * Dn <= 0.0)
        return t_old_minmod(DDn, DDc);
    return DDc;
}

double or_xder2(const double *d, int N, double H, int i, int j, int k)
{
    const int S = N + 1;
    line_t L = {d, IDX(i, j, k), (ptrdiff_t)S};
    return der2_axis(L, j, N, H, 1);
}
double or_yder2(const double *d, int N, double H, int i, int j, int k)
{
    const int S = N + 1;
    line_t L = {d, IDX(i, j, k), (ptrdiff_t)S * S};
    return der2_axis(L, i, N, H, 0);
}
double or_zder2(const double *d, int N, double H, int i, int j, int k)
{
    const int S = N + 1;
    line_t L = {d, IDX(i, j, k), 1};
    return der2_axis(L, k, N, H, 0);
}

/* ------------------------------------------------------------------ */
/* Cross derivatives (finite_difference3D.c:393-721)                   */
/* ------------------------------------------------------------------ */
/* Plane spanned by axes a (first index of the reference's dxy[di][dj]) and
 * b (second); P(u,v) is the value u steps along a and v steps along b. */
typedef struct {
    const double *d;
    size_t base;
    ptrdiff_t sa, sb;
} plane_t;
#define PV(P, u, v) ((P).d[(size_t)((ptrdiff_t)(P).base + (ptrdiff_t)(u) * (P).sa + (ptrdiff_t)(v) * (P).sb)])

static double cross_plane(plane_t P, int ca, int cb, int N, double H)
{
    static const double coef[3] = {1.0, -4.0, 3.0};
    static const double allcoef[3][3] = {{1.0, -4.0, 3.0}, {-4.0, 16.0, -12.0}, {3.0, -12.0, 9.0}};
    if ((ca == 0) || (ca == N) || (cb == 0) || (cb == N)) return 0.0;
    if ((ca < 2) || (ca > N - 2) || (cb < 2) || (cb > N - 2))
        return (PV(P, 1, 1) - PV(P, -1, 1) - PV(P, 1, -1) + PV(P, -1, -1)) / (4.0 * H * H);
    double fin = OR_LARGENUM;
    for (int di = 0; di < 3; di++)
        for (int dj = 0; dj < 3; dj++) {
            double v = 0.0;
            if ((di == 1) && (dj == 1)) {
                v = (PV(P, 1, 1) - PV(P, -1, 1) - PV(P, 1, -1) + PV(P, -1, -1));
            } else if (di == 1) {
                int sign = dj - 1;
                for (int c = 2; c >= 0; c--)
                    v += (-1.0 * (double)(sign)*coef[2 - c] * (PV(P, 1, sign * c) - PV(P, -1, sign * c)));
            } else if (dj == 1) {
                int sign = di - 1;
                for (int c = 2; c >= 0; c--)
                    v += (-1.0 * (double)(sign)*coef[2 - c] * (PV(P, sign * c, 1) - PV(P, sign * c, -1)));
            } else {
                int si = di - 1, sj = dj - 1, sij = si * sj;
                for (int ci = 2; ci >= 0; ci--)
                    for (int cj = 2; cj >= 0; cj--)
                        v += (allcoef[2 - ci][2 - cj] * (double)(sij)*PV(P, si * ci, sj * cj));
            }
            if (fabs(v) < fabs(fin)) fin = v;
        }
    return fin / (4.0 * H * H);
}

double or_dxy(const double *d, int N, double H, int i, int j, int k)
{
    const int S = N + 1;
    plane_t P = {d, IDX(i, j, k), (ptrdiff_t)S * S, (ptrdiff_t)S};
    return cross_plane(P, i, j, N, H);
}
double or_dxz(const double *d, int N, double H, int i, int j, int k)
{
    const int S = N + 1;
    plane_t P = {d, IDX(i, j, k), (ptrdiff_t)S, 1};
    return cross_plane(P, j, k, N, H);
}
double or_dyz(const double *d, int N, double H, int i, int j, int k)
{
    const int S = N + 1;
    plane_t P = {d, IDX(i, j, k), (ptrdiff_t)S * S, 1};
    return cross_plane(P, i, k, N, H);
}

/* distance_application3D.c:35-53 */
void or_curvatures(int N, double H, const double *d, double *mcurv, double *gcurv)
{
    const int S = N + 1;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < S; i++)
        for (int j = 0; j < S; j++)
            for (int k = 0; k < S; k++) {
                double dxx = or_xder2(d, N, H, i, j, k);
                double dyy = or_yder2(d, N, H, i, j, k);
                double dzz = or_zder2(d, N, H, i, j, k);
                double dxy = or_dxy(d, N, H, i, j, k);
                double dxz = or_dxz(d, N, H, i, j, k);
                double dyz = or_dyz(d, N, H, i, j, k);
                double diag = dxx * dyy + dyy * dzz + dxx * dzz;
                double cross = dxy * dxy + dyz * dyz + dxz * dxz;
                mcurv[IDX(i, j, k)] = -0.5 * (dxx + dyy + dzz);
                gcurv[IDX(i, j, k)] = diag - cross;
            }
}

/* ------------------------------------------------------------------ */
/* Tube (large3Dexample2.c:548-597)                                    */
/* ------------------------------------------------------------------ */
int64_t or_tube(int N, const double *d, double eps, int64_t *idx)
{
    const size_t S = (size_t)N + 1, total = S * S * S;
    int64_t c = 0;
    for (size_t o = 0; o < total; o++)
        if (fabs(d[o]) <= eps) {
            if (idx) idx[c] = (int64_t)o;
            c++;
        }
    return c;
}

/* ------------------------------------------------------------------ */
/* Tube point initialisation (large3Dexample2.c:4340-4452)             */
/* ------------------------------------------------------------------ */
static double tri8(double lll, double llh, double lhl, double lhh, double hll, double hlh,
                   double hhl, double hhh, double lx, double ly, double lz, double H)
{
    /* interpolate3D.c:49-53: letters are (x,y,z) = (j,i,k) low/high */
    return (lll * (H - lx) * (H - ly) * (H - lz) + llh * (H - lx) * (H - ly) * lz +
            lhl * (H - lx) * ly * (H - lz) + lhh * (H - lx) * ly * lz + hll * lx * (H - ly) * (H - lz) +
            hlh * lx * (H - ly) * lz + hhl * lx * ly * (H - lz) + hhh * lx * ly * lz) /
           (H * H * H);
}

/* interpolate3D.c:5-102 (cal_interpgrad).  Returns 0 ok, 1 norm far from 1,
 * -1 when the cell lies outside the grid (the reference calls exit there). */
static int interp_grad(int N, double H, double int_l, double xj, double yj, double zj,
                       const double *gx, const double *gy, const double *gz, double *ox,
                       double *oy, double *oz)
{
    const int S = N + 1;
    int i = (int)((yj - int_l) / H);
    int j = (int)((xj - int_l) / H);
    int k = (int)((zj - int_l) / H);
    double lowx = xj - int_l - (double)(j)*H;
    double lowy = yj - int_l - (double)(i)*H;
    double lowz = zj - int_l - (double)(k)*H;
    if ((lowx > H) || (lowx < 0.0) || (lowy > H) || (lowy < 0.0) || (lowz < 0.0) || (lowz > H)) return -1;
    if (i < 0 || j < 0 || k < 0 || i >= N || j >= N || k >= N) return -1;
    const double *g[3] = {gx, gy, gz};
    double r[3];
    for (int c = 0; c < 3; c++) {
        const double *a = g[c];
        r[c] = tri8(a[IDX(i, j, k)], a[IDX(i, j, k + 1)], a[IDX(i + 1, j, k)], a[IDX(i + 1, j, k + 1)],
                    a[IDX(i, j + 1, k)], a[IDX(i, j + 1, k + 1)], a[IDX(i + 1, j + 1, k)],
                    a[IDX(i + 1, j + 1, k + 1)], lowx, lowy, lowz, H);
    }
    double nrm = sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
    *ox = r[0] / nrm;
    *oy = r[1] / nrm;
    *oz = r[2] / nrm;
    return (fabs(nrm - 1.0) > 0.5) ? 1 : 0;
}

/* interpolate3D.c:569-605 (cal_BothCurvs) */
static int interp_curv(int N, double H, double int_l, double x, double y, double z,
                       const double *mc, const double *gc, double *om, double *og)
{
    const int S = N + 1;
    int j = (int)((x + 1e-19 - int_l) / H);
    int i = (int)((y + 1e-19 - int_l) / H);
    int k = (int)((z + 1e-19 - int_l) / H);
    if (i < 0 || j < 0 || k < 0 || i >= N || j >= N || k >= N) return -1;
    double lowx = x - int_l - (double)(j)*H;
    double lowy = y - int_l - (double)(i)*H;
    double lowz = z - int_l - (double)(k)*H;
    double hc = H * H * H;
    const double *a[2] = {mc, gc};
    double r[2];
    for (int c = 0; c < 2; c++) {
        const double *m = a[c];
        r[c] = (m[IDX(i, j, k)] * (H - lowx) * (H - lowy) * (H - lowz) +
                m[IDX(i + 1, j, k)] * (H - lowx) * lowy * (H - lowz) +
                m[IDX(i, j + 1, k)] * lowx * (H - lowy) * (H - lowz) +
                m[IDX(i + 1, j + 1, k)] * lowx * lowy * (H - lowz) +
                m[IDX(i, j, k + 1)] * (H - lowx) * (H - lowy) * lowz +
                m[IDX(i + 1, j, k + 1)] * (H - lowx) * lowy * lowz +
                m[IDX(i, j + 1, k + 1)] * lowx * (H - lowy) * lowz +
                m[IDX(i + 1, j + 1, k + 1)] * lowx * lowy * lowz) /
               hc;
    }
    *om = r[0];
    *og = r[1];
    return 0;
}

/* functions.c:366-374 (cosine mode) */
static double cal_delta(double epsilon, double x)
{
    if (fabs(x) <= epsilon) return (1.0 / (2.0 * epsilon)) * (1.0 + cos(OR_PI * x / epsilon));
    return 0.0;
}

int or_tube_init(const or_params *p, const double *d, const double *gx, const double *gy,
                 const double *gz, const double *mcurv, const double *gcurv, int64_t n,
                 const int64_t *idx, double *xs, double *nrm, double *delta, double *jac,
                 double *reg, double *w)
{
    const int N = p->N, S = N + 1;
    const double H = or_h(p), eps = p->factor * H, tau = H * p->tau_factor;
    const double HC = H * H * H, W = p->wave;
    int bad = 0;
    for (int64_t c = 0; c < n; c++) {
        int64_t o = idx[c];
        int i = (int)(o / ((int64_t)S * S)), j = (int)((o / S) % S), k = (int)(o % S);
        double zy = p->int_l + H * (double)(i);
        double zx = p->int_l + H * (double)(j);
        double zz = p->int_l + H * (double)(k);
        double dd = d[o];
        double tx = zx - dd * gx[o], ty = zy - dd * gy[o], tz = zz - dd * gz[o];
        xs[3 * c + 0] = tx;
        xs[3 * c + 1] = ty;
        xs[3 * c + 2] = tz;
        delta[c] = cal_delta(eps, dd);
        jac[c] = 1 + 2. * dd * mcurv[o] + dd * dd * gcurv[o];
        double nx, ny, nz;
        int st = interp_grad(N, H, p->int_l, tx, ty, tz, gx, gy, gz, &nx, &ny, &nz);
        if (st < 0) {
            if (!bad) bad = (int)(c + 1);
            nx = ny = nz = 0.0;
        } else {
            /* the driver normalises the returned unit vector again (:4409-4412) */
            double gn = sqrt(nx * nx + ny * ny + nz * nz);
            nx = nx / gn;
            ny = ny / gn;
            nz = nz / gn;
        }
        nrm[3 * c + 0] = nx;
        nrm[3 * c + 1] = ny;
        nrm[3 * c + 2] = nz;
        double cm = 0.0, cg = 0.0;
        if (interp_curv(N, H, p->int_l, tx, ty, tz, mcurv, gcurv, &cm, &cg) < 0 && !bad) bad = (int)(c + 1);
        double r1 = cm / (4. * OR_PI * tau);
        double r2 = -5. * tau * (2. * cm) * (4. * cm * cm - cg) / (512. * OR_PI);
        double r3 = -25. * tau * (2. * cm) * cg / (1536. * OR_PI);
        double r4 = W * W * tau * 2. * cm / (48. * OR_PI);
        if (p->interior == 1) reg[c] = r1 + r2 + r3 + r4;
        else reg[c] = -1. * (r1 + r2 + r3 + r4);
        w[c] = HC * delta[c] * jac[c];
    }
    return bad;
}

/* ------------------------------------------------------------------ */
/* Pair kernel (large3Dexample2.c:4463-4564)                           */
/* ------------------------------------------------------------------ */
static inline void pair_entry(double W, double tau, int dirichlet, int interior, const double *xs,
                              const double *nrm, const double *reg, const double *w, int64_t pi,
                              int64_t pj, double *re, double *im)
{
    static const double recipfourpi = 1. / (4. * OR_PI);
    double xmy1 = xs[3 * pi + 0] - xs[3 * pj + 0];
    double xmy2 = xs[3 * pi + 1] - xs[3 * pj + 1];
    double xmy3 = xs[3 * pi + 2] - xs[3 * pj + 2];
    double rho = sqrt(xmy1 * xmy1 + xmy2 * xmy2 + xmy3 * xmy3);
    double partial, partialimg;
    if (rho > tau) {
        double rec = 1. / rho;
        double par = W * rho;
        double S = sin(par), C = cos(par);
        double eS = S * rec, eC = C * rec;
        double denom = recipfourpi * rec * rec;
        double ct1 = -1. * (W * S + eC) * denom;
        double ct2 = (W * C - eS) * denom;
        int64_t q = dirichlet ? pj : pi;
        double inner = xmy1 * nrm[3 * q + 0] + xmy2 * nrm[3 * q + 1] + xmy3 * nrm[3 * q + 2];
        if (interior == 1) {
            partial = (-1.0) * ct1 * inner;
            partialimg = (-1.0) * ct2 * inner;
        } else {
            partial = ct1 * inner;
            partialimg = ct2 * inner;
        }
    } else {
        partial = dirichlet ? reg[pj] : reg[pi];
        partialimg = 0.0;
    }
    *re = w[pj] * partial;
    *im = w[pj] * partialimg;
    if (pi == pj) *re += 0.5;
}

void or_entry(const or_params *p, const double *xs, const double *nrm, const double *reg,
              const double *w, int64_t pi, int64_t pj, double *re, double *im)
{
    const double H = or_h(p);
    pair_entry(p->wave, H * p->tau_factor, p->dirichlet, p->interior, xs, nrm, reg, w, pi, pj, re, im);
}

void or_dense_rows(const or_params *p, int64_t n, const double *xs, const double *nrm,
                   const double *reg, const double *w, int64_t r0, int64_t r1, double *are,
                   double *aim)
{
    const double H = or_h(p), tau = H * p->tau_factor;
#pragma omp parallel for schedule(static)
    for (int64_t i = r0; i < r1; i++)
        for (int64_t j = 0; j < n; j++)
            pair_entry(p->wave, tau, p->dirichlet, p->interior, xs, nrm, reg, w, i, j,
                       &are[(i - r0) * n + j], &aim[(i - r0) * n + j]);
}

void or_matvec(const or_params *p, int64_t n, const double *xs, const double *nrm,
               const double *reg, const double *w, const double *pre, const double *pim,
               double *qre, double *qim, int adjoint, int64_t r0, int64_t r1, int nthreads)
{
    const double H = or_h(p), tau = H * p->tau_factor;
#ifdef _OPENMP
    if (nthreads < 1) nthreads = 1;
#pragma omp parallel for schedule(dynamic, 16) num_threads(nthreads)
#endif
    for (int64_t i = r0; i < r1; i++) {
        double sr = 0.0, si = 0.0;
        for (int64_t k = 0; k < n; k++) {
            double a, b;
            if (!adjoint) {
                /* large3Dexample2.c:3243-3244 */
                pair_entry(p->wave, tau, p->dirichlet, p->interior, xs, nrm, reg, w, i, k, &a, &b);
                sr += (a * pre[k] - b * pim[k]);
                si += (a * pim[k] + b * pre[k]);
            } else {
                /* large3Dexample2.c:3301-3302: conj(A[k][i]) */
                pair_entry(p->wave, tau, p->dirichlet, p->interior, xs, nrm, reg, w, k, i, &a, &b);
                sr += (a * pre[k] + b * pim[k]);
                si += (a * pim[k] - b * pre[k]);
            }
        }
        qre[i - r0] = sr;
        qim[i - r0] = si;
    }
}

/* ------------------------------------------------------------------ */
/* Complex BiCG (BICGSTAB.c:104-308; large3Dexample2.c:3131-3433)      */
/* ------------------------------------------------------------------ */
static double inner(int64_t n, const double *a, const double *b)
{
    double s = 0.0;
    for (int64_t i = 0; i < n; i++) s += a[i] * b[i];
    return s;
}

typedef void (*apply_fn)(void *ctx, const double *pre, const double *pim, double *qre,
                         double *qim, int adjoint);

static int bicg_core(int64_t n, apply_fn apply, void *ctx, const double *b, const double *bimg,
                     double *xo, double *xio, double accuracy, int maxit, double *resid)
{
    size_t sz = (size_t)n * sizeof(double);
    double *x = calloc(n, 8), *ximg = calloc(n, 8), *r = malloc(sz), *rimg = malloc(sz);
    double *rt = malloc(sz), *rtimg = malloc(sz), *pv = malloc(sz), *pimg = malloc(sz);
    double *pt = malloc(sz), *ptimg = malloc(sz), *Ap = malloc(sz), *Apimg = malloc(sz);
    double *Apt = malloc(sz), *Aptimg = malloc(sz);
    double normb = sqrt(inner(n, b, b) + inner(n, bimg, bimg));
    for (int64_t c = 0; c < n; c++) {
        r[c] = b[c];
        rimg[c] = bimg[c];
        pv[c] = r[c];
        pimg[c] = rimg[c];
        rt[c] = r[c];
        rtimg[c] = (-1.0) * rimg[c];
        pt[c] = rt[c];
        ptimg[c] = rtimg[c];
    }
    double innerrold = inner(n, r, rt) + inner(n, rimg, rtimg);
    double innerroldimg = inner(n, rimg, rt) - inner(n, r, rtimg);
    double bcsum = 0.0;
    for (int64_t c = 0; c < n; c++) {
        bcsum += fabs(r[c]);
        bcsum += fabs(rimg[c]);
    }
    double errornorm = 1.0, preerrornorm;
    int countrun = 0;
    if (bcsum < 1e-15) {
        errornorm = 0.0;
        goto done;
    }
    for (int it = 1; it <= maxit; it++) {
        apply(ctx, pv, pimg, Ap, Apimg, 0);
        apply(ctx, pt, ptimg, Apt, Aptimg, 1);
        double ca = inner(n, r, rt) + inner(n, rimg, rtimg);
        double cb = inner(n, rimg, rt) - inner(n, r, rtimg);
        double cc = inner(n, Ap, pt) + inner(n, Apimg, ptimg);
        double cd = inner(n, Apimg, pt) - inner(n, Ap, ptimg);
        double num = ca * cc + cb * cd, numi = cb * cc - ca * cd, den = cc * cc + cd * cd;
        double alpha = num / den, alphaimg = numi / den;
        for (int64_t j = 0; j < n; j++) {
            x[j] = x[j] + alpha * pv[j] - alphaimg * pimg[j];
            ximg[j] = ximg[j] + alphaimg * pv[j] + alpha * pimg[j];
            r[j] = r[j] - alpha * Ap[j] + alphaimg * Apimg[j];
            rimg[j] = rimg[j] - alphaimg * Ap[j] - alpha * Apimg[j];
            rt[j] = rt[j] - alpha * Apt[j] - alphaimg * Aptimg[j];
            rtimg[j] = rtimg[j] + alphaimg * Apt[j] - alpha * Aptimg[j];
        }
        cc = innerrold;
        cd = innerroldimg;
        ca = inner(n, r, rt) + inner(n, rimg, rtimg);
        cb = inner(n, rimg, rt) - inner(n, r, rtimg);
        num = ca * cc + cb * cd;
        numi = cb * cc - ca * cd;
        den = cc * cc + cd * cd;
        double beta = num / den, betaimg = numi / den;
        innerrold = ca;
        innerroldimg = cb;
        for (int64_t j = 0; j < n; j++) {
            double po = pv[j], poi = pimg[j], pto = pt[j], ptoi = ptimg[j];
            pv[j] = r[j] + beta * po - betaimg * poi;
            pimg[j] = rimg[j] + betaimg * po + beta * poi;
            pt[j] = rt[j] + beta * pto + betaimg * ptoi;
            ptimg[j] = rtimg[j] - betaimg * pto + beta * ptoi;
        }
        preerrornorm = errornorm;
        errornorm = sqrt(inner(n, r, r) + inner(n, rimg, rimg)) / normb;
        countrun++;
        if (errornorm < accuracy) break;
        if (errornorm != errornorm) break;
        if (fabs(preerrornorm - errornorm) < 1e-3 * accuracy) break;
    }
done:
    memcpy(xo, x, sz);
    memcpy(xio, ximg, sz);
    if (resid) *resid = errornorm;
    free(x); free(ximg); free(r); free(rimg); free(rt); free(rtimg); free(pv); free(pimg);
    free(pt); free(ptimg); free(Ap); free(Apimg); free(Apt); free(Aptimg);
    return countrun;
}

typedef struct {
    const or_params *p;
    int64_t n;
    const double *xs, *nrm, *reg, *w;
    int nthreads;
} free_ctx;

static void apply_free(void *c, const double *pre, const double *pim, double *qre, double *qim,
                       int adjoint)
{
    free_ctx *f = (free_ctx *)c;
    or_matvec(f->p, f->n, f->xs, f->nrm, f->reg, f->w, pre, pim, qre, qim, adjoint, 0, f->n,
              f->nthreads);
}

int or_bicg(const or_params *p, int64_t n, const double *xs, const double *nrm,
            const double *reg, const double *w, const double *bre, const double *bim,
            double *xre, double *xim, double acc, int maxit, int nthreads, double *resid)
{
    free_ctx f = {p, n, xs, nrm, reg, w, nthreads};
    return bicg_core(n, apply_free, &f, bre, bim, xre, xim, acc, maxit, resid);
}

typedef struct {
    int64_t n;
    const double *are, *aim;
} dense_ctx;

static void apply_dense(void *c, const double *pre, const double *pim, double *qre, double *qim,
                        int adjoint)
{
    dense_ctx *f = (dense_ctx *)c;
    int64_t n = f->n;
    for (int64_t j = 0; j < n; j++) {
        double s = 0.0, si = 0.0;
        for (int64_t k = 0; k < n; k++) {
            if (!adjoint) {
                double a = f->are[j * n + k], b = f->aim[j * n + k];
                s += (a * pre[k] - b * pim[k]);
                si += (a * pim[k] + b * pre[k]);
            } else {
                double a = f->are[k * n + j], b = f->aim[k * n + j];
                s += (a * pre[k] + b * pim[k]);
                si += (a * pim[k] - b * pre[k]);
            }
        }
        qre[j] = s;
        qim[j] = si;
    }
}

int or_bicg_dense(int64_t n, const double *are, const double *aim, const double *bre,
                  const double *bim, double *xre, double *xim, double acc, int maxit,
                  double *resid)
{
    dense_ctx f = {n, are, aim};
    return bicg_core(n, apply_dense, &f, bre, bim, xre, xim, acc, maxit, resid);
}

/* ------------------------------------------------------------------ */
/* Off-surface evaluation                                              */
/* ------------------------------------------------------------------ */
void or_eval(const or_params *p, int64_t n, const double *xs, const double *nrm,
             const double *w, const double *sre, const double *sim, int64_t m,
             const double *rx, double *ure, double *uim, int double_layer, int nthreads)
{
    const double H = or_h(p), tau = H * p->tau_factor, W = p->wave;
    static const double recipfourpi = 1. / (4. * OR_PI);
#ifdef _OPENMP
    if (nthreads < 1) nthreads = 1;
#pragma omp parallel for schedule(static) num_threads(nthreads)
#endif
    for (int64_t r = 0; r < m; r++) {
        double sx = rx[3 * r], sy = rx[3 * r + 1], sz = rx[3 * r + 2];
        double u = 0.0, ui = 0.0;
        for (int64_t c = 0; c < n; c++) {
            double zx = xs[3 * c], zy = xs[3 * c + 1], zz = xs[3 * c + 2];
            /* large3Dexample2.c:1810-1824 */
            double sn = sqrt((zx - sx) * (zx - sx) + (zy - sy) * (zy - sy) + (zz - sz) * (zz - sz));
            double ph, phi;
            if (!double_layer) {
                if (sn > tau) {
                    ph = cos(W * sn) / (-4. * OR_PI * sn);
                    phi = sin(W * sn) / (-4. * OR_PI * sn);
                } else {
                    ph = 0.;
                    phi = 0.;
                }
            } else {
                if (sn > tau) {
                    double xmy1 = sx - zx, xmy2 = sy - zy, xmy3 = sz - zz;
                    double rec = 1. / sn, par = W * sn;
                    double S = sin(par), C = cos(par);
                    double denom = recipfourpi * rec * rec;
                    double ct1 = -1. * (W * S + C * rec) * denom;
                    double ct2 = (W * C - S * rec) * denom;
                    double in = xmy1 * nrm[3 * c] + xmy2 * nrm[3 * c + 1] + xmy3 * nrm[3 * c + 2];
                    double sg = (p->interior == 1) ? -1.0 : 1.0;
                    ph = sg * ct1 * in;
                    phi = sg * ct2 * in;
                } else {
                    ph = 0.;
                    phi = 0.;
                }
            }
            u += ((ph * sre[c] - phi * sim[c]) * w[c]);
            ui += ((ph * sim[c] + phi * sre[c]) * w[c]);
        }
        ure[r] = u;
        uim[r] = ui;
    }
}

/* ------------------------------------------------------------------ */
/* Boundary data                                                       */
/* ------------------------------------------------------------------ */
void or_point_source_rhs(const or_params *p, int64_t n, const double *xs, const double *nrm,
                         const double *src, int kind, double *bre, double *bim)
{
    const double W = p->wave;
    for (int64_t c = 0; c < n; c++) {
        double dx = xs[3 * c] - src[0], dy = xs[3 * c + 1] - src[1], dz = xs[3 * c + 2] - src[2];
        double r = sqrt(dx * dx + dy * dy + dz * dz);
        double C = cos(W * r), S = sin(W * r);
        if (kind == 0) {
            /* g = e^{ikr}/(4 pi r) */
            bre[c] = C / (4. * OR_PI * r);
            bim[c] = S / (4. * OR_PI * r);
        } else if (kind == 1) {
            /* dg/dn_out with n_out = -n (n = grad d points inward):
             * grad g = g'(r) (x-s)/r, g'(r) = e^{ikr}(ikr-1)/(4 pi r^2) */
            double dn = -(dx * nrm[3 * c] + dy * nrm[3 * c + 1] + dz * nrm[3 * c + 2]) / r;
            double gr = (-C - W * r * S) / (4. * OR_PI * r * r);
            double gi = (W * r * C - S) / (4. * OR_PI * r * r);
            bre[c] = gr * dn;
            bim[c] = gi * dn;
        } else if (kind == 2) {
            /* reference monopole Neumann data, large3Dexample2.c:4778,4840 */
            bre[c] = (sin(W * r) / r) + (cos(W * r) / (W * r * r));
            bim[c] = (sin(W * r) / (W * r * r)) - (cos(W * r) / r);
        } else {
            /* reference monopole Dirichlet data, large3Dexample2.c:4642,4724 */
            bre[c] = -1.0 * cos(W * r) / (W * r);
            bim[c] = -1.0 * sin(W * r) / (W * r);
        }
    }
}

/* ------------------------------------------------------------------ */
/* Dense assemblers (HelmholtzKernel.c)                                */
/* ------------------------------------------------------------------ */
/* functions.h:25-26 (MOMENT_ORDER 1 constants of SineWeight) */
#define OR_CONSTA1 -759.2781934172483
#define OR_CONSTB1 446.2604260472818

/* functions.c:793-833: first moment with smooth ends */
double or_poly_weight(double t, double tau)
{
    if ((t <= tau) || (t >= 1.0)) return 0.0;
    double tau2 = tau * tau;
    double term1 = 7. * (1 + tau) * t;
    double term2 = -2. * (2. + 3. * tau + 2. * tau2);
    return 60. * (t - 1.) * (t - 1.) * (t - tau) * (t - tau) * (term1 + term2) / pow(tau - 1., 7.0);
}

/* functions.c:835-866, MOMENT_ORDER 1 */
double or_sine_weight(double t, double tau)
{
    if ((t <= tau) || (t >= 1.0)) return 0.0;
    return exp(0.5 / ((t - 0.1) * (t - 1.))) * (OR_CONSTA1 * t + OR_CONSTB1);
}

/* functions.c:433-456 (cal_phi, LAPLACE 0) */
static double fd_phi_re(double wave, double xi, double yi, double zi, double xj, double yj, double zj)
{
    double norm = sqrt(fabs((xi - xj) * (xi - xj) + (yi - yj) * (yi - yj) + (zi - zj) * (zi - zj)));
    if (norm == 0.0) return 0.0;
    return cos(wave * norm) / (-4.0 * OR_PI * norm);
}

/* functions.c:481-504 (phiimg) */
static double fd_phi_im(double wave, double xi, double yi, double zi, double xj, double yj, double zj)
{
    double norm = sqrt(fabs(pow(xi - xj, 2.0) + pow(yi - yj, 2.0) + pow(zi - zj, 2.0)));
    if (norm == 0.0) return 0.0;
    return sin(wave * norm) / (-4.0 * OR_PI * norm);
}

/* functions.c:121-155 (cal_partial): central difference of the fundamental
 * solution in the second variable, step H; modes 1-3 real, 4-6 imaginary. */
static void fd_partials(double H, double wave, const double *a, const double *b, double re[3], double im[3])
{
    re[0] = (fd_phi_re(wave, a[0], a[1], a[2], b[0] + H, b[1], b[2]) -
             fd_phi_re(wave, a[0], a[1], a[2], b[0] - H, b[1], b[2])) / (2.0 * H);
    re[1] = (fd_phi_re(wave, a[0], a[1], a[2], b[0], b[1] + H, b[2]) -
             fd_phi_re(wave, a[0], a[1], a[2], b[0], b[1] - H, b[2])) / (2.0 * H);
    re[2] = (fd_phi_re(wave, a[0], a[1], a[2], b[0], b[1], b[2] + H) -
             fd_phi_re(wave, a[0], a[1], a[2], b[0], b[1], b[2] - H)) / (2.0 * H);
    im[0] = (fd_phi_im(wave, a[0], a[1], a[2], b[0] + H, b[1], b[2]) -
             fd_phi_im(wave, a[0], a[1], a[2], b[0] - H, b[1], b[2])) / (2.0 * H);
    im[1] = (fd_phi_im(wave, a[0], a[1], a[2], b[0], b[1] + H, b[2]) -
             fd_phi_im(wave, a[0], a[1], a[2], b[0], b[1] - H, b[2])) / (2.0 * H);
    im[2] = (fd_phi_im(wave, a[0], a[1], a[2], b[0], b[1], b[2] + H) -
             fd_phi_im(wave, a[0], a[1], a[2], b[0], b[1], b[2] - H)) / (2.0 * H);
}

/* Is node value d in the point set of the assembler? */
static int dense_member(int kind, const or_dense_opts *o, double d)
{
    if (kind == OR_DENSE_DOUBLE_LAYER) { /* HelmholtzKernel.c:653-662 */
        if (o->onesided == 0) return !(fabs(d) > o->epsilon);
        return !((d > o->epsilon) || (d < 0.));
    }
    if (kind == OR_DENSE_COMBO) { /* :247-265 */
        if (o->onesided == 0) return !((fabs(d) > o->epsilon) || (fabs(d) < o->delta0));
        if (o->combo_interior == 1) return !((d > o->epsilon) || (d < o->delta0));
        return !((d < -1. * o->epsilon) || (d > -1. * o->delta0));
    }
    /* :46-55 */
    if (o->onesided == 0) return !((fabs(d) > o->epsilon) || (fabs(d) < o->delta0));
    return !((d > o->epsilon) | (d < o->delta0));
}

static void dense_weights(const or_dense_opts *o, double hcubed, double dist, double jac, double *row, int64_t n,
                          int64_t c)
{
    const double eps = o->epsilon;
    if (o->poly) {
        double w = (o->onesided == 0) ? or_poly_weight(fabs(dist / eps), o->delta0 / eps) / (2.0 * eps)
                                      : or_poly_weight(fabs(dist / eps), o->delta0 / eps) / (eps);
        row[OR_DP_POLYW * n + c] = w;
        row[OR_DP_POLYRES * n + c] = hcubed * jac * w;
    }
    if (o->sine) {
        double w = (o->onesided == 0) ? or_sine_weight(fabs(dist / eps), o->delta0 / eps) / (2.0 * eps)
                                      : or_sine_weight(fabs(dist / eps), o->delta0 / eps) / (eps);
        row[OR_DP_SINEW * n + c] = w;
        row[OR_DP_SINERES * n + c] = hcubed * jac * w;
    }
}

int64_t or_dense_points(int kind, const or_params *p, const or_dense_opts *o, const double *d,
                        const double *gx, const double *gy, const double *gz, const double *mcurv,
                        const double *gcurv, int64_t n_alloc, double *pts)
{
    const int N = p->N, S = N + 1;
    const double H = or_h(p), hcubed = H * H * H, int_l = p->int_l, W = p->wave;
    int64_t count = 0;
    for (int i = 0; i < S; i++) {
        const double zy = int_l + H * (double)(i);
        for (int j = 0; j < S; j++) {
            const double zx = int_l + H * (double)(j);
            for (int k = 0; k < S; k++) {
                const double zz = int_l + H * (double)(k);
                double dd;
                if (kind == OR_DENSE_SPHERE)
                    dd = o->radius - sqrt((zx - o->cx) * (zx - o->cx) + (zy - o->cy) * (zy - o->cy) +
                                          (zz - o->cz) * (zz - o->cz));
                else
                    dd = d[IDX(i, j, k)];
                if (!dense_member(kind, o, dd)) continue;
                const int64_t c = count++;
                if (!pts || n_alloc <= 0) continue;
                if (c >= n_alloc) continue;
                const int64_t n = n_alloc;
                double *row = pts;
                row[OR_DP_ZX * n + c] = zx;
                row[OR_DP_ZY * n + c] = zy;
                row[OR_DP_ZZ * n + c] = zz;
                row[OR_DP_DIST * n + c] = dd;
                if (kind == OR_DENSE_SPHERE) {
                    /* :57-98 */
                    const double r0 = sqrt((zx - o->cx) * (zx - o->cx) + (zy - o->cy) * (zy - o->cy) +
                                           (zz - o->cz) * (zz - o->cz));
                    const double tgx = (o->cx - zx) / r0, tgy = (o->cy - zy) / r0, tgz = (o->cz - zz) / r0;
                    const double sx = zx - dd * tgx, sy = zy - dd * tgy, sz = zz - dd * tgz;
                    const double r1 = sqrt((sx - o->cx) * (sx - o->cx) + (sy - o->cy) * (sy - o->cy) +
                                           (sz - o->cz) * (sz - o->cz));
                    row[OR_DP_XS * n + c] = sx;
                    row[OR_DP_YS * n + c] = sy;
                    row[OR_DP_ZS * n + c] = sz;
                    row[OR_DP_GX * n + c] = (o->cx - sx) / r1;
                    row[OR_DP_GY * n + c] = (o->cy - sy) / r1;
                    row[OR_DP_GZ * n + c] = (o->cz - sz) / r1;
                    const double curv = 1. / (o->radius - dd);
                    const double jac = 1. + dd * curv;
                    row[OR_DP_CURV * n + c] = curv;
                    row[OR_DP_JAC * n + c] = jac;
                    dense_weights(o, hcubed, dd, jac, row, n, c);
                    continue;
                }
                const size_t q = IDX(i, j, k);
                const double sx = zx - dd * gx[q], sy = zy - dd * gy[q], sz = zz - dd * gz[q];
                row[OR_DP_XS * n + c] = sx;
                row[OR_DP_YS * n + c] = sy;
                row[OR_DP_ZS * n + c] = sz;
                double nx, ny, nz, cm, cg;
                if (interp_grad(N, H, int_l, sx, sy, sz, gx, gy, gz, &nx, &ny, &nz) < 0) return -(1 + c);
                if (kind == OR_DENSE_COMBO) { /* :299-303 second normalisation */
                    double gn = sqrt(nx * nx + ny * ny + nz * nz);
                    nx = nx / gn;
                    ny = ny / gn;
                    nz = nz / gn;
                }
                row[OR_DP_GX * n + c] = nx;
                row[OR_DP_GY * n + c] = ny;
                row[OR_DP_GZ * n + c] = nz;
                const double jac = 1 + 2. * dd * mcurv[q] + dd * dd * gcurv[q];
                row[OR_DP_JAC * n + c] = jac;
                if (interp_curv(N, H, int_l, sx, sy, sz, mcurv, gcurv, &cm, &cg) < 0) return -(1 + c);
                const double tau = H * p->tau_factor;
                const double t1 = cm / (4. * OR_PI * tau);
                const double t2 = -5. * tau * (2. * cm) * (4. * cm * cm - cg) / (512. * OR_PI);
                const double t3 = -25. * tau * (2. * cm) * cg / (1536. * OR_PI);
                const double t4 = W * W * tau * 2. * cm / (48. * OR_PI);
                if (kind == OR_DENSE_DOUBLE_LAYER) { /* :700-725 */
                    const double delta = (o->onesided == 0) ? cal_delta(o->epsilon, dd)
                                                            : 2. * cal_delta(o->epsilon, dd);
                    row[OR_DP_DELTA * n + c] = delta;
                    row[OR_DP_REG * n + c] = t1 + t2 + t3 + t4;
                    row[OR_DP_REGIMG * n + c] = 0.0;
                    row[OR_DP_RESULT * n + c] = hcubed * delta * jac;
                } else { /* :350-385 */
                    row[OR_DP_REG * n + c] = (p->interior == 1) ? t1 + t2 + t3 + t4 : -1. * (t1 + t2 + t3 + t4);
                    row[OR_DP_REGIMG * n + c] = 0.0;
                    dense_weights(o, hcubed, dd, jac, row, n, c);
                }
            }
        }
    }
    return count;
}

int64_t or_dense_matrix(int kind, const or_params *p, const or_dense_opts *o, int64_t n, const double *pts,
                        double *k1re, double *k1im, double *k2re, double *k2im)
{
    const double H = or_h(p), W = p->wave;
    const double *xs = pts + OR_DP_XS * n, *ys = pts + OR_DP_YS * n, *zs = pts + OR_DP_ZS * n;
    const double *gx = pts + OR_DP_GX * n, *gy = pts + OR_DP_GY * n, *gz = pts + OR_DP_GZ * n;
    const double *reg = pts + OR_DP_REG * n, *dist = pts + OR_DP_DIST * n;
    const double *pres = pts + OR_DP_POLYRES * n, *sres = pts + OR_DP_SINERES * n, *res = pts + OR_DP_RESULT * n;
    int64_t regcount = 0;
    if (kind == OR_DENSE_DOUBLE_LAYER || kind == OR_DENSE_SPHERE) {
        /* :726-758 and :125-166: finite-difference kernel gradients */
        const double tau = (kind == OR_DENSE_DOUBLE_LAYER) ? H * p->tau_factor : 0.1 * H;
        const double threshold = (kind == OR_DENSE_DOUBLE_LAYER) ? tau * tau : 0.01 * H * H;
        double sreg = 0.0;
        if (kind == OR_DENSE_SPHERE) { /* :19-32 */
            const double R = o->radius;
            const double r1 = 1.0 / (4.0 * OR_PI * tau * R);
            const double r2 = (-5.0 * tau) / (256.0 * pow(R, 3.0) * OR_PI);
            const double r3 = (-50.0 * tau) / (1536.0 * pow(R, 3.0) * OR_PI);
            const double r4 = (pow(W, 2.0) * tau) / (24.0 * OR_PI * R);
            sreg = (p->interior == 1) ? r1 + r2 + r3 + r4 : -1.0 * (r1 + r2 + r3 + r4);
        }
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < n; i++) {
            const double a[3] = {xs[i], ys[i], zs[i]};
            for (int64_t j = 0; j < n; j++) {
                const double b[3] = {xs[j], ys[j], zs[j]};
                double pr[3], pi[3];
                fd_partials(H, W, a, b, pr, pi);
                double part, parti;
                const double n2 = (a[0] - b[0]) * (a[0] - b[0]) + (a[1] - b[1]) * (a[1] - b[1]) +
                                  (a[2] - b[2]) * (a[2] - b[2]);
                if (kind == OR_DENSE_DOUBLE_LAYER) {
                    part = pr[0] * gx[i] + pr[1] * gy[i] + pr[2] * gz[i];
                    parti = pi[0] * gx[i] + pi[1] * gy[i] + pi[2] * gz[i];
                    if (n2 < threshold) {
                        part = reg[i];
                        parti = 0.0;
                    }
                    k1re[i * n + j] = res[j] * part;
                    k1im[i * n + j] = res[j] * parti;
                    if (i == j) k1re[i * n + j] += 0.5;
                } else {
                    part = -1. * (pr[0] * gx[i] + pr[1] * gy[i] + pr[2] * gz[i]);
                    parti = -1. * (pi[0] * gx[i] + pi[1] * gy[i] + pi[2] * gz[i]);
                    if (n2 < threshold) {
                        part = sreg;
                        parti = 0.0;
                    }
                    if (o->poly && k1re) {
                        k1re[i * n + j] = part * pres[j];
                        k1im[i * n + j] = parti * pres[j];
                        if (i == j) k1re[i * n + j] -= 0.5;
                    }
                    if (o->sine && k2re) {
                        k2re[i * n + j] = part * sres[j];
                        k2im[i * n + j] = parti * sres[j];
                        if (i == j) k2re[i * n + j] -= 0.5;
                    }
                }
            }
        }
        return 0;
    }
    /* Combo, :399-607 */
    const double tau = p->tau_factor * H;
    const double recipfourpi = 1. / (4. * OR_PI);
    const double k = o->wavenum, eta = o->eta;
#pragma omp parallel for schedule(static) reduction(+ : regcount)
    for (int64_t i = 0; i < n; i++) {
        const double sxi = xs[i], syi = ys[i], szi = zs[i];
        for (int64_t j = 0; j < n; j++) {
            const double sxj = xs[j], syj = ys[j], szj = zs[j];
            const double m1 = sxi - sxj, m2 = syi - syj, m3 = szi - szj;
            const double mn = sqrt(m1 * m1 + m2 * m2 + m3 * m3);
            double part, parti;
            if (mn > tau) {
                const double rn = 1. / mn;
                const double prm = W * mn;
                const double sv = sin(prm), cv = cos(prm);
                const double es = sv * rn, ec = cv * rn;
                const double den = recipfourpi * rn * rn;
                const double c1 = -1. * (W * sv + ec) * den;
                const double c2 = (W * cv - es) * den;
                const double sip = -1. * (m1 * gx[i] + m2 * gy[i] + m3 * gz[i]);
                part = c1 * sip;
                parti = c2 * sip;
            } else {
                regcount += 1;
                part = reg[i];
                parti = 0.0;
            }
            double psr = 0, psi = 0, ssr = 0, ssi = 0;
            if (o->poly) {
                double tr = part * pres[j], ti = parti * pres[j];
                if (i == j) tr -= 0.5;
                psr = eta * ti;
                psi = -1. * eta * tr;
            }
            if (o->sine) {
                double tr = part * sres[j], ti = parti * sres[j];
                if (i == j) tr -= 0.5;
                ssr = eta * ti;
                ssi = -1. * eta * tr;
            }
            const double x1 = sxi + fabs(dist[j]) * gx[i];
            const double x2 = syi + fabs(dist[j]) * gy[i];
            const double x3 = szi + fabs(dist[j]) * gz[i];
            const double y1 = x1 - sxj, y2 = x2 - syj, y3 = x3 - szj;
            const double yn = sqrt(y1 * y1 + y2 * y2 + y3 * y3);
            const double rn = 1. / yn;
            const double prm = k * yn;
            const double ip1 = gx[i] * gx[j] + gy[i] * gy[j] + gz[i] * gz[j];
            const double ip2 = y1 * gx[i] + y2 * gy[i] + y3 * gz[i];
            const double ip3 = y1 * gx[j] + y2 * gy[j] + y3 * gz[j];
            const double cm1 = ip1 * rn;
            const double cm2 = ip2 * rn * ip3 * rn;
            const double cv = cos(prm) * rn, sv = sin(prm) * rn;
            const double t1r = -1. * (cv * rn + k * sv) * cm1;
            const double t1i = (k * cv - sv * rn) * cm1;
            const double t2r = -1. * k * k * cv * cm2;
            const double t2i = -1. * k * k * sv * cm2;
            const double t3r = 3. * k * sv * cm2 * rn;
            const double t3i = -3. * k * cv * cm2 * rn;
            const double t4r = 3. * cv * rn * cm2 * rn;
            const double t4i = 3. * sv * rn * cm2 * rn;
            if (o->poly && k1re) {
                k1re[i * n + j] = psr + pres[j] * (t1r + t2r + t3r + t4r) * recipfourpi;
                k1im[i * n + j] = psi + pres[j] * (t1i + t2i + t3i + t4i) * recipfourpi;
            }
            if (o->sine && k2re) {
                k2re[i * n + j] = ssr + sres[j] * (t1r + t2r + t3r + t4r) * recipfourpi;
                k2im[i * n + j] = ssi + sres[j] * (t1i + t2i + t3i + t4i) * recipfourpi;
            }
        }
    }
    return regcount;
}
