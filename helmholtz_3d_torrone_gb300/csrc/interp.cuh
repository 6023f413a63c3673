// interp.cuh -- trilinear interpolation of the grids at a projected point,
// in the reference's operation order (units built with -fmad=false keep it
// bit for bit): the gradient of interpolate3D.c:5-102 (cal_interpgrad) and
// the curvatures of interpolate3D.c:569-605 (cal_BothCurvs).
#pragma once

#include "hz_internal.cuh"

namespace hz {

// interpolate3D.c:49-53 term order; letters are (x,y,z) = (j,i,k) low/high.
__device__ __forceinline__ double tri8(double lll, double llh, double lhl, double lhh, double hll, double hlh,
                                       double hhl, double hhh, double lx, double ly, double lz, double H)
{
    return (lll * (H - lx) * (H - ly) * (H - lz) + llh * (H - lx) * (H - ly) * lz +
            lhl * (H - lx) * ly * (H - lz) + lhh * (H - lx) * ly * lz + hll * lx * (H - ly) * (H - lz) +
            hlh * lx * (H - ly) * lz + hhl * lx * ly * (H - lz) + hhh * lx * ly * lz) /
           (H * H * H);
}

// cal_interpgrad: cell of (tx,ty,tz), trilinear gradient, normalised once.
// Returns DEV_ERR_GRID when the cell lies outside the grid (the reference
// exits there), DEV_ERR_NORMAL when the interpolated norm is off by > 0.5
// (the reference prints and goes on), 0 otherwise.
__device__ __forceinline__ unsigned interp_gradient(int N, double H, double int_l, double tx, double ty, double tz,
                                                    const double *gx, const double *gy, const double *gz,
                                                    double &nx, double &ny, double &nz)
{
    const long long S = N + 1;
    const int gi = (int)((ty - int_l) / H), gj = (int)((tx - int_l) / H), gk = (int)((tz - int_l) / H);
    const double lowx = tx - int_l - (double)(gj)*H;
    const double lowy = ty - int_l - (double)(gi)*H;
    const double lowz = tz - int_l - (double)(gk)*H;
    nx = ny = nz = 0.0;
    if ((lowx > H) || (lowx < 0.0) || (lowy > H) || (lowy < 0.0) || (lowz < 0.0) || (lowz > H) || gi < 0 || gj < 0 ||
        gk < 0 || gi >= N || gj >= N || gk >= N)
        return DEV_ERR_GRID;
    double r[3];
    const double *g[3] = {gx, gy, gz};
#pragma unroll
    for (int cc = 0; cc < 3; cc++) {
        const double *q = g[cc];
        const long long b0 = (gi * S + gj) * S + gk;
        r[cc] = tri8(q[b0], q[b0 + 1], q[b0 + S * S], q[b0 + S * S + 1], q[b0 + S], q[b0 + S + 1], q[b0 + S * S + S],
                     q[b0 + S * S + S + 1], lowx, lowy, lowz, H);
    }
    const double nrm = sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
    nx = r[0] / nrm;
    ny = r[1] / nrm;
    nz = r[2] / nrm;
    return (fabs(nrm - 1.0) > 0.5) ? DEV_ERR_NORMAL : 0u;
}

// cal_BothCurvs: mean and Gaussian curvature at (tx,ty,tz), cell found with
// a 1e-19 nudge.  Returns DEV_ERR_GRID outside the grid, 0 otherwise.
__device__ __forceinline__ unsigned interp_curvatures(int N, double H, double int_l, double tx, double ty, double tz,
                                                      const double *mc, const double *gc, double &cm, double &cg)
{
    const long long S = N + 1;
    const int cj = (int)((tx + 1e-19 - int_l) / H);
    const int ci = (int)((ty + 1e-19 - int_l) / H);
    const int ck = (int)((tz + 1e-19 - int_l) / H);
    cm = cg = 0.0;
    if (ci < 0 || cj < 0 || ck < 0 || ci >= N || cj >= N || ck >= N) return DEV_ERR_GRID;
    const double lx = tx - int_l - (double)(cj)*H;
    const double ly = ty - int_l - (double)(ci)*H;
    const double lz = tz - int_l - (double)(ck)*H;
    const double hc = H * H * H;
    const long long b0 = (ci * S + cj) * S + ck;
    const double *m2[2] = {mc, gc};
    double r[2];
#pragma unroll
    for (int cc = 0; cc < 2; cc++) {
        const double *m = m2[cc];
        r[cc] = (m[b0] * (H - lx) * (H - ly) * (H - lz) + m[b0 + S * S] * (H - lx) * ly * (H - lz) +
                 m[b0 + S] * lx * (H - ly) * (H - lz) + m[b0 + S * S + S] * lx * ly * (H - lz) +
                 m[b0 + 1] * (H - lx) * (H - ly) * lz + m[b0 + S * S + 1] * (H - lx) * ly * lz +
                 m[b0 + S + 1] * lx * (H - ly) * lz + m[b0 + S * S + S + 1] * lx * ly * lz) /
                hc;
    }
    cm = r[0];
    cg = r[1];
    return 0u;
}

}  // namespace hz
