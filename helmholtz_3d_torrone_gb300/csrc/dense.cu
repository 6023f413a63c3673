// dense.cu -- the dense assemblers of HelmholtzKernel.c on the device:
//   DoubleLayerKernel        (HelmholtzKernel.c:613-761)
//   new_HelmholtzKernelCombo (HelmholtzKernel.c:173-610)
//   new_HelmholtzKernel      (HelmholtzKernel.c:3-169, analytic sphere)
// They are the reference's small-n parity path: every entry of an n x n
// complex matrix is written (16 B per entry and matrix), so they are
// HBM-write bound once the kernel values are cheap (Combo), and FP64-bound
// where each entry takes six finite-difference evaluations of the
// fundamental solution (double layer, sphere kernel).
//
// Built with -fmad=false: the per-point arrays (projection, normals,
// Jacobian, regularisation, weights) keep the reference's operation order,
// so they match it bit for bit up to the libm/CUDA differences of cos, sin,
// exp and pow; the matrix entries follow the reference's term order too.
#include "hz_internal.cuh"
#include "interp.cuh"

#include <cmath>

namespace hz {
namespace {

constexpr double kPi = 3.14159265358979323846264338328;  // constants.h:5
// functions.h:25-26, SineWeight with MOMENT_ORDER 1
constexpr double kConstA1 = -759.2781934172483;
constexpr double kConstB1 = 446.2604260472818;

struct DenseArgs {
    int kind;
    int N;
    double H, int_l, wave, tau_factor;
    int interior;
    double delta0, epsilon, wavenum, eta;
    int poly, sine, onesided, combo_interior;
    double radius, cx, cy, cz;
};

// Is node value d in the assembler's point set?
__device__ __forceinline__ bool dense_member(const DenseArgs &a, double d)
{
    if (a.kind == HZ_DENSE_DOUBLE_LAYER) {  // HelmholtzKernel.c:653-662
        if (a.onesided == 0) return !(fabs(d) > a.epsilon);
        return !((d > a.epsilon) || (d < 0.));
    }
    if (a.kind == HZ_DENSE_COMBO) {  // :247-265
        if (a.onesided == 0) return !((fabs(d) > a.epsilon) || (fabs(d) < a.delta0));
        if (a.combo_interior == 1) return !((d > a.epsilon) || (d < a.delta0));
        return !((d < -1. * a.epsilon) || (d > -1. * a.delta0));
    }
    if (a.onesided == 0) return !((fabs(d) > a.epsilon) || (fabs(d) < a.delta0));  // :46-55
    return !((d > a.epsilon) | (d < a.delta0));
}

__device__ __forceinline__ double sphere_dist(const DenseArgs &a, double zx, double zy, double zz)
{
    return a.radius - sqrt((zx - a.cx) * (zx - a.cx) + (zy - a.cy) * (zy - a.cy) + (zz - a.cz) * (zz - a.cz));
}

// Membership flags (0 member, 1 not) over the (N+1)^3 nodes, for the
// ordered compaction of tube.cu.
__global__ void dense_flag_kernel(DenseArgs a, const double *__restrict__ d, double *__restrict__ flag)
{
    const long long S = a.N + 1, total = S * S * S;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < total;
         q += (long long)gridDim.x * blockDim.x) {
        double dd;
        if (a.kind == HZ_DENSE_SPHERE) {
            const int i = (int)(q / (S * S)), j = (int)((q / S) % S), k = (int)(q % S);
            dd = sphere_dist(a, a.int_l + (double)(j)*a.H, a.int_l + (double)(i)*a.H, a.int_l + (double)(k)*a.H);
        } else {
            dd = d[q];
        }
        flag[q] = dense_member(a, dd) ? 0.0 : 1.0;
    }
}

// functions.c:793-833 (first moment, smooth ends)
__device__ __forceinline__ double poly_weight(double t, double tau)
{
    if ((t <= tau) || (t >= 1.0)) return 0.0;
    const double tau2 = tau * tau;
    const double term1 = 7. * (1 + tau) * t;
    const double term2 = -2. * (2. + 3. * tau + 2. * tau2);
    return 60. * (t - 1.) * (t - 1.) * (t - tau) * (t - tau) * (term1 + term2) / pow(tau - 1., 7.0);
}

// functions.c:835-866, MOMENT_ORDER 1
__device__ __forceinline__ double sine_weight(double t, double tau)
{
    if ((t <= tau) || (t >= 1.0)) return 0.0;
    return exp(0.5 / ((t - 0.1) * (t - 1.))) * (kConstA1 * t + kConstB1);
}

__device__ __forceinline__ void put(double *pts, int64_t n, int row, int64_t c, double v) { pts[row * n + c] = v; }

__device__ __forceinline__ void dense_weights(const DenseArgs &a, double hcubed, double dist, double jac,
                                              double *pts, int64_t n, int64_t c)
{
    const double eps = a.epsilon;
    if (a.poly) {
        const double w = (a.onesided == 0) ? poly_weight(fabs(dist / eps), a.delta0 / eps) / (2.0 * eps)
                                           : poly_weight(fabs(dist / eps), a.delta0 / eps) / (eps);
        put(pts, n, HZ_DP_POLYW, c, w);
        put(pts, n, HZ_DP_POLYRES, c, hcubed * jac * w);
    }
    if (a.sine) {
        const double w = (a.onesided == 0) ? sine_weight(fabs(dist / eps), a.delta0 / eps) / (2.0 * eps)
                                           : sine_weight(fabs(dist / eps), a.delta0 / eps) / (eps);
        put(pts, n, HZ_DP_SINEW, c, w);
        put(pts, n, HZ_DP_SINERES, c, hcubed * jac * w);
    }
}

// Per-point arrays, one thread per point (HelmholtzKernel.c:646-730,
// :222-389 and :33-110).
__global__ void dense_points_kernel(DenseArgs a, int64_t n, const int64_t *__restrict__ idx,
                                    const double *__restrict__ d, const double *__restrict__ gx,
                                    const double *__restrict__ gy, const double *__restrict__ gz,
                                    const double *__restrict__ mc, const double *__restrict__ gc, double *pts,
                                    unsigned *err)
{
    const long long S = a.N + 1;
    const double H = a.H, hcubed = H * H * H, W = a.wave;
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x) {
        const long long o = idx[c];
        const int i = (int)(o / (S * S)), j = (int)((o / S) % S), k = (int)(o % S);
        const double zy = a.int_l + H * (double)(i);
        const double zx = a.int_l + H * (double)(j);
        const double zz = a.int_l + H * (double)(k);
        put(pts, n, HZ_DP_ZX, c, zx);
        put(pts, n, HZ_DP_ZY, c, zy);
        put(pts, n, HZ_DP_ZZ, c, zz);
        if (a.kind == HZ_DENSE_SPHERE) {
            const double dd = sphere_dist(a, zx, zy, zz);
            const double r0 = sqrt((zx - a.cx) * (zx - a.cx) + (zy - a.cy) * (zy - a.cy) + (zz - a.cz) * (zz - a.cz));
            const double tgx = (a.cx - zx) / r0, tgy = (a.cy - zy) / r0, tgz = (a.cz - zz) / r0;
            const double sx = zx - dd * tgx, sy = zy - dd * tgy, sz = zz - dd * tgz;
            const double r1 = sqrt((sx - a.cx) * (sx - a.cx) + (sy - a.cy) * (sy - a.cy) + (sz - a.cz) * (sz - a.cz));
            put(pts, n, HZ_DP_DIST, c, dd);
            put(pts, n, HZ_DP_XS, c, sx);
            put(pts, n, HZ_DP_YS, c, sy);
            put(pts, n, HZ_DP_ZS, c, sz);
            put(pts, n, HZ_DP_GX, c, (a.cx - sx) / r1);
            put(pts, n, HZ_DP_GY, c, (a.cy - sy) / r1);
            put(pts, n, HZ_DP_GZ, c, (a.cz - sz) / r1);
            const double curv = 1. / (a.radius - dd);
            const double jac = 1. + dd * curv;
            put(pts, n, HZ_DP_CURV, c, curv);
            put(pts, n, HZ_DP_JAC, c, jac);
            dense_weights(a, hcubed, dd, jac, pts, n, c);
            continue;
        }
        const double dd = d[o];
        put(pts, n, HZ_DP_DIST, c, dd);
        const double sx = zx - dd * gx[o], sy = zy - dd * gy[o], sz = zz - dd * gz[o];
        put(pts, n, HZ_DP_XS, c, sx);
        put(pts, n, HZ_DP_YS, c, sy);
        put(pts, n, HZ_DP_ZS, c, sz);
        double nx, ny, nz, cm, cg;
        unsigned bad = interp_gradient(a.N, H, a.int_l, sx, sy, sz, gx, gy, gz, nx, ny, nz) & DEV_ERR_GRID;
        if (a.kind == HZ_DENSE_COMBO && !bad) {  // :299-303 normalised again
            const double gn = sqrt(nx * nx + ny * ny + nz * nz);
            nx = nx / gn;
            ny = ny / gn;
            nz = nz / gn;
        }
        put(pts, n, HZ_DP_GX, c, nx);
        put(pts, n, HZ_DP_GY, c, ny);
        put(pts, n, HZ_DP_GZ, c, nz);
        const double jac = 1 + 2. * dd * mc[o] + dd * dd * gc[o];
        put(pts, n, HZ_DP_JAC, c, jac);
        bad |= interp_curvatures(a.N, H, a.int_l, sx, sy, sz, mc, gc, cm, cg);
        const double tau = H * a.tau_factor;
        const double t1 = cm / (4. * kPi * tau);
        const double t2 = -5. * tau * (2. * cm) * (4. * cm * cm - cg) / (512. * kPi);
        const double t3 = -25. * tau * (2. * cm) * cg / (1536. * kPi);
        const double t4 = W * W * tau * 2. * cm / (48. * kPi);
        if (a.kind == HZ_DENSE_DOUBLE_LAYER) {  // :700-725, cosine delta (functions.c:366-374)
            const double de = (fabs(dd) <= a.epsilon) ? (1.0 / (2.0 * a.epsilon)) * (1.0 + cos(kPi * dd / a.epsilon))
                                                       : 0.0;
            const double delta = (a.onesided == 0) ? de : 2. * de;
            put(pts, n, HZ_DP_DELTA, c, delta);
            put(pts, n, HZ_DP_REG, c, t1 + t2 + t3 + t4);
            put(pts, n, HZ_DP_REGIMG, c, 0.0);
            put(pts, n, HZ_DP_RESULT, c, hcubed * delta * jac);
        } else {  // :350-385
            put(pts, n, HZ_DP_REG, c, (a.interior == 1) ? t1 + t2 + t3 + t4 : -1. * (t1 + t2 + t3 + t4));
            put(pts, n, HZ_DP_REGIMG, c, 0.0);
            dense_weights(a, hcubed, dd, jac, pts, n, c);
        }
        if (bad) atomicOr(err, bad);
    }
}

// One finite-difference evaluation of the fundamental solution at |a - b|
// (functions.c:433-504): re = cos(k r)/(-4 pi r), im = sin(k r)/(-4 pi r),
// 0 at r = 0 as the reference returns there.
__device__ __forceinline__ void phi_pair(double W, double a0, double a1, double a2, double b0, double b1, double b2,
                                         double &re, double &im)
{
    const double norm = sqrt(fabs((a0 - b0) * (a0 - b0) + (a1 - b1) * (a1 - b1) + (a2 - b2) * (a2 - b2)));
    if (norm == 0.0) {
        re = 0.0;
        im = 0.0;
        return;
    }
    double sv, cv;
    sincos(W * norm, &sv, &cv);
    re = cv / (-4.0 * kPi * norm);
    im = sv / (-4.0 * kPi * norm);
}

// Double layer (:731-758) and sphere kernel (:125-166): entries from the
// central differences of cal_partial (functions.c:121-155), step H in the
// second variable.  One thread per entry (row i = blockIdx.y stride,
// column j along x), so every row is written with coalesced stores.
template <int KIND>
__global__ void __launch_bounds__(256) dense_fd_kernel(DenseArgs a, int64_t n, const double *__restrict__ pts,
                                                       double sreg, double *k1re, double *k1im, double *k2re,
                                                       double *k2im)
{
    const double H = a.H, W = a.wave;
    const double *xs = pts + HZ_DP_XS * n, *ys = pts + HZ_DP_YS * n, *zs = pts + HZ_DP_ZS * n;
    const double tau = (KIND == HZ_DENSE_DOUBLE_LAYER) ? H * a.tau_factor : 0.1 * H;
    const double threshold = (KIND == HZ_DENSE_DOUBLE_LAYER) ? tau * tau : 0.01 * H * H;
    const int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (j >= n) return;
    const double b0 = xs[j], b1 = ys[j], b2 = zs[j];
    for (int64_t i = blockIdx.y; i < n; i += gridDim.y) {
        const double a0 = xs[i], a1 = ys[i], a2 = zs[i];
        double pr[3], pi[3];
#pragma unroll
        for (int ax = 0; ax < 3; ax++) {
            const double dp0 = (ax == 0) ? b0 + H : b0, dp1 = (ax == 1) ? b1 + H : b1, dp2 = (ax == 2) ? b2 + H : b2;
            const double dm0 = (ax == 0) ? b0 - H : b0, dm1 = (ax == 1) ? b1 - H : b1, dm2 = (ax == 2) ? b2 - H : b2;
            double rp, ip, rm, im;
            phi_pair(W, a0, a1, a2, dp0, dp1, dp2, rp, ip);
            phi_pair(W, a0, a1, a2, dm0, dm1, dm2, rm, im);
            pr[ax] = (rp - rm) / (2.0 * H);
            pi[ax] = (ip - im) / (2.0 * H);
        }
        const double gxi = pts[HZ_DP_GX * n + i], gyi = pts[HZ_DP_GY * n + i], gzi = pts[HZ_DP_GZ * n + i];
        const double n2 = (a0 - b0) * (a0 - b0) + (a1 - b1) * (a1 - b1) + (a2 - b2) * (a2 - b2);
        const int64_t e = i * n + j;
        if (KIND == HZ_DENSE_DOUBLE_LAYER) {
            double part = pr[0] * gxi + pr[1] * gyi + pr[2] * gzi;
            double parti = pi[0] * gxi + pi[1] * gyi + pi[2] * gzi;
            if (n2 < threshold) {
                part = pts[HZ_DP_REG * n + i];
                parti = 0.0;
            }
            const double r = pts[HZ_DP_RESULT * n + j];
            double v = r * part;
            if (i == j) v += 0.5;
            k1re[e] = v;
            k1im[e] = r * parti;
        } else {
            double part = -1. * (pr[0] * gxi + pr[1] * gyi + pr[2] * gzi);
            double parti = -1. * (pi[0] * gxi + pi[1] * gyi + pi[2] * gzi);
            if (n2 < threshold) {
                part = sreg;
                parti = 0.0;
            }
            if (k1re) {
                const double r = pts[HZ_DP_POLYRES * n + j];
                double v = part * r;
                if (i == j) v -= 0.5;
                k1re[e] = v;
                k1im[e] = parti * r;
            }
            if (k2re) {
                const double r = pts[HZ_DP_SINERES * n + j];
                double v = part * r;
                if (i == j) v -= 0.5;
                k2re[e] = v;
                k2im[e] = parti * r;
            }
        }
    }
}

// Combo (:399-607): -i eta times the regularised single layer dG(x*_i,
// y*_j)/dn_x, plus the hypersingular double layer at the offset point
// x*_i + |d_j| n_i.  Counts the regularised pairs.
__global__ void __launch_bounds__(256) dense_combo_kernel(DenseArgs a, int64_t n, const double *__restrict__ pts,
                                                          double *k1re, double *k1im, double *k2re, double *k2im,
                                                          unsigned long long *regcount)
{
    const double W = a.wave, k = a.wavenum, eta = a.eta;
    const double tau = a.tau_factor * a.H;
    const double recipfourpi = 1. / (4. * kPi);
    const double *xs = pts + HZ_DP_XS * n, *ys = pts + HZ_DP_YS * n, *zs = pts + HZ_DP_ZS * n;
    const double *gx = pts + HZ_DP_GX * n, *gy = pts + HZ_DP_GY * n, *gz = pts + HZ_DP_GZ * n;
    const int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    unsigned long long cnt = 0;
    if (j < n) {
        const double sxj = xs[j], syj = ys[j], szj = zs[j], gxj = gx[j], gyj = gy[j], gzj = gz[j];
        const double dj = fabs(pts[HZ_DP_DIST * n + j]);
        const double pres = a.poly ? pts[HZ_DP_POLYRES * n + j] : 0.0;
        const double sres = a.sine ? pts[HZ_DP_SINERES * n + j] : 0.0;
        for (int64_t i = blockIdx.y; i < n; i += gridDim.y) {
            const double sxi = xs[i], syi = ys[i], szi = zs[i], gxi = gx[i], gyi = gy[i], gzi = gz[i];
            const double m1 = sxi - sxj, m2 = syi - syj, m3 = szi - szj;
            const double mn = sqrt(m1 * m1 + m2 * m2 + m3 * m3);
            double part, parti;
            if (mn > tau) {
                const double rn = 1. / mn;
                double sv, cv;
                sincos(W * mn, &sv, &cv);
                const double es = sv * rn, ec = cv * rn;
                const double den = recipfourpi * rn * rn;
                const double c1 = -1. * (W * sv + ec) * den;
                const double c2 = (W * cv - es) * den;
                const double sip = -1. * (m1 * gxi + m2 * gyi + m3 * gzi);
                part = c1 * sip;
                parti = c2 * sip;
            } else {
                cnt++;
                part = pts[HZ_DP_REG * n + i];
                parti = 0.0;
            }
            const double x1 = sxi + dj * gxi, x2 = syi + dj * gyi, x3 = szi + dj * gzi;
            const double y1 = x1 - sxj, y2 = x2 - syj, y3 = x3 - szj;
            const double yn = sqrt(y1 * y1 + y2 * y2 + y3 * y3);
            const double rn = 1. / yn;
            const double ip1 = gxi * gxj + gyi * gyj + gzi * gzj;
            const double ip2 = y1 * gxi + y2 * gyi + y3 * gzi;
            const double ip3 = y1 * gxj + y2 * gyj + y3 * gzj;
            const double cm1 = ip1 * rn;
            const double cm2 = ip2 * rn * ip3 * rn;
            double s0, c0;
            sincos(k * yn, &s0, &c0);
            const double cv = c0 * rn, sv = s0 * rn;
            const double t1r = -1. * (cv * rn + k * sv) * cm1;
            const double t1i = (k * cv - sv * rn) * cm1;
            const double t2r = -1. * k * k * cv * cm2;
            const double t2i = -1. * k * k * sv * cm2;
            const double t3r = 3. * k * sv * cm2 * rn;
            const double t3i = -3. * k * cv * cm2 * rn;
            const double t4r = 3. * cv * rn * cm2 * rn;
            const double t4i = 3. * sv * rn * cm2 * rn;
            const double sr = t1r + t2r + t3r + t4r, si = t1i + t2i + t3i + t4i;
            const int64_t e = i * n + j;
            if (k1re) {
                double tr = part * pres;
                const double ti = parti * pres;
                if (i == j) tr -= 0.5;
                k1re[e] = eta * ti + pres * sr * recipfourpi;
                k1im[e] = -1. * eta * tr + pres * si * recipfourpi;
            }
            if (k2re) {
                double tr = part * sres;
                const double ti = parti * sres;
                if (i == j) tr -= 0.5;
                k2re[e] = eta * ti + sres * sr * recipfourpi;
                k2im[e] = -1. * eta * tr + sres * si * recipfourpi;
            }
        }
    }
    // per-block count, one atomic per block
    for (int o = 16; o > 0; o >>= 1) cnt += __shfl_down_sync(0xffffffffu, cnt, o);
    __shared__ unsigned long long sh[8];
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = cnt;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long t = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += sh[w];
        if (t) atomicAdd(regcount, t);
    }
}

int grid_for(long long work)
{
    long long b = (work + 255) / 256;
    if (b > 152LL * 16) b = 152LL * 16;
    return (int)(b < 1 ? 1 : b);
}

DenseArgs make_args(int kind, const hz_params &p, const hz_dense_opts &o)
{
    DenseArgs a;
    a.kind = kind;
    a.N = p.N;
    a.H = (p.int_u - p.int_l) / p.N;
    a.int_l = p.int_l;
    a.wave = p.wave;
    a.tau_factor = p.tau_factor;
    a.interior = p.interior;
    a.delta0 = o.delta0;
    a.epsilon = o.epsilon;
    a.wavenum = o.wavenum;
    a.eta = o.eta;
    a.poly = o.poly;
    a.sine = o.sine;
    a.onesided = o.onesided;
    a.combo_interior = o.combo_interior;
    a.radius = o.radius;
    a.cx = o.center[0];
    a.cy = o.center[1];
    a.cz = o.center[2];
    return a;
}

int check_dense(int kind, const hz_params *p, const hz_dense_opts *o)
{
    if (!p || !o || kind < HZ_DENSE_DOUBLE_LAYER || kind > HZ_DENSE_SPHERE) {
        set_error("dense assembler: bad kind or NULL parameters");
        return HZ_ERR_ARG;
    }
    if (p->N < 8 || p->N > 4096 || !(p->int_u > p->int_l) || !(o->epsilon > 0) || !(p->tau_factor > 0)) {
        set_error("dense assembler: bad N, domain, epsilon or tau_factor");
        return HZ_ERR_ARG;
    }
    if (kind == HZ_DENSE_SPHERE && !(o->radius > 0)) {
        set_error("dense assembler: sphere radius must be positive");
        return HZ_ERR_ARG;
    }
    return HZ_OK;
}

// Selected nodes (lexicographic) of one assembler; d on the device.
int dense_select(const DenseArgs &a, const double *d, DevBuf &idx, int64_t &n, cudaStream_t s)
{
    const long long S = a.N + 1, total = S * S * S;
    DevBuf flag, scratch;
    HZ_TRY(flag.ensure((size_t)total * sizeof(double)));
    dense_flag_kernel<<<grid_for(total), 256, 0, s>>>(a, d, flag.as<double>());
    HZ_CHECK_LAUNCH();
    return tube_build(a.N, 0.5, flag.as<double>(), idx, n, scratch, s);
}

}  // namespace

// Device form of the three assemblers; every pointer is on the device.
int dense_assemble_device(int kind, const hz_params &p, const hz_dense_opts &o, const double *d, const double *gx,
                          const double *gy, const double *gz, const double *mc, const double *gc, int64_t n_expected,
                          double *pts, double *k1re, double *k1im, double *k2re, double *k2im,
                          long long *regcount, unsigned *err, cudaStream_t s)
{
    const DenseArgs a = make_args(kind, p, o);
    DevBuf idx;
    int64_t n = 0;
    HZ_TRY(dense_select(a, d, idx, n, s));
    if (n != n_expected) {
        set_error("dense assembler selects %lld points, size given %lld", (long long)n, (long long)n_expected);
        return HZ_ERR_ARG;
    }
    if (n == 0) return HZ_OK;
    dense_points_kernel<<<grid_for(n), 256, 0, s>>>(a, n, idx.as<int64_t>(), d, gx, gy, gz, mc, gc, pts, err);
    HZ_CHECK_LAUNCH();
    const dim3 grid((unsigned)((n + 255) / 256), (unsigned)(n < 65535 ? n : 65535));
    if (kind == HZ_DENSE_DOUBLE_LAYER) {
        if (k1re && k1im) {
            dense_fd_kernel<HZ_DENSE_DOUBLE_LAYER><<<grid, 256, 0, s>>>(a, n, pts, 0.0, k1re, k1im, nullptr, nullptr);
            HZ_CHECK_LAUNCH();
        }
    } else if (kind == HZ_DENSE_SPHERE) {
        // :19-32, a constant regularisation factor of the sphere
        const double H = a.H, tau = 0.1 * H, R = a.radius;
        const double r1 = 1.0 / (4.0 * kPi * tau * R);
        const double r2 = (-5.0 * tau) / (256.0 * pow(R, 3.0) * kPi);
        const double r3 = (-50.0 * tau) / (1536.0 * pow(R, 3.0) * kPi);
        const double r4 = (pow(a.wave, 2.0) * tau) / (24.0 * kPi * R);
        const double sreg = (a.interior == 1) ? r1 + r2 + r3 + r4 : -1.0 * (r1 + r2 + r3 + r4);
        double *p1r = (o.poly && k1re && k1im) ? k1re : nullptr, *p1i = p1r ? k1im : nullptr;
        double *p2r = (o.sine && k2re && k2im) ? k2re : nullptr, *p2i = p2r ? k2im : nullptr;
        if (p1r || p2r) {
            dense_fd_kernel<HZ_DENSE_SPHERE><<<grid, 256, 0, s>>>(a, n, pts, sreg, p1r, p1i, p2r, p2i);
            HZ_CHECK_LAUNCH();
        }
    } else {
        DevBuf cnt;
        HZ_TRY(cnt.ensure(sizeof(unsigned long long)));
        HZ_CHECK_CUDA(cudaMemsetAsync(cnt.ptr, 0, sizeof(unsigned long long), s));
        double *p1r = (o.poly && k1re && k1im) ? k1re : nullptr, *p1i = p1r ? k1im : nullptr;
        double *p2r = (o.sine && k2re && k2im) ? k2re : nullptr, *p2i = p2r ? k2im : nullptr;
        dense_combo_kernel<<<grid, 256, 0, s>>>(a, n, pts, p1r, p1i, p2r, p2i, cnt.as<unsigned long long>());
        HZ_CHECK_LAUNCH();
        unsigned long long hc = 0;
        HZ_CHECK_CUDA(cudaMemcpyAsync(&hc, cnt.ptr, sizeof(hc), cudaMemcpyDeviceToHost, s));
        HZ_CHECK_CUDA(cudaStreamSynchronize(s));
        if (regcount) *regcount = (long long)hc;
    }
    return HZ_OK;
}

int dense_points_device(int kind, const hz_params &p, const hz_dense_opts &o, const double *d, const double *gx,
                        const double *gy, const double *gz, const double *mc, const double *gc, DevBuf &idx,
                        int64_t &n, DevBuf &pts, unsigned *err, cudaStream_t s)
{
    const DenseArgs a = make_args(kind, p, o);
    HZ_TRY(dense_select(a, d, idx, n, s));
    const size_t rows = (size_t)HZ_DENSE_ROWS * (size_t)(n > 0 ? n : 1);
    HZ_TRY(pts.ensure(rows * sizeof(double)));
    HZ_CHECK_CUDA(cudaMemsetAsync(pts.ptr, 0, rows * sizeof(double), s));
    if (n == 0) return HZ_OK;
    dense_points_kernel<<<grid_for(n), 256, 0, s>>>(a, n, idx.as<int64_t>(), d, gx, gy, gz, mc, gc, pts.as<double>(),
                                                     err);
    HZ_CHECK_LAUNCH();
    return HZ_OK;
}

int dense_count_device(int kind, const hz_params &p, const hz_dense_opts &o, const double *d, int64_t &n,
                       cudaStream_t s)
{
    const DenseArgs a = make_args(kind, p, o);
    DevBuf idx;
    HZ_TRY(dense_select(a, d, idx, n, s));
    HZ_CHECK_CUDA(cudaStreamSynchronize(s));
    return HZ_OK;
}

}  // namespace hz

using namespace hz;

extern "C" {

void hz_dense_opts_default(hz_dense_opts *o, int kind, const hz_params *p)
{
    if (!o) return;
    const double H = p ? (p->int_u - p->int_l) / p->N : 0.0;
    o->delta0 = 0.1 * H;                               // large3Dexample2.c:61,303
    o->epsilon = (kind == HZ_DENSE_DOUBLE_LAYER) ? (p ? p->factor * H : 0.0)  // :350
                                                 : sqrt(H);                    // :63,301
    o->wavenum = p ? p->wave : 0.0;
    o->eta = -1.0;  // DEFAULT_ETA, :37
    o->poly = 0;    // PDE.h POLY_TEST
    o->sine = 1;    // PDE.h SINE_TEST
    o->onesided = 0;
    o->combo_interior = 0;
    o->radius = 1.0;  // frame.h
    o->center[0] = o->center[1] = o->center[2] = 0.0;
}

int hz_dense_count(int kind, const hz_params *p, const hz_dense_opts *o, const double *d, int where, int64_t *n)
{
    HZ_TRY(check_dense(kind, p, o));
    HZ_TRY(where_ok(where));
    if (!n || (kind != HZ_DENSE_SPHERE && !d)) {
        set_error("hz_dense_count: NULL argument");
        return HZ_ERR_ARG;
    }
    const size_t S = (size_t)p->N + 1, nodes = S * S * S;
    cudaStream_t s = nullptr;
    DevBuf dbuf;
    const double *dd = nullptr;
    if (kind != HZ_DENSE_SPHERE) {
        if (where == HZ_HOST) {
            HZ_TRY(dbuf.ensure(nodes * sizeof(double)));
            HZ_TRY(stage_in(dbuf.as<double>(), d, nodes, where, s));
            dd = dbuf.as<double>();
        } else {
            dd = d;
        }
    }
    int64_t cnt = 0;
    HZ_TRY(dense_count_device(kind, *p, *o, dd, cnt, s));
    *n = cnt;
    return HZ_OK;
}

int hz_dense_assemble(int kind, const hz_params *p, const hz_dense_opts *o, const double *d, const double *gx,
                      const double *gy, const double *gz, const double *mc, const double *gc, int64_t n,
                      double *pts, double *k1_re, double *k1_im, double *k2_re, double *k2_im, int64_t *regcount,
                      int where)
{
    HZ_TRY(check_dense(kind, p, o));
    HZ_TRY(where_ok(where));
    if (kind != HZ_DENSE_SPHERE && !d) {
        set_error("hz_dense_assemble: NULL distance grid");
        return HZ_ERR_ARG;
    }
    if (n < 0 || n > (int64_t)1 << 20) {
        set_error("hz_dense_assemble: n = %lld out of range", (long long)n);
        return HZ_ERR_ARG;
    }
    const bool have_grids = gx && gy && gz && mc && gc;
    const size_t S = (size_t)p->N + 1, nodes = S * S * S;
    const double H = (p->int_u - p->int_l) / p->N;
    cudaStream_t s = nullptr;
    // device staging: 6 grids, per-point rows, matrices
    DevBuf grids, pbuf, mbuf, ebuf;
    const double *dd = nullptr, *g[5] = {gx, gy, gz, mc, gc};
    if (kind != HZ_DENSE_SPHERE) {
        if (where == HZ_HOST || !have_grids) {
            HZ_TRY(grids.ensure(6 * nodes * sizeof(double)));
            double *b = grids.as<double>();
            HZ_TRY(stage_in(b, d, nodes, where, s));
            dd = b;
            if (have_grids) {
                for (int q = 0; q < 5; q++) HZ_TRY(stage_in(b + (q + 1) * nodes, g[q], nodes, where, s));
            } else {
                HZ_TRY(launch_grid_stencils(p->N, H, b, b + nodes, b + 2 * nodes, b + 3 * nodes, b + 4 * nodes,
                                            b + 5 * nodes, p->weno_order == 3 ? 3 : 5, s));
            }
            for (int q = 0; q < 5; q++) g[q] = b + (q + 1) * nodes;
        } else {
            dd = d;
        }
    }
    HZ_TRY(pbuf.ensure((size_t)HZ_DENSE_ROWS * (n > 0 ? n : 1) * sizeof(double)));
    double *dpts = pbuf.as<double>();
    if (pts && where == HZ_HOST)  // rows the assembler does not write keep the caller's values
        HZ_TRY(stage_in(dpts, pts, (size_t)HZ_DENSE_ROWS * n, where, s));
    else if (pts)
        dpts = pts;
    else
        HZ_CHECK_CUDA(cudaMemsetAsync(dpts, 0, (size_t)HZ_DENSE_ROWS * (n > 0 ? n : 1) * sizeof(double), s));
    const size_t nn = (size_t)n * (size_t)n;
    double *m[4] = {k1_re, k1_im, k2_re, k2_im};
    double *dm[4] = {nullptr, nullptr, nullptr, nullptr};
    int want = 0;
    for (int q = 0; q < 4; q++) want += m[q] ? 1 : 0;
    if (where == HZ_HOST && want > 0 && nn > 0) {
        HZ_TRY(mbuf.ensure((size_t)want * nn * sizeof(double)));
        int used = 0;
        for (int q = 0; q < 4; q++)
            if (m[q]) dm[q] = mbuf.as<double>() + (size_t)(used++) * nn;
    } else {
        for (int q = 0; q < 4; q++) dm[q] = m[q];
    }
    HZ_TRY(ebuf.ensure(sizeof(unsigned)));
    HZ_CHECK_CUDA(cudaMemsetAsync(ebuf.ptr, 0, sizeof(unsigned), s));
    long long rc = 0;
    HZ_TRY(dense_assemble_device(kind, *p, *o, dd, g[0], g[1], g[2], g[3], g[4], n, dpts, dm[0], dm[1], dm[2], dm[3],
                                 &rc, ebuf.as<unsigned>(), s));
    unsigned e = 0;
    HZ_CHECK_CUDA(cudaMemcpyAsync(&e, ebuf.ptr, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
    if (where == HZ_HOST) {
        if (pts) HZ_TRY(stage_out(pts, dpts, (size_t)HZ_DENSE_ROWS * n, where, s));
        for (int q = 0; q < 4; q++)
            if (m[q] && nn > 0) HZ_TRY(stage_out(m[q], dm[q], nn, where, s));
    }
    HZ_CHECK_CUDA(cudaStreamSynchronize(s));
    if (regcount) *regcount = (int64_t)rc;
    if (e & DEV_ERR_GRID) {
        set_error("dense assembler: a projected point's interpolation cell lies outside the grid");
        return HZ_ERR_GRID;
    }
    return HZ_OK;
}

}  // extern "C"
