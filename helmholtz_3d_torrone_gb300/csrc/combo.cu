// combo.cu -- the Combo formulation (new_HelmholtzKernelCombo,
// HelmholtzKernel.c:173-610) as a matrix-free FP64 operator, and its
// off-surface evaluation (Combo_NeumannTest, large3Dexample2.c:1907-2059).
//
// With r_j the annulus weight H^3 J_j W(|d_j|) of the source and
// kappa_ij = (eta parti_ij + c4 D_ij) + i (-eta part_ij + c4 Dimg_ij), the
// reference's dense entry is K_ij = r_j kappa_ij, plus i eta / 2 on the
// diagonal (the -1/2 of the single layer times -i eta).  Here:
//   part + i parti = the regularised single-layer gradient dG(x*_i, x*_j)/dn_i
//                    (reg_i within tau = TAU_FACTOR H),
//   D + i Dimg     = the hypersingular double layer d^2G/dn_x dn_y at the
//                    offset point x*_i + |d_j| n_i and x*_j.
// A p:    q_i  = sum_j kappa_ij (r_j p_j) + (i eta / 2) p_i,
// A^H pt: qt_j = r_j sum_i conj(kappa_ij) pt_i - (i eta / 2) pt_j.
// Every entry is recomputed per product, so the sweep is bound by the FP64
// pipe: 1/r and 1/|y| come from rsqrt, both sin/cos pairs from the table
// method of sincos64.cuh, and the near-field test sqrt(r^2) > tau is
// evaluated exactly only where r^2 lies within a relative 1e-12 of tau^2.
// Sources are staged in shared memory tile by tile.
#include "hz_internal.cuh"
#include "sincos64.cuh"

namespace hz {
namespace {

constexpr double kPi = 3.14159265358979323846264338328;
constexpr int kComboThreads = 128;
constexpr int kComboTile = 128;

struct ComboArgs {
    int64_t n;
    double wave, wavenum, k2, eta, tau, tau2;
    const double4_32a *pos;  // (x*, reg)
    const double4_32a *nrm;  // (n, r)
    const double *adist;     // |d|
    const double *p_re, *p_im;
    double *q_re, *q_im;
};

// kappa_ij of the header: target point i (x*_i, n_i, reg_i) and source
// point j (x*_j, n_j, |d_j|), in the reference's term order
// (HelmholtzKernel.c:441-576).
__device__ __forceinline__ void combo_kappa(const ComboArgs &a, const double2 *tab, double xi, double yi, double zi,
                                            double nxi, double nyi, double nzi, double regi, double xj, double yj,
                                            double zj, double nxj, double nyj, double nzj, double dj, double &kr,
                                            double &ki)
{
    const double W = a.wave, k = a.wavenum;
    const double c4 = 1. / (4. * kPi);
    const double m1 = xi - xj, m2 = yi - yj, m3 = zi - zj;
    const double r2 = m1 * m1 + m2 * m2 + m3 * m3;
    bool far = r2 > a.tau2;
    if (fabs(r2 - a.tau2) <= 1e-12 * a.tau2) far = sqrt(r2) > a.tau;
    double part, parti;
    if (far) {
        const double rn = rsqrt(r2);
        const double mn = r2 * rn;
        double sv, cv;
        table_sincos(W * mn, tab, sv, cv);
        const double es = sv * rn, ec = cv * rn;
        const double den = c4 * rn * rn;
        const double c1 = -1. * (W * sv + ec) * den;
        const double c2 = (W * cv - es) * den;
        const double sip = -1. * (m1 * nxi + m2 * nyi + m3 * nzi);
        part = c1 * sip;
        parti = c2 * sip;
    } else {
        part = regi;
        parti = 0.0;
    }
    const double y1 = xi + dj * nxi - xj, y2 = yi + dj * nyi - yj, y3 = zi + dj * nzi - zj;
    const double ysq = y1 * y1 + y2 * y2 + y3 * y3;
    const double rn = rsqrt(ysq);
    const double yn = ysq * rn;
    const double ip1 = nxi * nxj + nyi * nyj + nzi * nzj;
    const double ip2 = y1 * nxi + y2 * nyi + y3 * nzi;
    const double ip3 = y1 * nxj + y2 * nyj + y3 * nzj;
    const double cm1 = ip1 * rn;
    const double cm2 = ip2 * rn * ip3 * rn;
    double s0, c0;
    table_sincos(k * yn, tab, s0, c0);
    // the reference's four terms t1..t4 (HelmholtzKernel.c:539-571)
    // regrouped: with e1 = k sin + cos/|y| and e2 = k cos - sin/|y|,
    //   t1 + .. + t4 = (1/|y|) [-cm1 e1 + cm2 (3 e1/|y| - k^2 cos)]  (real)
    //                  (1/|y|) [ cm1 e2 - cm2 (3 e2/|y| + k^2 sin)]  (imaginary)
    const double e1 = c0 * rn + k * s0, e2 = k * c0 - s0 * rn;
    const double g3 = 3. * rn;
    const double tr = rn * (cm2 * (g3 * e1 - a.k2 * c0) - cm1 * e1);
    const double ti = rn * (cm1 * e2 - cm2 * (g3 * e2 + a.k2 * s0));
    kr = a.eta * parti + tr * c4;
    ki = -1. * a.eta * part + ti * c4;
}

// One thread per output point; the other points come through shared
// memory in tiles.  ADJ = false: q = A p (thread = target i); ADJ = true:
// q = A^H p (thread = source j, loop over targets i).
template <bool ADJ>
__global__ void __launch_bounds__(kComboThreads) combo_sweep_kernel(ComboArgs a)
{
    __shared__ double4_32a sp[kComboTile], sn[kComboTile];
    __shared__ double2 sd[kComboTile];  // ADJ: pt_i; else r_j p_j
    __shared__ double sdist[kComboTile];
    __shared__ double2 tab[kSinTable];
    fill_sin_table(tab);
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const bool valid = t < a.n;
    double4_32a tp = make_double4_32a(0, 0, 0, 0), tn = make_double4_32a(0, 0, 0, 0);
    double td = 0.0;
    if (valid) {
        tp = a.pos[t];
        tn = a.nrm[t];
        td = a.adist[t];
    }
    double ar = 0.0, ai = 0.0;
    for (int64_t base = 0; base < a.n; base += kComboTile) {
        const int cnt = (int)((a.n - base < kComboTile) ? (a.n - base) : kComboTile);
        __syncthreads();
        for (int q = threadIdx.x; q < cnt; q += blockDim.x) {
            const double4_32a p = a.pos[base + q], m = a.nrm[base + q];
            sp[q] = p;
            sn[q] = m;
            sdist[q] = a.adist[base + q];
            const double pr = a.p_re[base + q], pi = a.p_im[base + q];
            sd[q] = ADJ ? make_double2(pr, pi) : make_double2(m.w * pr, m.w * pi);
        }
        __syncthreads();
        if (!valid) continue;
        for (int q = 0; q < cnt; q++) {
            const double4_32a o = sp[q], on = sn[q];
            double kr, ki;
            if (!ADJ)
                combo_kappa(a, tab, tp.x, tp.y, tp.z, tn.x, tn.y, tn.z, tp.w, o.x, o.y, o.z, on.x, on.y, on.z,
                            sdist[q], kr, ki);
            else
                combo_kappa(a, tab, o.x, o.y, o.z, on.x, on.y, on.z, o.w, tp.x, tp.y, tp.z, tn.x, tn.y, tn.z, td,
                            kr, ki);
            const double2 d = sd[q];
            if (!ADJ) {
                ar += kr * d.x - ki * d.y;
                ai += kr * d.y + ki * d.x;
            } else {  // conj(kappa) pt
                ar += kr * d.x + ki * d.y;
                ai += kr * d.y - ki * d.x;
            }
        }
    }
    if (!valid) return;
    const double pr = a.p_re[t], pi = a.p_im[t], he = 0.5 * a.eta;
    if (!ADJ) {
        a.q_re[t] = ar - he * pi;
        a.q_im[t] = ai + he * pr;
    } else {
        const double r = tn.w;
        a.q_re[t] = r * ar + he * pi;
        a.q_im[t] = r * ai - he * pr;
    }
}

// Rows of the Combo per-point array into the operator's arrays.
__global__ void combo_pack_kernel(int64_t n, const double *__restrict__ pts, int weight_row, double *xs,
                                  double *nrm, double *delta, double *jac, double *reg, double *w, double *adist,
                                  double4_32a *pos64, double4_32a *nrm64)
{
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x) {
        const double x = pts[HZ_DP_XS * n + c], y = pts[HZ_DP_YS * n + c], z = pts[HZ_DP_ZS * n + c];
        const double gx = pts[HZ_DP_GX * n + c], gy = pts[HZ_DP_GY * n + c], gz = pts[HZ_DP_GZ * n + c];
        const double r = pts[(int64_t)weight_row * n + c], rg = pts[HZ_DP_REG * n + c];
        xs[3 * c] = x;
        xs[3 * c + 1] = y;
        xs[3 * c + 2] = z;
        nrm[3 * c] = gx;
        nrm[3 * c + 1] = gy;
        nrm[3 * c + 2] = gz;
        delta[c] = 0.0;
        jac[c] = pts[HZ_DP_JAC * n + c];
        reg[c] = rg;
        w[c] = r;
        adist[c] = fabs(pts[HZ_DP_DIST * n + c]);
        pos64[c] = make_double4_32a(x, y, z, rg);
        nrm64[c] = make_double4_32a(gx, gy, gz, r);
    }
}

// Combo_NeumannTest (large3Dexample2.c:1975-2055): one block per receiver,
// u(x) = sum_i [dG(x, y*_i)/dn_y - i eta G(x, y*_i)] sigma_i r_i, with
// reg_i for |x - y*_i| <= tau (the reference indexes its regularisation
// with an unset loop variable there when DIRICHLET is 1; reg_i is used).
__global__ void __launch_bounds__(256) combo_eval_kernel(int64_t n, const double4_32a *__restrict__ pos,
                                                         const double4_32a *__restrict__ nrm,
                                                         const double *__restrict__ s_re,
                                                         const double *__restrict__ s_im, const double *__restrict__ rx,
                                                         double wave, double tau, double eta, double *u_re,
                                                         double *u_im)
{
    const int64_t m = blockIdx.x;
    const double sx = rx[3 * m], sy = rx[3 * m + 1], sz = rx[3 * m + 2];
    double ur = 0.0, ui = 0.0;
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
        const double4_32a p = pos[i], q = nrm[i];
        const double x1 = sx - p.x, x2 = sy - p.y, x3 = sz - p.z;
        const double rho = sqrt(x1 * x1 + x2 * x2 + x3 * x3);
        double sv, cv;
        sincos(wave * rho, &sv, &cv);
        const double inner = x1 * q.x + x2 * q.y + x3 * q.z;
        const double f1 = 4. * kPi * rho, f2 = f1 * rho;
        double pr, pi;
        if (rho > tau) {
            pr = (cv / rho + wave * sv) * inner / f2;
            pi = (sv / rho - wave * cv) * inner / f2;
        } else {
            pr = p.w;
            pi = 0.0;
        }
        const double kr = pr + eta * sv / f1, ki = pi + (-1. * eta * cv / f1);
        const double a = s_re[i], b = s_im[i];
        ur += (kr * a - ki * b) * q.w;
        ui += (ki * a + kr * b) * q.w;
    }
    __shared__ double sh[2][8];
    for (int o = 16; o > 0; o >>= 1) {
        ur += __shfl_down_sync(0xffffffffu, ur, o);
        ui += __shfl_down_sync(0xffffffffu, ui, o);
    }
    if ((threadIdx.x & 31) == 0) {
        sh[0][threadIdx.x >> 5] = ur;
        sh[1][threadIdx.x >> 5] = ui;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0, b = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) {
            a += sh[0][w];
            b += sh[1][w];
        }
        u_re[m] = a;
        u_im[m] = b;
    }
}

}  // namespace

int combo_pack(int64_t n, const double *pts, int sine, double *xs, double *nrm, double *delta, double *jac,
               double *reg, double *w, double *adist, double4_32a *pos64, double4_32a *nrm64, cudaStream_t s)
{
    if (n <= 0) return HZ_OK;
    long long b = (n + 255) / 256;
    if (b > 4096) b = 4096;
    combo_pack_kernel<<<(unsigned)b, 256, 0, s>>>(n, pts, sine ? HZ_DP_SINERES : HZ_DP_POLYRES, xs, nrm, delta, jac,
                                                  reg, w, adist, pos64, nrm64);
    HZ_CHECK_LAUNCH();
    return HZ_OK;
}

int sweep_combo64(int64_t n, double wave, double wavenum, double eta, double tau, const double4_32a *pos,
                  const double4_32a *nrm, const double *adist, int mode, const double *p_re, const double *p_im,
                  const double *pt_re, const double *pt_im, double *q_re, double *q_im, double *qt_re, double *qt_im,
                  cudaStream_t s, cudaEvent_t ev0, cudaEvent_t ev1)
{
    if (n <= 0) return HZ_OK;
    ComboArgs a;
    a.n = n;
    a.wave = wave;
    a.wavenum = wavenum;
    a.k2 = wavenum * wavenum;
    a.eta = eta;
    a.tau = tau;
    a.tau2 = tau * tau;
    a.pos = pos;
    a.nrm = nrm;
    a.adist = adist;
    const unsigned blocks = (unsigned)((n + kComboThreads - 1) / kComboThreads);
    if (ev0) HZ_CHECK_CUDA(record_timing_event(ev0, s));
    if (mode & SWEEP_A) {
        a.p_re = p_re;
        a.p_im = p_im;
        a.q_re = q_re;
        a.q_im = q_im;
        combo_sweep_kernel<false><<<blocks, kComboThreads, 0, s>>>(a);
        HZ_CHECK_LAUNCH();
    }
    if (mode & SWEEP_AH) {
        a.p_re = pt_re;
        a.p_im = pt_im;
        a.q_re = qt_re;
        a.q_im = qt_im;
        combo_sweep_kernel<true><<<blocks, kComboThreads, 0, s>>>(a);
        HZ_CHECK_LAUNCH();
    }
    if (ev1) HZ_CHECK_CUDA(record_timing_event(ev1, s));
    return HZ_OK;
}

int launch_eval_combo(int64_t n, const double4_32a *pos, const double4_32a *nrm, const double *s_re,
                      const double *s_im, int64_t m, const double *rx, double wave, double tau, double eta,
                      double *u_re, double *u_im, cudaStream_t s)
{
    if (m <= 0) return HZ_OK;
    combo_eval_kernel<<<(unsigned)m, 256, 0, s>>>(n, pos, nrm, s_re, s_im, rx, wave, tau, eta, u_re, u_im);
    HZ_CHECK_LAUNCH();
    return HZ_OK;
}

}  // namespace hz
