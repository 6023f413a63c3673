// shape_grad.cu -- misfit gradient with respect to the distance-grid values.
//
// J = sum_m |u_m - t_m|^2, u = E sigma, A sigma = b (Dirichlet formulation,
// double-layer receivers, boundary data b = G(x* - src), G(r) = e^{ikr}/(4 pi r)).
// With the adjoint A^H lambda = E^H r (r = u - t), for any parameter theta
//   dJ/dtheta = 2 Re[r^H (dE/dtheta) sigma] + 2 Re[lambda^H (db/dtheta)]
//             - 2 Re[lambda^H (dA/dtheta) sigma].
// The grid phi enters through the tube points' projections x*, normals n,
// weights w and regularisation factors reg, and those through the WENO
// gradient and the curvature grids.  This file computes
//   (1) per point p the sensitivities dJ/dx*_p, dJ/dn_p, dJ/dreg_p (an FP64
//       pair sweep with the kernel's derivatives; dJ/dw_p is closed form), and
//   (2) their pull-back through the projection, the trilinear
//       interpolations, the normalisations, delta_eps and the Jacobian into
//       adjoints of the grids (gx, gy, gz, mc, gc) and of phi itself;
// the stencils' own pull-back (grids -> phi) is stencil_adjoint_kernel
// (stencils.cu).  Kernel of the Dirichlet matrix (large3Dexample2.c:4471-4534):
//   A_ts = w_s sg f(rho) (x_t - x_s).n_s for rho > tau, w_s reg_s otherwise,
//   f(rho) = e^{ik rho} (ik - 1/rho) / (4 pi rho^2) = G'(rho)/rho,
//   f'(rho) = e^{ik rho} (-k^2 - 3ik/rho + 3/rho^2) / (4 pi rho^2),
// so d[f(rho) (d.n)]/dd = B(d; n) = (f'/rho)(d.n) d + f n.
#include "hz_internal.cuh"

namespace hz {
namespace {

constexpr double kPi = 3.14159265358979323846264338328;
constexpr int kShT = 128;

struct Cplx {
    double re, im;
};

__device__ __forceinline__ void kernel_fs(double k, double rho, Cplx &f, Cplx &fp)
{
    double S, C;
    sincos(k * rho, &S, &C);
    const double q = 1.0 / (4.0 * kPi * rho * rho);
    // f = (C + iS)(ik - 1/rho) q
    const double ar = -1.0 / rho, ai = k;
    f.re = (C * ar - S * ai) * q;
    f.im = (C * ai + S * ar) * q;
    // f' = (C + iS)(-k^2 + 3/rho^2 - 3ik/rho) q
    const double br = -k * k + 3.0 / (rho * rho), bi = -3.0 * k / rho;
    fp.re = (C * br - S * bi) * q;
    fp.im = (C * bi + S * br) * q;
}

// Per point p: S1 = sum_t conj(lambda_t) B(x_t - x_p; n_p), S2 = sum_s
// B(x_p - x_s; n_s) w_s sigma_s, S3 = sum_t conj(lambda_t) f (x_t - x_p) over
// rho > tau, S4 = sum over rho <= tau of conj(lambda_t); then the receiver
// sums and the boundary-data term.  Outputs gx (3n), gn (3n), greg (n).
__global__ void __launch_bounds__(kShT) shape_sens_kernel(int64_t n, const double4_32a *__restrict__ pos,
                                                          const double4_32a *__restrict__ nrm,
                                                          const double *__restrict__ s_re,
                                                          const double *__restrict__ s_im,
                                                          const double *__restrict__ l_re,
                                                          const double *__restrict__ l_im, int64_t m,
                                                          const double *__restrict__ rx, const double *__restrict__ r_re,
                                                          const double *__restrict__ r_im, double wave, double tau,
                                                          double sg, double srcx, double srcy, double srcz,
                                                          double *gxs, double *gn, double *greg)
{
    __shared__ double4_32a sp[kShT], sn[kShT];
    __shared__ double4_32a sv[kShT];  // (sigma re, im, lambda re, im)
    const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const bool valid = p < n;
    double4_32a xp = make_double4_32a(0, 0, 0, 0), np_ = make_double4_32a(0, 0, 0, 0);
    double sr = 0, si = 0, lr = 0, li = 0;
    if (valid) {
        xp = pos[p];
        np_ = nrm[p];
        sr = s_re[p];
        si = s_im[p];
        lr = l_re[p];
        li = l_im[p];
    }
    Cplx S1[3] = {{0, 0}, {0, 0}, {0, 0}}, S2[3] = {{0, 0}, {0, 0}, {0, 0}}, S3[3] = {{0, 0}, {0, 0}, {0, 0}};
    Cplx S4 = {0, 0};
    for (int64_t base = 0; base < n; base += kShT) {
        const int cnt = (int)((n - base < kShT) ? (n - base) : kShT);
        __syncthreads();
        for (int q = threadIdx.x; q < cnt; q += blockDim.x) {
            sp[q] = pos[base + q];
            sn[q] = nrm[base + q];
            sv[q] = make_double4_32a(s_re[base + q], s_im[base + q], l_re[base + q], l_im[base + q]);
        }
        __syncthreads();
        if (!valid) continue;
        for (int q = 0; q < cnt; q++) {
            const double4_32a xt = sp[q], nt = sn[q], v = sv[q];
            const double d0 = xt.x - xp.x, d1 = xt.y - xp.y, d2 = xt.z - xp.z;
            const double rho = sqrt(d0 * d0 + d1 * d1 + d2 * d2);
            // conj(lambda_t)
            const double cl_r = v.z, cl_i = -v.w;
            if (!(rho > tau)) {
                S4.re += cl_r;
                S4.im += cl_i;
                continue;
            }
            Cplx f, fp;
            kernel_fs(wave, rho, f, fp);
            const double dnp = d0 * np_.x + d1 * np_.y + d2 * np_.z;
            const double dnt = d0 * nt.x + d1 * nt.y + d2 * nt.z;
            const double dv[3] = {d0, d1, d2}, npv[3] = {np_.x, np_.y, np_.z}, ntv[3] = {nt.x, nt.y, nt.z};
            // w_t sigma_t
            const double ws_r = nt.w * v.x, ws_i = nt.w * v.y;
#pragma unroll
            for (int c = 0; c < 3; c++) {
                // B1 = (f'/rho)(d.n_p) d + f n_p ; B2 = (f'/rho)(d.n_t) d + f n_t
                const double b1r = fp.re / rho * dnp * dv[c] + f.re * npv[c];
                const double b1i = fp.im / rho * dnp * dv[c] + f.im * npv[c];
                const double b2r = fp.re / rho * dnt * dv[c] + f.re * ntv[c];
                const double b2i = fp.im / rho * dnt * dv[c] + f.im * ntv[c];
                S1[c].re += cl_r * b1r - cl_i * b1i;
                S1[c].im += cl_r * b1i + cl_i * b1r;
                S2[c].re += b2r * ws_r - b2i * ws_i;
                S2[c].im += b2r * ws_i + b2i * ws_r;
                const double fdr = f.re * dv[c], fdi = f.im * dv[c];
                S3[c].re += cl_r * fdr - cl_i * fdi;
                S3[c].im += cl_r * fdi + cl_i * fdr;
            }
        }
    }
    // receivers: R1 = sum_m conj(r_m) B(x_m - x_p; n_p), R2 = sum_m conj(r_m) f (x_m - x_p)
    Cplx R1[3] = {{0, 0}, {0, 0}, {0, 0}}, R2[3] = {{0, 0}, {0, 0}, {0, 0}};
    for (int64_t base = 0; base < m; base += kShT) {
        const int cnt = (int)((m - base < kShT) ? (m - base) : kShT);
        __syncthreads();
        for (int q = threadIdx.x; q < cnt; q += blockDim.x) {
            sv[q] = make_double4_32a(rx[3 * (base + q)], rx[3 * (base + q) + 1], rx[3 * (base + q) + 2], 0.0);
            sp[q] = make_double4_32a(r_re[base + q], r_im[base + q], 0.0, 0.0);
        }
        __syncthreads();
        if (!valid) continue;
        for (int q = 0; q < cnt; q++) {
            const double d0 = sv[q].x - xp.x, d1 = sv[q].y - xp.y, d2 = sv[q].z - xp.z;
            const double rho = sqrt(d0 * d0 + d1 * d1 + d2 * d2);
            if (!(rho > tau)) continue;
            Cplx f, fp;
            kernel_fs(wave, rho, f, fp);
            const double cr_r = sp[q].x, cr_i = -sp[q].y;
            const double dnp = d0 * np_.x + d1 * np_.y + d2 * np_.z;
            const double dv[3] = {d0, d1, d2}, npv[3] = {np_.x, np_.y, np_.z};
#pragma unroll
            for (int c = 0; c < 3; c++) {
                const double br = fp.re / rho * dnp * dv[c] + f.re * npv[c];
                const double bi = fp.im / rho * dnp * dv[c] + f.im * npv[c];
                R1[c].re += cr_r * br - cr_i * bi;
                R1[c].im += cr_r * bi + cr_i * br;
                R2[c].re += cr_r * f.re * dv[c] - cr_i * f.im * dv[c];
                R2[c].im += cr_r * f.im * dv[c] + cr_i * f.re * dv[c];
            }
        }
    }
    if (!valid) return;
    // boundary data b_p = G(|x*_p - src|): db/dx* = f(rho_s) (x*_p - src)
    const double e0 = xp.x - srcx, e1 = xp.y - srcy, e2 = xp.z - srcz;
    const double rs = sqrt(e0 * e0 + e1 * e1 + e2 * e2);
    Cplx fs, fsp;
    kernel_fs(wave, rs, fs, fsp);
    const double ev[3] = {e0, e1, e2};
    const double w = np_.w;
    // 2 Re(a z) with a = w sg sigma_p (complex) for S1 / R1 / S3 / R2
    const double ar = w * sg * sr, ai = w * sg * si;
#pragma unroll
    for (int c = 0; c < 3; c++) {
        double g = 2.0 * (ar * S1[c].re - ai * S1[c].im);                  // + 2Re[w sg sigma S1]
        g -= 2.0 * sg * (lr * S2[c].re + li * S2[c].im);                   // - 2Re[conj(l_p) sg S2]
        g -= 2.0 * (ar * R1[c].re - ai * R1[c].im);                        // - 2Re[w sg sigma R1]
        g += 2.0 * (lr * fs.re * ev[c] + li * fs.im * ev[c]);             // + 2Re[conj(l_p) db/dx]
        gxs[3 * p + c] = g;
        gn[3 * p + c] = -2.0 * (ar * S3[c].re - ai * S3[c].im) + 2.0 * (ar * R2[c].re - ai * R2[c].im);
    }
    greg[p] = -2.0 * (w * sr * S4.re - w * si * S4.im);
}

struct ChainArgs {
    int N, interior, order;
    double H, int_l, eps, tau, wave;
    int64_t n;
    const int64_t *idx;
    const double *d, *gx, *gy, *gz, *mc, *gc;
    const double *xs;  // 3n
    const double *w, *s_re, *s_im, *l_re, *l_im;
    const double *gxs, *gn, *greg;
    double *Gbx, *Gby, *Gbz, *mcb, *gcb, *phib;
};

// Pull the per-point sensitivities back to the grids (one thread per point).
__global__ void __launch_bounds__(128) shape_chain_kernel(ChainArgs a)
{
    const long long S = a.N + 1;
    const double H = a.H, H3 = H * H * H;
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < a.n; p += (int64_t)gridDim.x * blockDim.x) {
        const long long o = a.idx[p];
        const double phi = a.d[o];
        const double G0 = a.gx[o], G1 = a.gy[o], G2 = a.gz[o];
        const double tx = a.xs[3 * p], ty = a.xs[3 * p + 1], tz = a.xs[3 * p + 2];
        double xb[3] = {a.gxs[3 * p], a.gxs[3 * p + 1], a.gxs[3 * p + 2]};
        // ---- normal: n = normalise(normalise(v)), v trilinear in the gradient grids
        {
            const int gi = (int)((ty - a.int_l) / H), gj = (int)((tx - a.int_l) / H), gk = (int)((tz - a.int_l) / H);
            if (gi >= 0 && gj >= 0 && gk >= 0 && gi < a.N && gj < a.N && gk < a.N) {
                const double lx = tx - a.int_l - (double)gj * H, ly = ty - a.int_l - (double)gi * H,
                             lz = tz - a.int_l - (double)gk * H;
                double v[3] = {0, 0, 0};
                double wc[8], dwc[8][3];
                long long qc[8];
                for (int c = 0; c < 8; c++) {
                    const int ai_ = (c >> 2) & 1, bj = (c >> 1) & 1, ck = c & 1;  // i (y), j (x), k (z) offsets
                    const double fx = bj ? lx : H - lx, fy = ai_ ? ly : H - ly, fz = ck ? lz : H - lz;
                    const double sx = bj ? 1.0 : -1.0, sy = ai_ ? 1.0 : -1.0, sz = ck ? 1.0 : -1.0;
                    wc[c] = fx * fy * fz / H3;
                    dwc[c][0] = sx * fy * fz / H3;
                    dwc[c][1] = fx * sy * fz / H3;
                    dwc[c][2] = fx * fy * sz / H3;
                    qc[c] = ((gi + ai_) * S + gj + bj) * S + gk + ck;
                    v[0] += wc[c] * a.gx[qc[c]];
                    v[1] += wc[c] * a.gy[qc[c]];
                    v[2] += wc[c] * a.gz[qc[c]];
                }
                const double nv = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
                if (nv > 0) {
                    const double nn[3] = {v[0] / nv, v[1] / nv, v[2] / nv};
                    const double gnv[3] = {a.gn[3 * p], a.gn[3 * p + 1], a.gn[3 * p + 2]};
                    const double dot = gnv[0] * nn[0] + gnv[1] * nn[1] + gnv[2] * nn[2];
                    const double vb[3] = {(gnv[0] - dot * nn[0]) / nv, (gnv[1] - dot * nn[1]) / nv,
                                          (gnv[2] - dot * nn[2]) / nv};
                    for (int c = 0; c < 8; c++) {
                        atomicAdd(a.Gbx + qc[c], wc[c] * vb[0]);
                        atomicAdd(a.Gby + qc[c], wc[c] * vb[1]);
                        atomicAdd(a.Gbz + qc[c], wc[c] * vb[2]);
                        const double gv = a.gx[qc[c]] * vb[0] + a.gy[qc[c]] * vb[1] + a.gz[qc[c]] * vb[2];
                        xb[0] += dwc[c][0] * gv;
                        xb[1] += dwc[c][1] * gv;
                        xb[2] += dwc[c][2] * gv;
                    }
                }
            }
        }
        // ---- regularisation factor from the curvatures interpolated at x*
        {
            const double gr = a.greg[p];
            const int cj = (int)((tx + 1e-19 - a.int_l) / H), ci = (int)((ty + 1e-19 - a.int_l) / H),
                      ck = (int)((tz + 1e-19 - a.int_l) / H);
            if (gr != 0.0 && ci >= 0 && cj >= 0 && ck >= 0 && ci < a.N && cj < a.N && ck < a.N) {
                const double lx = tx - a.int_l - (double)cj * H, ly = ty - a.int_l - (double)ci * H,
                             lz = tz - a.int_l - (double)ck * H;
                double wc[8], dwc[8][3], cm = 0, cg = 0;
                long long qc[8];
                for (int c = 0; c < 8; c++) {
                    const int ai_ = (c >> 2) & 1, bj = (c >> 1) & 1, kk = c & 1;
                    const double fx = bj ? lx : H - lx, fy = ai_ ? ly : H - ly, fz = kk ? lz : H - lz;
                    const double sx = bj ? 1.0 : -1.0, sy = ai_ ? 1.0 : -1.0, sz = kk ? 1.0 : -1.0;
                    wc[c] = fx * fy * fz / H3;
                    dwc[c][0] = sx * fy * fz / H3;
                    dwc[c][1] = fx * sy * fz / H3;
                    dwc[c][2] = fx * fy * sz / H3;
                    qc[c] = ((ci + ai_) * S + cj + bj) * S + ck + kk;
                    cm += wc[c] * a.mc[qc[c]];
                    cg += wc[c] * a.gc[qc[c]];
                }
                const double t = a.tau, sgn = (a.interior == 1) ? 1.0 : -1.0;
                const double dcm = sgn * (1.0 / (4. * kPi * t) - 5. * t * (24. * cm * cm - 2. * cg) / (512. * kPi) -
                                          50. * t * cg / (1536. * kPi) + 2. * a.wave * a.wave * t / (48. * kPi));
                const double dcg = sgn * (10. * t * cm / (512. * kPi) - 50. * t * cm / (1536. * kPi));
                for (int c = 0; c < 8; c++) {
                    atomicAdd(a.mcb + qc[c], gr * dcm * wc[c]);
                    atomicAdd(a.gcb + qc[c], gr * dcg * wc[c]);
                    const double gv = gr * (dcm * a.mc[qc[c]] + dcg * a.gc[qc[c]]);
                    xb[0] += dwc[c][0] * gv;
                    xb[1] += dwc[c][1] * gv;
                    xb[2] += dwc[c][2] * gv;
                }
            }
        }
        // ---- weight w = H^3 delta(phi) J, J = 1 + 2 phi mc + phi^2 gc; dJ/dw = Re(conj(l) sigma)/w
        {
            const double wv = a.w[p];
            const double gw = (wv != 0.0) ? (a.l_re[p] * a.s_re[p] + a.l_im[p] * a.s_im[p]) / wv : 0.0;
            const double e = a.eps;
            const double dl = (fabs(phi) <= e) ? (1.0 / (2.0 * e)) * (1.0 + cos(kPi * phi / e)) : 0.0;
            const double ddl = (fabs(phi) <= e) ? -(kPi / (2.0 * e * e)) * sin(kPi * phi / e) : 0.0;
            const double mco = a.mc[o], gco = a.gc[o];
            const double J = 1 + 2. * phi * mco + phi * phi * gco;
            atomicAdd(a.phib + o, gw * H3 * (ddl * J + dl * (2. * mco + 2. * phi * gco)));
            atomicAdd(a.mcb + o, gw * H3 * dl * 2. * phi);
            atomicAdd(a.gcb + o, gw * H3 * dl * phi * phi);
        }
        // ---- projection x* = z - phi grad(phi)(z)
        atomicAdd(a.phib + o, -(xb[0] * G0 + xb[1] * G1 + xb[2] * G2));
        atomicAdd(a.Gbx + o, -phi * xb[0]);
        atomicAdd(a.Gby + o, -phi * xb[1]);
        atomicAdd(a.Gbz + o, -phi * xb[2]);
    }
}

}  // namespace

int shape_gradient_device(const hz_params &p, double H, double eps, double tau, int64_t n, const int64_t *idx,
                          const double *d, const double *gx, const double *gy, const double *gz, const double *mc,
                          const double *gc, const double *xs, const double *w, const double4_32a *pos,
                          const double4_32a *nrm, const double *s_re, const double *s_im, const double *l_re,
                          const double *l_im, int64_t m, const double *rx, const double *r_re, const double *r_im,
                          const double *src, double *work, double *phib, cudaStream_t s)
{
    const long long S = p.N + 1, nodes = S * S * S;
    double *gxs = work, *gn = work + 3 * n, *greg = work + 6 * n;
    double *Gb = work + 7 * n;  // 5 grids: Gbx, Gby, Gbz, mcb, gcb
    HZ_CHECK_CUDA(cudaMemsetAsync(Gb, 0, 5 * nodes * sizeof(double), s));
    HZ_CHECK_CUDA(cudaMemsetAsync(phib, 0, nodes * sizeof(double), s));
    if (n > 0) {
        const double sg = (p.interior == 1) ? -1.0 : 1.0;
        shape_sens_kernel<<<(unsigned)((n + kShT - 1) / kShT), kShT, 0, s>>>(
            n, pos, nrm, s_re, s_im, l_re, l_im, m, rx, r_re, r_im, p.wave, tau, sg, src[0], src[1], src[2], gxs, gn,
            greg);
        HZ_CHECK_LAUNCH();
        ChainArgs a;
        a.N = p.N;
        a.interior = p.interior;
        a.order = p.weno_order;
        a.H = H;
        a.int_l = p.int_l;
        a.eps = eps;
        a.tau = tau;
        a.wave = p.wave;
        a.n = n;
        a.idx = idx;
        a.d = d;
        a.gx = gx;
        a.gy = gy;
        a.gz = gz;
        a.mc = mc;
        a.gc = gc;
        a.xs = xs;
        a.w = w;
        a.s_re = s_re;
        a.s_im = s_im;
        a.l_re = l_re;
        a.l_im = l_im;
        a.gxs = gxs;
        a.gn = gn;
        a.greg = greg;
        a.Gbx = Gb;
        a.Gby = Gb + nodes;
        a.Gbz = Gb + 2 * nodes;
        a.mcb = Gb + 3 * nodes;
        a.gcb = Gb + 4 * nodes;
        a.phib = phib;
        long long b = (n + 127) / 128;
        if (b > 4096) b = 4096;
        shape_chain_kernel<<<(unsigned)b, 128, 0, s>>>(a);
        HZ_CHECK_LAUNCH();
    }
    // grids -> phi through the stencils (local central differences, step 1e-7)
    return launch_stencil_adjoint(p.N, H, d, Gb, Gb + nodes, Gb + 2 * nodes, Gb + 3 * nodes, Gb + 4 * nodes, phib,
                                  p.weno_order, 1e-7, s);
}

size_t shape_gradient_work_bytes(int64_t n, int N)
{
    const size_t S = (size_t)N + 1;
    return (7 * (size_t)n + 5 * S * S * S) * sizeof(double);
}

}  // namespace hz
