// adjoint.cu -- kernels of the adjoint (gradient) path for the receiver
// misfit J = sum_m |u(x_m) - t_m|^2, u = E sigma, A sigma = b:
//   * eval_adj:  s = E^H r                       (reverse of evaluate.cu)
//   * eval_dk:   (dE/dk) sigma at the receivers
//   * sweep_dk:  (dA/dk) sigma over all pairs (FP64)
// Kernel values are recomputed here, never stored.  With
//   c1 + i c2 = (-(k sin kr + cos kr / r) + i (k cos kr - sin kr / r)) / (4 pi r^2)
// (the matrix kernel of large3Dexample2.c:4471-4497) one has
//   d(c1 + i c2)/dk = -(k / (4 pi r)) (cos kr + i sin kr),
// and for the single layer -Phi = (cos kr + i sin kr)/(-4 pi r):
//   d(-Phi)/dk = (sin kr - i cos kr)/(4 pi).
// Near pairs (r <= tau) carry w_s reg, whose k-derivative is w_s dreg
// (dreg stored per point by the tube initialisation).
#include "hz_internal.cuh"

namespace hz {
namespace {

constexpr double kPi = 3.14159265358979323846264338328;
constexpr int kRecvChunk = 256;

// s_c = sum_m conj(E_mc) r_m for every tube point c (one thread per point,
// receivers staged through shared memory).
__global__ void __launch_bounds__(256) eval_adj_kernel(int64_t n, const double4_32a *__restrict__ pos,
                                                       const double4_32a *__restrict__ nrm, int64_t m,
                                                       const double *__restrict__ rx, const double *__restrict__ r_re,
                                                       const double *__restrict__ r_im, double wave, double tau,
                                                       double sg, int layer, double *s_re, double *s_im)
{
    __shared__ double srx[kRecvChunk][5];
    const int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const bool valid = c < n;
    double4_32a p = make_double4_32a(0, 0, 0, 0), q = make_double4_32a(0, 0, 0, 0);
    if (valid) {
        p = pos[c];
        q = nrm[c];
    }
    const double c4 = 1.0 / (4.0 * kPi);
    double ar = 0.0, ai = 0.0;
    for (int64_t m0 = 0; m0 < m; m0 += kRecvChunk) {
        const int cnt = (int)((m - m0 < kRecvChunk) ? (m - m0) : kRecvChunk);
        __syncthreads();
        for (int t = threadIdx.x; t < cnt; t += blockDim.x) {
            srx[t][0] = rx[3 * (m0 + t)];
            srx[t][1] = rx[3 * (m0 + t) + 1];
            srx[t][2] = rx[3 * (m0 + t) + 2];
            srx[t][3] = r_re[m0 + t];
            srx[t][4] = r_im[m0 + t];
        }
        __syncthreads();
        if (!valid) continue;
        for (int t = 0; t < cnt; t++) {
            const double sx = srx[t][0], sy = srx[t][1], sz = srx[t][2];
            const double sn = sqrt((p.x - sx) * (p.x - sx) + (p.y - sy) * (p.y - sy) + (p.z - sz) * (p.z - sz));
            if (!(sn > tau)) continue;
            double S, C, er, ei;
            sincos(wave * sn, &S, &C);
            if (layer == HZ_SINGLE_LAYER) {
                er = C / (-4. * kPi * sn);
                ei = S / (-4. * kPi * sn);
            } else {
                const double rec = 1. / sn, denom = c4 * rec * rec;
                const double ct1 = -1. * (wave * S + C * rec) * denom, ct2 = (wave * C - S * rec) * denom;
                const double in = (sx - p.x) * q.x + (sy - p.y) * q.y + (sz - p.z) * q.z;
                er = sg * ct1 * in;
                ei = sg * ct2 * in;
            }
            // conj(E) r with E = (er + i ei) w
            ar += er * srx[t][3] + ei * srx[t][4];
            ai += er * srx[t][4] - ei * srx[t][3];
        }
    }
    if (valid) {
        s_re[c] = ar * q.w;
        s_im[c] = ai * q.w;
    }
}

// ((dE/dk) sigma)_m, one block per receiver.
__global__ void __launch_bounds__(256) eval_dk_kernel(int64_t n, const double4_32a *__restrict__ pos,
                                                      const double4_32a *__restrict__ nrm,
                                                      const double *__restrict__ s_re, const double *__restrict__ s_im,
                                                      const double *__restrict__ rx, double wave, double tau, double sg,
                                                      int layer, double *u_re, double *u_im)
{
    const int64_t r = blockIdx.x;
    const double sx = rx[3 * r], sy = rx[3 * r + 1], sz = rx[3 * r + 2];
    double ur = 0.0, ui = 0.0;
    for (int64_t c = threadIdx.x; c < n; c += blockDim.x) {
        const double4_32a p = pos[c], q = nrm[c];
        const double sn = sqrt((p.x - sx) * (p.x - sx) + (p.y - sy) * (p.y - sy) + (p.z - sz) * (p.z - sz));
        if (!(sn > tau)) continue;
        double S, C, er, ei;
        sincos(wave * sn, &S, &C);
        if (layer == HZ_SINGLE_LAYER) {
            er = S / (4. * kPi);
            ei = -C / (4. * kPi);
        } else {
            const double f = -wave / (4. * kPi * sn);
            const double in = (sx - p.x) * q.x + (sy - p.y) * q.y + (sz - p.z) * q.z;
            er = sg * f * C * in;
            ei = sg * f * S * in;
        }
        const double a = s_re[c], b = s_im[c];
        ur += (er * a - ei * b) * q.w;
        ui += (er * b + ei * a) * q.w;
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
        u_re[r] = a;
        u_im[r] = b;
    }
}

// ((dA/dk) sigma)_t over all sources (one thread per target, sources read
// through the cache).  Far: w_s sg d(c1+ic2)/dk (x_t-x_s).n_a; near: w_s dreg.
template <bool DIR>
__global__ void __launch_bounds__(128) sweep_dk_kernel(int64_t n, const double4_32a *__restrict__ pos,
                                                       const double4_32a *__restrict__ nrm,
                                                       const double *__restrict__ dreg, const double *__restrict__ s_re,
                                                       const double *__restrict__ s_im, double wave, double tau, double sg,
                                                       double *q_re, double *q_im)
{
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= n) return;
    const double4_32a tp = pos[t], tn = nrm[t];
    const double dt = dreg[t];
    double ar = 0.0, ai = 0.0;
    for (int64_t s = 0; s < n; s++) {
        const double4_32a sp = pos[s], snn = nrm[s];
        const double x1 = tp.x - sp.x, x2 = tp.y - sp.y, x3 = tp.z - sp.z;
        const double rho = sqrt(x1 * x1 + x2 * x2 + x3 * x3);
        double vr, vi;
        if (rho > tau) {
            double S, C;
            sincos(wave * rho, &S, &C);
            const double f = -wave / (4. * kPi * rho);
            const double in = DIR ? (x1 * snn.x + x2 * snn.y + x3 * snn.z) : (x1 * tn.x + x2 * tn.y + x3 * tn.z);
            vr = sg * f * C * in;
            vi = sg * f * S * in;
        } else {
            vr = DIR ? dreg[s] : dt;
            vi = 0.0;
        }
        const double a = snn.w * s_re[s], b = snn.w * s_im[s];
        ar += vr * a - vi * b;
        ai += vr * b + vi * a;
    }
    q_re[t] = ar;
    q_im[t] = ai;
}

}  // namespace

int launch_eval_adjoint(int64_t n, const double4_32a *pos, const double4_32a *nrm, int64_t m, const double *rx,
                        const double *r_re, const double *r_im, double wave, double tau, int interior, int layer,
                        double *s_re, double *s_im, cudaStream_t s)
{
    if (n <= 0) return HZ_OK;
    eval_adj_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(n, pos, nrm, m, rx, r_re, r_im, wave, tau,
                                                                interior == 1 ? -1.0 : 1.0, layer, s_re, s_im);
    HZ_CHECK_LAUNCH();
    return HZ_OK;
}

int launch_eval_dk(int64_t n, const double4_32a *pos, const double4_32a *nrm, const double *s_re,
                   const double *s_im, int64_t m, const double *rx, double wave, double tau, int interior, int layer,
                   double *u_re, double *u_im, cudaStream_t s)
{
    if (m <= 0) return HZ_OK;
    eval_dk_kernel<<<(unsigned)m, 256, 0, s>>>(n, pos, nrm, s_re, s_im, rx, wave, tau, interior == 1 ? -1.0 : 1.0,
                                               layer, u_re, u_im);
    HZ_CHECK_LAUNCH();
    return HZ_OK;
}

int launch_sweep_dk(int64_t n, const double4_32a *pos, const double4_32a *nrm, const double *dreg,
                    const double *s_re, const double *s_im, double wave, double tau, int interior, int dirichlet,
                    double *q_re, double *q_im, cudaStream_t s)
{
    if (n <= 0) return HZ_OK;
    const unsigned blocks = (unsigned)((n + 127) / 128);
    const double sg = interior == 1 ? -1.0 : 1.0;
    if (dirichlet) sweep_dk_kernel<true><<<blocks, 128, 0, s>>>(n, pos, nrm, dreg, s_re, s_im, wave, tau, sg, q_re, q_im);
    else sweep_dk_kernel<false><<<blocks, 128, 0, s>>>(n, pos, nrm, dreg, s_re, s_im, wave, tau, sg, q_re, q_im);
    HZ_CHECK_LAUNCH();
    return HZ_OK;
}

}  // namespace hz
