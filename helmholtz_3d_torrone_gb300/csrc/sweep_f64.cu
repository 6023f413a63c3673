// sweep_f64.cu -- FP64 matrix-free pair sweep: q = A p, qt = A^H pt.
//
// The operator is the reference's omp_get_Ccomp entry (large3Dexample2.c:
// 4463-4564) applied on the fly:
//   rho > tau:  A_ts = w_s sg (ct1 + i ct2) (x_t - x_s).n_a,
//               ct1 = -(k sin(k rho) + cos(k rho)/rho) / (4 pi rho^2),
//               ct2 =  (k cos(k rho) - sin(k rho)/rho) / (4 pi rho^2),
//               a = t (Neumann) or s (Dirichlet), sg = -1 for interior;
//   rho <= tau: A_ts = w_s reg_t (Neumann) or w_s reg_s (Dirichlet);
//   A_tt += 1/2.
// A^H row t uses conj(A_st) = w_t conj(...) with the roles of t and s swapped.
//
// One thread owns one target; source tiles of kTile64 records (position+reg,
// normal+weight, prescaled density) are staged in shared memory by TMA bulk
// copies, double-buffered on mbarriers.  FP64 throughout; the 1/2 diagonal
// and the weights are applied in the epilogue.
//
// GB300 runs FP64 at about 1/60 of its FP32 rate, so the FP64 arithmetic is
// kept short: 1/rho comes from rsqrt(rho^2) and rho = rho^2 / rho, and
// sin/cos use the table-driven method of sincos64.cuh.  The near-field
// decision keeps the reference's test sqrt(rho^2) > tau exactly: it is
// evaluated whenever rho^2 lies within a relative 1e-12 of tau^2, where
// rho^2 > tau^2 could disagree.
#include "hz_internal.cuh"
#include "bulk_copy.cuh"
#include "sincos64.cuh"

namespace hz {
namespace {

struct Args64 {
    int64_t n;
    double wave, tau, tau2;
    double inv_scale;  // 4 pi sg: the near-field value times this cancels the density prescale
    const double4_32a *pos, *nrm;
    const double4_32a *dens;  // (w_s p_re, w_s p_im, pt_re, pt_im)
    const double *p_re, *p_im, *pt_re, *pt_im;
    double *q_re, *q_im, *qt_re, *qt_im;
    unsigned *err;
};

// dens = scale (w p, pt), scale = sg / (4 pi): the kernel's common factor.
__global__ void prep64_kernel(int64_t n, const double4_32a *__restrict__ nrm, const double *__restrict__ p_re,
                              const double *__restrict__ p_im, const double *__restrict__ pt_re,
                              const double *__restrict__ pt_im, double scale, double4_32a *__restrict__ dens)
{
    for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < n; s += (int64_t)gridDim.x * blockDim.x) {
        const double w = nrm[s].w * scale;
        double a = 0, b = 0, c = 0, d = 0;
        if (p_re) {
            a = w * p_re[s];
            b = w * p_im[s];
        }
        if (pt_re) {
            c = scale * pt_re[s];
            d = scale * pt_im[s];
        }
        dens[s] = make_double4_32a(a, b, c, d);
    }
}

constexpr double kPi64 = 3.14159265358979323846264338328;

template <int MODE, bool DIR>
__global__ void __launch_bounds__(kThreads64) sweep64_kernel(Args64 a)
{
    constexpr int T = kTile64;
    __shared__ alignas(128) double4_32a sp[2][T];
    __shared__ alignas(128) double4_32a sn[2][T];
    __shared__ alignas(128) double4_32a sd[2][T];
    __shared__ alignas(8) uint64_t bar[2];
    __shared__ double2 tab[kSinTable];
    fill_sin_table(tab);
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = t < a.n;
    double4_32a tp = make_double4_32a(0, 0, 0, 0), tn = make_double4_32a(0, 0, 0, 0);
    if (valid) {
        tp = a.pos[t];
        tn = a.nrm[t];
    }
    const int64_t ntiles = (a.n + T - 1) / T;
    if (threadIdx.x == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        fence_barrier_init();
    }
    __syncthreads();
    auto issue = [&](int64_t tile, int buf) {
        const int64_t base = tile * T;
        const int64_t cnt = (a.n - base < T) ? (a.n - base) : T;
        const uint32_t bytes = (uint32_t)(cnt * sizeof(double4_32a));
        mbar_arrive_expect_tx(&bar[buf], 3 * bytes);
        bulk_g2s(&sp[buf][0], a.pos + base, bytes, &bar[buf]);
        bulk_g2s(&sn[buf][0], a.nrm + base, bytes, &bar[buf]);
        bulk_g2s(&sd[buf][0], a.dens + base, bytes, &bar[buf]);
    };
    if (threadIdx.x == 0 && ntiles > 0) issue(0, 0);
    double aAr = 0, aAi = 0, aHr = 0, aHi = 0;
    for (int64_t tile = 0; tile < ntiles; tile++) {
        const int buf = (int)(tile & 1);
        if (threadIdx.x == 0 && tile + 1 < ntiles) issue(tile + 1, buf ^ 1);
        const bool ok = mbar_wait_bounded(&bar[buf], (uint32_t)((tile >> 1) & 1), g_data_wait_limit);
        if (__syncthreads_or(!ok)) {
            if (threadIdx.x == 0) {
                atomicOr(a.err, DEV_ERR_WAIT);
                // let the issued copies land before the block exits (bounded)
                mbar_drain(&bar[buf], (uint32_t)((tile >> 1) & 1), &bar[buf ^ 1], (uint32_t)(((tile + 1) >> 1) & 1),
                           tile + 1 < ntiles);
            }
            return;
        }
        const int64_t base = tile * T;
        const int cnt = (int)((a.n - base < T) ? (a.n - base) : T);
        if (valid) {
            for (int j = 0; j < cnt; j++) {
                const double4_32a sp_ = sp[buf][j];
                const double4_32a sn_ = sn[buf][j];
                const double4_32a sd_ = sd[buf][j];
                const double xmy1 = tp.x - sp_.x, xmy2 = tp.y - sp_.y, xmy3 = tp.z - sp_.z;
                const double r2 = xmy1 * xmy1 + xmy2 * xmy2 + xmy3 * xmy3;
                bool far = r2 > a.tau2;
                if (fabs(r2 - a.tau2) <= 1e-12 * a.tau2) far = sqrt(r2) > a.tau;
                double vAr = 0.0, vAi = 0.0, vHr = 0.0, vHi = 0.0;
                if (far) {
                    const double rec = rsqrt(r2);
                    const double rho = r2 * rec;
                    double S, C;
                    table_sincos(a.wave * rho, tab, S, C);
                    // sg / (4 pi) rides on the densities
                    const double eS = S * rec, eC = C * rec;
                    const double denom = rec * rec;
                    const double ct1 = -1. * (a.wave * S + eC) * denom;
                    const double ct2 = (a.wave * C - eS) * denom;
                    if (MODE & SWEEP_A) {
                        const double in = DIR ? (xmy1 * sn_.x + xmy2 * sn_.y + xmy3 * sn_.z)
                                              : (xmy1 * tn.x + xmy2 * tn.y + xmy3 * tn.z);
                        vAr = ct1 * in;
                        vAi = ct2 * in;
                    }
                    if (MODE & SWEEP_AH) {
                        const double in = -(DIR ? (xmy1 * tn.x + xmy2 * tn.y + xmy3 * tn.z)
                                                : (xmy1 * sn_.x + xmy2 * sn_.y + xmy3 * sn_.z));
                        vHr = ct1 * in;
                        vHi = -(ct2 * in);
                    }
                } else {
                    vAr = (DIR ? sp_.w : tp.w) * a.inv_scale;
                    vHr = (DIR ? tp.w : sp_.w) * a.inv_scale;
                    vAi = 0.0;
                    vHi = 0.0;
                }
                if (MODE & SWEEP_A) {
                    aAr += vAr * sd_.x - vAi * sd_.y;
                    aAi += vAr * sd_.y + vAi * sd_.x;
                }
                if (MODE & SWEEP_AH) {
                    aHr += vHr * sd_.z - vHi * sd_.w;
                    aHi += vHr * sd_.w + vHi * sd_.z;
                }
            }
        }
        __syncthreads();
    }
    if (!valid) return;
    if (MODE & SWEEP_A) {
        double r = aAr, i = aAi;
        if (!isfinite(r) || !isfinite(i)) atomicOr(a.err, DEV_ERR_NONFINITE);
        a.q_re[t] = r + 0.5 * a.p_re[t];
        a.q_im[t] = i + 0.5 * a.p_im[t];
    }
    if (MODE & SWEEP_AH) {
        const double w = tn.w;
        double r = w * aHr, i = w * aHi;
        if (!isfinite(r) || !isfinite(i)) atomicOr(a.err, DEV_ERR_NONFINITE);
        a.qt_re[t] = r + 0.5 * a.pt_re[t];
        a.qt_im[t] = i + 0.5 * a.pt_im[t];
    }
}

template <int MODE>
void launch64(const Args64 &a, bool dir, cudaStream_t s)
{
    const unsigned blocks = (unsigned)((a.n + kThreads64 - 1) / kThreads64);
    if (dir) sweep64_kernel<MODE, true><<<blocks, kThreads64, 0, s>>>(a);
    else sweep64_kernel<MODE, false><<<blocks, kThreads64, 0, s>>>(a);
}

}  // namespace

int sweep_f64(const SweepConst &c, const Rec64 &r, int mode, const double *p_re, const double *p_im,
              const double *pt_re, const double *pt_im, double *q_re, double *q_im, double *qt_re,
              double *qt_im, double2 *scratch, cudaStream_t s, cudaEvent_t ev0,
              cudaEvent_t ev1)
{
    if (c.n <= 0) return HZ_OK;
    double4_32a *dens = reinterpret_cast<double4_32a *>(scratch);
    const bool useA = (mode & SWEEP_A) != 0, useH = (mode & SWEEP_AH) != 0;
    {
        int dev = 0, sms = 152;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        long long b = (c.n + 255) / 256;
        if (b > sms * 8) b = sms * 8;
        prep64_kernel<<<(unsigned)b, 256, 0, s>>>(c.n, r.nrm, useA ? p_re : nullptr, useA ? p_im : nullptr,
                                                  useH ? pt_re : nullptr, useH ? pt_im : nullptr,
                                                  ((c.interior == 1) ? -1.0 : 1.0) / (4.0 * kPi64), dens);
        HZ_CHECK_LAUNCH();
    }
    Args64 a;
    a.n = c.n;
    a.wave = c.wave;
    a.tau = c.tau;
    a.tau2 = c.tau * c.tau;
    a.inv_scale = ((c.interior == 1) ? -1.0 : 1.0) * (4.0 * kPi64);
    a.pos = r.pos;
    a.nrm = r.nrm;
    a.dens = dens;
    a.p_re = p_re; a.p_im = p_im; a.pt_re = pt_re; a.pt_im = pt_im;
    a.q_re = q_re; a.q_im = q_im; a.qt_re = qt_re; a.qt_im = qt_im;
    a.err = c.err;
    if (ev0) HZ_CHECK_CUDA(record_timing_event(ev0, s));
    if (mode == SWEEP_PAIR) launch64<SWEEP_PAIR>(a, c.dirichlet != 0, s);
    else if (mode == SWEEP_A) launch64<SWEEP_A>(a, c.dirichlet != 0, s);
    else launch64<SWEEP_AH>(a, c.dirichlet != 0, s);
    HZ_CHECK_LAUNCH();
    if (ev1) HZ_CHECK_CUDA(record_timing_event(ev1, s));
    return HZ_OK;
}

HZ_DEFINE_WAIT_LIMIT_SETTER(set_wait_limit_f64)

}  // namespace hz
