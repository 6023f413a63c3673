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
// One thread owns two targets (kTgt64); source tiles of kSrc64 records
// (position+reg, normal+weight, prescaled density) are staged in shared
// memory by TMA bulk copies, double-buffered on mbarriers, and each staged
// record serves both targets.  FP64 throughout; the 1/2 diagonal and the
// weights are applied in the epilogue.
//
// GB300 runs FP64 at about 1/64 of its FP32 rate and the kernel is bound by
// the FP64 pipe, so each far pair costs as few FP64 operations as the
// result's accuracy allows (pair64.cuh): 1/rho from an SFU seed and one
// third-order correction, sin/cos of k rho from a 2048-entry table and two
// short series, the table index from FP32 arithmetic, and the entry formed
// as e^{i k rho} (-1/rho + i k) / rho^2 (six FP64 multiplies fewer than the
// reference's separate ct1 and ct2).  The near-field decision keeps the
// reference's test sqrt(rho^2) > tau exactly: rho^2 and tau^2 are compared
// as integers (their bit patterns order like the values), and within 8192
// ulps of tau^2 the reference's own arithmetic (rho^2 summed without fused
// multiply-adds, IEEE square root) decides.
#include "hz_internal.cuh"
#include "bulk_copy.cuh"
#include "pair64.cuh"

namespace hz {
namespace {

struct Args64 {
    int64_t n;
    double wave, tau, tau2;
    float kscale;       // k * 2048 / (2 pi) (2048 / (2 pi) on scaled coordinates): the phase table index
    long long tau2b;    // bit pattern of tau^2 ((k tau)^2 on scaled coordinates)
    double inv_scale;  // 4 pi sg (/ k^2 scaled): the near-field value times this cancels the density prescale
    const double4_32a *pos, *nrm;
    const double4_32a *posu;  // unscaled positions (the near-field tie test of the scaled sweep)
    const double4_32a *dens;  // (w_s p_re, w_s p_im, pt_re, pt_im)
    const double *p_re, *p_im, *pt_re, *pt_im;
    double *q_re, *q_im, *qt_re, *qt_im;
    unsigned *err;
};

constexpr int kSrc64 = 64;   // sources per shared-memory tile
constexpr int kTgt64 = 2;    // targets per thread
constexpr long long kTieUlps = 8192;

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

// The reference's near-field decision sqrt(rho^2) > tau, rho^2 summed
// without fused multiply-adds, on unscaled coordinate differences.
__device__ __forceinline__ bool far_exact(double dx, double dy, double dz, double tau)
{
    const double r2ref = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
    return __dsqrt_rn(r2ref) > tau;
}

// One (target t, source s) pair added to acc = (A re, A im, A^H re, A^H im).
// SCALED: positions are k x, so the differences, rho^2 and the projection
// carry factors of k (the densities carry the k^2 of the entry).
template <int MODE, bool DIR, bool SCALED>
__device__ __forceinline__ void pair64(const Args64 &a, const double2 *tab, const double4_32a &tp,
                                       const double4_32a &tn, const double4_32a &sp, const double4_32a &sn,
                                       const double4_32a &sd, int64_t t, int64_t s, double *acc)
{
    const double dx = tp.x - sp.x, dy = tp.y - sp.y, dz = tp.z - sp.z;
    const double r2 = fma(dz, dz, fma(dy, dy, dx * dx));
    const long long rb = __double_as_longlong(r2);
    bool far = rb > a.tau2b;
    if ((unsigned long long)(rb - a.tau2b + kTieUlps) <= (unsigned long long)(2 * kTieUlps)) {
        if (SCALED) {
            const double4_32a u = a.posu[t], v = a.posu[s];
            far = far_exact(u.x - v.x, u.y - v.y, u.z - v.z, a.tau);
        } else {
            far = far_exact(dx, dy, dz, a.tau);
        }
    }
    if (far) {
        double ur, ui, y2;
        far_factor64<SCALED>(r2, a.wave, a.kscale, tab, ur, ui, y2);
        if (MODE & SWEEP_A) {
            const double in = DIR ? fma(dz, sn.z, fma(dy, sn.y, dx * sn.x)) : fma(dz, tn.z, fma(dy, tn.y, dx * tn.x));
            const double f = in * y2;
            const double vr = ur * f, vi = ui * f;
            acc[0] = fma(-vi, sd.y, fma(vr, sd.x, acc[0]));
            acc[1] = fma(vi, sd.x, fma(vr, sd.y, acc[1]));
        }
        if (MODE & SWEEP_AH) {
            const double in = DIR ? fma(dz, tn.z, fma(dy, tn.y, dx * tn.x)) : fma(dz, sn.z, fma(dy, sn.y, dx * sn.x));
            // conj of the entry with the roles swapped: in -> -in, imaginary part negated
            const double f = -(in * y2);
            const double vr = ur * f, vi = -(ui * f);
            acc[2] = fma(-vi, sd.w, fma(vr, sd.z, acc[2]));
            acc[3] = fma(vi, sd.z, fma(vr, sd.w, acc[3]));
        }
    } else {
        if (MODE & SWEEP_A) {
            const double v = (DIR ? sp.w : tp.w) * a.inv_scale;
            acc[0] = fma(v, sd.x, acc[0]);
            acc[1] = fma(v, sd.y, acc[1]);
        }
        if (MODE & SWEEP_AH) {
            const double v = (DIR ? tp.w : sp.w) * a.inv_scale;
            acc[2] = fma(v, sd.z, acc[2]);
            acc[3] = fma(v, sd.w, acc[3]);
        }
    }
}

template <int MODE, bool DIR, bool SCALED>
__global__ void __launch_bounds__(kThreads64, 4) sweep64_kernel(Args64 a)
{
    constexpr int T = kSrc64;
    __shared__ alignas(128) double4_32a sp[2][T];
    __shared__ alignas(128) double4_32a sn[2][T];
    __shared__ alignas(128) double4_32a sd[2][T];
    __shared__ alignas(8) uint64_t bar[2];
    __shared__ alignas(16) double2 tab[kPhaseTable];
    fill_phase_table(tab);
    const int64_t t0 = (int64_t)blockIdx.x * (blockDim.x * kTgt64) + threadIdx.x;
    double4_32a tp[kTgt64], tn[kTgt64];
    bool valid[kTgt64];
#pragma unroll
    for (int g = 0; g < kTgt64; g++) {
        const int64_t t = t0 + (int64_t)g * blockDim.x;
        valid[g] = t < a.n;
        tp[g] = valid[g] ? a.pos[t] : make_double4_32a(0, 0, 0, 0);
        tn[g] = valid[g] ? a.nrm[t] : make_double4_32a(0, 0, 0, 0);
    }
    const bool any = valid[0];
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
    double acc[kTgt64][4];
#pragma unroll
    for (int g = 0; g < kTgt64; g++) acc[g][0] = acc[g][1] = acc[g][2] = acc[g][3] = 0.0;
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
        if (any) {
            for (int j = 0; j < cnt; j++) {
                const double4_32a sp_ = sp[buf][j];
                const double4_32a sn_ = sn[buf][j];
                const double4_32a sd_ = sd[buf][j];
#pragma unroll
                for (int g = 0; g < kTgt64; g++)
                    pair64<MODE, DIR, SCALED>(a, tab, tp[g], tn[g], sp_, sn_, sd_, t0 + (int64_t)g * blockDim.x,
                                              base + j, acc[g]);
            }
        }
        __syncthreads();
    }
#pragma unroll
    for (int g = 0; g < kTgt64; g++) {
        if (!valid[g]) continue;
        const int64_t t = t0 + (int64_t)g * blockDim.x;
        if (MODE & SWEEP_A) {
            const double r = acc[g][0], i = acc[g][1];
            if (!isfinite(r) || !isfinite(i)) atomicOr(a.err, DEV_ERR_NONFINITE);
            a.q_re[t] = r + 0.5 * a.p_re[t];
            a.q_im[t] = i + 0.5 * a.p_im[t];
        }
        if (MODE & SWEEP_AH) {
            const double w = tn[g].w;
            const double r = w * acc[g][2], i = w * acc[g][3];
            if (!isfinite(r) || !isfinite(i)) atomicOr(a.err, DEV_ERR_NONFINITE);
            a.qt_re[t] = r + 0.5 * a.pt_re[t];
            a.qt_im[t] = i + 0.5 * a.pt_im[t];
        }
    }
}

template <int MODE, bool SCALED>
void launch64(const Args64 &a, bool dir, cudaStream_t s)
{
    const int per_block = kThreads64 * kTgt64;
    const unsigned blocks = (unsigned)((a.n + per_block - 1) / per_block);
    if (dir) sweep64_kernel<MODE, true, SCALED><<<blocks, kThreads64, 0, s>>>(a);
    else sweep64_kernel<MODE, false, SCALED><<<blocks, kThreads64, 0, s>>>(a);
}

template <bool SCALED>
void launch64_mode(const Args64 &a, int mode, bool dir, cudaStream_t s)
{
    if (mode == SWEEP_PAIR) launch64<SWEEP_PAIR, SCALED>(a, dir, s);
    else if (mode == SWEEP_A) launch64<SWEEP_A, SCALED>(a, dir, s);
    else launch64<SWEEP_AH, SCALED>(a, dir, s);
}

// posk[i] = (k x*, k y*, k z*, reg): the records of the scaled sweep.
__global__ void scale_records64_kernel(int64_t n, double k, const double4_32a *__restrict__ pos,
                                       double4_32a *__restrict__ posk)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double4_32a p = pos[i];
        posk[i] = make_double4_32a(k * p.x, k * p.y, k * p.z, p.w);
    }
}

}  // namespace

int sweep_f64(const SweepConst &c, const Rec64 &r, int mode, const double *p_re, const double *p_im,
              const double *pt_re, const double *pt_im, double *q_re, double *q_im, double *qt_re,
              double *qt_im, double2 *scratch, cudaStream_t s, cudaEvent_t ev0,
              cudaEvent_t ev1)
{
    if (c.n <= 0) return HZ_OK;
    if (!(c.wave * c.extent <= kMaxPhase64)) {
        set_error("FP64 sweep: k * domain diagonal = %g exceeds the phase reduction's range (%g)",
                  c.wave * c.extent, kMaxPhase64);
        return HZ_ERR_ARG;
    }
    double4_32a *dens = reinterpret_cast<double4_32a *>(scratch);
    const bool useA = (mode & SWEEP_A) != 0, useH = (mode & SWEEP_AH) != 0;
    // Coordinates scaled by k (records built by scale_records64) save three
    // FP64 operations per pair; below k = 1 (and for records without a
    // scaled copy) the unscaled sweep runs.
    const bool scaled = r.posk != nullptr && c.wave >= 1.0;
    const double sg = (c.interior == 1) ? -1.0 : 1.0;
    const double k2 = scaled ? c.wave * c.wave : 1.0;
    Args64 a;
    a.n = c.n;
    a.wave = c.wave;
    a.tau = c.tau;
    a.tau2 = scaled ? (c.wave * c.tau) * (c.wave * c.tau) : c.tau * c.tau;
    a.tau2b = __builtin_bit_cast(long long, a.tau2);
    a.kscale = (float)((scaled ? 1.0 : c.wave) * (kPhaseTable / (2.0 * kPi64)));
    a.inv_scale = sg * (4.0 * kPi64) / k2;
    a.pos = scaled ? r.posk : r.pos;
    a.posu = r.pos;
    a.nrm = r.nrm;
    a.dens = dens;
    a.p_re = p_re; a.p_im = p_im; a.pt_re = pt_re; a.pt_im = pt_im;
    a.q_re = q_re; a.q_im = q_im; a.qt_re = qt_re; a.qt_im = qt_im;
    a.err = c.err;
    {
        int dev = 0, sms = 152;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        long long b = (c.n + 255) / 256;
        if (b > sms * 8) b = sms * 8;
        prep64_kernel<<<(unsigned)b, 256, 0, s>>>(c.n, r.nrm, useA ? p_re : nullptr, useA ? p_im : nullptr,
                                                  useH ? pt_re : nullptr, useH ? pt_im : nullptr,
                                                  sg * k2 / (4.0 * kPi64), dens);
        HZ_CHECK_LAUNCH();
    }
    if (ev0) HZ_CHECK_CUDA(record_timing_event(ev0, s));
    if (scaled) launch64_mode<true>(a, mode, c.dirichlet != 0, s);
    else launch64_mode<false>(a, mode, c.dirichlet != 0, s);
    HZ_CHECK_LAUNCH();
    if (ev1) HZ_CHECK_CUDA(record_timing_event(ev1, s));
    return HZ_OK;
}

int scale_records64(int64_t n, double k, const double4_32a *pos, double4_32a *posk, cudaStream_t s)
{
    if (n <= 0) return HZ_OK;
    long long b = (n + 255) / 256;
    if (b > 4096) b = 4096;
    scale_records64_kernel<<<(unsigned)b, 256, 0, s>>>(n, k, pos, posk);
    HZ_CHECK_LAUNCH();
    return HZ_OK;
}

HZ_DEFINE_WAIT_LIMIT_SETTER(set_wait_limit_f64)

}  // namespace hz
