// krylov.cu -- device-resident complex BiCG / BiCGSTAB with FP64 vectors
// and FP64, deterministically ordered inner products.
//
// BiCG follows the reference's CompBiCG / parallel_BiCGcomplex recurrences
// (BICGSTAB.c:104-308, large3Dexample2.c:3131-3433) with <a,b> = sum a conj(b):
//   x0 = 0, r = p = b, rt = pt = conj(b);
//   q = A p, qt = A^H pt;  alpha = <r,rt>/<q,pt>;
//   x += alpha p;  r -= alpha q;  rt -= conj(alpha) qt;
//   beta = <r,rt>_new/<r,rt>_old;  p = r + beta p;  pt = rt + conj(beta) pt;
//   stop at ||r||/||b|| < tol, NaN, or |change of ||r||/||b||| < 1e-3 tol.
// The two products of an iteration come from one fused pair sweep.
// BiCGSTAB is the standard complex form (two A products per iteration).
// Scalars stay on the device; the host reads one residual per iteration.
// The per-iteration launch sequence is captured once into a CUDA graph.
#include "hz_internal.cuh"
#include "krylov.cuh"

#include <cmath>
#include <chrono>

namespace hz {
namespace {

constexpr int kDotBlocks = 256;   // fixed: the partial-sum order is deterministic
constexpr int kDotThreads = 256;
constexpr int kMaxDots = 4;

// Block-reduce up to kMaxDots doubles; thread 0 writes partial[blockIdx][d].
template <int ND>
__device__ void block_reduce_store(double (&v)[ND], double *partial)
{
    __shared__ double sh[kDotThreads / 32][kMaxDots];
#pragma unroll
    for (int d = 0; d < ND; d++) {
        double x = v[d];
        for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
        if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5][d] = x;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
#pragma unroll
        for (int d = 0; d < ND; d++) {
            double s = 0.0;
            for (int w = 0; w < kDotThreads / 32; w++) s += sh[w][d];
            partial[blockIdx.x * kMaxDots + d] = s;
        }
    }
}

__device__ void sum_partials(const double *partial, int nd, double *out)
{
    for (int d = 0; d < nd; d++) {
        double s = 0.0;
        for (int b = 0; b < kDotBlocks; b++) s += partial[b * kMaxDots + d];
        out[d] = s;
    }
}

// <a, b> = sum a conj(b): (sum ar br + ai bi, sum ai br - ar bi); optionally
// also ||a||^2.
__global__ void __launch_bounds__(kDotThreads) cdot_kernel(int64_t n, const double *__restrict__ ar,
                                                           const double *__restrict__ ai,
                                                           const double *__restrict__ br,
                                                           const double *__restrict__ bi, double *partial)
{
    double v[3] = {0.0, 0.0, 0.0};
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double a0 = ar[i], a1 = ai[i], b0 = br[i], b1 = bi[i];
        v[0] += a0 * b0 + a1 * b1;
        v[1] += a1 * b0 - a0 * b1;
        v[2] += a0 * a0 + a1 * a1;
    }
    block_reduce_store<3>(v, partial);
}

// ----------------------------------------------------------------- BiCG
__global__ void bicg_init_kernel(int64_t n, const double *__restrict__ b_re, const double *__restrict__ b_im,
                                 double *x_re, double *x_im, double *r_re, double *r_im, double *rt_re,
                                 double *rt_im, double *p_re, double *p_im, double *pt_re, double *pt_im)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double br = b_re[i], bi = b_im[i];
        x_re[i] = 0.0;
        x_im[i] = 0.0;
        r_re[i] = br;
        r_im[i] = bi;
        p_re[i] = br;
        p_im[i] = bi;
        rt_re[i] = br;
        rt_im[i] = (-1.0) * bi;
        pt_re[i] = br;
        pt_im[i] = (-1.0) * bi;
    }
}

// after init: <r, rt> and ||b||
__global__ void bicg_start_kernel(const double *partial, KrylovScalars *sc)
{
    double s[3];
    sum_partials(partial, 3, s);
    sc->rho_re = s[0];
    sc->rho_im = s[1];
    sc->normb = sqrt(s[2]);
    sc->err = 1.0;
    sc->preerr = 1.0;
    sc->status = (s[2] > 0.0) ? 0 : 1;
}

// alpha = <r,rt> / <q,pt>
__global__ void bicg_alpha_kernel(const double *partial, KrylovScalars *sc)
{
    double s[3];
    sum_partials(partial, 3, s);
    const double ca = sc->rho_re, cb = sc->rho_im, cc = s[0], cd = s[1];
    const double num = ca * cc + cb * cd, numi = cb * cc - ca * cd, den = cc * cc + cd * cd;
    sc->alpha_re = num / den;
    sc->alpha_im = numi / den;
    if (den == 0.0) sc->status = 2;
}

__global__ void __launch_bounds__(kDotThreads) bicg_update_kernel(
    int64_t n, const KrylovScalars *__restrict__ sc, double *x_re, double *x_im, double *r_re, double *r_im,
    double *rt_re, double *rt_im, const double *__restrict__ p_re, const double *__restrict__ p_im,
    const double *__restrict__ q_re, const double *__restrict__ q_im, const double *__restrict__ qt_re,
    const double *__restrict__ qt_im, double *partial)
{
    const double al = sc->alpha_re, ali = sc->alpha_im;
    double v[3] = {0.0, 0.0, 0.0};
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x) {
        const double pr = p_re[j], pi = p_im[j], qr = q_re[j], qi = q_im[j], tr = qt_re[j], ti = qt_im[j];
        x_re[j] = x_re[j] + al * pr - ali * pi;
        x_im[j] = x_im[j] + ali * pr + al * pi;
        const double rr = r_re[j] - al * qr + ali * qi;
        const double ri = r_im[j] - ali * qr - al * qi;
        const double sr = rt_re[j] - al * tr - ali * ti;
        const double si = rt_im[j] + ali * tr - al * ti;
        r_re[j] = rr;
        r_im[j] = ri;
        rt_re[j] = sr;
        rt_im[j] = si;
        v[0] += rr * sr + ri * si;
        v[1] += ri * sr - rr * si;
        v[2] += rr * rr + ri * ri;
    }
    block_reduce_store<3>(v, partial);
}

__global__ void bicg_beta_kernel(const double *partial, KrylovScalars *sc, double *host_err)
{
    double s[3];
    sum_partials(partial, 3, s);
    const double cc = sc->rho_re, cd = sc->rho_im, ca = s[0], cb = s[1];
    const double num = ca * cc + cb * cd, numi = cb * cc - ca * cd, den = cc * cc + cd * cd;
    sc->beta_re = num / den;
    sc->beta_im = numi / den;
    sc->rho_re = ca;
    sc->rho_im = cb;
    sc->preerr = sc->err;
    sc->err = sqrt(s[2]) / sc->normb;
    if (den == 0.0) sc->status = 2;
    host_err[0] = sc->err;
    host_err[1] = sc->preerr;
    host_err[2] = (double)sc->status;
}

__global__ void bicg_p_kernel(int64_t n, const KrylovScalars *__restrict__ sc, const double *__restrict__ r_re,
                              const double *__restrict__ r_im, const double *__restrict__ rt_re,
                              const double *__restrict__ rt_im, double *p_re, double *p_im, double *pt_re,
                              double *pt_im)
{
    const double be = sc->beta_re, bi = sc->beta_im;
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x) {
        const double po = p_re[j], poi = p_im[j], to = pt_re[j], toi = pt_im[j];
        p_re[j] = r_re[j] + be * po - bi * poi;
        p_im[j] = r_im[j] + bi * po + be * poi;
        pt_re[j] = rt_re[j] + be * to + bi * toi;
        pt_im[j] = rt_im[j] - bi * to + be * toi;
    }
}

// ------------------------------------------------------------- BiCGSTAB
// Vectors: x, r, rh (shadow = b), p, v, s, t.  rho = <r, rh>.
__global__ void stab_init_kernel(int64_t n, const double *__restrict__ b_re, const double *__restrict__ b_im,
                                 double *x_re, double *x_im, double *r_re, double *r_im, double *rh_re,
                                 double *rh_im, double *p_re, double *p_im, double *v_re, double *v_im)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        x_re[i] = x_im[i] = 0.0;
        r_re[i] = rh_re[i] = b_re[i];
        r_im[i] = rh_im[i] = b_im[i];
        p_re[i] = p_im[i] = 0.0;
        v_re[i] = v_im[i] = 0.0;
    }
}

__global__ void stab_start_kernel(const double *partial, KrylovScalars *sc)
{
    double s[3];
    sum_partials(partial, 3, s);
    sc->normb = sqrt(s[2]);
    sc->rho_re = 1.0;  // rho_0 = alpha = omega = 1
    sc->rho_im = 0.0;
    sc->alpha_re = 1.0;
    sc->alpha_im = 0.0;
    sc->omega_re = 1.0;
    sc->omega_im = 0.0;
    sc->err = 1.0;
    sc->preerr = 1.0;
    sc->status = (s[2] > 0.0) ? 0 : 1;
}

__device__ void cdiv(double ar, double ai, double br, double bi, double &cr, double &ci)
{
    const double den = br * br + bi * bi;
    cr = (ar * br + ai * bi) / den;
    ci = (ai * br - ar * bi) / den;
}

// rho_new = <r, rh>; beta = (rho_new/rho)(alpha/omega); p = r + beta (p - omega v)
__global__ void stab_beta_kernel(const double *partial, KrylovScalars *sc)
{
    double s[3];
    sum_partials(partial, 3, s);
    double q1r, q1i, q2r, q2i;
    cdiv(s[0], s[1], sc->rho_re, sc->rho_im, q1r, q1i);
    cdiv(sc->alpha_re, sc->alpha_im, sc->omega_re, sc->omega_im, q2r, q2i);
    sc->beta_re = q1r * q2r - q1i * q2i;
    sc->beta_im = q1r * q2i + q1i * q2r;
    if (s[0] == 0.0 && s[1] == 0.0) sc->status = 2;
    sc->rho_re = s[0];
    sc->rho_im = s[1];
}

__global__ void stab_p_kernel(int64_t n, const KrylovScalars *__restrict__ sc, const double *r_re,
                              const double *r_im, double *p_re, double *p_im, const double *v_re,
                              const double *v_im)
{
    const double br = sc->beta_re, bi = sc->beta_im, wr = sc->omega_re, wi = sc->omega_im;
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x) {
        const double tr = p_re[j] - (wr * v_re[j] - wi * v_im[j]);
        const double ti = p_im[j] - (wr * v_im[j] + wi * v_re[j]);
        p_re[j] = r_re[j] + br * tr - bi * ti;
        p_im[j] = r_im[j] + br * ti + bi * tr;
    }
}

// alpha = rho / <v, rh>
__global__ void stab_alpha_kernel(const double *partial, KrylovScalars *sc)
{
    double s[3];
    sum_partials(partial, 3, s);
    if (s[0] == 0.0 && s[1] == 0.0) sc->status = 2;
    cdiv(sc->rho_re, sc->rho_im, s[0], s[1], sc->alpha_re, sc->alpha_im);
}

// s = r - alpha v  (stored in r)
__global__ void stab_s_kernel(int64_t n, const KrylovScalars *__restrict__ sc, double *r_re, double *r_im,
                              const double *v_re, const double *v_im)
{
    const double ar = sc->alpha_re, ai = sc->alpha_im;
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x) {
        r_re[j] = r_re[j] - (ar * v_re[j] - ai * v_im[j]);
        r_im[j] = r_im[j] - (ar * v_im[j] + ai * v_re[j]);
    }
}

// omega = <s, t>/<t, t> from partials of cdot(s, t) (v[0], v[1]) and ||t||^2
// computed as cdot(t, t).
__global__ void stab_omega_kernel(const double *partial_st, const double *partial_tt, KrylovScalars *sc)
{
    double a[3], b[3];
    sum_partials(partial_st, 3, a);
    sum_partials(partial_tt, 3, b);
    // omega = t^H s / t^H t, and t^H s = sum conj(t) s = cdot(s, t)
    const double tt = b[2];
    sc->omega_re = a[0] / tt;
    sc->omega_im = a[1] / tt;
    if (tt == 0.0) sc->status = 2;
}

// x += alpha p + omega s; r = s - omega t; partial ||r||^2 and <r, rh>
__global__ void __launch_bounds__(kDotThreads) stab_update_kernel(
    int64_t n, const KrylovScalars *__restrict__ sc, double *x_re, double *x_im, double *r_re, double *r_im,
    const double *p_re, const double *p_im, const double *t_re, const double *t_im, const double *rh_re,
    const double *rh_im, double *partial)
{
    const double ar = sc->alpha_re, ai = sc->alpha_im, wr = sc->omega_re, wi = sc->omega_im;
    double v[3] = {0.0, 0.0, 0.0};
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x) {
        const double sr = r_re[j], si = r_im[j];
        x_re[j] += (ar * p_re[j] - ai * p_im[j]) + (wr * sr - wi * si);
        x_im[j] += (ar * p_im[j] + ai * p_re[j]) + (wr * si + wi * sr);
        const double nr = sr - (wr * t_re[j] - wi * t_im[j]);
        const double ni = si - (wr * t_im[j] + wi * t_re[j]);
        r_re[j] = nr;
        r_im[j] = ni;
        const double hr = rh_re[j], hi = rh_im[j];
        v[0] += nr * hr + ni * hi;
        v[1] += ni * hr - nr * hi;
        v[2] += nr * nr + ni * ni;
    }
    block_reduce_store<3>(v, partial);
}

__global__ void stab_err_kernel(const double *partial, KrylovScalars *sc, double *host_err)
{
    double s[3];
    sum_partials(partial, 3, s);
    sc->preerr = sc->err;
    sc->err = sqrt(s[2]) / sc->normb;
    host_err[0] = sc->err;
    host_err[1] = sc->preerr;
    host_err[2] = (double)sc->status;
}

// ------------------------------------------------------------ refinement
__global__ void axpy_scale_kernel(int64_t n, double a, const double *e_re, const double *e_im, double *x_re,
                                  double *x_im)
{
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x) {
        x_re[j] += a * e_re[j];
        x_im[j] += a * e_im[j];
    }
}

__global__ void residual_kernel(int64_t n, const double *b_re, const double *b_im, const double *q_re,
                                const double *q_im, double *r_re, double *r_im, double inv_scale_unused)
{
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x) {
        r_re[j] = b_re[j] - q_re[j];
        r_im[j] = b_im[j] - q_im[j];
    }
}

__global__ void scale_kernel(int64_t n, double a, const double *x_re, const double *x_im, double *y_re,
                             double *y_im)
{
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x) {
        y_re[j] = a * x_re[j];
        y_im[j] = a * x_im[j];
    }
}

__global__ void norm_kernel(const double *partial, double *out)
{
    double s[3];
    sum_partials(partial, 3, s);
    out[0] = sqrt(s[2]);
}

int vec_blocks(int64_t n)
{
    long long b = (n + 255) / 256;
    if (b > 1184) b = 1184;
    if (b < 1) b = 1;
    return (int)b;
}

}  // namespace

// ---------------------------------------------------------------- Krylov
Krylov::~Krylov()
{
    if (graph_exec) cudaGraphExecDestroy(graph_exec);
    if (host_err) cudaFreeHost(host_err);
}

int Krylov::reserve(int64_t n_)
{
    n = n_;
    const size_t vec = (size_t)n * sizeof(double);
    void *before = vecs.ptr;
    HZ_TRY(vecs.ensure(vec * 2 * kVecs));
    if (vecs.ptr != before) invalidate_graph();  // the graph holds the old vectors
    HZ_TRY(partial.ensure((size_t)kDotBlocks * kMaxDots * sizeof(double) * 2));
    HZ_TRY(scal.ensure(sizeof(KrylovScalars)));
    if (!host_err) HZ_CHECK_CUDA(cudaMallocHost(&host_err, 4 * sizeof(double)));
    return HZ_OK;
}

int Krylov::keep_best(cudaStream_t s)
{
    const size_t bytes = (size_t)n * sizeof(double);
    HZ_CHECK_CUDA(cudaMemcpyAsync(re(XB), re(X), bytes, cudaMemcpyDeviceToDevice, s));
    HZ_CHECK_CUDA(cudaMemcpyAsync(im(XB), im(X), bytes, cudaMemcpyDeviceToDevice, s));
    return HZ_OK;
}

double *Krylov::re(int v) { return vecs.as<double>() + (size_t)(2 * v) * n; }
double *Krylov::im(int v) { return vecs.as<double>() + (size_t)(2 * v + 1) * n; }

int Krylov::bicg_iteration(LinOp &A, cudaStream_t s)
{
    double *pp = partial.as<double>();
    KrylovScalars *sc = scal.as<KrylovScalars>();
    const int vb = vec_blocks(n);
    HZ_TRY(A.apply(SWEEP_PAIR, re(P), im(P), re(PT), im(PT), re(Q), im(Q), re(QT), im(QT), s));
    cdot_kernel<<<kDotBlocks, kDotThreads, 0, s>>>(n, re(Q), im(Q), re(PT), im(PT), pp);
    HZ_CHECK_LAUNCH();
    bicg_alpha_kernel<<<1, 1, 0, s>>>(pp, sc);
    HZ_CHECK_LAUNCH();
    bicg_update_kernel<<<kDotBlocks, kDotThreads, 0, s>>>(n, sc, re(X), im(X), re(R), im(R), re(RT), im(RT),
                                                          re(P), im(P), re(Q), im(Q), re(QT), im(QT), pp);
    HZ_CHECK_LAUNCH();
    bicg_beta_kernel<<<1, 1, 0, s>>>(pp, sc, host_err);
    HZ_CHECK_LAUNCH();
    bicg_p_kernel<<<vb, 256, 0, s>>>(n, sc, re(R), im(R), re(RT), im(RT), re(P), im(P), re(PT), im(PT));
    HZ_CHECK_LAUNCH();
    return HZ_OK;
}

int Krylov::stab_iteration(LinOp &A, cudaStream_t s)
{
    double *pp = partial.as<double>();
    double *pp2 = pp + kDotBlocks * kMaxDots;
    KrylovScalars *sc = scal.as<KrylovScalars>();
    const int vb = vec_blocks(n);
    // rho_new = <r, rh>, beta, p = r + beta (p - omega v)
    cdot_kernel<<<kDotBlocks, kDotThreads, 0, s>>>(n, re(R), im(R), re(RH), im(RH), pp);
    HZ_CHECK_LAUNCH();
    stab_beta_kernel<<<1, 1, 0, s>>>(pp, sc);
    HZ_CHECK_LAUNCH();
    stab_p_kernel<<<vb, 256, 0, s>>>(n, sc, re(R), im(R), re(P), im(P), re(V), im(V));
    HZ_CHECK_LAUNCH();
    HZ_TRY(A.apply(SWEEP_A, re(P), im(P), nullptr, nullptr, re(V), im(V), nullptr, nullptr, s));
    cdot_kernel<<<kDotBlocks, kDotThreads, 0, s>>>(n, re(V), im(V), re(RH), im(RH), pp);
    HZ_CHECK_LAUNCH();
    stab_alpha_kernel<<<1, 1, 0, s>>>(pp, sc);
    HZ_CHECK_LAUNCH();
    stab_s_kernel<<<vb, 256, 0, s>>>(n, sc, re(R), im(R), re(V), im(V));
    HZ_CHECK_LAUNCH();
    HZ_TRY(A.apply(SWEEP_A, re(R), im(R), nullptr, nullptr, re(Q), im(Q), nullptr, nullptr, s));
    cdot_kernel<<<kDotBlocks, kDotThreads, 0, s>>>(n, re(R), im(R), re(Q), im(Q), pp);
    HZ_CHECK_LAUNCH();
    cdot_kernel<<<kDotBlocks, kDotThreads, 0, s>>>(n, re(Q), im(Q), re(Q), im(Q), pp2);
    HZ_CHECK_LAUNCH();
    stab_omega_kernel<<<1, 1, 0, s>>>(pp, pp2, sc);
    HZ_CHECK_LAUNCH();
    stab_update_kernel<<<kDotBlocks, kDotThreads, 0, s>>>(n, sc, re(X), im(X), re(R), im(R), re(P), im(P),
                                                          re(Q), im(Q), re(RH), im(RH), pp);
    HZ_CHECK_LAUNCH();
    stab_err_kernel<<<1, 1, 0, s>>>(pp, sc, host_err);
    HZ_CHECK_LAUNCH();
    return HZ_OK;
}

int Krylov::solve(LinOp &A, int method, const double *b_re, const double *b_im, double tol, int maxit,
                  bool stagnation, bool use_graph, cudaStream_t s, int &iters, double &resid, int &status, int stall)
{
    double *pp = partial.as<double>();
    KrylovScalars *sc = scal.as<KrylovScalars>();
    const int vb = vec_blocks(n);
    iters = 0;
    status = HZ_OK;
    history.clear();
    if (method == HZ_BICG) {
        bicg_init_kernel<<<vb, 256, 0, s>>>(n, b_re, b_im, re(X), im(X), re(R), im(R), re(RT), im(RT), re(P),
                                            im(P), re(PT), im(PT));
        HZ_CHECK_LAUNCH();
        cdot_kernel<<<kDotBlocks, kDotThreads, 0, s>>>(n, re(R), im(R), re(RT), im(RT), pp);
        HZ_CHECK_LAUNCH();
        bicg_start_kernel<<<1, 1, 0, s>>>(pp, sc);
        HZ_CHECK_LAUNCH();
    } else {
        stab_init_kernel<<<vb, 256, 0, s>>>(n, b_re, b_im, re(X), im(X), re(R), im(R), re(RH), im(RH), re(P),
                                            im(P), re(V), im(V));
        HZ_CHECK_LAUNCH();
        cdot_kernel<<<kDotBlocks, kDotThreads, 0, s>>>(n, re(R), im(R), re(R), im(R), pp);
        HZ_CHECK_LAUNCH();
        stab_start_kernel<<<1, 1, 0, s>>>(pp, sc);
        HZ_CHECK_LAUNCH();
    }
    KrylovScalars h{};
    HZ_CHECK_CUDA(cudaMemcpyAsync(&h, sc, sizeof(h), cudaMemcpyDeviceToHost, s));
    HZ_CHECK_CUDA(cudaStreamSynchronize(s));
    resid = 0.0;
    if (h.status == 1 || h.normb < 1e-15) {  // zero data: x = 0 (BICGSTAB.c:152-160)
        resid = 0.0;
        return HZ_OK;
    }
    // capture one iteration into a graph (re-captured when the operator or
    // stream changes; the graph is keyed by method and operator)
    cudaGraphExec_t exec = nullptr;
    if (use_graph) {
        if (graph_exec && graph_key != 0 && graph_key == A.key() && graph_key_method == method && graph_stream == s) {
            exec = graph_exec;
        } else {
            if (graph_exec) {
                cudaGraphExecDestroy(graph_exec);
                graph_exec = nullptr;
            }
            cudaGraph_t g = nullptr;
            cudaStream_t cs = s;
            bool captured = false;
            if (cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
                A.capture_begin();
                int rc = (method == HZ_BICG) ? bicg_iteration(A, cs) : stab_iteration(A, cs);
                cudaError_t e = cudaStreamEndCapture(cs, &g);
                A.capture_end();
                if (rc == HZ_OK && e == cudaSuccess && g) {
                    if (cudaGraphInstantiate(&graph_exec, g, 0) == cudaSuccess) captured = true;
                }
                if (g) cudaGraphDestroy(g);
            }
            cudaGetLastError();
            if (captured) {
                graph_key = A.key();
                graph_key_method = method;
                graph_stream = s;
                exec = graph_exec;
            } else {
                graph_exec = nullptr;
            }
        }
    }
    double err = 1.0, best = 1e300;
    int best_it = 0;
    for (int it = 1; it <= maxit; it++) {
        if (exec) {
            HZ_CHECK_CUDA(cudaGraphLaunch(exec, s));
            note_launch(method == HZ_BICG ? 7 : 14);
        } else {
            HZ_TRY(method == HZ_BICG ? bicg_iteration(A, s) : stab_iteration(A, s));
        }
        HZ_CHECK_CUDA(cudaStreamSynchronize(s));
        A.iteration_done(exec != nullptr);
        iters = it;
        const double preerr = host_err[1];
        err = host_err[0];
        history.push_back(err);
        const int st = (int)host_err[2];
        if (err < tol) break;
        if (err != err) {
            status = HZ_ERR_NONFINITE;
            break;
        }
        if (st == 2) {
            status = HZ_ERR_BREAKDOWN;
            break;
        }
        if (stagnation && fabs(preerr - err) < 1e-3 * tol) break;
        if (err < best) {
            best = err;
            best_it = it;
            if (stall > 0) HZ_TRY(keep_best(s));
        } else if (stall > 0 && it - best_it >= (stall > best_it ? stall : best_it)) {
            break;  // no new minimum for max(stall, best_it) iterations
        }
    }
    resid = err;
    if (stall > 0 && best < 1e300 && !(err <= best)) {
        // the last iterate is worse than the best one seen: return that
        const size_t bytes = (size_t)n * sizeof(double);
        HZ_CHECK_CUDA(cudaMemcpyAsync(re(X), re(XB), bytes, cudaMemcpyDeviceToDevice, s));
        HZ_CHECK_CUDA(cudaMemcpyAsync(im(X), im(XB), bytes, cudaMemcpyDeviceToDevice, s));
        resid = best;
        if (status == HZ_ERR_NONFINITE) status = HZ_OK;
    }
    return HZ_OK;
}

// helpers used by the refinement driver
int vec_axpy(int64_t n, double a, const double *e_re, const double *e_im, double *x_re, double *x_im,
             cudaStream_t s)
{
    axpy_scale_kernel<<<vec_blocks(n), 256, 0, s>>>(n, a, e_re, e_im, x_re, x_im);
    HZ_CHECK_LAUNCH();
    return HZ_OK;
}

int vec_sub(int64_t n, const double *b_re, const double *b_im, const double *q_re, const double *q_im,
            double *r_re, double *r_im, cudaStream_t s)
{
    residual_kernel<<<vec_blocks(n), 256, 0, s>>>(n, b_re, b_im, q_re, q_im, r_re, r_im, 0.0);
    HZ_CHECK_LAUNCH();
    return HZ_OK;
}

int vec_scale(int64_t n, double a, const double *x_re, const double *x_im, double *y_re, double *y_im,
              cudaStream_t s)
{
    scale_kernel<<<vec_blocks(n), 256, 0, s>>>(n, a, x_re, x_im, y_re, y_im);
    HZ_CHECK_LAUNCH();
    return HZ_OK;
}

int vec_norm(int64_t n, const double *x_re, const double *x_im, double *dev_partial, double *dev_out,
             double &host_out, cudaStream_t s)
{
    cdot_kernel<<<kDotBlocks, kDotThreads, 0, s>>>(n, x_re, x_im, x_re, x_im, dev_partial);
    HZ_CHECK_LAUNCH();
    norm_kernel<<<1, 1, 0, s>>>(dev_partial, dev_out);
    HZ_CHECK_LAUNCH();
    HZ_CHECK_CUDA(cudaMemcpyAsync(&host_out, dev_out, sizeof(double), cudaMemcpyDeviceToHost, s));
    HZ_CHECK_CUDA(cudaStreamSynchronize(s));
    return HZ_OK;
}

size_t vec_partial_bytes() { return (size_t)kDotBlocks * kMaxDots * sizeof(double) + 64; }

}  // namespace hz
