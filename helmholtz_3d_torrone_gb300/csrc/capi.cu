// capi.cu -- the extern "C" boundary (include/helmholtz_gb300.h).
#include "hz_internal.cuh"
#include "krylov.cuh"
#include "krylov_multi.cuh"

#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <new>
#include <vector>

namespace hz {

static thread_local char g_err[1024] = "";
static std::atomic<long long> g_launches{0};

void set_error(const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
}

void note_launch(int count) { g_launches.fetch_add(count, std::memory_order_relaxed); }

int DevBuf::ensure(size_t nbytes)
{
    if (nbytes <= bytes && ptr) return HZ_OK;
    release();
    if (nbytes == 0) nbytes = 16;
    cudaError_t e = cudaMalloc(&ptr, nbytes);
    if (e != cudaSuccess) {
        ptr = nullptr;
        bytes = 0;
        set_error("cudaMalloc(%zu bytes): %s", nbytes, cudaGetErrorString(e));
        cudaGetLastError();
        return HZ_ERR_CUDA;
    }
    bytes = nbytes;
    return HZ_OK;
}

void DevBuf::release()
{
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    bytes = 0;
}

// evaluate.cu
int launch_eval(int64_t n, const double4_32a *pos, const double4_32a *nrm, const double *s_re, const double *s_im,
                int64_t m, const double *rx, double wave, double tau, int interior, int layer, double *u_re,
                double *u_im, cudaStream_t s);
int launch_rhs(int64_t n, const double4_32a *pos, const double4_32a *nrm, const double *src, double wave, int kind,
               double *b_re, double *b_im, cudaStream_t s);
int launch_eval_adjoint(int64_t n, const double4_32a *pos, const double4_32a *nrm, int64_t m, const double *rx,
                        const double *r_re, const double *r_im, double wave, double tau, int interior, int layer,
                        double *s_re, double *s_im, cudaStream_t s);
int launch_eval_dk(int64_t n, const double4_32a *pos, const double4_32a *nrm, const double *s_re,
                   const double *s_im, int64_t m, const double *rx, double wave, double tau, int interior, int layer,
                   double *u_re, double *u_im, cudaStream_t s);
int launch_sweep_dk(int64_t n, const double4_32a *pos, const double4_32a *nrm, const double *dreg,
                    const double *s_re, const double *s_im, double wave, double tau, int interior, int dirichlet,
                    double *q_re, double *q_im, cudaStream_t s);
int launch_slice(int axis, double c, int n2, double lo, double h2, double mask, int N, double H, double int_l,
                 const double *d, double *rx, unsigned char *keep, cudaStream_t s);
int launch_mask(int64_t m, const unsigned char *keep, double *u_re, double *u_im, cudaStream_t s);
int launch_plane_waves(int64_t n, const double4_32a *pos, const double4_32a *nrm, int ndir, const double *dirs,
                       double wave, int kind, double *b_re, double *b_im, cudaStream_t s);
size_t dense_partial_elems(int64_t n);
int launch_dense(int64_t n, const double *are, const double *aim, const double *p_re, const double *p_im,
                 const double *pt_re, const double *pt_im, double *q_re, double *q_im, double *qt_re,
                 double *qt_im, double *part_re, double *part_im, cudaStream_t s);

SweepConst sweep_const(const hz_operator *op)
{
    SweepConst c;
    c.n = op->n;
    c.wave = op->p.wave;
    c.tau = op->tau;
    c.dirichlet = op->p.dirichlet;
    c.interior = op->p.interior;
    c.err = op->err.as<unsigned>();
    c.phase_split = op->phase_mode == HZ_PHASE_SPLIT;
    c.extent = 1.7320508075688772 * (op->p.int_u - op->p.int_l);
    return c;
}

Rec64 rec64(hz_operator *op)
{
    Rec64 r;
    r.pos = op->pos64.as<double4_32a>();
    r.nrm = op->nrm64.as<double4_32a>();
    r.posk = op->posk64.ptr ? op->posk64.as<double4_32a>() : nullptr;
    return r;
}

int check_device_error(hz_operator *op, const char *where)
{
    unsigned e = 0;
    HZ_CHECK_CUDA(cudaMemcpyAsync(&e, op->err.ptr, sizeof(unsigned), cudaMemcpyDeviceToHost, op->stream));
    HZ_CHECK_CUDA(cudaStreamSynchronize(op->stream));
    if (e & DEV_ERR_WAIT) {
        set_error("%s: a bounded device wait gave up (error word 0x%x)", where, e);
        return HZ_ERR_DEVICE_WAIT;
    }
    if (e & DEV_ERR_GRID) {
        set_error("%s: a projected point or its interpolation cell lies outside the grid", where);
        return HZ_ERR_GRID;
    }
    if (e & DEV_ERR_NONFINITE) {
        set_error("%s: non-finite value", where);
        return HZ_ERR_NONFINITE;
    }
    return HZ_OK;
}

// Matrix-free operator over the tube (FP64 or FP32 sweep).
struct MatrixFreeOp final : LinOp {
    hz_operator *op;
    int precision;
    MatrixFreeOp(hz_operator *o, int prec) : op(o), precision(prec) {}
    int apply(int mode, const double *p_re, const double *p_im, const double *pt_re, const double *pt_im,
              double *q_re, double *q_im, double *qt_re, double *qt_im, cudaStream_t s) override
    {
        const SweepConst c = sweep_const(op);
        const int slot = op->timer.slot();
        cudaEvent_t e0 = slot >= 0 ? op->timer.start[slot] : nullptr;
        cudaEvent_t e1 = slot >= 0 ? op->timer.stop[slot] : nullptr;
        if (op->combo) {
            if (precision != HZ_PREC_F64)
                return sweep_combo32(c, op->r32, op->pos64.as<double4_32a>(), op->combo_opts.wavenum,
                                     op->combo_opts.eta, mode, p_re, p_im, pt_re, pt_im, q_re, q_im, qt_re, qt_im,
                                     op->dens32.as<float4>(), s, e0, e1);
            return sweep_combo64(op->n, op->p.wave, op->combo_opts.wavenum, op->combo_opts.eta, op->tau,
                                 op->pos64.as<double4_32a>(), op->nrm64.as<double4_32a>(), op->adist.as<double>(),
                                 mode, p_re, p_im, pt_re, pt_im, q_re, q_im, qt_re, qt_im, s, e0, e1);
        }
        if (precision == HZ_PREC_F64)
            return sweep_f64(c, rec64(op), mode, p_re, p_im, pt_re, pt_im, q_re, q_im, qt_re, qt_im,
                             op->scratch.as<double2>(), s, e0, e1);
        const int cfg = (mode == SWEEP_PAIR || op->sweep_cfg_a < 0) ? op->sweep_cfg : op->sweep_cfg_a;
        return sweep_f32(c, op->r32, op->pos64.as<double4_32a>(), mode, p_re, p_im, pt_re, pt_im, q_re, q_im, qt_re,
                         qt_im, op->dens32.as<float4>(), s, e0, e1, cfg);
    }
    void capture_begin() override { op->timer.next = 0; }
    void capture_end() override
    {
        op->timer.graph_slots = op->timer.next;
        op->timer.next = 0;
    }
    void iteration_done(bool graph) override
    {
        if (graph) {
            op->timer.harvest(op->timer.graph_slots);
        } else {
            op->timer.harvest(op->timer.next);
            op->timer.next = 0;
        }
    }
    uint64_t key() const override
    {
        return ((uint64_t)(uintptr_t)op << 8) ^ (uint64_t)(precision * 16 + op->sweep_cfg) ^
               ((uint64_t)op->phase_mode << 6) ^ ((uint64_t)(op->sweep_cfg_a + 1) << 32) ^ 1ull;
    }
};

int SweepTimer::slot()
{
    if (!on || next >= kSlots) return -1;
    return next++;
}

void SweepTimer::harvest(int count)
{
    for (int i = 0; i < count && i < kSlots; i++) {
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, start[i], stop[i]) == cudaSuccess) {
            total_ms += ms;
            launches++;
        } else {
            cudaGetLastError();
        }
    }
}

struct DenseOp final : LinOp {
    int64_t n;
    const double *are, *aim;
    double *part_re, *part_im;
    int apply(int mode, const double *p_re, const double *p_im, const double *pt_re, const double *pt_im,
              double *q_re, double *q_im, double *qt_re, double *qt_im, cudaStream_t s) override
    {
        return launch_dense(n, are, aim, (mode & SWEEP_A) ? p_re : nullptr, p_im,
                            (mode & SWEEP_AH) ? pt_re : nullptr, pt_im, q_re, q_im, qt_re, qt_im, part_re, part_im,
                            s);
    }
    uint64_t key() const override { return ((uint64_t)(uintptr_t)are << 4) ^ 2ull; }
};

// Multi right-hand-side operator over the tube.
// Columns that stopped iterating are left out of the sweep: the others are
// packed into consecutive columns of `pack`, swept, and their products copied
// back (the stopped columns' products are not read).  `pairs` counts the
// kernel evaluations (one per pair and kernel pass, multi_rhs_passes).
struct MultiMatrixFreeOp final : MultiOp {
    hz_operator *op;
    int precision;
    DevBuf *scratch, *pack;
    std::vector<int> cols;  // empty: every column
    long long pairs = 0;
    MultiMatrixFreeOp(hz_operator *o, int prec, DevBuf *sc, DevBuf *pk)
        : op(o), precision(prec), scratch(sc), pack(pk) {}
    int apply(int R, const double *p_re, const double *p_im, double *q_re, double *q_im, cudaStream_t s) override
    {
        HZ_TRY(scratch->ensure(multi_rhs_scratch_bytes(op->n, op->r32.npad)));
        const int64_t n = op->n;
        const int m = cols.empty() ? R : (int)cols.size();
        pairs += (long long)n * n * multi_rhs_passes(precision, m);
        if (m == R)
            return sweep_multi(sweep_const(op), op->r32, rec64(op), precision, R, p_re, p_im, q_re, q_im,
                               scratch->ptr, s);
        const size_t col = (size_t)n * sizeof(double), mn = (size_t)m * n;
        HZ_TRY(pack->ensure(4 * mn * sizeof(double)));
        double *pr = pack->as<double>(), *pi = pr + mn, *qr = pr + 2 * mn, *qi = pr + 3 * mn;
        for (int j = 0; j < m; j++) {
            HZ_CHECK_CUDA(cudaMemcpyAsync(pr + j * n, p_re + cols[j] * n, col, cudaMemcpyDeviceToDevice, s));
            HZ_CHECK_CUDA(cudaMemcpyAsync(pi + j * n, p_im + cols[j] * n, col, cudaMemcpyDeviceToDevice, s));
        }
        HZ_TRY(sweep_multi(sweep_const(op), op->r32, rec64(op), precision, m, pr, pi, qr, qi, scratch->ptr, s));
        for (int j = 0; j < m; j++) {
            HZ_CHECK_CUDA(cudaMemcpyAsync(q_re + cols[j] * n, qr + j * n, col, cudaMemcpyDeviceToDevice, s));
            HZ_CHECK_CUDA(cudaMemcpyAsync(q_im + cols[j] * n, qi + j * n, col, cudaMemcpyDeviceToDevice, s));
        }
        return HZ_OK;
    }
    int restrict_to(const std::vector<int> &c, cudaStream_t s) override
    {
        (void)s;
        cols = c;
        return HZ_OK;
    }
};

// Copy count doubles in (host or device) to a device pointer.
int stage_in(double *dst, const double *src, size_t count, int where, cudaStream_t s)
{
    if (!src) {
        set_error("input pointer is NULL");
        return HZ_ERR_ARG;
    }
    HZ_CHECK_CUDA(cudaMemcpyAsync(dst, src, count * sizeof(double),
                                  where == HZ_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice, s));
    return HZ_OK;
}

int stage_out(double *dst, const double *src, size_t count, int where, cudaStream_t s)
{
    if (!dst) return HZ_OK;
    HZ_CHECK_CUDA(cudaMemcpyAsync(dst, src, count * sizeof(double),
                                  where == HZ_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice, s));
    return HZ_OK;
}

int where_ok(int where)
{
    if (where != HZ_HOST && where != HZ_DEVICE) {
        set_error("where must be HZ_HOST or HZ_DEVICE");
        return HZ_ERR_ARG;
    }
    return HZ_OK;
}

}  // namespace hz

using namespace hz;

// An inner FP32 solve stops after this many iterations without a new
// minimum residual: rounding the densities to FP32 bounds what it can reach.
constexpr int kInnerStall = 30;

// Per-operator solver state (kept out of the public struct layout).
struct hz_solver_state {
    Krylov outer, inner;
    KrylovMulti multi;
    DevBuf vec;  // b, x, r, q (re/im) for refinement
    DevBuf small;
    DevBuf mvec, mscratch, mpack;  // multi right-hand side staging, sweep scratch, packed columns
    DevBuf gwork, gsmall, gx;  // GMRES basis, Hessenberg partials, inner solution
    DevBuf mgwork, mgsmall, mgx;  // lockstep multi right-hand-side GMRES: basis, partials, inner solutions
    DevBuf xbest;              // refinement: best iterate so far (re/im)
    std::vector<double> history;  // per-iteration residuals of the last hz_solve (BiCG/BiCGSTAB)
};

namespace {

hz_solver_state *solver_of(hz_operator *op) { return op->solver; }

int check_params(const hz_params *p)
{
    if (!p) {
        set_error("params is NULL");
        return HZ_ERR_ARG;
    }
    if (p->N < 8 || p->N > 4096) {
        set_error("N = %d out of range [8, 4096]", p->N);
        return HZ_ERR_ARG;
    }
    if (!(p->int_u > p->int_l)) {
        set_error("int_u must exceed int_l");
        return HZ_ERR_ARG;
    }
    if (!(p->factor > 0) || !(p->tau_factor > 0) || !std::isfinite(p->wave)) {
        set_error("factor, tau_factor must be positive and wave finite");
        return HZ_ERR_ARG;
    }
    if (p->weno_order != 3 && p->weno_order != 5) {
        set_error("weno_order must be 3 or 5");
        return HZ_ERR_ARG;
    }
    return HZ_OK;
}

int need_built(hz_operator *op)
{
    if (!op) {
        set_error("operator is NULL");
        return HZ_ERR_ARG;
    }
    if (!op->built) {
        set_error("hz_build has not been run");
        return HZ_ERR_STATE;
    }
    return HZ_OK;
}

}  // namespace

// FP32 sweep records of the tube (or annulus) points in blocked order.
static int build_records32(hz_operator *op, double reg_scale)
{
    cudaStream_t s = op->stream;
    const int N = op->p.N;
    const int64_t n = op->n;
    const int64_t unit = (int64_t)kThreads32 * kTgt32;  // multiple of kTile32
    const int64_t npad = ((n + unit - 1) / unit) * unit;
    op->r32.npad = npad;
    if (npad > 0) {
        HZ_TRY(op->perm.ensure(npad * sizeof(int)));
        HZ_TRY(op->pos32.ensure(npad * sizeof(float4)));
        HZ_TRY(op->nrm32.ensure(npad * sizeof(float4)));
        HZ_TRY(op->tpos32.ensure(npad * sizeof(double4_32a)));
        const int64_t ntiles = npad / kTile32;
        op->r32.mwords = (ntiles + 31) / 32;
        HZ_TRY(op->origin32.ensure(ntiles * sizeof(double4_32a)));
        HZ_TRY(op->split32.ensure((2 * npad + 2 * ntiles) * sizeof(float4)));
        HZ_TRY(op->nearmask32.ensure(ntiles * op->r32.mwords * sizeof(uint32_t)));
        HZ_TRY(op->dens32.ensure(npad * sizeof(float4)));
        HZ_TRY(sweep_order(N, n, op->idx.as<int64_t>(), op->perm.as<int>(), npad, op->scratch, s));
    }
    op->r32.perm = op->perm.as<int>();
    op->r32.pos = op->pos32.as<float4>();
    op->r32.nrm = op->nrm32.as<float4>();
    op->r32.origin = op->origin32.as<double4_32a>();
    op->r32.tpos = op->tpos32.as<double4_32a>();
    {
        float4 *sp = op->split32.as<float4>();
        const int64_t ntiles = npad / kTile32;
        op->r32.thi = sp;
        op->r32.tlo = sp ? sp + npad : nullptr;
        op->r32.ohi = sp ? sp + 2 * npad : nullptr;
        op->r32.olo = sp ? sp + 2 * npad + ntiles : nullptr;
        op->r32.nearmask = op->nearmask32.as<uint32_t>();
    }
    if (npad > 0) {
        const size_t pb = sweep32_partial_bytes();
        HZ_TRY(op->partial32.ensure(pb));
        op->r32.partial = op->partial32.as<double4_32a>();
        op->r32.partial_bytes = pb;
    }
    if (npad > 0)
        HZ_TRY(build_rec32(op->r32, op->pos64.as<double4_32a>(), op->nrm64.as<double4_32a>(),
                           reg_scale, op->tau, s));
    return HZ_OK;
}

// hz_build for the Combo formulation: annulus selection and per-point rows
// of new_HelmholtzKernelCombo (dense.cu), packed into the operator's arrays.
static int build_combo(hz_operator *op, int64_t *n_out)
{
    cudaStream_t s = op->stream;
    int64_t n = 0;
    HZ_TRY(dense_points_device(HZ_DENSE_COMBO, op->p, op->combo_opts, op->d.as<double>(), op->gx.as<double>(),
                               op->gy.as<double>(), op->gz.as<double>(), op->mc.as<double>(), op->gc.as<double>(),
                               op->idx, n, op->cpts, op->err.as<unsigned>(), s));
    op->n = n;
    const size_t nn = (size_t)(n > 0 ? n : 1);
    HZ_TRY(op->xs.ensure(3 * nn * sizeof(double)));
    HZ_TRY(op->nrm.ensure(3 * nn * sizeof(double)));
    for (DevBuf *b : {&op->delta, &op->jac, &op->reg, &op->w, &op->dreg, &op->adist})
        HZ_TRY(b->ensure(nn * sizeof(double)));
    HZ_TRY(op->pos64.ensure(nn * sizeof(double4_32a)));
    HZ_TRY(op->nrm64.ensure(nn * sizeof(double4_32a)));
    HZ_TRY(combo_pack(n, op->cpts.as<double>(), op->combo_opts.sine, op->xs.as<double>(), op->nrm.as<double>(),
                      op->delta.as<double>(), op->jac.as<double>(), op->reg.as<double>(), op->w.as<double>(),
                      op->adist.as<double>(), op->pos64.as<double4_32a>(), op->nrm64.as<double4_32a>(), s));
    HZ_CHECK_CUDA(cudaMemsetAsync(op->dreg.ptr, 0, nn * sizeof(double), s));
    HZ_TRY(check_device_error(op, "hz_build (Combo)"));
    // FP32 records as the classic operator's (reg scaled by 4 pi: the Combo
    // kernel's c4 = 1/(4 pi) is folded into the densities), |d| in nrm32.w
    HZ_TRY(build_records32(op, 4.0 * 3.14159265358979323846264338328));
    HZ_TRY(combo32_set_distances(op->r32, op->adist.as<double>(), s));
    HZ_TRY(op->scratch.ensure(nn * sizeof(double4_32a) + 256));
    HZ_TRY(op->io.ensure(nn * sizeof(double) * 8));
    HZ_CHECK_CUDA(cudaStreamSynchronize(s));
    op->built = true;
    hz_solver_state *st = solver_of(op);
    if (st) {
        st->outer.invalidate_graph();
        st->inner.invalidate_graph();
    }
    if (n_out) *n_out = n;
    return HZ_OK;
}

static int need_classic(hz_operator *op, const char *who)
{
    if (op && op->combo) {
        set_error("%s is not available for the Combo formulation", who);
        return HZ_ERR_STATE;
    }
    return HZ_OK;
}

extern "C" {

const char *hz_last_error(void) { return g_err; }

int hz_set_phase_mode(hz_operator *op, int mode)
{
    if (!op || (mode != HZ_PHASE_DIRECT && mode != HZ_PHASE_SPLIT)) {
        set_error("hz_set_phase_mode: need an operator and HZ_PHASE_DIRECT or HZ_PHASE_SPLIT");
        return HZ_ERR_ARG;
    }
    op->phase_mode = mode;
    return HZ_OK;
}

int hz_set_combo(hz_operator *op, const hz_dense_opts *o)
{
    if (!op) {
        set_error("operator is NULL");
        return HZ_ERR_ARG;
    }
    if (o && (!(o->epsilon > o->delta0) || !(o->delta0 >= 0) || (!o->poly && !o->sine) || (o->poly && o->sine))) {
        set_error("hz_set_combo: need 0 <= delta0 < epsilon and exactly one of poly / sine");
        return HZ_ERR_ARG;
    }
    op->combo = o ? 1 : 0;
    if (o) op->combo_opts = *o;
    op->built = false;
    return HZ_OK;
}

int64_t hz_kernel_launches(void) { return g_launches.load(); }

int hz_set_wait_limit(long long polls)
{
    if (polls < 0) polls = kWaitLimit;
    if (set_wait_limit_f32(polls) || set_wait_limit_combo32(polls) || set_wait_limit_f64(polls) ||
        set_wait_limit_multi(polls)) {
        set_error("hz_set_wait_limit: cudaMemcpyToSymbol failed");
        cudaGetLastError();
        return HZ_ERR_CUDA;
    }
    return HZ_OK;
}

void hz_params_default(hz_params *p, int N, double wave)
{
    p->N = N;
    p->int_l = -2.0;
    p->int_u = 2.0;
    p->wave = wave;
    p->factor = 2.0;
    p->tau_factor = 2.0;
    p->dirichlet = 0;
    p->interior = 0;
    p->weno_order = 5;
}

void hz_solve_opts_default(hz_solve_opts *o)
{
    o->method = HZ_BICG;
    o->precision = HZ_PREC_F64;
    o->tol = 1e-7;  // BICGSTAB.h:12 DEFAULTACC
    o->maxit = 2000;
    o->inner_tol = 1e-5;
    o->max_outer = 20;
    o->stagnation = 1;
    o->restart = 40;
}

int hz_create(const hz_params *p, hz_operator **out)
{
    HZ_TRY(check_params(p));
    if (!out) {
        set_error("out is NULL");
        return HZ_ERR_ARG;
    }
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0) {
        set_error("no CUDA device: %s", cudaGetErrorString(e));
        cudaGetLastError();
        return HZ_ERR_CUDA;
    }
    hz_operator *op = new (std::nothrow) hz_operator();
    if (!op) {
        set_error("out of host memory");
        return HZ_ERR_ARG;
    }
    op->p = *p;
    HZ_CHECK_CUDA(cudaGetDevice(&op->device));
    HZ_CHECK_CUDA(cudaStreamCreateWithFlags(&op->own_stream, cudaStreamNonBlocking));
    op->stream = op->own_stream;
    op->H = (p->int_u - p->int_l) / p->N;  // large3Dexample2.c:174
    op->eps = p->factor * op->H;           // :350
    op->tau = op->H * p->tau_factor;       // :4286
    int rc = op->err.ensure(64);
    if (rc == HZ_OK) rc = (cudaMemsetAsync(op->err.ptr, 0, 64, op->stream) == cudaSuccess) ? HZ_OK : HZ_ERR_CUDA;
    if (rc != HZ_OK) {
        delete op;
        return rc;
    }
    op->solver = new (std::nothrow) hz_solver_state();
    if (!op->solver) {
        delete op;
        set_error("out of host memory");
        return HZ_ERR_ARG;
    }
    *out = op;
    return HZ_OK;
}

void hz_destroy(hz_operator *op)
{
    if (!op) return;
    cudaSetDevice(op->device);
    if (op->stream) cudaStreamSynchronize(op->stream);
    delete op->solver;
    op->solver = nullptr;
    if (op->own_stream) cudaStreamDestroy(op->own_stream);
    for (int i = 0; i < SweepTimer::kSlots; i++) {
        if (op->timer.start[i]) cudaEventDestroy(op->timer.start[i]);
        if (op->timer.stop[i]) cudaEventDestroy(op->timer.stop[i]);
    }
    delete op;
}

int hz_set_stream(hz_operator *op, void *stream)
{
    if (!op) {
        set_error("operator is NULL");
        return HZ_ERR_ARG;
    }
    op->stream = stream ? static_cast<cudaStream_t>(stream) : op->own_stream;
    return HZ_OK;
}

void *hz_get_stream(hz_operator *op) { return op ? (void *)op->stream : nullptr; }

int hz_set_distance(hz_operator *op, const double *d, int where)
{
    if (!op) {
        set_error("operator is NULL");
        return HZ_ERR_ARG;
    }
    HZ_TRY(where_ok(where));
    HZ_CHECK_CUDA(cudaSetDevice(op->device));
    const size_t S = (size_t)op->p.N + 1, nodes = S * S * S;
    HZ_TRY(op->d.ensure(nodes * sizeof(double)));
    HZ_TRY(stage_in(op->d.as<double>(), d, nodes, where, op->stream));
    op->have_distance = true;
    op->built = false;
    return HZ_OK;
}

int hz_build(hz_operator *op, int64_t *n_out)
{
    if (!op) {
        set_error("operator is NULL");
        return HZ_ERR_ARG;
    }
    if (!op->have_distance) {
        set_error("hz_set_distance has not been called");
        return HZ_ERR_STATE;
    }
    HZ_CHECK_CUDA(cudaSetDevice(op->device));
    cudaStream_t s = op->stream;
    const int N = op->p.N;
    const size_t S = (size_t)N + 1, nodes = S * S * S;
    for (DevBuf *b : {&op->gx, &op->gy, &op->gz, &op->mc, &op->gc}) HZ_TRY(b->ensure(nodes * sizeof(double)));
    HZ_CHECK_CUDA(cudaMemsetAsync(op->err.ptr, 0, sizeof(unsigned), s));
    HZ_TRY(launch_grid_stencils(N, op->H, op->d.as<double>(), op->gx.as<double>(), op->gy.as<double>(),
                                op->gz.as<double>(), op->mc.as<double>(), op->gc.as<double>(), op->p.weno_order, s));
    int64_t n = 0;
    if (op->combo) return build_combo(op, n_out);
    HZ_TRY(tube_build(N, op->eps, op->d.as<double>(), op->idx, n, op->scratch, s));
    op->n = n;
    const size_t nn = (size_t)(n > 0 ? n : 1);
    HZ_TRY(op->xs.ensure(3 * nn * sizeof(double)));
    HZ_TRY(op->nrm.ensure(3 * nn * sizeof(double)));
    for (DevBuf *b : {&op->delta, &op->jac, &op->reg, &op->w, &op->dreg}) HZ_TRY(b->ensure(nn * sizeof(double)));
    HZ_TRY(op->pos64.ensure(nn * sizeof(double4_32a)));
    HZ_TRY(op->nrm64.ensure(nn * sizeof(double4_32a)));
    HZ_TRY(tube_init(op->p, op->d.as<double>(), op->gx.as<double>(), op->gy.as<double>(), op->gz.as<double>(),
                     op->mc.as<double>(), op->gc.as<double>(), n, op->idx.as<int64_t>(), op->xs.as<double>(),
                     op->nrm.as<double>(), op->delta.as<double>(), op->jac.as<double>(), op->reg.as<double>(),
                     op->w.as<double>(), op->pos64.as<double4_32a>(), op->nrm64.as<double4_32a>(), op->err.as<unsigned>(), s,
                     op->dreg.as<double>()));
    HZ_TRY(check_device_error(op, "hz_build"));
    if (op->p.wave >= 1.0) {
        HZ_TRY(op->posk64.ensure(nn * sizeof(double4_32a)));
        HZ_TRY(scale_records64(n, op->p.wave, op->pos64.as<double4_32a>(), op->posk64.as<double4_32a>(), s));
    } else {
        op->posk64.release();
    }
    HZ_TRY(build_records32(op, sweep32_reg_scale(op->p.interior)));
    // scratch for the FP64 sweep densities (double4_32a per point) and staging
    HZ_TRY(op->scratch.ensure(nn * sizeof(double4_32a) + 256));
    HZ_TRY(op->io.ensure(nn * sizeof(double) * 8));
    HZ_CHECK_CUDA(cudaStreamSynchronize(s));
    op->built = true;
    hz_solver_state *st = solver_of(op);
    if (st) {
        st->outer.invalidate_graph();
        st->inner.invalidate_graph();
    }
    if (n_out) *n_out = n;
    return HZ_OK;
}

int64_t hz_tube_size(const hz_operator *op) { return op ? op->n : -1; }

int hz_autotune(hz_operator *op, int *chosen, double *ms_per_sweep)
{
    HZ_TRY(need_classic(op, "hz_autotune"));
    HZ_TRY(need_built(op));
    HZ_CHECK_CUDA(cudaSetDevice(op->device));
    cudaStream_t s = op->stream;
    const size_t n = (size_t)op->n;
    if (n == 0) {
        if (chosen) *chosen = op->sweep_cfg;
        return HZ_OK;
    }
    // unit densities in the staging buffer (values do not change the timing)
    double *io = op->io.as<double>();
    HZ_CHECK_CUDA(cudaMemsetAsync(io, 0, 8 * n * sizeof(double), s));
    cudaEvent_t e0, e1;
    HZ_CHECK_CUDA(cudaEventCreate(&e0));
    HZ_CHECK_CUDA(cudaEventCreate(&e1));
    const SweepConst c = sweep_const(op);
    // the fused pass (BiCG) and the single-product pass (GMRES, BiCGSTAB,
    // the refinement's inner products) are timed and chosen separately
    int best = 0, best_a = 0;
    float best_ms = 1e30f, best_a_ms = 1e30f;
    int rc = HZ_OK;
    for (int mode : {SWEEP_PAIR, SWEEP_A}) {
        for (int cfg = 0; cfg < sweep32_num_configs() && rc == HZ_OK; cfg++) {
            float ms_min = 1e30f;
            for (int rep = 0; rep < 2 && rc == HZ_OK; rep++) {
                rc = sweep_f32(c, op->r32, op->pos64.as<double4_32a>(), mode, io, io + n, io + 2 * n, io + 3 * n,
                               io + 4 * n, io + 5 * n, io + 6 * n, io + 7 * n, op->dens32.as<float4>(), s, e0, e1,
                               cfg);
                if (rc == HZ_OK && cudaEventSynchronize(e1) == cudaSuccess) {
                    float ms = 0.f;
                    cudaEventElapsedTime(&ms, e0, e1);
                    if (ms < ms_min) ms_min = ms;
                }
            }
            if (mode == SWEEP_PAIR && ms_min < best_ms) {
                best_ms = ms_min;
                best = cfg;
            } else if (mode == SWEEP_A && ms_min < best_a_ms) {
                best_a_ms = ms_min;
                best_a = cfg;
            }
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc != HZ_OK) return rc;
    HZ_TRY(check_device_error(op, "hz_autotune"));
    if (best != op->sweep_cfg || best_a != op->sweep_cfg_a) {
        op->sweep_cfg = best;
        op->sweep_cfg_a = best_a;
        op->solver->outer.invalidate_graph();
        op->solver->inner.invalidate_graph();
    }
    if (chosen) *chosen = best;
    if (ms_per_sweep) *ms_per_sweep = best_ms;
    return HZ_OK;
}

int hz_set_sweep_config(hz_operator *op, int cfg)
{
    if (!op || cfg < 0 || cfg >= sweep32_num_configs()) {
        set_error("hz_set_sweep_config: config must be in [0, %d)", sweep32_num_configs());
        return HZ_ERR_ARG;
    }
    if (cfg != op->sweep_cfg || op->sweep_cfg_a != -1) {
        op->sweep_cfg = cfg;
        op->sweep_cfg_a = -1;
        op->solver->outer.invalidate_graph();
        op->solver->inner.invalidate_graph();
    }
    return HZ_OK;
}

int hz_sweep_timing(hz_operator *op, int enable, double *total_ms, int64_t *launches)
{
    if (!op) {
        set_error("operator is NULL");
        return HZ_ERR_ARG;
    }
    if (total_ms) *total_ms = op->timer.total_ms;
    if (launches) *launches = op->timer.launches;
    if (enable >= 0) {
        HZ_CHECK_CUDA(cudaSetDevice(op->device));
        if (enable && !op->timer.start[0]) {
            for (int i = 0; i < SweepTimer::kSlots; i++) {
                HZ_CHECK_CUDA(cudaEventCreate(&op->timer.start[i]));
                HZ_CHECK_CUDA(cudaEventCreate(&op->timer.stop[i]));
            }
        }
        if ((enable != 0) != op->timer.on) {
            // captured iteration graphs hold (or lack) the event nodes
            op->solver->outer.invalidate_graph();
            op->solver->inner.invalidate_graph();
        }
        op->timer.on = enable != 0;
        op->timer.total_ms = 0.0;
        op->timer.launches = 0;
        op->timer.next = 0;
    }
    return HZ_OK;
}

int hz_get_grids(hz_operator *op, double *gx, double *gy, double *gz, double *mcurv, double *gcurv, int where)
{
    HZ_TRY(need_built(op));
    HZ_TRY(where_ok(where));
    const size_t S = (size_t)op->p.N + 1, nodes = S * S * S;
    HZ_TRY(stage_out(gx, op->gx.as<double>(), nodes, where, op->stream));
    HZ_TRY(stage_out(gy, op->gy.as<double>(), nodes, where, op->stream));
    HZ_TRY(stage_out(gz, op->gz.as<double>(), nodes, where, op->stream));
    HZ_TRY(stage_out(mcurv, op->mc.as<double>(), nodes, where, op->stream));
    HZ_TRY(stage_out(gcurv, op->gc.as<double>(), nodes, where, op->stream));
    HZ_CHECK_CUDA(cudaStreamSynchronize(op->stream));
    return HZ_OK;
}

int hz_get_tube(hz_operator *op, int64_t *idx, double *xs, double *nrm, double *delta, double *jac, double *reg,
                double *w, int where)
{
    HZ_TRY(need_built(op));
    HZ_TRY(where_ok(where));
    const size_t n = (size_t)op->n;
    cudaStream_t s = op->stream;
    if (idx)
        HZ_CHECK_CUDA(cudaMemcpyAsync(idx, op->idx.ptr, n * sizeof(int64_t),
                                      where == HZ_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice, s));
    HZ_TRY(stage_out(xs, op->xs.as<double>(), 3 * n, where, s));
    HZ_TRY(stage_out(nrm, op->nrm.as<double>(), 3 * n, where, s));
    HZ_TRY(stage_out(delta, op->delta.as<double>(), n, where, s));
    HZ_TRY(stage_out(jac, op->jac.as<double>(), n, where, s));
    HZ_TRY(stage_out(reg, op->reg.as<double>(), n, where, s));
    HZ_TRY(stage_out(w, op->w.as<double>(), n, where, s));
    HZ_CHECK_CUDA(cudaStreamSynchronize(s));
    return HZ_OK;
}

static int matvec_common(hz_operator *op, int precision, int mode, const double *p_re, const double *p_im,
                         const double *pt_re, const double *pt_im, double *q_re, double *q_im, double *qt_re,
                         double *qt_im, int where)
{
    HZ_TRY(need_built(op));
    HZ_TRY(where_ok(where));
    if (precision < HZ_PREC_F64 || precision > HZ_PREC_F32_REFINED) {
        set_error("unknown precision %d", precision);
        return HZ_ERR_ARG;
    }
    HZ_CHECK_CUDA(cudaSetDevice(op->device));
    cudaStream_t s = op->stream;
    const size_t n = (size_t)op->n;
    if (n == 0) return HZ_OK;
    double *io = op->io.as<double>();
    const double *dp_re = p_re, *dp_im = p_im, *dpt_re = pt_re, *dpt_im = pt_im;
    double *dq_re = q_re, *dq_im = q_im, *dqt_re = qt_re, *dqt_im = qt_im;
    if (where == HZ_HOST) {
        if (mode & SWEEP_A) {
            HZ_TRY(stage_in(io + 0 * n, p_re, n, where, s));
            HZ_TRY(stage_in(io + 1 * n, p_im, n, where, s));
            dp_re = io;
            dp_im = io + n;
            dq_re = io + 4 * n;
            dq_im = io + 5 * n;
        }
        if (mode & SWEEP_AH) {
            HZ_TRY(stage_in(io + 2 * n, pt_re, n, where, s));
            HZ_TRY(stage_in(io + 3 * n, pt_im, n, where, s));
            dpt_re = io + 2 * n;
            dpt_im = io + 3 * n;
            dqt_re = io + 6 * n;
            dqt_im = io + 7 * n;
        }
    } else {
        if (((mode & SWEEP_A) && (!p_re || !p_im || !q_re || !q_im)) ||
            ((mode & SWEEP_AH) && (!pt_re || !pt_im || !qt_re || !qt_im))) {
            set_error("matvec: NULL vector");
            return HZ_ERR_ARG;
        }
    }
    HZ_CHECK_CUDA(cudaMemsetAsync(op->err.ptr, 0, sizeof(unsigned), s));
    MatrixFreeOp A(op, precision == HZ_PREC_F64 ? HZ_PREC_F64 : HZ_PREC_F32);
    HZ_TRY(A.apply(mode, dp_re, dp_im, dpt_re, dpt_im, dq_re, dq_im, dqt_re, dqt_im, s));
    if (where == HZ_HOST) {
        if (mode & SWEEP_A) {
            HZ_TRY(stage_out(q_re, dq_re, n, where, s));
            HZ_TRY(stage_out(q_im, dq_im, n, where, s));
        }
        if (mode & SWEEP_AH) {
            HZ_TRY(stage_out(qt_re, dqt_re, n, where, s));
            HZ_TRY(stage_out(qt_im, dqt_im, n, where, s));
        }
    }
    const int rc = check_device_error(op, "matvec");
    A.iteration_done(false);
    return rc;
}

int hz_matvec(hz_operator *op, int precision, int adjoint, const double *p_re, const double *p_im, double *q_re,
              double *q_im, int where)
{
    if (adjoint)
        return matvec_common(op, precision, SWEEP_AH, nullptr, nullptr, p_re, p_im, nullptr, nullptr, q_re, q_im,
                             where);
    return matvec_common(op, precision, SWEEP_A, p_re, p_im, nullptr, nullptr, q_re, q_im, nullptr, nullptr, where);
}

int hz_matvec_pair(hz_operator *op, int precision, const double *p_re, const double *p_im, const double *pt_re,
                   const double *pt_im, double *q_re, double *q_im, double *qt_re, double *qt_im, int where)
{
    return matvec_common(op, precision, SWEEP_PAIR, p_re, p_im, pt_re, pt_im, q_re, q_im, qt_re, qt_im, where);
}

int hz_matvec_multi(hz_operator *op, int precision, int nrhs, const double *p_re, const double *p_im,
                    double *q_re, double *q_im, int where)
{
    HZ_TRY(need_classic(op, "hz_matvec_multi"));
    HZ_TRY(need_built(op));
    HZ_TRY(where_ok(where));
    if (nrhs < 1 || precision < HZ_PREC_F64 || precision > HZ_PREC_F32_REFINED) {
        set_error("hz_matvec_multi: nrhs must be >= 1 and precision valid");
        return HZ_ERR_ARG;
    }
    HZ_CHECK_CUDA(cudaSetDevice(op->device));
    cudaStream_t s = op->stream;
    hz_solver_state *st = op->solver;
    const size_t n = (size_t)op->n, tot = n * (size_t)nrhs;
    if (n == 0) return HZ_OK;
    const double *dpr = p_re, *dpi = p_im;
    double *dqr = q_re, *dqi = q_im;
    if (where == HZ_HOST) {
        HZ_TRY(st->mvec.ensure(4 * tot * sizeof(double)));
        double *b = st->mvec.as<double>();
        HZ_TRY(stage_in(b, p_re, tot, where, s));
        HZ_TRY(stage_in(b + tot, p_im, tot, where, s));
        dpr = b;
        dpi = b + tot;
        dqr = b + 2 * tot;
        dqi = b + 3 * tot;
    }
    HZ_CHECK_CUDA(cudaMemsetAsync(op->err.ptr, 0, sizeof(unsigned), s));
    MultiMatrixFreeOp A(op, precision == HZ_PREC_F64 ? HZ_PREC_F64 : HZ_PREC_F32, &st->mscratch, &st->mpack);
    HZ_TRY(A.apply(nrhs, dpr, dpi, dqr, dqi, s));
    if (where == HZ_HOST) {
        HZ_TRY(stage_out(q_re, dqr, tot, where, s));
        HZ_TRY(stage_out(q_im, dqi, tot, where, s));
    }
    return check_device_error(op, "hz_matvec_multi");
}

int hz_solve_multi(hz_operator *op, const hz_solve_opts *opts_in, int nrhs, const double *b_re, const double *b_im,
                   double *x_re, double *x_im, int where, hz_solve_info *info, double *resid)
{
    HZ_TRY(need_classic(op, "hz_solve_multi"));
    HZ_TRY(need_built(op));
    HZ_TRY(where_ok(where));
    hz_solve_opts o;
    if (opts_in) o = *opts_in;
    else hz_solve_opts_default(&o);
    if (nrhs < 1 || !(o.tol > 0) || o.maxit < 1 || o.precision < HZ_PREC_F64 || o.precision > HZ_PREC_F32_REFINED ||
        (o.method == HZ_GMRES && (o.restart < 2 || o.restart > 127))) {
        set_error("hz_solve_multi: bad arguments");
        return HZ_ERR_ARG;
    }
    const bool gm = o.method == HZ_GMRES;
    HZ_CHECK_CUDA(cudaSetDevice(op->device));
    if (gm) {
        // the lockstep GMRES basis is (restart + 3) x nrhs x n complex
        // doubles: say so plainly when it cannot fit
        const size_t need = gmres_multi_work_bytes(op->n, nrhs, o.restart);
        size_t free_b = 0, total_b = 0;
        HZ_CHECK_CUDA(cudaMemGetInfo(&free_b, &total_b));
        const size_t have = op->solver->mgwork.bytes;
        if (need > have && need - have > free_b) {
            set_error("hz_solve_multi: the GMRES basis for %d columns and restart %d needs %.1f GB, %.1f GB free "
                      "(lower restart or solve fewer columns per call)",
                      nrhs, o.restart, need / 1e9, (free_b + have) / 1e9);
            return HZ_ERR_ARG;
        }
    }
    cudaStream_t s = op->stream;
    hz_solver_state *st = op->solver;
    const int64_t n = op->n;
    const size_t tot = (size_t)n * (size_t)nrhs;
    hz_solve_info inf{};
    auto t0 = std::chrono::steady_clock::now();
    std::vector<double> res(nrhs, 0.0);
    if (n == 0) {
        if (info) *info = inf;
        return HZ_OK;
    }
    // staging: b, x, r, q  ([R][n] each, re/im)
    HZ_TRY(st->mvec.ensure(8 * tot * sizeof(double)));
    double *B0 = st->mvec.as<double>(), *B1 = B0 + tot, *X0 = B0 + 2 * tot, *X1 = B0 + 3 * tot, *R0 = B0 + 4 * tot,
           *R1 = B0 + 5 * tot, *Q0 = B0 + 6 * tot, *Q1 = B0 + 7 * tot;
    HZ_TRY(stage_in(B0, b_re, tot, where, s));
    HZ_TRY(stage_in(B1, b_im, tot, where, s));
    HZ_CHECK_CUDA(cudaMemsetAsync(op->err.ptr, 0, sizeof(unsigned), s));
    HZ_TRY(st->multi.reserve(n, nrhs));
    int iters = 0, outer = 0;
    long long pairs = 0;
    if (o.precision != HZ_PREC_F32_REFINED) {
        MultiMatrixFreeOp A(op, o.precision, &st->mscratch, &st->mpack);
        if (gm) {
            HZ_TRY(gmres_multi_solve(A, n, nrhs, o.restart, B0, B1, X0, X1, o.tol, o.maxit, 0, st->mgwork, st->mgsmall,
                                     s, iters, res));
        } else {
            HZ_TRY(st->multi.solve(A, B0, B1, o.tol, o.maxit, o.stagnation != 0, s, iters, res));
            HZ_CHECK_CUDA(cudaMemcpyAsync(X0, st->multi.re(KrylovMulti::X), tot * sizeof(double),
                                          cudaMemcpyDeviceToDevice, s));
            HZ_CHECK_CUDA(cudaMemcpyAsync(X1, st->multi.im(KrylovMulti::X), tot * sizeof(double),
                                          cudaMemcpyDeviceToDevice, s));
        }
        pairs = A.pairs;
    } else {
        // FP64 iterative refinement of every column still above tol:
        // X += ||r_j|| A32^{-1} (r_j/||r_j||)
        MultiMatrixFreeOp A32(op, HZ_PREC_F32, &st->mscratch, &st->mpack),
            A64(op, HZ_PREC_F64, &st->mscratch, &st->mpack);
        HZ_TRY(st->small.ensure(vec_partial_bytes() + 64));
        double *part = st->small.as<double>();
        double *dout = part + (vec_partial_bytes() / sizeof(double));
        std::vector<double> normb(nrhs), nr(nrhs);
        for (int r = 0; r < nrhs; r++) HZ_TRY(vec_norm(n, B0 + r * n, B1 + r * n, part, dout, normb[r], s));
        HZ_CHECK_CUDA(cudaMemsetAsync(X0, 0, tot * sizeof(double), s));
        HZ_CHECK_CUDA(cudaMemsetAsync(X1, 0, tot * sizeof(double), s));
        HZ_CHECK_CUDA(cudaMemcpyAsync(R0, B0, tot * sizeof(double), cudaMemcpyDeviceToDevice, s));
        HZ_CHECK_CUDA(cudaMemcpyAsync(R1, B1, tot * sizeof(double), cudaMemcpyDeviceToDevice, s));
        nr = normb;
        for (int r = 0; r < nrhs; r++) res[r] = normb[r] > 0 ? 1.0 : 0.0;
        auto worst = [&]() {
            double w = 0;
            for (double v : res) w = v > w ? v : w;
            return w;
        };
        std::vector<int> open;
        while (worst() >= o.tol && outer < o.max_outer) {
            outer++;
            open.clear();
            for (int r = 0; r < nrhs; r++) {
                if (res[r] >= o.tol) {
                    open.push_back(r);
                    HZ_TRY(vec_scale(n, 1.0 / nr[r], R0 + r * n, R1 + r * n, Q0 + r * n, Q1 + r * n, s));
                } else {
                    // a zero right-hand side: the column does not iterate
                    HZ_CHECK_CUDA(cudaMemsetAsync(Q0 + r * n, 0, n * sizeof(double), s));
                    HZ_CHECK_CUDA(cudaMemsetAsync(Q1 + r * n, 0, n * sizeof(double), s));
                }
            }
            int it = 0;
            std::vector<double> ires;
            const double itol = refine_inner_tol(o, worst());
            const double *E0 = st->multi.re(KrylovMulti::X), *E1 = st->multi.im(KrylovMulti::X);
            if (gm) {
                HZ_TRY(st->mgx.ensure(2 * tot * sizeof(double)));
                double *G0 = st->mgx.as<double>(), *G1 = G0 + tot;
                HZ_TRY(gmres_multi_solve(A32, n, nrhs, o.restart, Q0, Q1, G0, G1, itol, o.maxit, kInnerStall,
                                         st->mgwork, st->mgsmall, s, it, ires));
                E0 = G0;
                E1 = G1;
            } else {
                HZ_TRY(st->multi.solve(A32, Q0, Q1, itol, o.maxit, o.stagnation != 0, s, it, ires, kInnerStall));
            }
            iters += it;
            for (int r : open) HZ_TRY(vec_axpy(n, nr[r], E0 + r * n, E1 + r * n, X0 + r * n, X1 + r * n, s));
            HZ_TRY(A64.restrict_to(open, s));
            HZ_TRY(A64.apply(nrhs, X0, X1, Q0, Q1, s));
            for (int r : open) {
                HZ_TRY(vec_sub(n, B0 + r * n, B1 + r * n, Q0 + r * n, Q1 + r * n, R0 + r * n, R1 + r * n, s));
                HZ_TRY(vec_norm(n, R0 + r * n, R1 + r * n, part, dout, nr[r], s));
                res[r] = normb[r] > 0 ? nr[r] / normb[r] : 0.0;
            }
            if (inf.steps < HZ_MAX_STEPS) {
                inf.step_iters[inf.steps] = it;
                inf.step_inner_tol[inf.steps] = itol;
                inf.step_resid[inf.steps] = worst();
                inf.steps++;
            }
        }
        pairs = A32.pairs + A64.pairs;
    }
    HZ_TRY(stage_out(x_re, X0, tot, where, s));
    HZ_TRY(stage_out(x_im, X1, tot, where, s));
    HZ_CHECK_CUDA(cudaStreamSynchronize(s));
    const int rc = check_device_error(op, "hz_solve_multi");
    double worst = 0;
    for (int r = 0; r < nrhs; r++) {
        worst = res[r] > worst ? res[r] : worst;
        if (resid) resid[r] = res[r];
    }
    inf.iterations = iters;
    inf.outer = outer;
    inf.resid = worst;
    inf.resid_f64 = (o.precision == HZ_PREC_F32) ? -1.0 : worst;
    inf.pair_evals = pairs;
    inf.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    inf.status = rc;
    inf.converged = worst < o.tol ? 1 : 0;
    if (info) *info = inf;
    return rc;
}

int hz_rhs_plane_waves(hz_operator *op, int ndir, const double *dirs, int kind, double *b_re, double *b_im,
                       int where)
{
    HZ_TRY(need_built(op));
    HZ_TRY(where_ok(where));
    if (ndir < 1 || !dirs || (kind != HZ_RHS_POINT_DIRICHLET && kind != HZ_RHS_POINT_NEUMANN)) {
        set_error("hz_rhs_plane_waves: bad arguments");
        return HZ_ERR_ARG;
    }
    cudaStream_t s = op->stream;
    const size_t n = (size_t)op->n, tot = n * (size_t)ndir;
    hz_solver_state *st = op->solver;
    DevBuf dd;
    HZ_TRY(dd.ensure(3 * (size_t)ndir * sizeof(double)));
    HZ_CHECK_CUDA(cudaMemcpyAsync(dd.ptr, dirs, 3 * (size_t)ndir * sizeof(double), cudaMemcpyHostToDevice, s));
    double *dre = b_re, *dim = b_im;
    if (where == HZ_HOST) {
        HZ_TRY(st->mvec.ensure(2 * tot * sizeof(double)));
        dre = st->mvec.as<double>();
        dim = dre + tot;
    }
    HZ_TRY(launch_plane_waves(op->n, op->pos64.as<double4_32a>(), op->nrm64.as<double4_32a>(), ndir, dd.as<double>(),
                              op->p.wave, kind, dre, dim, s));
    if (where == HZ_HOST) {
        HZ_TRY(stage_out(b_re, dre, tot, where, s));
        HZ_TRY(stage_out(b_im, dim, tot, where, s));
    }
    HZ_CHECK_CUDA(cudaStreamSynchronize(s));
    return HZ_OK;
}

// Solve A x = b (adjoint = false) or A^H x = b (adjoint = true) with the
// options o; b and x are device vectors (x must not alias the solver's
// workspace).  Fills inf; returns HZ_OK or an error, status in *status.
static int solve_device(hz_operator *op, const hz_solve_opts &o, bool adjoint, const double *b0, const double *b1,
                        double *x0, double *x1, hz_solve_info &inf, int &status)
{
    cudaStream_t s = op->stream;
    hz_solver_state *st = solver_of(op);
    const int64_t n = op->n;
    HZ_TRY(st->vec.ensure((size_t)n * sizeof(double) * 4));
    HZ_TRY(st->small.ensure(vec_partial_bytes() + 64));
    double *r0 = st->vec.as<double>(), *r1 = r0 + n, *q0 = r0 + 2 * n, *q1 = r0 + 3 * n;
    int iters = 0;
    status = HZ_OK;
    double resid = 0.0;
    {
        // a NaN or Inf in b would read as "no data" (x = 0) to the Krylov
        // start test; the reference exits on it (large3Dexample2.c:2641)
        double nb = 0.0;
        double *part = st->small.as<double>();
        HZ_TRY(vec_norm(n, b0, b1, part, part + (vec_partial_bytes() / sizeof(double)), nb, s));
        if (!std::isfinite(nb)) {
            HZ_CHECK_CUDA(cudaMemsetAsync(x0, 0, n * sizeof(double), s));
            HZ_CHECK_CUDA(cudaMemsetAsync(x1, 0, n * sizeof(double), s));
            status = HZ_ERR_NONFINITE;
            inf.converged = 0;
            return HZ_OK;
        }
    }
    st->history.clear();
    if (o.precision != HZ_PREC_F32_REFINED && o.method == HZ_GMRES) {
        MatrixFreeOp Af(op, o.precision);
        AdjointOp Aa(Af);
        LinOp &A = adjoint ? static_cast<LinOp &>(Aa) : static_cast<LinOp &>(Af);
        int products = 0;
        HZ_TRY(gmres_solve(A, n, o.restart, b0, b1, x0, x1, o.tol, o.maxit, 0, st->gwork, st->gsmall, s, iters,
                           resid, products));
        inf.iterations = iters;
        inf.resid = resid;
        inf.resid_f64 = (o.precision == HZ_PREC_F64) ? resid : -1.0;
        inf.pair_evals = (long long)products * n * n;
        inf.converged = resid < o.tol ? 1 : 0;
        return HZ_OK;
    }
    if (o.precision != HZ_PREC_F32_REFINED) {
        HZ_TRY(st->outer.reserve(n));
        MatrixFreeOp Af(op, o.precision);
        AdjointOp Aa(Af);
        LinOp &A = adjoint ? static_cast<LinOp &>(Aa) : static_cast<LinOp &>(Af);
        HZ_TRY(st->outer.solve(A, o.method, b0, b1, o.tol, o.maxit, o.stagnation != 0, true, s, iters, resid, status));
        st->history = st->outer.history;
        HZ_CHECK_CUDA(cudaMemcpyAsync(x0, st->outer.re(Krylov::X), n * sizeof(double), cudaMemcpyDeviceToDevice, s));
        HZ_CHECK_CUDA(cudaMemcpyAsync(x1, st->outer.im(Krylov::X), n * sizeof(double), cudaMemcpyDeviceToDevice, s));
        inf.iterations = iters;
        inf.resid = resid;
        inf.resid_f64 = (o.precision == HZ_PREC_F64) ? resid : -1.0;
        // two matrix products per iteration (A p and A^H pt, or two A products)
        inf.pair_evals = 2LL * iters * n * n;
        inf.converged = resid < o.tol ? 1 : 0;
        return HZ_OK;
    }
    // FP64 iterative refinement around FP32 inner solves.
    HZ_TRY(st->inner.reserve(n));
    st->history.clear();
    MatrixFreeOp A32f(op, HZ_PREC_F32), A64f(op, HZ_PREC_F64);
    AdjointOp A32a(A32f), A64a(A64f);
    LinOp &A32 = adjoint ? static_cast<LinOp &>(A32a) : static_cast<LinOp &>(A32f);
    LinOp &A64 = adjoint ? static_cast<LinOp &>(A64a) : static_cast<LinOp &>(A64f);
    double *part = st->small.as<double>();
    double *dout = part + (vec_partial_bytes() / sizeof(double));
    double normb = 0.0, nr = 0.0;
    HZ_TRY(vec_norm(n, b0, b1, part, dout, normb, s));
    HZ_CHECK_CUDA(cudaMemsetAsync(x0, 0, n * sizeof(double), s));
    HZ_CHECK_CUDA(cudaMemsetAsync(x1, 0, n * sizeof(double), s));
    HZ_CHECK_CUDA(cudaMemcpyAsync(r0, b0, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
    HZ_CHECK_CUDA(cudaMemcpyAsync(r1, b1, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
    nr = normb;
    double res = (normb > 0) ? 1.0 : 0.0;
    int outer = 0;
    long long products = 0;
    const bool gm = o.method == HZ_GMRES;
    HZ_TRY(st->gx.ensure((size_t)n * 2 * sizeof(double)));
    // The best iterate (lowest FP64 residual) and its residual are kept.  A
    // step that does not lower the residual goes back to them; the step is
    // then repeated once with GMRES, whose inner residual cannot grow (a
    // BiCG inner solve can stall on a rough residual), and a second failure
    // ends the refinement with the best iterate.
    HZ_TRY(st->xbest.ensure((size_t)n * 4 * sizeof(double)));
    double *xb0 = st->xbest.as<double>(), *xb1 = xb0 + n, *rb0 = xb0 + 2 * n, *rb1 = xb0 + 3 * n;
    const int restart = (o.restart >= 2 && o.restart <= 127) ? o.restart : 40;
    double best = res;
    bool stalled = false, retry = false;
    auto copy2 = [&](double *d0, double *d1, const double *s0, const double *s1) -> int {
        HZ_CHECK_CUDA(cudaMemcpyAsync(d0, s0, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
        HZ_CHECK_CUDA(cudaMemcpyAsync(d1, s1, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
        return HZ_OK;
    };
    HZ_TRY(copy2(xb0, xb1, x0, x1));
    HZ_TRY(copy2(rb0, rb1, r0, r1));
    while (normb > 0 && res >= o.tol && outer < o.max_outer) {
        outer++;
        // inner right-hand side r / ||r|| (into q)
        HZ_TRY(vec_scale(n, 1.0 / nr, r0, r1, q0, q1, s));
        int it = 0, ist = HZ_OK;
        double ires = 0.0;
        const double itol = refine_inner_tol(o, res);
        const double *e0, *e1;
        if (gm || retry) {
            int prods = 0;
            double *g0 = st->gx.as<double>(), *g1 = g0 + n;
            HZ_TRY(gmres_solve(A32, n, restart, q0, q1, g0, g1, itol, o.maxit, kInnerStall, st->gwork, st->gsmall, s,
                               it, ires, prods));
            products += prods;
            e0 = g0;
            e1 = g1;
        } else {
            HZ_TRY(st->inner.solve(A32, o.method, q0, q1, itol, o.maxit, o.stagnation != 0, true, s, it, ires, ist,
                                   kInnerStall));
            st->history.insert(st->history.end(), st->inner.history.begin(), st->inner.history.end());
            products += 2LL * it;
            e0 = st->inner.re(Krylov::X);
            e1 = st->inner.im(Krylov::X);
        }
        iters += it;
        if (ist != HZ_OK && ist != HZ_ERR_BREAKDOWN) {
            status = ist;
            break;
        }
        HZ_TRY(vec_axpy(n, nr, e0, e1, x0, x1, s));
        // r = b - A x with the FP64 sweep
        HZ_TRY(A64.apply(SWEEP_A, x0, x1, nullptr, nullptr, q0, q1, nullptr, nullptr, s));
        HZ_TRY(vec_sub(n, b0, b1, q0, q1, r0, r1, s));
        HZ_TRY(vec_norm(n, r0, r1, part, dout, nr, s));
        A64.iteration_done(false);
        res = nr / normb;
        if (inf.steps < HZ_MAX_STEPS) {
            inf.step_iters[inf.steps] = (gm || retry) ? -it : it;
            inf.step_inner_tol[inf.steps] = itol;
            inf.step_resid[inf.steps] = res;
            inf.steps++;
        }
        if (!(res < best)) {
            // no progress (or a non-finite residual): back to the best iterate
            HZ_TRY(copy2(x0, x1, xb0, xb1));
            HZ_TRY(copy2(r0, r1, rb0, rb1));
            res = best;
            nr = best * normb;
            if (!gm && !retry) {
                retry = true;
                continue;
            }
            stalled = true;
            if (ist == HZ_ERR_BREAKDOWN) status = HZ_ERR_BREAKDOWN;
            break;
        }
        best = res;
        retry = false;
        if (res >= o.tol && outer < o.max_outer) {
            HZ_TRY(copy2(xb0, xb1, x0, x1));
            HZ_TRY(copy2(rb0, rb1, r0, r1));
        }
    }
    inf.iterations = iters;
    inf.outer = outer;
    inf.resid = res;
    inf.resid_f64 = res;
    inf.converged = (!stalled && res < o.tol) ? 1 : 0;
    // inner products (two per BiCG iteration); one FP64 residual product per step
    inf.pair_evals = (products + outer) * (long long)n * n;
    return HZ_OK;
}

static int check_opts(const hz_solve_opts &o)
{
    if (o.method != HZ_BICG && o.method != HZ_BICGSTAB && o.method != HZ_GMRES) {
        set_error("unknown method %d", o.method);
        return HZ_ERR_ARG;
    }
    if (o.precision < HZ_PREC_F64 || o.precision > HZ_PREC_F32_REFINED || !(o.tol > 0) || o.maxit < 1 ||
        (o.method == HZ_GMRES && (o.restart < 2 || o.restart > 127))) {
        set_error("bad solve options");
        return HZ_ERR_ARG;
    }
    return HZ_OK;
}

int hz_solve(hz_operator *op, const hz_solve_opts *opts_in, const double *b_re, const double *b_im, double *x_re,
             double *x_im, int where, hz_solve_info *info)
{
    HZ_TRY(need_built(op));
    HZ_TRY(where_ok(where));
    hz_solve_opts o;
    if (opts_in) o = *opts_in;
    else hz_solve_opts_default(&o);
    HZ_TRY(check_opts(o));
    HZ_CHECK_CUDA(cudaSetDevice(op->device));
    cudaStream_t s = op->stream;
    const int64_t n = op->n;
    hz_solve_info inf{};
    auto t0 = std::chrono::steady_clock::now();
    if (n == 0) {
        if (info) *info = inf;
        return HZ_OK;
    }
    // b and x staging: the operator's io buffer (8 n doubles)
    double *io = op->io.as<double>();
    double *b0 = io, *b1 = io + n, *x0 = io + 2 * n, *x1 = io + 3 * n;
    HZ_TRY(stage_in(b0, b_re, n, where, s));
    HZ_TRY(stage_in(b1, b_im, n, where, s));
    HZ_CHECK_CUDA(cudaMemsetAsync(op->err.ptr, 0, sizeof(unsigned), s));
    int status = HZ_OK;
    HZ_TRY(solve_device(op, o, false, b0, b1, x0, x1, inf, status));
    HZ_TRY(stage_out(x_re, x0, n, where, s));
    HZ_TRY(stage_out(x_im, x1, n, where, s));
    HZ_CHECK_CUDA(cudaStreamSynchronize(s));
    int rc = check_device_error(op, "hz_solve");
    inf.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    inf.status = (rc != HZ_OK) ? rc : status;
    if (info) *info = inf;
    if (rc != HZ_OK) return rc;
    if (status != HZ_OK) {
        if (status == HZ_ERR_NONFINITE) set_error("hz_solve: non-finite value in the right-hand side or an iterate");
        else if (status == HZ_ERR_BREAKDOWN) set_error("hz_solve: Krylov breakdown (a zero denominator)");
        else set_error("hz_solve: solver stopped early (status %d)", status);
        return status;
    }
    return HZ_OK;
}

int hz_residual_history(hz_operator *op, double *out, int cap, int *count)
{
    if (!op || !count || cap < 0 || (cap > 0 && !out)) {
        set_error("hz_residual_history: bad arguments");
        return HZ_ERR_ARG;
    }
    const std::vector<double> &h = op->solver->history;
    const int m = (int)h.size();
    for (int i = 0; i < m && i < cap; i++) out[i] = h[i];
    *count = m;
    return HZ_OK;
}

int hz_misfit_gradient(hz_operator *op, const hz_solve_opts *opts_in, const double *b_re, const double *b_im,
                       int layer, int64_t m, const double *rx, const double *t_re, const double *t_im, double *J,
                       double *g_re, double *g_im, double *dJ_dk, double *dJ_dw, int where, hz_solve_info *info)
{
    HZ_TRY(need_classic(op, "hz_misfit_gradient"));
    HZ_TRY(need_built(op));
    HZ_TRY(where_ok(where));
    hz_solve_opts o;
    if (opts_in) o = *opts_in;
    else hz_solve_opts_default(&o);
    HZ_TRY(check_opts(o));
    if (m < 1 || !rx || !t_re || !t_im || (layer != HZ_SINGLE_LAYER && layer != HZ_DOUBLE_LAYER)) {
        set_error("hz_misfit_gradient: bad arguments");
        return HZ_ERR_ARG;
    }
    HZ_CHECK_CUDA(cudaSetDevice(op->device));
    cudaStream_t s = op->stream;
    const int64_t n = op->n;
    auto t0 = std::chrono::steady_clock::now();
    // device layout: b, sigma, lambda, s, dA sigma (re/im, n each); receivers
    // (3m), targets, u, r, dE sigma (re/im, m each)
    DevBuf buf;
    HZ_TRY(buf.ensure((10 * (size_t)n + 11 * (size_t)m) * sizeof(double)));
    double *b0 = buf.as<double>(), *b1 = b0 + n, *sg0 = b0 + 2 * n, *sg1 = b0 + 3 * n, *l0 = b0 + 4 * n,
           *l1 = b0 + 5 * n, *s0 = b0 + 6 * n, *s1 = b0 + 7 * n, *d0 = b0 + 8 * n, *d1 = b0 + 9 * n;
    double *R = b0 + 10 * n, *T0 = R + 3 * m, *T1 = T0 + m, *U0 = T1 + m, *U1 = U0 + m, *E0 = U1 + m, *E1 = E0 + m,
           *Q0 = E1 + m, *Q1 = Q0 + m;
    HZ_TRY(stage_in(b0, b_re, n, where, s));
    HZ_TRY(stage_in(b1, b_im, n, where, s));
    HZ_TRY(stage_in(R, rx, 3 * m, where, s));
    HZ_TRY(stage_in(T0, t_re, m, where, s));
    HZ_TRY(stage_in(T1, t_im, m, where, s));
    HZ_CHECK_CUDA(cudaMemsetAsync(op->err.ptr, 0, sizeof(unsigned), s));
    hz_solve_info fwd{}, adj{};
    int status = HZ_OK, status2 = HZ_OK;
    // forward: A sigma = b, u = E sigma, residual r = u - t
    HZ_TRY(solve_device(op, o, false, b0, b1, sg0, sg1, fwd, status));
    HZ_TRY(launch_eval(n, op->pos64.as<double4_32a>(), op->nrm64.as<double4_32a>(), sg0, sg1, m, R, op->p.wave, op->tau,
                       op->p.interior, layer, U0, U1, s));
    HZ_TRY(vec_sub(m, U0, U1, T0, T1, E0, E1, s));  // E := r
    // adjoint: A^H lambda = E^H r
    HZ_TRY(launch_eval_adjoint(n, op->pos64.as<double4_32a>(), op->nrm64.as<double4_32a>(), m, R, E0, E1, op->p.wave,
                               op->tau, op->p.interior, layer, s0, s1, s));
    HZ_TRY(solve_device(op, o, true, s0, s1, l0, l1, adj, status2));
    // k-derivatives: (dE/dk) sigma at the receivers, (dA/dk) sigma over the tube
    HZ_TRY(launch_eval_dk(n, op->pos64.as<double4_32a>(), op->nrm64.as<double4_32a>(), sg0, sg1, m, R, op->p.wave,
                          op->tau, op->p.interior, layer, Q0, Q1, s));
    HZ_TRY(launch_sweep_dk(n, op->pos64.as<double4_32a>(), op->nrm64.as<double4_32a>(), op->dreg.as<double>(), sg0,
                           sg1, op->p.wave, op->tau, op->p.interior, op->p.dirichlet, d0, d1, s));
    // host side of the small reductions
    std::vector<double> hr0(m), hr1(m), hq0(m), hq1(m);
    HZ_CHECK_CUDA(cudaMemcpyAsync(hr0.data(), E0, m * sizeof(double), cudaMemcpyDeviceToHost, s));
    HZ_CHECK_CUDA(cudaMemcpyAsync(hr1.data(), E1, m * sizeof(double), cudaMemcpyDeviceToHost, s));
    HZ_CHECK_CUDA(cudaMemcpyAsync(hq0.data(), Q0, m * sizeof(double), cudaMemcpyDeviceToHost, s));
    HZ_CHECK_CUDA(cudaMemcpyAsync(hq1.data(), Q1, m * sizeof(double), cudaMemcpyDeviceToHost, s));
    std::vector<double> hl0(n), hl1(n), hd0(n), hd1(n), hs0(n), hs1(n), hw(n);
    HZ_CHECK_CUDA(cudaMemcpyAsync(hl0.data(), l0, n * sizeof(double), cudaMemcpyDeviceToHost, s));
    HZ_CHECK_CUDA(cudaMemcpyAsync(hl1.data(), l1, n * sizeof(double), cudaMemcpyDeviceToHost, s));
    HZ_CHECK_CUDA(cudaMemcpyAsync(hd0.data(), d0, n * sizeof(double), cudaMemcpyDeviceToHost, s));
    HZ_CHECK_CUDA(cudaMemcpyAsync(hd1.data(), d1, n * sizeof(double), cudaMemcpyDeviceToHost, s));
    HZ_CHECK_CUDA(cudaMemcpyAsync(hs0.data(), sg0, n * sizeof(double), cudaMemcpyDeviceToHost, s));
    HZ_CHECK_CUDA(cudaMemcpyAsync(hs1.data(), sg1, n * sizeof(double), cudaMemcpyDeviceToHost, s));
    HZ_CHECK_CUDA(cudaMemcpyAsync(hw.data(), op->w.ptr, n * sizeof(double), cudaMemcpyDeviceToHost, s));
    HZ_CHECK_CUDA(cudaStreamSynchronize(s));
    // J = sum |r|^2;  dJ/dk = 2 Re(r^H (dE/dk) sigma) - 2 Re(lambda^H (dA/dk) sigma)
    double jv = 0.0, dk = 0.0;
    for (int64_t i = 0; i < m; i++) {
        jv += hr0[i] * hr0[i] + hr1[i] * hr1[i];
        dk += 2.0 * (hr0[i] * hq0[i] + hr1[i] * hq1[i]);
    }
    for (int64_t i = 0; i < n; i++) dk -= 2.0 * (hl0[i] * hd0[i] + hl1[i] * hd1[i]);
    if (J) *J = jv;
    if (dJ_dk) *dJ_dk = dk;
    // dJ/db = 2 lambda (gradient w.r.t. Re b and Im b)
    if (g_re || g_im) {
        HZ_TRY(vec_scale(n, 2.0, l0, l1, s0, s1, s));
        HZ_TRY(stage_out(g_re, s0, n, where, s));
        HZ_TRY(stage_out(g_im, s1, n, where, s));
    }
    // dJ/dw_s = Re(conj(lambda_s) sigma_s) / w_s  (A = K W + I/2, E = E' W)
    if (dJ_dw) {
        std::vector<double> gw(n);
        for (int64_t i = 0; i < n; i++)
            gw[i] = hw[i] != 0.0 ? (hl0[i] * hs0[i] + hl1[i] * hs1[i]) / hw[i] : 0.0;
        if (where == HZ_HOST) memcpy(dJ_dw, gw.data(), n * sizeof(double));
        else HZ_CHECK_CUDA(cudaMemcpyAsync(dJ_dw, gw.data(), n * sizeof(double), cudaMemcpyHostToDevice, s));
    }
    HZ_CHECK_CUDA(cudaStreamSynchronize(s));
    int rc = check_device_error(op, "hz_misfit_gradient");
    if (info) {
        hz_solve_info inf = fwd;
        inf.iterations = fwd.iterations + adj.iterations;
        inf.outer = fwd.outer + adj.outer;
        inf.resid = fwd.resid > adj.resid ? fwd.resid : adj.resid;
        inf.resid_f64 = fwd.resid_f64 > adj.resid_f64 ? fwd.resid_f64 : adj.resid_f64;
        inf.pair_evals = fwd.pair_evals + adj.pair_evals + n * n;
        inf.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        inf.status = rc != HZ_OK ? rc : (status != HZ_OK ? status : status2);
        inf.converged = (fwd.converged && adj.converged) ? 1 : 0;
        *info = inf;
    }
    if (rc != HZ_OK) return rc;
    if (status != HZ_OK || status2 != HZ_OK) {
        set_error("solver stopped early (status %d / %d)", status, status2);
        return status != HZ_OK ? status : status2;
    }
    return HZ_OK;
}

int hz_shape_gradient(hz_operator *op, const hz_solve_opts *opts_in, const double *src, int64_t m, const double *rx,
                      const double *t_re, const double *t_im, double *J, double *dJ_dphi, int where,
                      hz_solve_info *info)
{
    HZ_TRY(need_classic(op, "hz_shape_gradient"));
    HZ_TRY(need_built(op));
    HZ_TRY(where_ok(where));
    hz_solve_opts o;
    if (opts_in) o = *opts_in;
    else hz_solve_opts_default(&o);
    HZ_TRY(check_opts(o));
    if (!op->p.dirichlet || m < 1 || !src || !rx || !t_re || !t_im) {
        set_error("hz_shape_gradient: needs the Dirichlet formulation, receivers, targets and a source");
        return HZ_ERR_ARG;
    }
    HZ_CHECK_CUDA(cudaSetDevice(op->device));
    cudaStream_t s = op->stream;
    const int64_t n = op->n;
    const size_t S = (size_t)op->p.N + 1, nodes = S * S * S;
    auto t0 = std::chrono::steady_clock::now();
    DevBuf buf, work;
    HZ_TRY(buf.ensure((8 * (size_t)n + 9 * (size_t)m + nodes) * sizeof(double)));
    HZ_TRY(work.ensure(shape_gradient_work_bytes(n, op->p.N)));
    double *b0 = buf.as<double>(), *b1 = b0 + n, *sg0 = b0 + 2 * n, *sg1 = b0 + 3 * n, *l0 = b0 + 4 * n,
           *l1 = b0 + 5 * n, *e0 = b0 + 6 * n, *e1 = b0 + 7 * n;
    double *R = b0 + 8 * n, *T0 = R + 3 * m, *T1 = T0 + m, *U0 = T1 + m, *U1 = U0 + m, *E0 = U1 + m, *E1 = E0 + m;
    double *phib = E1 + m;
    HZ_TRY(stage_in(R, rx, 3 * m, where, s));
    HZ_TRY(stage_in(T0, t_re, m, where, s));
    HZ_TRY(stage_in(T1, t_im, m, where, s));
    HZ_CHECK_CUDA(cudaMemsetAsync(op->err.ptr, 0, sizeof(unsigned), s));
    HZ_TRY(launch_rhs(n, op->pos64.as<double4_32a>(), op->nrm64.as<double4_32a>(), src, op->p.wave,
                      HZ_RHS_POINT_DIRICHLET, b0, b1, s));
    hz_solve_info fwd{}, adj{};
    int status = HZ_OK, status2 = HZ_OK;
    HZ_TRY(solve_device(op, o, false, b0, b1, sg0, sg1, fwd, status));
    HZ_TRY(launch_eval(n, op->pos64.as<double4_32a>(), op->nrm64.as<double4_32a>(), sg0, sg1, m, R, op->p.wave, op->tau,
                       op->p.interior, HZ_DOUBLE_LAYER, U0, U1, s));
    HZ_TRY(vec_sub(m, U0, U1, T0, T1, E0, E1, s));  // r = u - t
    HZ_TRY(launch_eval_adjoint(n, op->pos64.as<double4_32a>(), op->nrm64.as<double4_32a>(), m, R, E0, E1, op->p.wave,
                               op->tau, op->p.interior, HZ_DOUBLE_LAYER, e0, e1, s));
    HZ_TRY(solve_device(op, o, true, e0, e1, l0, l1, adj, status2));
    HZ_TRY(shape_gradient_device(op->p, op->H, op->eps, op->tau, n, op->idx.as<int64_t>(), op->d.as<double>(),
                                 op->gx.as<double>(), op->gy.as<double>(), op->gz.as<double>(), op->mc.as<double>(),
                                 op->gc.as<double>(), op->xs.as<double>(), op->w.as<double>(),
                                 op->pos64.as<double4_32a>(), op->nrm64.as<double4_32a>(), sg0, sg1, l0, l1, m, R, E0,
                                 E1, src, work.as<double>(), phib, s));
    std::vector<double> hr0(m), hr1(m);
    HZ_CHECK_CUDA(cudaMemcpyAsync(hr0.data(), E0, m * sizeof(double), cudaMemcpyDeviceToHost, s));
    HZ_CHECK_CUDA(cudaMemcpyAsync(hr1.data(), E1, m * sizeof(double), cudaMemcpyDeviceToHost, s));
    HZ_TRY(stage_out(dJ_dphi, phib, nodes, where, s));
    HZ_CHECK_CUDA(cudaStreamSynchronize(s));
    double jv = 0.0;
    for (int64_t i = 0; i < m; i++) jv += hr0[i] * hr0[i] + hr1[i] * hr1[i];
    if (J) *J = jv;
    int rc = check_device_error(op, "hz_shape_gradient");
    if (info) {
        hz_solve_info inf = fwd;
        inf.iterations = fwd.iterations + adj.iterations;
        inf.outer = fwd.outer + adj.outer;
        inf.resid = fwd.resid > adj.resid ? fwd.resid : adj.resid;
        inf.resid_f64 = fwd.resid_f64 > adj.resid_f64 ? fwd.resid_f64 : adj.resid_f64;
        inf.pair_evals = fwd.pair_evals + adj.pair_evals + n * n;
        inf.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        inf.status = rc != HZ_OK ? rc : (status != HZ_OK ? status : status2);
        inf.converged = (fwd.converged && adj.converged) ? 1 : 0;
        *info = inf;
    }
    if (rc != HZ_OK) return rc;
    if (status != HZ_OK || status2 != HZ_OK) {
        set_error("solver stopped early (status %d / %d)", status, status2);
        return status != HZ_OK ? status : status2;
    }
    return HZ_OK;
}

int hz_rhs_point_source(hz_operator *op, const double *src, int kind, double *b_re, double *b_im, int where)
{
    HZ_TRY(need_built(op));
    HZ_TRY(where_ok(where));
    if (!src || kind < 0 || kind > 3) {
        set_error("bad point source arguments");
        return HZ_ERR_ARG;
    }
    const size_t n = (size_t)op->n;
    cudaStream_t s = op->stream;
    double *io = op->io.as<double>();
    double *dre = (where == HZ_HOST) ? io : b_re, *dim = (where == HZ_HOST) ? io + n : b_im;
    HZ_TRY(launch_rhs(op->n, op->pos64.as<double4_32a>(), op->nrm64.as<double4_32a>(), src, op->p.wave, kind, dre, dim, s));
    if (where == HZ_HOST) {
        HZ_TRY(stage_out(b_re, dre, n, where, s));
        HZ_TRY(stage_out(b_im, dim, n, where, s));
    }
    HZ_CHECK_CUDA(cudaStreamSynchronize(s));
    return HZ_OK;
}

int hz_eval(hz_operator *op, int layer, int64_t m, const double *rx, const double *s_re, const double *s_im,
            double *u_re, double *u_im, int where)
{
    HZ_TRY(need_built(op));
    HZ_TRY(where_ok(where));
    if (layer != HZ_SINGLE_LAYER && layer != HZ_DOUBLE_LAYER && layer != HZ_COMBO_LAYER) {
        set_error("unknown layer %d", layer);
        return HZ_ERR_ARG;
    }
    if ((layer == HZ_COMBO_LAYER) != (op->combo != 0)) {
        set_error("HZ_COMBO_LAYER goes with (and only with) the Combo formulation");
        return HZ_ERR_ARG;
    }
    if (m < 0) {
        set_error("negative receiver count");
        return HZ_ERR_ARG;
    }
    if (m == 0) return HZ_OK;
    cudaStream_t s = op->stream;
    const size_t n = (size_t)op->n;
    const double *drx = rx, *dsr = s_re, *dsi = s_im;
    double *dur = u_re, *dui = u_im;
    DevBuf tmp;
    if (where == HZ_HOST) {
        HZ_TRY(tmp.ensure((3 * (size_t)m + 2 * n + 2 * (size_t)m) * sizeof(double)));
        double *t = tmp.as<double>();
        HZ_TRY(stage_in(t, rx, 3 * m, where, s));
        HZ_TRY(stage_in(t + 3 * m, s_re, n, where, s));
        HZ_TRY(stage_in(t + 3 * m + n, s_im, n, where, s));
        drx = t;
        dsr = t + 3 * m;
        dsi = t + 3 * m + n;
        dur = t + 3 * m + 2 * n;
        dui = dur + m;
    }
    if (layer == HZ_COMBO_LAYER)
        HZ_TRY(launch_eval_combo(op->n, op->pos64.as<double4_32a>(), op->nrm64.as<double4_32a>(), dsr, dsi, m, drx,
                                 op->p.wave, op->tau, op->combo_opts.eta, dur, dui, s));
    else
        HZ_TRY(launch_eval(op->n, op->pos64.as<double4_32a>(), op->nrm64.as<double4_32a>(), dsr, dsi, m, drx,
                           op->p.wave, op->tau, op->p.interior, layer, dur, dui, s));
    if (where == HZ_HOST) {
        HZ_TRY(stage_out(u_re, dur, m, where, s));
        HZ_TRY(stage_out(u_im, dui, m, where, s));
    }
    HZ_CHECK_CUDA(cudaStreamSynchronize(s));
    return HZ_OK;
}

int hz_eval_slice(hz_operator *op, int layer, int axis, double c, int n2, double lo, double h2, double mask,
                  const double *s_re, const double *s_im, double *u_re, double *u_im, int where)
{
    HZ_TRY(need_built(op));
    HZ_TRY(where_ok(where));
    if (axis < 0 || axis > 2 || n2 < 1 || n2 > 16384 || !(h2 > 0) ||
        (layer != HZ_SINGLE_LAYER && layer != HZ_DOUBLE_LAYER)) {
        set_error("hz_eval_slice: bad arguments");
        return HZ_ERR_ARG;
    }
    cudaStream_t s = op->stream;
    const int64_t m = (int64_t)n2 * n2;
    const size_t n = (size_t)op->n;
    DevBuf tmp;
    HZ_TRY(tmp.ensure((3 * (size_t)m + 2 * (size_t)m + 2 * n) * sizeof(double) + (size_t)m + 64));
    double *rx = tmp.as<double>(), *ur = rx + 3 * m, *ui = ur + m, *sr = ui + m, *si = sr + n;
    unsigned char *keep = reinterpret_cast<unsigned char *>(si + n);
    const double *dsr = s_re, *dsi = s_im;
    if (where == HZ_HOST) {
        HZ_TRY(stage_in(sr, s_re, n, where, s));
        HZ_TRY(stage_in(si, s_im, n, where, s));
        dsr = sr;
        dsi = si;
    }
    HZ_TRY(launch_slice(axis, c, n2, lo, h2, mask, op->p.N, op->H, op->p.int_l, op->d.as<double>(), rx, keep, s));
    HZ_TRY(launch_eval(op->n, op->pos64.as<double4_32a>(), op->nrm64.as<double4_32a>(), dsr, dsi, m, rx, op->p.wave,
                       op->tau, op->p.interior, layer, ur, ui, s));
    HZ_TRY(launch_mask(m, keep, ur, ui, s));
    HZ_TRY(stage_out(u_re, ur, m, where, s));
    HZ_TRY(stage_out(u_im, ui, m, where, s));
    HZ_CHECK_CUDA(cudaStreamSynchronize(s));
    return HZ_OK;
}

int hz_assign_gradient(int N, double H, const double *d, double *gx, double *gy, double *gz, int weno_order,
                       int where)
{
    HZ_TRY(where_ok(where));
    if (N < 8 || !d || !gx || !gy || !gz || (weno_order != 3 && weno_order != 5)) {
        set_error("hz_assign_gradient: bad arguments");
        return HZ_ERR_ARG;
    }
    const size_t S = (size_t)N + 1, nodes = S * S * S;
    cudaStream_t s = nullptr;
    if (where == HZ_DEVICE) {
        HZ_TRY(launch_grid_stencils(N, H, d, gx, gy, gz, nullptr, nullptr, weno_order, s));
        HZ_CHECK_CUDA(cudaStreamSynchronize(s));
        return HZ_OK;
    }
    DevBuf buf;
    HZ_TRY(buf.ensure(4 * nodes * sizeof(double)));
    double *b = buf.as<double>();
    HZ_TRY(stage_in(b, d, nodes, where, s));
    HZ_TRY(launch_grid_stencils(N, H, b, b + nodes, b + 2 * nodes, b + 3 * nodes, nullptr, nullptr, weno_order, s));
    HZ_TRY(stage_out(gx, b + nodes, nodes, where, s));
    HZ_TRY(stage_out(gy, b + 2 * nodes, nodes, where, s));
    HZ_TRY(stage_out(gz, b + 3 * nodes, nodes, where, s));
    HZ_CHECK_CUDA(cudaStreamSynchronize(s));
    return HZ_OK;
}

int hz_reinitialize(int N, double H, double *phi, int iters, double cfl, int weno_order, int where)
{
    HZ_TRY(where_ok(where));
    if (N < 8 || !phi || iters < 0 || !(cfl > 0) || cfl > 1.0 || (weno_order != 3 && weno_order != 5)) {
        set_error("hz_reinitialize: bad arguments");
        return HZ_ERR_ARG;
    }
    const size_t S = (size_t)N + 1, nodes = S * S * S;
    cudaStream_t s = nullptr;
    DevBuf buf;
    HZ_TRY(buf.ensure(4 * nodes * sizeof(double)));
    double *b = buf.as<double>();
    double *dphi = b + 3 * nodes;
    HZ_TRY(stage_in(dphi, phi, nodes, where, s));
    HZ_CHECK_CUDA(cudaMemcpyAsync(b, dphi, nodes * sizeof(double), cudaMemcpyDeviceToDevice, s));  // phi0
    HZ_TRY(launch_reinit(N, H, dphi, b + nodes, b + 2 * nodes, b, iters, cfl, weno_order, s));
    HZ_TRY(stage_out(phi, dphi, nodes, where, s));
    HZ_CHECK_CUDA(cudaStreamSynchronize(s));
    return HZ_OK;
}

int hz_assign_curvatures(int N, double H, const double *d, double *mcurv, double *gcurv, int where)
{
    HZ_TRY(where_ok(where));
    if (N < 8 || !d || !mcurv || !gcurv) {
        set_error("hz_assign_curvatures: bad arguments");
        return HZ_ERR_ARG;
    }
    const size_t S = (size_t)N + 1, nodes = S * S * S;
    cudaStream_t s = nullptr;
    if (where == HZ_DEVICE) {
        HZ_TRY(launch_grid_stencils(N, H, d, nullptr, nullptr, nullptr, mcurv, gcurv, 5, s));
        HZ_CHECK_CUDA(cudaStreamSynchronize(s));
        return HZ_OK;
    }
    DevBuf buf;
    HZ_TRY(buf.ensure(3 * nodes * sizeof(double)));
    double *b = buf.as<double>();
    HZ_TRY(stage_in(b, d, nodes, where, s));
    HZ_TRY(launch_grid_stencils(N, H, b, nullptr, nullptr, nullptr, b + nodes, b + 2 * nodes, 5, s));
    HZ_TRY(stage_out(mcurv, b + nodes, nodes, where, s));
    HZ_TRY(stage_out(gcurv, b + 2 * nodes, nodes, where, s));
    HZ_CHECK_CUDA(cudaStreamSynchronize(s));
    return HZ_OK;
}

int hz_dense_bicg(int64_t n, const double *a_re, const double *a_im, const double *b_re, const double *b_im,
                  double *x_re, double *x_im, double tol, int maxit, int where, hz_solve_info *info)
{
    HZ_TRY(where_ok(where));
    if (n < 1 || !a_re || !a_im || !(tol > 0) || maxit < 1) {
        set_error("hz_dense_bicg: bad arguments");
        return HZ_ERR_ARG;
    }
    auto t0 = std::chrono::steady_clock::now();
    cudaStream_t s = nullptr;
    const size_t nn = (size_t)n * (size_t)n;
    DevBuf mat, vec, part;
    const double *dre = a_re, *dim = a_im;
    if (where == HZ_HOST) {
        HZ_TRY(mat.ensure(2 * nn * sizeof(double)));
        HZ_TRY(stage_in(mat.as<double>(), a_re, nn, where, s));
        HZ_TRY(stage_in(mat.as<double>() + nn, a_im, nn, where, s));
        dre = mat.as<double>();
        dim = dre + nn;
    }
    HZ_TRY(vec.ensure(2 * (size_t)n * sizeof(double)));
    HZ_TRY(stage_in(vec.as<double>(), b_re, n, where, s));
    HZ_TRY(stage_in(vec.as<double>() + n, b_im, n, where, s));
    HZ_TRY(part.ensure(2 * dense_partial_elems(n) * sizeof(double)));
    DenseOp A;
    A.n = n;
    A.are = dre;
    A.aim = dim;
    A.part_re = part.as<double>();
    A.part_im = A.part_re + dense_partial_elems(n);
    Krylov k;
    HZ_TRY(k.reserve(n));
    int iters = 0, status = HZ_OK;
    double resid = 0.0;
    HZ_TRY(k.solve(A, HZ_BICG, vec.as<double>(), vec.as<double>() + n, tol, maxit, true, false, s, iters, resid, status));
    HZ_TRY(stage_out(x_re, k.re(Krylov::X), n, where, s));
    HZ_TRY(stage_out(x_im, k.im(Krylov::X), n, where, s));
    HZ_CHECK_CUDA(cudaStreamSynchronize(s));
    if (info) {
        hz_solve_info inf{};
        inf.iterations = iters;
        inf.resid = resid;
        inf.resid_f64 = resid;
        inf.status = status;
        inf.converged = resid < tol ? 1 : 0;
        inf.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        *info = inf;
    }
    return status;
}

}  // extern "C"
