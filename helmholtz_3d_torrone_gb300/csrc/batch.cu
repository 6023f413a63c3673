// batch.cu -- batches of independent operators solved together.
//
// The vectors of a batch of R operators are stored as [R][nmax] columns,
// each zero past its operator's tube size n_r; the products keep those
// tails zero, so lockstep BiCGSTAB (KrylovMulti) over the columns is exactly
// R independent BiCGSTAB solves.  The FP32 product is one persistent
// stream-K launch over the concatenated (operator, target block, source
// tile) units of all operators (sweep_f32.cu, sweep32_batch_kernel), and the
// whole BiCGSTAB iteration is captured once as a CUDA graph.  A system that
// has converged leaves the batch: the launch is re-described over the
// operators whose columns still iterate (and the graph captured again), and
// the refinement neither re-solves it nor recomputes its FP64 residual.  The
// FP64 products (refinement residuals) run one FP64 sweep per operator, the
// sweeps spread over side streams so that small operators share the GPU.
#include "hz_internal.cuh"
#include "krylov.cuh"
#include "krylov_multi.cuh"

#include <chrono>
#include <vector>

using namespace hz;

namespace {
constexpr int kBatchShapes = 4;
constexpr int kInnerStallBatch = 30;  // as the single-operator refinement
}  // namespace

struct hz_batch {
    std::vector<hz_operator *> ops;
    int R = 0;
    int64_t nmax = 0, max_npad = 0;
    int device = 0;
    cudaStream_t stream = nullptr;
    int shape = 1;  // FP32 batch sweep shape (hz_batch_autotune)
    DevBuf desc;    // kBatchShapes descriptor arrays
    int64_t units[kBatchShapes] = {}, blocks[kBatchShapes] = {};
    std::vector<Batch32Item> items;
    // the FP32 launch over a subset of the operators (sub_n > 0)
    DevBuf desc_sub;
    int sub_n = 0, sub_shape = -1;
    int64_t sub_units = 0, sub_blocks = 0;
    uint64_t sub_gen = 0;
    DevBuf partial;
    size_t partial_bytes = 0;
    KrylovMulti multi;
    DevBuf vec, small;
    // side streams for the per-operator FP64 products (fork / join on events)
    std::vector<cudaStream_t> side;
    std::vector<cudaEvent_t> side_done;
    cudaEvent_t fork = nullptr;
    ~hz_batch()
    {
        for (cudaStream_t x : side) cudaStreamDestroy(x);
        for (cudaEvent_t e : side_done) cudaEventDestroy(e);
        if (fork) cudaEventDestroy(fork);
    }
};

namespace {

struct BatchF32 final : MultiOp {
    hz_batch *b;
    bool sub = false;  // launch over b->desc_sub
    explicit BatchF32(hz_batch *bb) : b(bb) {}
    int apply(int R, const double *p_re, const double *p_im, double *q_re, double *q_im, cudaStream_t s) override
    {
        (void)R;
        if (sub && b->sub_shape == b->shape)
            return sweep_f32_batch(b->shape, b->desc_sub.ptr, b->sub_n, b->R, b->sub_units, b->sub_blocks,
                                   b->partial.as<double4_32a>(), b->partial_bytes, p_re, p_im, q_re, q_im, b->nmax,
                                   b->max_npad, s, nullptr, nullptr);
        const size_t db = batch32_desc_bytes(b->R);
        return sweep_f32_batch(b->shape, b->desc.as<char>() + (size_t)b->shape * db, b->R, b->R, b->units[b->shape],
                               b->blocks[b->shape], b->partial.as<double4_32a>(), b->partial_bytes, p_re, p_im, q_re,
                               q_im, b->nmax, b->max_npad, s, nullptr, nullptr);
    }
    uint64_t key() const override
    {
        const uint64_t g = sub ? b->sub_gen : 0;
        return ((uint64_t)(uintptr_t)b << 4) ^ (uint64_t)(b->shape + 1) ^ (g << 40);
    }
    int restrict_to(const std::vector<int> &cols, cudaStream_t s) override
    {
        if ((int)cols.size() == b->R) {
            sub = false;
            return HZ_OK;
        }
        sub = false;
        b->sub_n = 0;
        b->sub_shape = -1;
        HZ_TRY(batch32_describe(b->items.data(), (int)cols.size(), b->shape, b->desc_sub.ptr, b->sub_units,
                                b->sub_blocks, s, cols.data()));
        b->sub_n = (int)cols.size();
        b->sub_shape = b->shape;
        b->sub_gen++;
        sub = true;
        return HZ_OK;
    }
};

// The FP64 products (refinement residuals) are one FP64 sweep per
// operator.  A small operator's sweep fills few SMs, so the sweeps run
// concurrently on side streams forked from s and joined back to it (each
// operator has its own density scratch, output column and error word).
constexpr int kSideStreams = 8;

struct BatchF64 final : MultiOp {
    hz_batch *b;
    std::vector<int> cols;  // empty: every operator
    explicit BatchF64(hz_batch *bb) : b(bb) {}
    int ensure_side()
    {
        if (!b->side.empty()) return HZ_OK;
        HZ_CHECK_CUDA(cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming));
        for (int i = 0; i < kSideStreams; i++) {
            cudaStream_t x = nullptr;
            cudaEvent_t e = nullptr;
            HZ_CHECK_CUDA(cudaStreamCreateWithFlags(&x, cudaStreamNonBlocking));
            b->side.push_back(x);
            HZ_CHECK_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
            b->side_done.push_back(e);
        }
        return HZ_OK;
    }
    int apply(int R, const double *p_re, const double *p_im, double *q_re, double *q_im, cudaStream_t s) override
    {
        (void)R;
        HZ_CHECK_CUDA(cudaMemsetAsync(q_re, 0, (size_t)b->R * b->nmax * sizeof(double), s));
        HZ_CHECK_CUDA(cudaMemsetAsync(q_im, 0, (size_t)b->R * b->nmax * sizeof(double), s));
        const int m = cols.empty() ? b->R : (int)cols.size();
        HZ_TRY(ensure_side());
        HZ_CHECK_CUDA(cudaEventRecord(b->fork, s));
        const int used = m < kSideStreams ? m : kSideStreams;
        for (int k = 0; k < used; k++) HZ_CHECK_CUDA(cudaStreamWaitEvent(b->side[k], b->fork, 0));
        int rc = HZ_OK;
        for (int i = 0; i < m && rc == HZ_OK; i++) {
            const int r = cols.empty() ? i : cols[i];
            hz_operator *op = b->ops[r];
            const size_t off = (size_t)r * b->nmax;
            rc = sweep_f64(sweep_const(op), rec64(op), SWEEP_A, p_re + off, p_im + off, nullptr, nullptr, q_re + off,
                           q_im + off, nullptr, nullptr, op->scratch.as<double2>(), b->side[i % kSideStreams]);
        }
        // join every side stream that was forked, also after a failed launch
        for (int k = 0; k < used; k++) {
            HZ_CHECK_CUDA(cudaEventRecord(b->side_done[k], b->side[k]));
            HZ_CHECK_CUDA(cudaStreamWaitEvent(s, b->side_done[k], 0));
        }
        return rc;
    }
    int restrict_to(const std::vector<int> &c, cudaStream_t s) override
    {
        (void)s;
        cols = c;
        return HZ_OK;
    }
};

int check_batch(hz_batch *b)
{
    if (!b || b->R < 1) {
        set_error("batch is NULL or empty");
        return HZ_ERR_ARG;
    }
    for (hz_operator *op : b->ops)
        if (!op->built) {
            set_error("an operator of the batch was rebuilt or invalidated; create the batch again");
            return HZ_ERR_STATE;
        }
    return HZ_OK;
}

int clear_errors(hz_batch *b, cudaStream_t s)
{
    for (hz_operator *op : b->ops) HZ_CHECK_CUDA(cudaMemsetAsync(op->err.ptr, 0, sizeof(unsigned), s));
    return HZ_OK;
}

int batch_errors(hz_batch *b, const char *who)
{
    for (hz_operator *op : b->ops) HZ_TRY(check_device_error(op, who));
    return HZ_OK;
}

// per-operator vectors (host or device) <-> padded [R][nmax] device columns
int gather(hz_batch *b, const double *const *src, double *dst, int where, cudaStream_t s)
{
    HZ_CHECK_CUDA(cudaMemsetAsync(dst, 0, (size_t)b->R * b->nmax * sizeof(double), s));
    for (int r = 0; r < b->R; r++) {
        if (!src || !src[r]) {
            set_error("batch input vector %d is NULL", r);
            return HZ_ERR_ARG;
        }
        HZ_TRY(stage_in(dst + (size_t)r * b->nmax, src[r], (size_t)b->ops[r]->n, where, s));
    }
    return HZ_OK;
}

int scatter(hz_batch *b, const double *src, double *const *dst, int where, cudaStream_t s)
{
    if (!dst) return HZ_OK;
    for (int r = 0; r < b->R; r++) HZ_TRY(stage_out(dst[r], src + (size_t)r * b->nmax, (size_t)b->ops[r]->n, where, s));
    return HZ_OK;
}

}  // namespace

extern "C" {

int hz_batch_create(hz_operator *const *ops, int count, hz_batch **out)
{
    if (!ops || count < 1 || !out) {
        set_error("hz_batch_create: bad arguments");
        return HZ_ERR_ARG;
    }
    hz_batch *b = new hz_batch;
    b->R = count;
    for (int r = 0; r < count; r++) {
        hz_operator *op = ops[r];
        if (!op || !op->built || op->combo || op->r32.npad <= 0 || (r > 0 && op->device != ops[0]->device)) {
            delete b;
            set_error("hz_batch_create: operator %d is missing, not built, Combo, empty or on another device", r);
            return HZ_ERR_ARG;
        }
        b->ops.push_back(op);
        b->nmax = op->n > b->nmax ? op->n : b->nmax;
        b->max_npad = op->r32.npad > b->max_npad ? op->r32.npad : b->max_npad;
    }
    b->device = ops[0]->device;
    b->stream = ops[0]->stream;
    int rc = cudaSetDevice(b->device) == cudaSuccess ? HZ_OK : HZ_ERR_CUDA;
    const size_t db = batch32_desc_bytes(count);
    if (rc == HZ_OK) rc = b->desc.ensure(kBatchShapes * db);
    if (rc == HZ_OK) rc = b->desc_sub.ensure(db);
    std::vector<Batch32Item> &items = b->items;
    items.resize(count);
    for (int r = 0; r < count && rc == HZ_OK; r++) {
        hz_operator *op = ops[r];
        items[r].c = sweep_const(op);
        items[r].r = op->r32;
        items[r].pos64 = op->pos64.as<double4_32a>();
        items[r].dens = op->dens32.as<float4>();
    }
    for (int k = 0; k < kBatchShapes && rc == HZ_OK; k++)
        rc = batch32_describe(items.data(), count, k, b->desc.as<char>() + (size_t)k * db, b->units[k], b->blocks[k],
                              b->stream);
    if (rc == HZ_OK) {
        b->partial_bytes = batch32_partial_bytes();
        rc = b->partial.ensure(b->partial_bytes);
    }
    if (rc != HZ_OK) {
        delete b;
        return rc;
    }
    *out = b;
    return HZ_OK;
}

void hz_batch_destroy(hz_batch *b) { delete b; }

int hz_batch_autotune(hz_batch *b, int *chosen, double *ms_per_sweep)
{
    HZ_TRY(check_batch(b));
    HZ_CHECK_CUDA(cudaSetDevice(b->device));
    cudaStream_t s = b->stream;
    const size_t tot = (size_t)b->R * b->nmax;
    HZ_TRY(b->vec.ensure(4 * tot * sizeof(double)));
    double *v = b->vec.as<double>();
    HZ_CHECK_CUDA(cudaMemsetAsync(v, 0, 4 * tot * sizeof(double), s));
    cudaEvent_t e0, e1;
    HZ_CHECK_CUDA(cudaEventCreate(&e0));
    HZ_CHECK_CUDA(cudaEventCreate(&e1));
    int best = b->shape;
    float best_ms = 1e30f;
    int rc = HZ_OK;
    const size_t db = batch32_desc_bytes(b->R);
    for (int k = 0; k < kBatchShapes && rc == HZ_OK; k++) {
        float ms_min = 1e30f;
        for (int rep = 0; rep < 2 && rc == HZ_OK; rep++) {
            rc = sweep_f32_batch(k, b->desc.as<char>() + (size_t)k * db, b->R, b->R, b->units[k], b->blocks[k],
                                 b->partial.as<double4_32a>(), b->partial_bytes, v, v + tot, v + 2 * tot, v + 3 * tot,
                                 b->nmax, b->max_npad, s, e0, e1);
            if (rc == HZ_OK && cudaEventSynchronize(e1) == cudaSuccess) {
                float ms = 0.f;
                cudaEventElapsedTime(&ms, e0, e1);
                ms_min = ms < ms_min ? ms : ms_min;
            }
        }
        if (ms_min < best_ms) {
            best_ms = ms_min;
            best = k;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    HZ_TRY(rc);
    b->shape = best;
    if (chosen) *chosen = best;
    if (ms_per_sweep) *ms_per_sweep = best_ms;
    return HZ_OK;
}

int hz_batch_set_variant(hz_batch *b, int v)
{
    HZ_TRY(check_batch(b));
    if (v < 0 || v >= kBatchShapes) {
        set_error("hz_batch_set_variant: variant must be in [0, %d)", kBatchShapes);
        return HZ_ERR_ARG;
    }
    b->shape = v;
    return HZ_OK;
}

int hz_batch_matvec(hz_batch *b, int precision, const double *const *p_re, const double *const *p_im,
                    double *const *q_re, double *const *q_im, int where)
{
    HZ_TRY(check_batch(b));
    HZ_TRY(where_ok(where));
    if (precision != HZ_PREC_F64 && precision != HZ_PREC_F32) {
        set_error("hz_batch_matvec: precision must be HZ_PREC_F64 or HZ_PREC_F32");
        return HZ_ERR_ARG;
    }
    HZ_CHECK_CUDA(cudaSetDevice(b->device));
    cudaStream_t s = b->stream;
    const size_t tot = (size_t)b->R * b->nmax;
    HZ_TRY(b->vec.ensure(4 * tot * sizeof(double)));
    double *v = b->vec.as<double>();
    HZ_TRY(clear_errors(b, s));
    HZ_TRY(gather(b, p_re, v, where, s));
    HZ_TRY(gather(b, p_im, v + tot, where, s));
    if (precision == HZ_PREC_F32) {
        BatchF32 A(b);
        HZ_TRY(A.apply(b->R, v, v + tot, v + 2 * tot, v + 3 * tot, s));
    } else {
        BatchF64 A(b);
        HZ_TRY(A.apply(b->R, v, v + tot, v + 2 * tot, v + 3 * tot, s));
    }
    HZ_TRY(scatter(b, v + 2 * tot, q_re, where, s));
    HZ_TRY(scatter(b, v + 3 * tot, q_im, where, s));
    HZ_CHECK_CUDA(cudaStreamSynchronize(s));
    return batch_errors(b, "hz_batch_matvec");
}

int hz_batch_solve(hz_batch *b, const hz_solve_opts *opts_in, const double *const *b_re, const double *const *b_im,
                   double *const *x_re, double *const *x_im, int where, hz_solve_info *info, double *resid)
{
    HZ_TRY(check_batch(b));
    HZ_TRY(where_ok(where));
    hz_solve_opts o;
    if (opts_in) o = *opts_in;
    else hz_solve_opts_default(&o);
    if (!(o.tol > 0) || o.maxit < 1 || o.precision < HZ_PREC_F64 || o.precision > HZ_PREC_F32_REFINED) {
        set_error("hz_batch_solve: bad options");
        return HZ_ERR_ARG;
    }
    HZ_CHECK_CUDA(cudaSetDevice(b->device));
    cudaStream_t s = b->stream;
    const int R = b->R;
    const int64_t nm = b->nmax;
    const size_t tot = (size_t)R * nm;
    auto t0 = std::chrono::steady_clock::now();
    HZ_TRY(b->vec.ensure(8 * tot * sizeof(double)));
    double *B0 = b->vec.as<double>(), *B1 = B0 + tot, *X0 = B0 + 2 * tot, *X1 = B0 + 3 * tot, *R0 = B0 + 4 * tot,
           *R1 = B0 + 5 * tot, *Q0 = B0 + 6 * tot, *Q1 = B0 + 7 * tot;
    HZ_TRY(clear_errors(b, s));
    HZ_TRY(gather(b, b_re, B0, where, s));
    HZ_TRY(gather(b, b_im, B1, where, s));
    HZ_TRY(b->multi.reserve(nm, R));
    std::vector<double> res(R, 0.0);
    hz_solve_info inf{};
    int iters = 0, outer = 0;
    long long pairs = 0;
    std::vector<int> cit;
    auto pairs_of = [&](const std::vector<int> &its, int products) {
        long long p = 0;
        for (int r = 0; r < R; r++) p += (long long)products * its[r] * b->ops[r]->n * b->ops[r]->n;
        return p;
    };
    if (o.precision != HZ_PREC_F32_REFINED) {
        BatchF32 A32(b);
        BatchF64 A64(b);
        MultiOp &A = (o.precision == HZ_PREC_F32) ? static_cast<MultiOp &>(A32) : static_cast<MultiOp &>(A64);
        HZ_TRY(b->multi.solve(A, B0, B1, o.tol, o.maxit, o.stagnation != 0, s, iters, res, 0, &cit));
        HZ_CHECK_CUDA(cudaMemcpyAsync(X0, b->multi.re(KrylovMulti::X), tot * sizeof(double), cudaMemcpyDeviceToDevice, s));
        HZ_CHECK_CUDA(cudaMemcpyAsync(X1, b->multi.im(KrylovMulti::X), tot * sizeof(double), cudaMemcpyDeviceToDevice, s));
        pairs = pairs_of(cit, 2);
    } else {
        // FP64 iterative refinement of every system still above tol:
        // x_r += ||r_r|| A32^{-1}(r_r/||r_r||)
        BatchF32 A32(b);
        BatchF64 A64(b);
        HZ_TRY(b->small.ensure(vec_partial_bytes() + 64));
        double *part = b->small.as<double>();
        double *dout = part + (vec_partial_bytes() / sizeof(double));
        std::vector<double> normb(R), nr(R);
        for (int r = 0; r < R; r++) HZ_TRY(vec_norm(nm, B0 + r * nm, B1 + r * nm, part, dout, normb[r], s));
        HZ_CHECK_CUDA(cudaMemsetAsync(X0, 0, tot * sizeof(double), s));
        HZ_CHECK_CUDA(cudaMemsetAsync(X1, 0, tot * sizeof(double), s));
        HZ_CHECK_CUDA(cudaMemcpyAsync(R0, B0, tot * sizeof(double), cudaMemcpyDeviceToDevice, s));
        HZ_CHECK_CUDA(cudaMemcpyAsync(R1, B1, tot * sizeof(double), cudaMemcpyDeviceToDevice, s));
        nr = normb;
        for (int r = 0; r < R; r++) res[r] = normb[r] > 0 ? 1.0 : 0.0;
        auto worst = [&]() {
            double w = 0;
            for (double v : res) w = v > w ? v : w;
            return w;
        };
        std::vector<int> open;
        while (worst() >= o.tol && outer < o.max_outer) {
            outer++;
            open.clear();
            for (int r = 0; r < R; r++) {
                double *q0 = Q0 + r * nm, *q1 = Q1 + r * nm;
                if (res[r] >= o.tol) {
                    open.push_back(r);
                    HZ_TRY(vec_scale(nm, 1.0 / nr[r], R0 + r * nm, R1 + r * nm, q0, q1, s));
                } else {
                    // a zero right-hand side: the column does not iterate
                    HZ_CHECK_CUDA(cudaMemsetAsync(q0, 0, nm * sizeof(double), s));
                    HZ_CHECK_CUDA(cudaMemsetAsync(q1, 0, nm * sizeof(double), s));
                }
            }
            int it = 0;
            std::vector<double> ires;
            const double itol = refine_inner_tol(o, worst());
            HZ_TRY(b->multi.solve(A32, Q0, Q1, itol, o.maxit, o.stagnation != 0, s, it, ires, kInnerStallBatch,
                                  &cit));
            iters += it;
            pairs += pairs_of(cit, 2);
            A64.cols = open;
            for (int r : open) {
                const size_t off = (size_t)r * nm;
                HZ_TRY(vec_axpy(nm, nr[r], b->multi.re(KrylovMulti::X) + off, b->multi.im(KrylovMulti::X) + off,
                                X0 + off, X1 + off, s));
            }
            HZ_TRY(A64.apply(R, X0, X1, Q0, Q1, s));
            for (int r : open) {
                const size_t off = (size_t)r * nm;
                pairs += (long long)b->ops[r]->n * b->ops[r]->n;
                HZ_TRY(vec_sub(nm, B0 + off, B1 + off, Q0 + off, Q1 + off, R0 + off, R1 + off, s));
                HZ_TRY(vec_norm(nm, R0 + off, R1 + off, part, dout, nr[r], s));
                res[r] = normb[r] > 0 ? nr[r] / normb[r] : 0.0;
            }
            if (inf.steps < HZ_MAX_STEPS) {
                inf.step_iters[inf.steps] = it;
                inf.step_inner_tol[inf.steps] = itol;
                inf.step_resid[inf.steps] = worst();
                inf.steps++;
            }
        }
    }
    HZ_TRY(scatter(b, X0, x_re, where, s));
    HZ_TRY(scatter(b, X1, x_im, where, s));
    HZ_CHECK_CUDA(cudaStreamSynchronize(s));
    const int rc = batch_errors(b, "hz_batch_solve");
    double w = 0;
    for (int r = 0; r < R; r++) {
        w = res[r] > w ? res[r] : w;
        if (resid) resid[r] = res[r];
    }
    inf.iterations = iters;
    inf.outer = outer;
    inf.resid = w;
    inf.resid_f64 = (o.precision == HZ_PREC_F32) ? -1.0 : w;
    inf.pair_evals = pairs;
    inf.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    inf.status = rc;
    inf.converged = w < o.tol ? 1 : 0;
    if (info) *info = inf;
    return rc;
}

}  // extern "C"
