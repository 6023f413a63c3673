// krylov_multi.cu -- BiCGSTAB for many right-hand sides in lockstep, each
// with its own scalars, driven by the multi-RHS pair sweep (one kernel
// evaluation per pair for the whole batch).  FP64 vectors and
// deterministically ordered FP64 inner products, as in krylov.cu; a
// right-hand side stops updating once its own residual is below tol.
#include "hz_internal.cuh"
#include "krylov_multi.cuh"

#include <cmath>
#include <vector>

namespace hz {
namespace {

constexpr int kMB = 64;  // partial-sum blocks per right-hand side
constexpr int kMT = 256;

struct MScal {
    double rho_re, rho_im, alpha_re, alpha_im, omega_re, omega_im, beta_re, beta_im;
    double normb, err, best;
    int active, status, it, best_it, improved;
};

// per-RHS partial sums of (sum a conj(b)) and ||a||^2; grid (kMB, R)
__global__ void __launch_bounds__(kMT) mcdot_kernel(int64_t n, const double *__restrict__ ar,
                                                    const double *__restrict__ ai, const double *__restrict__ br,
                                                    const double *__restrict__ bi, double *partial)
{
    const int r = blockIdx.y;
    const double *a0 = ar + (int64_t)r * n, *a1 = ai + (int64_t)r * n, *b0 = br + (int64_t)r * n,
                 *b1 = bi + (int64_t)r * n;
    double v[3] = {0, 0, 0};
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double x0 = a0[i], x1 = a1[i], y0 = b0[i], y1 = b1[i];
        v[0] += x0 * y0 + x1 * y1;
        v[1] += x1 * y0 - x0 * y1;
        v[2] += x0 * x0 + x1 * x1;
    }
    __shared__ double sh[kMT / 32][3];
    for (int d = 0; d < 3; d++) {
        double x = v[d];
        for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
        if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5][d] = x;
    }
    __syncthreads();
    if (threadIdx.x == 0)
        for (int d = 0; d < 3; d++) {
            double s = 0;
            for (int w = 0; w < kMT / 32; w++) s += sh[w][d];
            partial[((int64_t)r * kMB + blockIdx.x) * 4 + d] = s;
        }
}

__device__ void msum(const double *partial, int r, double *out)
{
    for (int d = 0; d < 3; d++) {
        double s = 0;
        for (int b = 0; b < kMB; b++) s += partial[((int64_t)r * kMB + b) * 4 + d];
        out[d] = s;
    }
}

__device__ void cdivd(double ar, double ai, double br, double bi, double &cr, double &ci)
{
    const double den = br * br + bi * bi;
    cr = (ar * br + ai * bi) / den;
    ci = (ai * br - ar * bi) / den;
}

__global__ void minit_kernel(int64_t n, const double *b_re, const double *b_im, double *x_re, double *x_im,
                             double *r_re, double *r_im, double *rh_re, double *rh_im, double *p_re, double *p_im,
                             double *v_re, double *v_im)
{
    const int64_t off = (int64_t)blockIdx.y * n;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t j = off + i;
        x_re[j] = x_im[j] = 0.0;
        r_re[j] = rh_re[j] = b_re[j];
        r_im[j] = rh_im[j] = b_im[j];
        p_re[j] = p_im[j] = v_re[j] = v_im[j] = 0.0;
    }
}

__global__ void mstart_kernel(int R, const double *partial, MScal *sc, double *host)
{
    const int r = threadIdx.x + blockIdx.x * blockDim.x;
    if (r >= R) return;
    double s[3];
    msum(partial, r, s);
    MScal &c = sc[r];
    c.normb = sqrt(s[2]);
    c.rho_re = 1.0;
    c.rho_im = 0.0;
    c.alpha_re = 1.0;
    c.alpha_im = 0.0;
    c.omega_re = 1.0;
    c.omega_im = 0.0;
    c.err = (s[2] > 0) ? 1.0 : 0.0;
    c.active = (s[2] > 0) ? 1 : 0;
    c.status = 0;
    c.best = 1e300;
    c.it = 0;
    c.best_it = 0;
    c.improved = 0;
    host[2 * r] = c.err;
    host[2 * r + 1] = c.active ? 1.0 : 0.0;
}

__global__ void mbeta_kernel(int R, const double *partial, MScal *sc)
{
    const int r = threadIdx.x + blockIdx.x * blockDim.x;
    if (r >= R || !sc[r].active) return;
    double s[3], q1r, q1i, q2r, q2i;
    msum(partial, r, s);
    MScal &c = sc[r];
    cdivd(s[0], s[1], c.rho_re, c.rho_im, q1r, q1i);
    cdivd(c.alpha_re, c.alpha_im, c.omega_re, c.omega_im, q2r, q2i);
    c.beta_re = q1r * q2r - q1i * q2i;
    c.beta_im = q1r * q2i + q1i * q2r;
    if (s[0] == 0.0 && s[1] == 0.0) c.status = 2;
    c.rho_re = s[0];
    c.rho_im = s[1];
}

__global__ void mp_kernel(int64_t n, const MScal *sc, const double *r_re, const double *r_im, double *p_re,
                          double *p_im, const double *v_re, const double *v_im)
{
    const MScal c = sc[blockIdx.y];
    if (!c.active) return;
    const int64_t off = (int64_t)blockIdx.y * n;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t j = off + i;
        const double tr = p_re[j] - (c.omega_re * v_re[j] - c.omega_im * v_im[j]);
        const double ti = p_im[j] - (c.omega_re * v_im[j] + c.omega_im * v_re[j]);
        p_re[j] = r_re[j] + c.beta_re * tr - c.beta_im * ti;
        p_im[j] = r_im[j] + c.beta_re * ti + c.beta_im * tr;
    }
}

__global__ void malpha_kernel(int R, const double *partial, MScal *sc)
{
    const int r = threadIdx.x + blockIdx.x * blockDim.x;
    if (r >= R || !sc[r].active) return;
    double s[3];
    msum(partial, r, s);
    MScal &c = sc[r];
    if (s[0] == 0.0 && s[1] == 0.0) c.status = 2;
    cdivd(c.rho_re, c.rho_im, s[0], s[1], c.alpha_re, c.alpha_im);
}

__global__ void ms_kernel(int64_t n, const MScal *sc, double *r_re, double *r_im, const double *v_re,
                          const double *v_im)
{
    const MScal c = sc[blockIdx.y];
    if (!c.active) return;
    const int64_t off = (int64_t)blockIdx.y * n;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t j = off + i;
        r_re[j] -= c.alpha_re * v_re[j] - c.alpha_im * v_im[j];
        r_im[j] -= c.alpha_re * v_im[j] + c.alpha_im * v_re[j];
    }
}

__global__ void momega_kernel(int R, const double *pst, const double *ptt, MScal *sc)
{
    const int r = threadIdx.x + blockIdx.x * blockDim.x;
    if (r >= R || !sc[r].active) return;
    double a[3], b[3];
    msum(pst, r, a);
    msum(ptt, r, b);
    MScal &c = sc[r];
    c.omega_re = a[0] / b[2];
    c.omega_im = a[1] / b[2];
    if (b[2] == 0.0) c.status = 2;
}

__global__ void mupdate_kernel(int64_t n, const MScal *sc, double *x_re, double *x_im, double *r_re, double *r_im,
                               const double *p_re, const double *p_im, const double *t_re, const double *t_im)
{
    const MScal c = sc[blockIdx.y];
    if (!c.active) return;
    const int64_t off = (int64_t)blockIdx.y * n;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t j = off + i;
        const double sr = r_re[j], si = r_im[j];
        x_re[j] += (c.alpha_re * p_re[j] - c.alpha_im * p_im[j]) + (c.omega_re * sr - c.omega_im * si);
        x_im[j] += (c.alpha_re * p_im[j] + c.alpha_im * p_re[j]) + (c.omega_re * si + c.omega_im * sr);
        r_re[j] = sr - (c.omega_re * t_re[j] - c.omega_im * t_im[j]);
        r_im[j] = si - (c.omega_re * t_im[j] + c.omega_im * t_re[j]);
    }
}

__global__ void merr_kernel(int R, const double *partial, MScal *sc, double tol, int stagnation, int stall,
                            double *host)
{
    const int r = threadIdx.x + blockIdx.x * blockDim.x;
    if (r >= R) return;
    MScal &c = sc[r];
    c.improved = 0;
    if (c.active) {
        double s[3];
        msum(partial, r, s);
        const double pre = c.err;
        c.err = sqrt(s[2]) / c.normb;
        c.it++;
        if (c.err < c.best) {
            c.best = c.err;
            c.best_it = c.it;
            c.improved = 1;
        }
        if (c.err < tol || c.err != c.err || c.status != 0 || (stagnation && fabs(pre - c.err) < 1e-3 * tol) ||
            (stall > 0 && c.it - c.best_it >= max(stall, c.best_it)))
            c.active = 0;
    }
    host[2 * r] = c.err;
    host[2 * r + 1] = c.active ? 1.0 : (c.status ? -1.0 : 0.0);
}

// XB = X for the columns whose residual reached a new minimum
__global__ void mkeep_kernel(int64_t n, const MScal *sc, const double *x_re, const double *x_im, double *b_re,
                             double *b_im)
{
    if (!sc[blockIdx.y].improved) return;
    const int64_t off = (int64_t)blockIdx.y * n;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        b_re[off + i] = x_re[off + i];
        b_im[off + i] = x_im[off + i];
    }
}

// X = XB for the columns that ended above their best residual
__global__ void mrestore_kernel(int64_t n, const MScal *sc, double *x_re, double *x_im, const double *b_re,
                                const double *b_im)
{
    const MScal c = sc[blockIdx.y];
    if (!(c.best < 1e300) || c.err <= c.best) return;
    const int64_t off = (int64_t)blockIdx.y * n;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        x_re[off + i] = b_re[off + i];
        x_im[off + i] = b_im[off + i];
    }
}

__global__ void mresid_kernel(int R, const MScal *sc, double *host)
{
    const int r = threadIdx.x + blockIdx.x * blockDim.x;
    if (r >= R) return;
    const MScal c = sc[r];
    host[2 * r] = (c.best < 1e300 && !(c.err <= c.best)) ? c.best : c.err;
}

int grid_x(int64_t n)
{
    long long b = (n + kMT - 1) / kMT;
    if (b > 64) b = 64;
    return (int)(b < 1 ? 1 : b);
}

}  // namespace

KrylovMulti::~KrylovMulti()
{
    if (graph_exec) cudaGraphExecDestroy(graph_exec);
    if (host) cudaFreeHost(host);
}

int KrylovMulti::reserve(int64_t n_, int R_)
{
    // a captured iteration refers to the old buffers and sizes
    if (graph_exec) cudaGraphExecDestroy(graph_exec);
    graph_exec = nullptr;
    graph_key = 0;
    n = n_;
    R = R_;
    HZ_TRY(vecs.ensure((size_t)n * R * sizeof(double) * 2 * kVecs));
    HZ_TRY(partial.ensure((size_t)R * kMB * 4 * sizeof(double) * 2));
    HZ_TRY(scal.ensure((size_t)R * sizeof(MScal)));
    if (host) cudaFreeHost(host);
    host = nullptr;
    HZ_CHECK_CUDA(cudaMallocHost(&host, (size_t)R * 2 * sizeof(double)));
    return HZ_OK;
}

double *KrylovMulti::re(int v) { return vecs.as<double>() + (size_t)(2 * v) * n * R; }
double *KrylovMulti::im(int v) { return vecs.as<double>() + (size_t)(2 * v + 1) * n * R; }

int KrylovMulti::iteration(MultiOp &A, double tol, bool stagnation, int stall, cudaStream_t s)
{
    double *pp = partial.as<double>();
    double *pp2 = pp + (size_t)R * kMB * 4;
    MScal *sc = scal.as<MScal>();
    const dim3 g(grid_x(n), R);
    const int sb = (R + 127) / 128;
    mcdot_kernel<<<dim3(kMB, R), kMT, 0, s>>>(n, re(RV), im(RV), re(RH), im(RH), pp);
    HZ_CHECK_LAUNCH();
    mbeta_kernel<<<sb, 128, 0, s>>>(R, pp, sc);
    HZ_CHECK_LAUNCH();
    mp_kernel<<<g, kMT, 0, s>>>(n, sc, re(RV), im(RV), re(P), im(P), re(V), im(V));
    HZ_CHECK_LAUNCH();
    HZ_TRY(A.apply(R, re(P), im(P), re(V), im(V), s));
    mcdot_kernel<<<dim3(kMB, R), kMT, 0, s>>>(n, re(V), im(V), re(RH), im(RH), pp);
    HZ_CHECK_LAUNCH();
    malpha_kernel<<<sb, 128, 0, s>>>(R, pp, sc);
    HZ_CHECK_LAUNCH();
    ms_kernel<<<g, kMT, 0, s>>>(n, sc, re(RV), im(RV), re(V), im(V));
    HZ_CHECK_LAUNCH();
    HZ_TRY(A.apply(R, re(RV), im(RV), re(T), im(T), s));
    mcdot_kernel<<<dim3(kMB, R), kMT, 0, s>>>(n, re(RV), im(RV), re(T), im(T), pp);
    HZ_CHECK_LAUNCH();
    mcdot_kernel<<<dim3(kMB, R), kMT, 0, s>>>(n, re(T), im(T), re(T), im(T), pp2);
    HZ_CHECK_LAUNCH();
    momega_kernel<<<sb, 128, 0, s>>>(R, pp, pp2, sc);
    HZ_CHECK_LAUNCH();
    mupdate_kernel<<<g, kMT, 0, s>>>(n, sc, re(X), im(X), re(RV), im(RV), re(P), im(P), re(T), im(T));
    HZ_CHECK_LAUNCH();
    mcdot_kernel<<<dim3(kMB, R), kMT, 0, s>>>(n, re(RV), im(RV), re(RV), im(RV), pp);
    HZ_CHECK_LAUNCH();
    merr_kernel<<<sb, 128, 0, s>>>(R, pp, sc, tol, stagnation ? 1 : 0, stall, host);
    HZ_CHECK_LAUNCH();
    if (stall > 0) {
        mkeep_kernel<<<g, kMT, 0, s>>>(n, sc, re(X), im(X), re(XB), im(XB));
        HZ_CHECK_LAUNCH();
    }
    return HZ_OK;
}

int KrylovMulti::solve(MultiOp &A, const double *b_re, const double *b_im, double tol, int maxit, bool stagnation,
                       cudaStream_t s, int &iters, std::vector<double> &resid, int stall,
                       std::vector<int> *col_iters)
{
    double *pp = partial.as<double>();
    MScal *sc = scal.as<MScal>();
    const dim3 g(grid_x(n), R);
    const int sb = (R + 127) / 128;
    minit_kernel<<<g, kMT, 0, s>>>(n, b_re, b_im, re(X), im(X), re(RV), im(RV), re(RH), im(RH), re(P), im(P), re(V),
                                   im(V));
    HZ_CHECK_LAUNCH();
    mcdot_kernel<<<dim3(kMB, R), kMT, 0, s>>>(n, re(RV), im(RV), re(RV), im(RV), pp);
    HZ_CHECK_LAUNCH();
    mstart_kernel<<<sb, 128, 0, s>>>(R, pp, sc, host);
    HZ_CHECK_LAUNCH();
    HZ_CHECK_CUDA(cudaStreamSynchronize(s));
    iters = 0;
    resid.assign(R, 0.0);
    if (col_iters) col_iters->assign(R, 0);
    std::vector<int> cols;
    auto active_cols = [&](std::vector<int> &out) {
        out.clear();
        for (int r = 0; r < R; r++)
            if (host[2 * r + 1] > 0) out.push_back(r);
    };
    active_cols(cols);
    if (cols.empty()) return HZ_OK;
    HZ_TRY(A.restrict_to(cols, s));
    std::vector<int> now;
    const int flags = (stagnation ? 1 : 0) | (stall << 1);
    for (int it = 1; it <= maxit; it++) {
        const uint64_t key = A.key();
        if (key) {
            // one BiCGSTAB step per graph launch (captured on first use)
            if (!graph_exec || graph_key != key || graph_stream != s || graph_tol != tol || graph_flags != flags) {
                if (graph_exec) {
                    cudaGraphExecDestroy(graph_exec);
                    graph_exec = nullptr;
                }
                cudaGraph_t g = nullptr;
                HZ_CHECK_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
                const int rc = iteration(A, tol, stagnation, stall, s);
                const cudaError_t ec = cudaStreamEndCapture(s, &g);
                if (rc != HZ_OK) {
                    if (g) cudaGraphDestroy(g);
                    return rc;
                }
                if (ec != cudaSuccess) {
                    set_error("multi right-hand-side solver: graph capture failed: %s", cudaGetErrorString(ec));
                    return HZ_ERR_CUDA;
                }
                const cudaError_t ei = cudaGraphInstantiate(&graph_exec, g, 0);
                cudaGraphDestroy(g);
                if (ei != cudaSuccess) {
                    graph_exec = nullptr;
                    set_error("multi right-hand-side solver: graph instantiation failed: %s", cudaGetErrorString(ei));
                    return HZ_ERR_CUDA;
                }
                graph_key = key;
                graph_stream = s;
                graph_tol = tol;
                graph_flags = flags;
            }
            HZ_CHECK_CUDA(cudaGraphLaunch(graph_exec, s));
        } else {
            HZ_TRY(iteration(A, tol, stagnation, stall, s));
        }
        HZ_CHECK_CUDA(cudaStreamSynchronize(s));
        iters = it;
        for (int r = 0; r < R; r++) resid[r] = host[2 * r];
        if (col_iters)
            for (int r : cols) (*col_iters)[r]++;
        active_cols(now);
        if (now.empty()) break;
        if (now.size() != cols.size()) {
            cols.swap(now);
            HZ_TRY(A.restrict_to(cols, s));
        }
    }
    if (stall > 0) {
        mrestore_kernel<<<g, kMT, 0, s>>>(n, sc, re(X), im(X), re(XB), im(XB));
        HZ_CHECK_LAUNCH();
        mresid_kernel<<<sb, 128, 0, s>>>(R, sc, host);
        HZ_CHECK_LAUNCH();
        HZ_CHECK_CUDA(cudaStreamSynchronize(s));
        for (int r = 0; r < R; r++) resid[r] = host[2 * r];
    }
    return HZ_OK;
}

}  // namespace hz
