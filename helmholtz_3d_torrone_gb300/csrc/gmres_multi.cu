// gmres_multi.cu -- lockstep restarted GMRES(m) over R right-hand sides.
//
// Column r runs its own Arnoldi process (basis, Hessenberg matrix, Givens
// rotations) exactly as gmres.cu does for one system; what the columns
// share is the product: the k-th basis vectors of every column still
// iterating form one [R][n] block, and one multi right-hand-side pass
// evaluates each pair's kernel once for all of them.  The basis is stored
// as [m+1][R][n] so that block is contiguous.  Orthogonalisation is
// classical Gram-Schmidt applied twice per column (batched kernels over the
// active columns, FP64 sums in a fixed order); the small least-squares
// problems are solved on the host.  A column leaves when its residual
// estimate is below tol (or, with stall > 0, when it has not reached a new
// minimum for max(stall, iterations to its last minimum) iterations): its
// solution is formed at once and the operator is told to skip it.
#include "hz_internal.cuh"
#include "krylov_multi.cuh"

#include <cmath>
#include <complex>
#include <vector>

namespace hz {
namespace {

constexpr int kMB = 64;   // partial-sum blocks per column
constexpr int kMT = 256;
constexpr int kMaxM = 128;

// partial[(c * kMB + blk) * kMaxM + j] (complex) = block sum of
// conj(V_j[col]) w[col] for the c-th active column col = cols[c], j < k.
// Launched with exactly kMB blocks in x, so every partial slot is written.
__global__ void __launch_bounds__(kMT) mvh_kernel(int64_t n, int R, int k, const int *__restrict__ cols,
                                                  const double *__restrict__ vr, const double *__restrict__ vi,
                                                  const double *__restrict__ wr, const double *__restrict__ wi,
                                                  double *partial)
{
    __shared__ double sh[kMT / 32][2];
    const int c = blockIdx.y, col = cols[c];
    const double *w0 = wr + (int64_t)col * n, *w1 = wi + (int64_t)col * n;
    for (int j = 0; j < k; j++) {
        const double *a0 = vr + ((int64_t)j * R + col) * n, *a1 = vi + ((int64_t)j * R + col) * n;
        double s0 = 0.0, s1 = 0.0;
        for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
            const double x0 = a0[i], x1 = a1[i], y0 = w0[i], y1 = w1[i];
            s0 += x0 * y0 + x1 * y1;
            s1 += x0 * y1 - x1 * y0;
        }
        for (int o = 16; o > 0; o >>= 1) {
            s0 += __shfl_down_sync(0xffffffffu, s0, o);
            s1 += __shfl_down_sync(0xffffffffu, s1, o);
        }
        if ((threadIdx.x & 31) == 0) {
            sh[threadIdx.x >> 5][0] = s0;
            sh[threadIdx.x >> 5][1] = s1;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            double a = 0, b = 0;
            for (int q = 0; q < kMT / 32; q++) {
                a += sh[q][0];
                b += sh[q][1];
            }
            double *p = partial + (((int64_t)c * kMB + blockIdx.x) * kMaxM + j) * 2;
            p[0] = a;
            p[1] = b;
        }
        __syncthreads();
    }
}

// h[c][j] from the partials in block order; also into (pass 0) or added to
// (pass 1) hsum[c][j].
__global__ void mvh_reduce_kernel(int k, const double *partial, double *h, double *hsum, int pass)
{
    const int c = blockIdx.x, j = threadIdx.x;
    if (j >= k) return;
    double a = 0, b = 0;
    for (int q = 0; q < kMB; q++) {
        const double *p = partial + (((int64_t)c * kMB + q) * kMaxM + j) * 2;
        a += p[0];
        b += p[1];
    }
    double *o = h + ((int64_t)c * kMaxM + j) * 2, *t = hsum + ((int64_t)c * kMaxM + j) * 2;
    o[0] = a;
    o[1] = b;
    if (pass) {
        t[0] += a;
        t[1] += b;
    } else {
        t[0] = a;
        t[1] = b;
    }
}

// w[col] -= sum_j V_j[col] h[c][j]
__global__ void mvupdate_kernel(int64_t n, int R, int k, const int *__restrict__ cols, const double *__restrict__ vr,
                                const double *__restrict__ vi, const double *__restrict__ h, double *wr, double *wi)
{
    const int c = blockIdx.y, col = cols[c];
    const double *hc = h + (int64_t)c * kMaxM * 2;
    double *w0 = wr + (int64_t)col * n, *w1 = wi + (int64_t)col * n;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double a = w0[i], b = w1[i];
        for (int j = 0; j < k; j++) {
            const double x0 = vr[((int64_t)j * R + col) * n + i], x1 = vi[((int64_t)j * R + col) * n + i];
            const double h0 = hc[2 * j], h1 = hc[2 * j + 1];
            a -= x0 * h0 - x1 * h1;
            b -= x0 * h1 + x1 * h0;
        }
        w0[i] = a;
        w1[i] = b;
    }
}

// V_{k}[col] = w[col] / nrm[c]  (nrm[c] > 0; else left as is)
__global__ void mscale_kernel(int64_t n, int R, int k, const int *__restrict__ cols, const double *__restrict__ nrm,
                              const double *__restrict__ wr, const double *__restrict__ wi, double *vr, double *vi)
{
    const int c = blockIdx.y, col = cols[c];
    const double s = nrm[c];
    if (!(s > 0)) return;
    const double inv = 1.0 / s;
    const double *w0 = wr + (int64_t)col * n, *w1 = wi + (int64_t)col * n;
    double *v0 = vr + ((int64_t)k * R + col) * n, *v1 = vi + ((int64_t)k * R + col) * n;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        v0[i] = inv * w0[i];
        v1[i] = inv * w1[i];
    }
}

// x[col] += sum_j V_j[col] y_j  (y: kMaxM complex per column slot c)
__global__ void mxupdate_kernel(int64_t n, int R, int k, const int *__restrict__ cols, const double *__restrict__ vr,
                                const double *__restrict__ vi, const double *__restrict__ y, double *xr, double *xi)
{
    const int c = blockIdx.y, col = cols[c];
    const double *yc = y + (int64_t)c * kMaxM * 2;
    double *x0 = xr + (int64_t)col * n, *x1 = xi + (int64_t)col * n;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double a = x0[i], b = x1[i];
        for (int j = 0; j < k; j++) {
            const double v0 = vr[((int64_t)j * R + col) * n + i], v1 = vi[((int64_t)j * R + col) * n + i];
            a += v0 * yc[2 * j] - v1 * yc[2 * j + 1];
            b += v0 * yc[2 * j + 1] + v1 * yc[2 * j];
        }
        x0[i] = a;
        x1[i] = b;
    }
}

// w[col] = b[col] - t[col]
__global__ void msub_kernel(int64_t n, const int *__restrict__ cols, const double *br, const double *bi,
                            const double *tr, const double *ti, double *wr, double *wi)
{
    const int64_t off = (int64_t)cols[blockIdx.y] * n;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        wr[off + i] = br[off + i] - tr[off + i];
        wi[off + i] = bi[off + i] - ti[off + i];
    }
}

int mblocks(int64_t n)
{
    long long b = (n + kMT - 1) / kMT;
    if (b > kMB) b = kMB;
    return (int)(b < 1 ? 1 : b);
}

using cplx = std::complex<double>;

// Per-column Arnoldi state on the host.
struct Col {
    std::vector<cplx> H, cs, sn, g;
    double normb = 0, best = 1e300, resid = 0;
    int best_it = 0, its = 0;
    bool active = false;
};

}  // namespace

size_t gmres_multi_work_bytes(int64_t n, int R, int m)
{
    if (m > kMaxM - 1) m = kMaxM - 1;
    return ((size_t)(m + 1) + 2) * 2 * (size_t)R * (size_t)n * sizeof(double);
}

int gmres_multi_solve(MultiOp &A, int64_t n, int R, int m, const double *b_re, const double *b_im, double *x_re,
                      double *x_im, double tol, int maxit, int stall, DevBuf &work, DevBuf &small, cudaStream_t s,
                      int &iters, std::vector<double> &resid, std::vector<int> *col_iters)
{
    if (m < 2) m = 2;
    if (m > kMaxM - 1) m = kMaxM - 1;
    const size_t RN = (size_t)R * n;
    HZ_TRY(work.ensure(gmres_multi_work_bytes(n, R, m)));
    const size_t part = (size_t)R * kMB * kMaxM * 2, hsz = (size_t)R * kMaxM * 2;
    HZ_TRY(small.ensure((part + 3 * hsz + 2 * (size_t)R) * sizeof(double) + (size_t)R * sizeof(int) + 256));
    double *vr = work.as<double>(), *vi = vr + (size_t)(m + 1) * RN;
    double *wr = vi + (size_t)(m + 1) * RN, *wi = wr + RN;
    double *tr = wi + RN, *ti = tr + RN;
    double *partial = small.as<double>();
    double *hdev = partial + part, *hsum = hdev + hsz, *ydev = hsum + hsz;
    double *ndev = ydev + hsz;
    int *cdev = reinterpret_cast<int *>(ndev + 2 * R);
    const int gx = mblocks(n);
    std::vector<double> hh(hsz), hn_host(hsz), nrm(R);
    std::vector<Col> C(R);
    std::vector<int> act;  // active columns (device list order)
    iters = 0;
    resid.assign(R, 0.0);
    if (col_iters) col_iters->assign(R, 0);
    HZ_CHECK_CUDA(cudaMemsetAsync(x_re, 0, RN * sizeof(double), s));
    HZ_CHECK_CUDA(cudaMemsetAsync(x_im, 0, RN * sizeof(double), s));
    HZ_CHECK_CUDA(cudaMemcpyAsync(wr, b_re, RN * sizeof(double), cudaMemcpyDeviceToDevice, s));
    HZ_CHECK_CUDA(cudaMemcpyAsync(wi, b_im, RN * sizeof(double), cudaMemcpyDeviceToDevice, s));
    // ||w[col]|| for the columns in act (into nrm[col])
    auto norms = [&](const std::vector<int> &cl) -> int {
        if (cl.empty()) return HZ_OK;
        const int a = (int)cl.size();
        HZ_CHECK_CUDA(cudaMemcpyAsync(cdev, cl.data(), a * sizeof(int), cudaMemcpyHostToDevice, s));
        // conj(w) w: the basis pointer is w itself at "j = 0" with R = 0 stride
        mvh_kernel<<<dim3(kMB, a), kMT, 0, s>>>(n, 0, 1, cdev, wr, wi, wr, wi, partial);
        HZ_CHECK_LAUNCH();
        mvh_reduce_kernel<<<a, kMaxM, 0, s>>>(1, partial, hdev, hsum, 0);
        HZ_CHECK_LAUNCH();
        HZ_CHECK_CUDA(cudaMemcpyAsync(hn_host.data(), hdev, (size_t)a * kMaxM * 2 * sizeof(double),
                                      cudaMemcpyDeviceToHost, s));
        HZ_CHECK_CUDA(cudaStreamSynchronize(s));
        for (int c = 0; c < a; c++) nrm[cl[c]] = std::sqrt(std::fabs(hn_host[(size_t)c * kMaxM * 2]));
        return HZ_OK;
    };
    std::vector<int> all(R);
    for (int r = 0; r < R; r++) all[r] = r;
    HZ_TRY(norms(all));
    for (int r = 0; r < R; r++) {
        C[r].normb = nrm[r];
        C[r].active = nrm[r] > 0;
    }
    // Form x[col] += V y for the columns in `done` (their current cycle of k
    // steps), from the host rotations.
    auto finish = [&](const std::vector<int> &done, const std::vector<int> &ks) -> int {
        if (done.empty()) return HZ_OK;
        const int a = (int)done.size();
        std::vector<double> yh((size_t)a * kMaxM * 2, 0.0);
        int kmax = 0;
        for (int c = 0; c < a; c++) {
            const Col &q = C[done[c]];
            const int k = ks[c];
            kmax = k > kmax ? k : kmax;
            std::vector<cplx> y(k);
            for (int i = k - 1; i >= 0; i--) {
                cplx acc = q.g[i];
                for (int j = i + 1; j < k; j++) acc -= q.H[(size_t)i * m + j] * y[j];
                y[i] = acc / q.H[(size_t)i * m + i];
            }
            for (int i = 0; i < k; i++) {
                yh[((size_t)c * kMaxM + i) * 2] = y[i].real();
                yh[((size_t)c * kMaxM + i) * 2 + 1] = y[i].imag();
            }
        }
        HZ_CHECK_CUDA(cudaMemcpyAsync(ydev, yh.data(), yh.size() * sizeof(double), cudaMemcpyHostToDevice, s));
        HZ_CHECK_CUDA(cudaMemcpyAsync(cdev, done.data(), a * sizeof(int), cudaMemcpyHostToDevice, s));
        // ks differ only when a column stopped early; the shorter ones have
        // y_j = 0 beyond their k
        mxupdate_kernel<<<dim3(gx, a), kMT, 0, s>>>(n, R, kmax, cdev, vr, vi, ydev, x_re, x_im);
        HZ_CHECK_LAUNCH();
        HZ_CHECK_CUDA(cudaStreamSynchronize(s));
        return HZ_OK;
    };
    while (iters < maxit) {
        // start (or restart) a cycle for every active column: beta = ||w||
        act.clear();
        for (int r = 0; r < R; r++)
            if (C[r].active) act.push_back(r);
        if (act.empty()) break;
        HZ_TRY(norms(act));
        std::vector<int> go;
        for (int r : act) {
            Col &q = C[r];
            q.resid = nrm[r] / q.normb;
            resid[r] = q.resid;
            if (q.resid < tol || nrm[r] == 0.0) {
                q.active = false;
                continue;
            }
            q.H.assign((size_t)(m + 1) * m, cplx(0, 0));
            q.cs.assign(m, cplx(0, 0));
            q.sn.assign(m, cplx(0, 0));
            q.g.assign(m + 1, cplx(0, 0));
            q.g[0] = nrm[r];
            go.push_back(r);
        }
        if (go.empty()) break;
        {
            std::vector<double> nv(go.size());
            for (size_t c = 0; c < go.size(); c++) nv[c] = nrm[go[c]];
            HZ_CHECK_CUDA(cudaMemcpyAsync(ndev, nv.data(), nv.size() * sizeof(double), cudaMemcpyHostToDevice, s));
            HZ_CHECK_CUDA(cudaMemcpyAsync(cdev, go.data(), go.size() * sizeof(int), cudaMemcpyHostToDevice, s));
            mscale_kernel<<<dim3(gx, (unsigned)go.size()), kMT, 0, s>>>(n, R, 0, cdev, ndev, wr, wi, vr, vi);
            HZ_CHECK_LAUNCH();
        }
        std::vector<int> cyc = go;  // columns of this cycle still iterating
        std::vector<int> kdone(R, 0);
        int k = 0;
        for (; k < m && iters < maxit && !cyc.empty(); k++) {
            iters++;
            HZ_TRY(A.restrict_to(cyc, s));
            HZ_TRY(A.apply(R, vr + (size_t)k * RN, vi + (size_t)k * RN, wr, wi, s));
            const int a = (int)cyc.size();
            HZ_CHECK_CUDA(cudaMemcpyAsync(cdev, cyc.data(), a * sizeof(int), cudaMemcpyHostToDevice, s));
            for (int pass = 0; pass < 2; pass++) {
                mvh_kernel<<<dim3(kMB, a), kMT, 0, s>>>(n, R, k + 1, cdev, vr, vi, wr, wi, partial);
                HZ_CHECK_LAUNCH();
                mvh_reduce_kernel<<<a, kMaxM, 0, s>>>(k + 1, partial, hdev, hsum, pass);
                HZ_CHECK_LAUNCH();
                mvupdate_kernel<<<dim3(gx, a), kMT, 0, s>>>(n, R, k + 1, cdev, vr, vi, hdev, wr, wi);
                HZ_CHECK_LAUNCH();
            }
            HZ_CHECK_CUDA(cudaMemcpyAsync(hh.data(), hsum, (size_t)a * kMaxM * 2 * sizeof(double),
                                          cudaMemcpyDeviceToHost, s));
            HZ_TRY(norms(cyc));  // synchronises: hh (the h of this step) and nrm are ready
            const std::vector<double> &hs = hh;
            std::vector<int> keep, stop, stop_k;
            for (int c = 0; c < a; c++) {
                const int r = cyc[c];
                Col &q = C[r];
                q.its++;
                if (col_iters) (*col_iters)[r]++;
                const double hn = nrm[r];
                for (int j = 0; j <= k; j++)
                    q.H[(size_t)j * m + k] = cplx(hs[((size_t)c * kMaxM + j) * 2], hs[((size_t)c * kMaxM + j) * 2 + 1]);
                q.H[(size_t)(k + 1) * m + k] = hn;
                for (int j = 0; j < k; j++) {
                    const cplx x = q.H[(size_t)j * m + k], y = q.H[(size_t)(j + 1) * m + k];
                    q.H[(size_t)j * m + k] = std::conj(q.cs[j]) * x + std::conj(q.sn[j]) * y;
                    q.H[(size_t)(j + 1) * m + k] = -q.sn[j] * x + q.cs[j] * y;
                }
                const cplx x = q.H[(size_t)k * m + k], y = q.H[(size_t)(k + 1) * m + k];
                const double rr = std::sqrt(std::norm(x) + std::norm(y));
                q.cs[k] = (rr > 0) ? x / rr : cplx(1, 0);
                q.sn[k] = (rr > 0) ? y / rr : cplx(0, 0);
                q.H[(size_t)k * m + k] = rr;
                q.H[(size_t)(k + 1) * m + k] = 0;
                q.g[k + 1] = -q.sn[k] * q.g[k];
                q.g[k] = std::conj(q.cs[k]) * q.g[k];
                q.resid = std::abs(q.g[k + 1]) / q.normb;
                resid[r] = q.resid;
                if (q.resid < q.best) {
                    q.best = q.resid;
                    q.best_it = q.its;
                }
                const bool stalled = stall > 0 && q.its - q.best_it >= (stall > q.best_it ? stall : q.best_it);
                if (q.resid < tol || hn == 0.0 || stalled) {
                    q.active = false;
                    stop.push_back(r);
                    stop_k.push_back(k + 1);
                } else {
                    keep.push_back(r);
                }
            }
            // next basis vectors of the columns that go on
            if (!keep.empty()) {
                std::vector<double> nv(keep.size());
                for (size_t c = 0; c < keep.size(); c++) nv[c] = nrm[keep[c]];
                HZ_CHECK_CUDA(cudaMemcpyAsync(ndev, nv.data(), nv.size() * sizeof(double), cudaMemcpyHostToDevice, s));
                HZ_CHECK_CUDA(cudaMemcpyAsync(cdev, keep.data(), keep.size() * sizeof(int), cudaMemcpyHostToDevice, s));
                mscale_kernel<<<dim3(gx, (unsigned)keep.size()), kMT, 0, s>>>(n, R, k + 1, cdev, ndev, wr, wi, vr, vi);
                HZ_CHECK_LAUNCH();
            }
            HZ_TRY(finish(stop, stop_k));
            cyc.swap(keep);
        }
        // end of the cycle: the columns still iterating form their x and, if
        // the cycle ran out, restart from w = b - A x
        if (!cyc.empty()) {
            std::vector<int> ks(cyc.size(), k);
            HZ_TRY(finish(cyc, ks));
            if (iters >= maxit) break;
            HZ_TRY(A.restrict_to(cyc, s));
            HZ_TRY(A.apply(R, x_re, x_im, tr, ti, s));
            HZ_CHECK_CUDA(cudaMemcpyAsync(cdev, cyc.data(), cyc.size() * sizeof(int), cudaMemcpyHostToDevice, s));
            msub_kernel<<<dim3(gx, (unsigned)cyc.size()), kMT, 0, s>>>(n, cdev, b_re, b_im, tr, ti, wr, wi);
            HZ_CHECK_LAUNCH();
        }
    }
    return HZ_OK;
}

}  // namespace hz
