// gmres.cu -- restarted GMRES(m) with FP64 vectors on the device.
//
// Needs only A products (no A^H), minimises the residual at every step and
// is therefore insensitive to the small non-linearity of the FP32 sweep
// (densities rounded to FP32), which slows BiCG down as inner solver of the
// iterative refinement.  Orthogonalisation is classical Gram-Schmidt applied
// twice (CGS2): two passes of one block-wide batched product V^H w and one
// update w -= V h, with FP64 sums in a fixed order.  The small Hessenberg
// least-squares problem is solved on the host with complex Givens rotations.
#include "hz_internal.cuh"
#include "krylov.cuh"

#include <cmath>
#include <complex>
#include <vector>

namespace hz {
namespace {

constexpr int kGB = 128;  // partial-sum blocks
constexpr int kGT = 256;
constexpr int kMaxRestart = 128;

// h[j] = sum_i conj(V_j[i]) w[i] for j < k (partials per block)
__global__ void __launch_bounds__(kGT) vh_kernel(int64_t n, int k, const double *__restrict__ vr,
                                                 const double *__restrict__ vi, const double *__restrict__ wr,
                                                 const double *__restrict__ wi, double *partial)
{
    __shared__ double sh[kGT / 32][2];
    for (int j = 0; j < k; j++) {
        const double *a0 = vr + (int64_t)j * n, *a1 = vi + (int64_t)j * n;
        double s0 = 0.0, s1 = 0.0;
        for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
            const double x0 = a0[i], x1 = a1[i], y0 = wr[i], y1 = wi[i];
            s0 += x0 * y0 + x1 * y1;  // conj(v) w
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
            for (int w = 0; w < kGT / 32; w++) {
                a += sh[w][0];
                b += sh[w][1];
            }
            partial[((int64_t)blockIdx.x * kMaxRestart + j) * 2] = a;
            partial[((int64_t)blockIdx.x * kMaxRestart + j) * 2 + 1] = b;
        }
        __syncthreads();
    }
}

// h (k complex) from the partials, summed in block order, into hdev; also
// stored into (accumulate = 0) or added to (accumulate = 1) hsum if given.
__global__ void vh_reduce_kernel(int k, const double *partial, double *hdev, double *hsum, int accumulate)
{
    const int j = threadIdx.x;
    if (j >= k) return;
    double a = 0, b = 0;
    for (int q = 0; q < kGB; q++) {
        a += partial[((int64_t)q * kMaxRestart + j) * 2];
        b += partial[((int64_t)q * kMaxRestart + j) * 2 + 1];
    }
    hdev[2 * j] = a;
    hdev[2 * j + 1] = b;
    if (!hsum) return;
    if (accumulate) {
        hsum[2 * j] += a;
        hsum[2 * j + 1] += b;
    } else {
        hsum[2 * j] = a;
        hsum[2 * j + 1] = b;
    }
}

// w -= sum_j V_j h_j
__global__ void vupdate_kernel(int64_t n, int k, const double *__restrict__ vr, const double *__restrict__ vi,
                               const double *__restrict__ h, double *wr, double *wi)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double a = wr[i], b = wi[i];
        for (int j = 0; j < k; j++) {
            const double x0 = vr[(int64_t)j * n + i], x1 = vi[(int64_t)j * n + i];
            const double h0 = h[2 * j], h1 = h[2 * j + 1];
            a -= x0 * h0 - x1 * h1;
            b -= x0 * h1 + x1 * h0;
        }
        wr[i] = a;
        wi[i] = b;
    }
}

// x += sum_j V_j y_j   (y on the device)
__global__ void xupdate_kernel(int64_t n, int k, const double *__restrict__ vr, const double *__restrict__ vi,
                               const double *__restrict__ y, double *xr, double *xi)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double a = xr[i], b = xi[i];
        for (int j = 0; j < k; j++) {
            const double x0 = vr[(int64_t)j * n + i], x1 = vi[(int64_t)j * n + i];
            a += x0 * y[2 * j] - x1 * y[2 * j + 1];
            b += x0 * y[2 * j + 1] + x1 * y[2 * j];
        }
        xr[i] = a;
        xi[i] = b;
    }
}

__global__ void scale_into_kernel(int64_t n, double s, const double *ar, const double *ai, double *br, double *bi)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        br[i] = s * ar[i];
        bi[i] = s * ai[i];
    }
}

__global__ void sub_into_kernel(int64_t n, const double *ar, const double *ai, const double *br, const double *bi,
                                double *cr, double *ci)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        cr[i] = ar[i] - br[i];
        ci[i] = ai[i] - bi[i];
    }
}

int vblocks(int64_t n)
{
    long long b = (n + 255) / 256;
    if (b > 1184) b = 1184;
    return (int)(b < 1 ? 1 : b);
}

}  // namespace

using cplx = std::complex<double>;

int gmres_solve(LinOp &A, int64_t n, int m, const double *b_re, const double *b_im, double *x_re, double *x_im,
                double tol, int maxit, int stall, DevBuf &work, DevBuf &small, cudaStream_t s, int &iters,
                double &resid, int &products)
{
    products = 0;
    if (m < 2) m = 2;
    if (m > kMaxRestart - 1) m = kMaxRestart - 1;
    // V: (m+1) basis vectors; w; Ax scratch
    HZ_TRY(work.ensure(((size_t)(m + 1) + 2) * 2 * (size_t)n * sizeof(double)));
    HZ_TRY(small.ensure((size_t)kGB * kMaxRestart * 2 * sizeof(double) + 8 * kMaxRestart * sizeof(double) + 64));
    double *V = work.as<double>();
    double *vr = V, *vi = V + (size_t)(m + 1) * n;
    double *wr = V + 2 * (size_t)(m + 1) * n, *wi = wr + n;
    double *tr = wi + n, *ti = tr + n;
    double *partial = small.as<double>();
    double *hdev = partial + (size_t)kGB * kMaxRestart * 2;
    double *hsum = hdev + 2 * kMaxRestart;
    double *ydev = hsum + 2 * kMaxRestart;
    const int vb = vblocks(n);
    std::vector<double> hh(2 * kMaxRestart);
    auto norm2 = [&](const double *ar, const double *ai, double &out) -> int {
        vh_kernel<<<kGB, kGT, 0, s>>>(n, 1, ar, ai, ar, ai, partial);
        HZ_CHECK_LAUNCH();
        vh_reduce_kernel<<<1, kMaxRestart, 0, s>>>(1, partial, hdev, nullptr, 0);
        HZ_CHECK_LAUNCH();
        HZ_CHECK_CUDA(cudaMemcpyAsync(hh.data(), hdev, 2 * sizeof(double), cudaMemcpyDeviceToHost, s));
        HZ_CHECK_CUDA(cudaStreamSynchronize(s));
        out = sqrt(fabs(hh[0]));
        return HZ_OK;
    };
    HZ_CHECK_CUDA(cudaMemsetAsync(x_re, 0, n * sizeof(double), s));
    HZ_CHECK_CUDA(cudaMemsetAsync(x_im, 0, n * sizeof(double), s));
    double normb = 0;
    HZ_TRY(norm2(b_re, b_im, normb));
    iters = 0;
    resid = 0.0;
    if (!(normb > 0)) return HZ_OK;
    double best = 1e300;
    int best_it = 0;
    // r0 = b (x0 = 0)
    HZ_CHECK_CUDA(cudaMemcpyAsync(wr, b_re, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
    HZ_CHECK_CUDA(cudaMemcpyAsync(wi, b_im, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
    bool done = false;
    while (!done && iters < maxit) {
        double beta = 0;
        HZ_TRY(norm2(wr, wi, beta));
        resid = beta / normb;
        if (resid < tol || beta == 0.0) break;
        scale_into_kernel<<<vb, 256, 0, s>>>(n, 1.0 / beta, wr, wi, vr, vi);
        HZ_CHECK_LAUNCH();
        std::vector<cplx> H((size_t)(m + 1) * m, cplx(0, 0)), cs(m), sn(m), g(m + 1, cplx(0, 0));
        g[0] = beta;
        int k = 0;
        for (; k < m && iters < maxit; k++) {
            iters++;
            products++;
            HZ_TRY(A.apply(SWEEP_A, vr + (size_t)k * n, vi + (size_t)k * n, nullptr, nullptr, wr, wi, nullptr, nullptr,
                           s));
            // CGS2 against V_0..V_k
            for (int pass = 0; pass < 2; pass++) {
                vh_kernel<<<kGB, kGT, 0, s>>>(n, k + 1, vr, vi, wr, wi, partial);
                HZ_CHECK_LAUNCH();
                vh_reduce_kernel<<<1, kMaxRestart, 0, s>>>(k + 1, partial, hdev, hsum, pass);
                HZ_CHECK_LAUNCH();
                vupdate_kernel<<<vb, 256, 0, s>>>(n, k + 1, vr, vi, hdev, wr, wi);
                HZ_CHECK_LAUNCH();
            }
            double hn = 0;
            HZ_TRY(norm2(wr, wi, hn));
            HZ_CHECK_CUDA(cudaMemcpyAsync(hh.data(), hsum, 2 * (k + 1) * sizeof(double), cudaMemcpyDeviceToHost, s));
            HZ_CHECK_CUDA(cudaStreamSynchronize(s));
            A.iteration_done(false);
            for (int j = 0; j <= k; j++) H[(size_t)j * m + k] = cplx(hh[2 * j], hh[2 * j + 1]);
            H[(size_t)(k + 1) * m + k] = hn;
            if (hn > 0) {
                scale_into_kernel<<<vb, 256, 0, s>>>(n, 1.0 / hn, wr, wi, vr + (size_t)(k + 1) * n,
                                                     vi + (size_t)(k + 1) * n);
                HZ_CHECK_LAUNCH();
            }
            // previous rotations, then a new one zeroing H[k+1][k]
            for (int j = 0; j < k; j++) {
                const cplx a = H[(size_t)j * m + k], b = H[(size_t)(j + 1) * m + k];
                H[(size_t)j * m + k] = std::conj(cs[j]) * a + std::conj(sn[j]) * b;
                H[(size_t)(j + 1) * m + k] = -sn[j] * a + cs[j] * b;
            }
            const cplx a = H[(size_t)k * m + k], b = H[(size_t)(k + 1) * m + k];
            const double r = std::sqrt(std::norm(a) + std::norm(b));
            cs[k] = (r > 0) ? a / r : cplx(1, 0);
            sn[k] = (r > 0) ? b / r : cplx(0, 0);
            H[(size_t)k * m + k] = r;
            H[(size_t)(k + 1) * m + k] = 0;
            g[k + 1] = -sn[k] * g[k];
            g[k] = std::conj(cs[k]) * g[k];
            resid = std::abs(g[k + 1]) / normb;
            if (resid < best) {
                best = resid;
                best_it = iters;
            }
            if (resid < tol || hn == 0.0 || (stall > 0 && iters - best_it >= (stall > best_it ? stall : best_it))) {
                done = true;
                k++;
                break;
            }
        }
        // y = H^{-1} g (upper triangular k x k), x += V y
        std::vector<cplx> y(k);
        for (int i = k - 1; i >= 0; i--) {
            cplx acc = g[i];
            for (int j = i + 1; j < k; j++) acc -= H[(size_t)i * m + j] * y[j];
            y[i] = acc / H[(size_t)i * m + i];
        }
        std::vector<double> yh(2 * k);
        for (int i = 0; i < k; i++) {
            yh[2 * i] = y[i].real();
            yh[2 * i + 1] = y[i].imag();
        }
        HZ_CHECK_CUDA(cudaMemcpyAsync(ydev, yh.data(), 2 * k * sizeof(double), cudaMemcpyHostToDevice, s));
        xupdate_kernel<<<vb, 256, 0, s>>>(n, k, vr, vi, ydev, x_re, x_im);
        HZ_CHECK_LAUNCH();
        HZ_CHECK_CUDA(cudaStreamSynchronize(s));
        if (done || iters >= maxit) break;
        // restart: w = b - A x
        products++;
        HZ_TRY(A.apply(SWEEP_A, x_re, x_im, nullptr, nullptr, tr, ti, nullptr, nullptr, s));
        sub_into_kernel<<<vb, 256, 0, s>>>(n, b_re, b_im, tr, ti, wr, wi);
        HZ_CHECK_LAUNCH();
        A.iteration_done(false);
    }
    return HZ_OK;
}

}  // namespace hz
