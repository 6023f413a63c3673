// evaluate.cu -- off-surface field at receivers, boundary data at the tube
// points, and the dense complex matvec behind the CompBiCG drop-in.
#include "hz_internal.cuh"

namespace hz {
namespace {

constexpr int kEvalThreads = 256;

// One block per receiver; sources strided over the block, FP64, reduced in
// a fixed order.  Single layer: NeumannTest (large3Dexample2.c:1810-1824),
//   u += (-Phi) sigma w with -Phi = (cos(k r) + i sin(k r)) / (-4 pi r);
// double layer: the Dirichlet matrix's kernel (:4471-4497) off the surface,
//   u += sg (ct1 + i ct2) ((x - x_p).n_p) sigma w.
// Pairs with r <= tau are skipped, as in the reference.
__global__ void __launch_bounds__(kEvalThreads) eval_kernel(int64_t n, const double4_32a *__restrict__ pos,
                                                            const double4_32a *__restrict__ nrm,
                                                            const double *__restrict__ s_re,
                                                            const double *__restrict__ s_im,
                                                            const double *__restrict__ rx, double wave, double tau,
                                                            double sg, int layer, double *u_re, double *u_im)
{
    const double PI = 3.14159265358979323846264338328;
    const double c4 = 1. / (4. * PI);
    const int64_t r = blockIdx.x;
    const double sx = rx[3 * r], sy = rx[3 * r + 1], sz = rx[3 * r + 2];
    double ur = 0.0, ui = 0.0;
    for (int64_t c = threadIdx.x; c < n; c += blockDim.x) {
        const double4_32a p = pos[c];
        const double4_32a q = nrm[c];
        const double zx = p.x, zy = p.y, zz = p.z;
        const double sn = sqrt((zx - sx) * (zx - sx) + (zy - sy) * (zy - sy) + (zz - sz) * (zz - sz));
        if (!(sn > tau)) continue;
        double ph, phi;
        double S, C;
        sincos(wave * sn, &S, &C);
        if (layer == HZ_SINGLE_LAYER) {
            ph = C / (-4. * PI * sn);
            phi = S / (-4. * PI * sn);
        } else {
            const double xmy1 = sx - zx, xmy2 = sy - zy, xmy3 = sz - zz;
            const double rec = 1. / sn;
            const double denom = c4 * rec * rec;
            const double ct1 = -1. * (wave * S + C * rec) * denom;
            const double ct2 = (wave * C - S * rec) * denom;
            const double in = xmy1 * q.x + xmy2 * q.y + xmy3 * q.z;
            ph = sg * ct1 * in;
            phi = sg * ct2 * in;
        }
        const double w = q.w, a = s_re[c], b = s_im[c];
        ur += ((ph * a - phi * b) * w);
        ui += ((ph * b + phi * a) * w);
    }
    __shared__ double sh[2][kEvalThreads / 32];
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
        double a = 0.0, b = 0.0;
        for (int w = 0; w < kEvalThreads / 32; w++) {
            a += sh[0][w];
            b += sh[1][w];
        }
        u_re[r] = a;
        u_im[r] = b;
    }
}

// Boundary data at projected points (see HZ_RHS_*).
__global__ void rhs_kernel(int64_t n, const double4_32a *__restrict__ pos, const double4_32a *__restrict__ nrm, double sx,
                           double sy, double sz, double W, int kind, double *b_re, double *b_im)
{
    const double PI = 3.14159265358979323846264338328;
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x) {
        const double4_32a p = pos[c], q = nrm[c];
        const double dx = p.x - sx, dy = p.y - sy, dz = p.z - sz;
        const double r = sqrt(dx * dx + dy * dy + dz * dz);
        double S, C;
        sincos(W * r, &S, &C);
        double re, im;
        if (kind == HZ_RHS_POINT_DIRICHLET) {
            re = C / (4. * PI * r);
            im = S / (4. * PI * r);
        } else if (kind == HZ_RHS_POINT_NEUMANN) {
            const double dn = -(dx * q.x + dy * q.y + dz * q.z) / r;
            const double gr = (-C - W * r * S) / (4. * PI * r * r);
            const double gi = (W * r * C - S) / (4. * PI * r * r);
            re = gr * dn;
            im = gi * dn;
        } else if (kind == HZ_RHS_MONOPOLE_NEUMANN) {
            re = (S / r) + (C / (W * r * r));
            im = (S / (W * r * r)) - (C / r);
        } else {
            re = -1.0 * C / (W * r);
            im = -1.0 * S / (W * r);
        }
        b_re[c] = re;
        b_im[c] = im;
    }
}

// Receivers on a plane and a mask from the trilinearly interpolated
// distance grid (1 = keep, 0 = inside or within mask of the surface).
__global__ void slice_points_kernel(int axis, double c, int n2, double lo, double h2, double mask, int N, double H,
                                    double int_l, const double *__restrict__ d, double *rx, unsigned char *keep)
{
    const int64_t total = (int64_t)n2 * n2;
    const long long S = N + 1;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < total; q += (int64_t)gridDim.x * blockDim.x) {
        const int a = (int)(q / n2), b = (int)(q % n2);
        const double u = lo + a * h2, v = lo + b * h2;
        double x, y, z;
        if (axis == 0) { x = c; y = u; z = v; }
        else if (axis == 1) { x = u; y = c; z = v; }
        else { x = u; y = v; z = c; }
        rx[3 * q] = x;
        rx[3 * q + 1] = y;
        rx[3 * q + 2] = z;
        int i = (int)floor((y - int_l) / H), j = (int)floor((x - int_l) / H), k = (int)floor((z - int_l) / H);
        unsigned char kp = 1;
        if (i >= 0 && j >= 0 && k >= 0 && i < N && j < N && k < N) {
            const double ly = (y - int_l) / H - i, lx = (x - int_l) / H - j, lz = (z - int_l) / H - k;
            const long long o = ((long long)i * S + j) * S + k;
            double acc = 0.0;
            for (int di = 0; di < 2; di++)
                for (int dj = 0; dj < 2; dj++)
                    for (int dk = 0; dk < 2; dk++) {
                        const double wgt = (di ? ly : 1 - ly) * (dj ? lx : 1 - lx) * (dk ? lz : 1 - lz);
                        acc += wgt * d[o + di * S * S + dj * S + dk];
                    }
            if (acc > -mask) kp = 0;
        }
        keep[q] = kp;
    }
}

__global__ void apply_mask_kernel(int64_t m, const unsigned char *__restrict__ keep, double *u_re, double *u_im)
{
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < m; q += (int64_t)gridDim.x * blockDim.x)
        if (!keep[q]) {
            u_re[q] = 0.0;
            u_im[q] = 0.0;
        }
}

// Incident plane waves u = e^{ik d.x} at the projected points, one column
// [ndir][n] per direction: Dirichlet data (kind 0) or its derivative along
// the outward normal -n (kind 1).
__global__ void plane_wave_kernel(int64_t n, const double4_32a *__restrict__ pos, const double4_32a *__restrict__ nrm,
                                  int ndir, const double *__restrict__ dirs, double W, int kind, double *b_re,
                                  double *b_im)
{
    const int r = blockIdx.y;
    const double dx = dirs[3 * r], dy = dirs[3 * r + 1], dz = dirs[3 * r + 2];
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x) {
        const double4_32a p = pos[c];
        double S, C;
        sincos(W * (dx * p.x + dy * p.y + dz * p.z), &S, &C);
        double re = C, im = S;
        if (kind == HZ_RHS_POINT_NEUMANN) {
            const double4_32a q = nrm[c];
            const double dn = -(dx * q.x + dy * q.y + dz * q.z);  // d . n_out
            re = -W * dn * S;                                     // i k (d.n_out) e^{ik d.x}
            im = W * dn * C;
        }
        b_re[(int64_t)r * n + c] = re;
        b_im[(int64_t)r * n + c] = im;
    }
}

// Dense complex products on a row-major n x n matrix (real and imaginary
// parts), large3Dexample2.c:3262-3309: q = A p and qt = A^H pt in one pass
// over A.  A block owns kDenseRows rows; each warp walks its rows with
// coalesced column loads, and A^H contributions for the block's rows are
// written to partial[row_block][col] and reduced in a second, ordered pass.
constexpr int kDenseRows = 32;

__global__ void dense_rows_kernel(int64_t n, const double *__restrict__ are, const double *__restrict__ aim,
                                  const double *__restrict__ p_re, const double *__restrict__ p_im,
                                  const double *__restrict__ pt_re, const double *__restrict__ pt_im,
                                  double *__restrict__ q_re, double *__restrict__ q_im,
                                  double *__restrict__ part_re, double *__restrict__ part_im, int do_a, int do_adj)
{
    const int64_t r0 = (int64_t)blockIdx.x * kDenseRows;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int nwarps = blockDim.x >> 5;
    // A p: one warp per row
    for (int rr = warp; do_a && rr < kDenseRows; rr += nwarps) {
        const int64_t row = r0 + rr;
        if (row >= n) break;
        const double *ar = are + row * n, *ai = aim + row * n;
        double sr = 0.0, si = 0.0;
        for (int64_t k = lane; k < n; k += 32) {
            const double a = ar[k], b = ai[k];
            sr += (a * p_re[k] - b * p_im[k]);
            si += (a * p_im[k] + b * p_re[k]);
        }
        for (int o = 16; o > 0; o >>= 1) {
            sr += __shfl_down_sync(0xffffffffu, sr, o);
            si += __shfl_down_sync(0xffffffffu, si, o);
        }
        if (lane == 0) {
            q_re[row] = sr;
            q_im[row] = si;
        }
    }
    if (!do_adj) return;
    // A^H pt partials: column k accumulates conj(A[row][k]) pt[row] over the block's rows
    for (int64_t k = threadIdx.x; k < n; k += blockDim.x) {
        double sr = 0.0, si = 0.0;
        for (int rr = 0; rr < kDenseRows; rr++) {
            const int64_t row = r0 + rr;
            if (row >= n) break;
            const double a = are[row * n + k], b = aim[row * n + k];
            sr += (a * pt_re[row] + b * pt_im[row]);
            si += (a * pt_im[row] - b * pt_re[row]);
        }
        part_re[(int64_t)blockIdx.x * n + k] = sr;
        part_im[(int64_t)blockIdx.x * n + k] = si;
    }
}

__global__ void dense_adj_reduce_kernel(int64_t n, int64_t nblk, const double *__restrict__ part_re,
                                        const double *__restrict__ part_im, double *qt_re, double *qt_im)
{
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
        double sr = 0.0, si = 0.0;
        for (int64_t b = 0; b < nblk; b++) {
            sr += part_re[b * n + k];
            si += part_im[b * n + k];
        }
        qt_re[k] = sr;
        qt_im[k] = si;
    }
}

}  // namespace

int launch_eval(int64_t n, const double4_32a *pos, const double4_32a *nrm, const double *s_re, const double *s_im,
                int64_t m, const double *rx, double wave, double tau, int interior, int layer, double *u_re,
                double *u_im, cudaStream_t s)
{
    if (m <= 0) return HZ_OK;
    if (m > 0x7fffffffLL) {
        set_error("hz_eval: too many receivers");
        return HZ_ERR_ARG;
    }
    eval_kernel<<<(unsigned)m, kEvalThreads, 0, s>>>(n, pos, nrm, s_re, s_im, rx, wave, tau,
                                                     interior == 1 ? -1.0 : 1.0, layer, u_re, u_im);
    HZ_CHECK_LAUNCH();
    return HZ_OK;
}

int launch_rhs(int64_t n, const double4_32a *pos, const double4_32a *nrm, const double *src, double wave, int kind,
               double *b_re, double *b_im, cudaStream_t s)
{
    if (n <= 0) return HZ_OK;
    long long b = (n + 255) / 256;
    if (b > 4096) b = 4096;
    rhs_kernel<<<(unsigned)b, 256, 0, s>>>(n, pos, nrm, src[0], src[1], src[2], wave, kind, b_re, b_im);
    HZ_CHECK_LAUNCH();
    return HZ_OK;
}

int launch_plane_waves(int64_t n, const double4_32a *pos, const double4_32a *nrm, int ndir, const double *dirs,
                       double wave, int kind, double *b_re, double *b_im, cudaStream_t s)
{
    if (n <= 0) return HZ_OK;
    long long b = (n + 255) / 256;
    if (b > 256) b = 256;
    plane_wave_kernel<<<dim3((unsigned)b, (unsigned)ndir), 256, 0, s>>>(n, pos, nrm, ndir, dirs, wave, kind, b_re, b_im);
    HZ_CHECK_LAUNCH();
    return HZ_OK;
}

int launch_slice(int axis, double c, int n2, double lo, double h2, double mask, int N, double H, double int_l,
                 const double *d, double *rx, unsigned char *keep, cudaStream_t s)
{
    const int64_t total = (int64_t)n2 * n2;
    long long b = (total + 255) / 256;
    if (b > 4096) b = 4096;
    slice_points_kernel<<<(unsigned)b, 256, 0, s>>>(axis, c, n2, lo, h2, mask, N, H, int_l, d, rx, keep);
    HZ_CHECK_LAUNCH();
    return HZ_OK;
}

int launch_mask(int64_t m, const unsigned char *keep, double *u_re, double *u_im, cudaStream_t s)
{
    long long b = (m + 255) / 256;
    if (b > 4096) b = 4096;
    apply_mask_kernel<<<(unsigned)b, 256, 0, s>>>(m, keep, u_re, u_im);
    HZ_CHECK_LAUNCH();
    return HZ_OK;
}

size_t dense_partial_elems(int64_t n) { return (size_t)((n + kDenseRows - 1) / kDenseRows) * (size_t)n; }

int launch_dense(int64_t n, const double *are, const double *aim, const double *p_re, const double *p_im,
                 const double *pt_re, const double *pt_im, double *q_re, double *q_im, double *qt_re,
                 double *qt_im, double *part_re, double *part_im, cudaStream_t s)
{
    const int64_t nblk = (n + kDenseRows - 1) / kDenseRows;
    const int do_adj = (pt_re != nullptr), do_a = (p_re != nullptr);
    dense_rows_kernel<<<(unsigned)nblk, 256, 0, s>>>(n, are, aim, p_re, p_im, pt_re, pt_im, q_re, q_im, part_re,
                                                      part_im, do_a, do_adj);
    HZ_CHECK_LAUNCH();
    if (do_adj) {
        long long b = (n + 255) / 256;
        if (b > 4096) b = 4096;
        dense_adj_reduce_kernel<<<(unsigned)b, 256, 0, s>>>(n, nblk, part_re, part_im, qt_re, qt_im);
        HZ_CHECK_LAUNCH();
    }
    return HZ_OK;
}

}  // namespace hz
