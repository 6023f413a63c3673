// ref_api.cu -- the reference's library entry points with their original
// signatures (include/helmholtz_ref_api.h), backed by the device kernels.
// Ragged host arrays are gathered into contiguous staging buffers, the
// whole-grid / whole-matrix work runs on the GPU, and results are scattered
// back into the caller's arrays.
#include "hz_internal.cuh"
#include "../../include/helmholtz_ref_api.h"

#include <vector>

namespace {

int gather_grid(double ***g, int S, std::vector<double> &out)
{
    if (!g) return HZ_ERR_ARG;
    out.resize((size_t)S * S * S);
    for (int i = 0; i < S; i++) {
        if (!g[i]) return HZ_ERR_ARG;
        for (int j = 0; j < S; j++) {
            if (!g[i][j]) return HZ_ERR_ARG;
            memcpy(out.data() + ((size_t)i * S + j) * S, g[i][j], S * sizeof(double));
        }
    }
    return HZ_OK;
}

int scatter_grid(const std::vector<double> &in, int S, double ***g)
{
    if (!g) return HZ_ERR_ARG;
    for (int i = 0; i < S; i++) {
        if (!g[i]) return HZ_ERR_ARG;
        for (int j = 0; j < S; j++) {
            if (!g[i][j]) return HZ_ERR_ARG;
            memcpy(g[i][j], in.data() + ((size_t)i * S + j) * S, S * sizeof(double));
        }
    }
    return HZ_OK;
}

int dense_bicg_ragged(int size, double *density, double *densityimg, double **K, double **Ki, double *b,
                      double *bimg, int maxit)
{
    if (size < 1 || !density || !densityimg || !K || !Ki || !b || !bimg) {
        hz::set_error("CompBiCG: bad arguments");
        return HZ_ERR_ARG;
    }
    const size_t n = (size_t)size;
    std::vector<double> are(n * n), aim(n * n);
    for (size_t i = 0; i < n; i++) {
        if (!K[i] || !Ki[i]) {
            hz::set_error("CompBiCG: NULL matrix row %zu", i);
            return HZ_ERR_ARG;
        }
        memcpy(are.data() + i * n, K[i], n * sizeof(double));
        memcpy(aim.data() + i * n, Ki[i], n * sizeof(double));
    }
    hz_solve_info info;
    // BICGSTAB.h:12 DEFAULTACC (hz_ref_config.bicg_acc)
    hz_ref_config c;
    hz_ref_get_config(&c);
    return hz_dense_bicg((int64_t)n, are.data(), aim.data(), b, bimg, density, densityimg, c.bicg_acc, maxit,
                         HZ_HOST, &info);
}

}  // namespace

int ASSIGN_GRADIENT(int N, double H, double ***dist, double ***graddx, double ***graddy, double ***graddz,
                    int weno_mode)
{
    if (weno_mode != 3 && weno_mode != 5) {
        hz::set_error("ASSIGN_GRADIENT: weno_mode %d not supported (3 or 5)", weno_mode);
        return HZ_ERR_ARG;
    }
    const int S = N + 1;
    std::vector<double> d, gx(0), gy(0), gz(0);
    if (gather_grid(dist, S, d) != HZ_OK) {
        hz::set_error("ASSIGN_GRADIENT: ragged distance grid has NULL rows");
        return HZ_ERR_ARG;
    }
    gx.resize(d.size());
    gy.resize(d.size());
    gz.resize(d.size());
    HZ_TRY(hz_assign_gradient(N, H, d.data(), gx.data(), gy.data(), gz.data(), weno_mode, HZ_HOST));
    if (scatter_grid(gx, S, graddx) != HZ_OK || scatter_grid(gy, S, graddy) != HZ_OK ||
        scatter_grid(gz, S, graddz) != HZ_OK) {
        hz::set_error("ASSIGN_GRADIENT: ragged output grid has NULL rows");
        return HZ_ERR_ARG;
    }
    return 0;
}

int ASSIGN_CURVATURES(int N, double H, double ***dist, double ***mcurv, double ***gcurv)
{
    const int S = N + 1;
    std::vector<double> d, mc, gc;
    if (gather_grid(dist, S, d) != HZ_OK) {
        hz::set_error("ASSIGN_CURVATURES: ragged distance grid has NULL rows");
        return HZ_ERR_ARG;
    }
    mc.resize(d.size());
    gc.resize(d.size());
    HZ_TRY(hz_assign_curvatures(N, H, d.data(), mc.data(), gc.data(), HZ_HOST));
    if (scatter_grid(mc, S, mcurv) != HZ_OK || scatter_grid(gc, S, gcurv) != HZ_OK) {
        hz::set_error("ASSIGN_CURVATURES: ragged output grid has NULL rows");
        return HZ_ERR_ARG;
    }
    return 0;
}

int CompBiCG(int size, double *density, double *densityimg, double **Kernel, double **Kernelimg, double *b,
             double *bimg)
{
    // BICGSTAB.c:159 caps CompBiCG at 1000 iterations
    return dense_bicg_ragged(size, density, densityimg, Kernel, Kernelimg, b, bimg, 1000);
}

int omp_CompBiCG(int size, double *density, double *densityimg, double **Kernel, double **Kernelimg, double *b,
                 double *bimg, int chunk)
{
    (void)chunk;
    // BICGSTAB.c:497 caps omp_CompBiCG at 2000 iterations
    return dense_bicg_ragged(size, density, densityimg, Kernel, Kernelimg, b, bimg, 2000);
}

// ---------------------------------------------------------------------------
// Dense assemblers (HelmholtzKernel.c) with the reference's signatures.

// The driver globals the reference's dense assemblers read
// (HelmholtzKernel.h:16-18).  Weak definitions with the reference's initial
// values (large3Dexample2.c:46-51): a driver that defines them, as
// large3Dexample2.c does, supplies the values in use.
__attribute__((weak, visibility("default"))) int N = 20;
__attribute__((weak, visibility("default"))) int SIZE = 21;
__attribute__((weak, visibility("default"))) double H = 0.0;
__attribute__((weak, visibility("default"))) double HCUBED = 0.0;
__attribute__((weak, visibility("default"))) double WAVE = 15.0;

namespace {

// frame.h / PDE.h values of the reference build
hz_ref_config g_ref = {-2.0, 2.0, 2.0, 0, 0, 1, 0, 0, 0, 1.0, {0.0, 0.0, 0.0}, 1e-7};

struct DeviceGrids {
    hz::DevBuf buf;
    const double *g[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
};

// hz_params of the driver's globals and the configuration; checks that the
// driver's H is the configuration's (INT_U - INT_L)/N.
int driver_params(hz_params &p, const char *who)
{
    if (N < 8 || SIZE != N + 1) {
        hz::set_error("%s: driver globals N = %d, SIZE = %d are not set", who, N, SIZE);
        return HZ_ERR_STATE;
    }
    hz_params_default(&p, N, WAVE);
    p.int_l = g_ref.int_l;
    p.int_u = g_ref.int_u;
    p.tau_factor = g_ref.tau_factor;
    p.interior = g_ref.interior;
    const double h = (p.int_u - p.int_l) / p.N;
    if (!(fabs(h - H) <= 1e-12 * h)) {
        hz::set_error("%s: global H = %g differs from (INT_U - INT_L)/N = %g of the configuration", who, H, h);
        return HZ_ERR_STATE;
    }
    return HZ_OK;
}

int upload_grids(double ***grids[6], int S, DeviceGrids &dg, const char *who)
{
    const size_t nodes = (size_t)S * S * S;
    HZ_TRY(dg.buf.ensure(6 * nodes * sizeof(double)));
    std::vector<double> tmp;
    for (int q = 0; q < 6; q++) {
        if (gather_grid(grids[q], S, tmp) != HZ_OK) {
            hz::set_error("%s: ragged grid %d has NULL rows", who, q);
            return HZ_ERR_ARG;
        }
        double *dst = dg.buf.as<double>() + q * nodes;
        HZ_CHECK_CUDA(cudaMemcpy(dst, tmp.data(), nodes * sizeof(double), cudaMemcpyHostToDevice));
        dg.g[q] = dst;
    }
    return HZ_OK;
}

// Copy one row of the per-point array (device) into a caller's list.
int copy_row(double *dst, const double *dpts, int row, int64_t n)
{
    if (!dst || n == 0) return HZ_OK;
    HZ_CHECK_CUDA(cudaMemcpy(dst, dpts + (size_t)row * n, n * sizeof(double), cudaMemcpyDeviceToHost));
    return HZ_OK;
}

// Copy a device n x n matrix into caller rows (one copy per row).
int copy_rows(double **dst, const double *src, int64_t n, const char *who)
{
    if (!dst) return HZ_OK;
    for (int64_t i = 0; i < n; i++) {
        if (!dst[i]) {
            hz::set_error("%s: NULL matrix row %lld", who, (long long)i);
            return HZ_ERR_ARG;
        }
        HZ_CHECK_CUDA(cudaMemcpy(dst[i], src + (size_t)i * n, n * sizeof(double), cudaMemcpyDeviceToHost));
    }
    return HZ_OK;
}

// Assemble on the device: per-point rows into dpts, matrices into dm[0..3]
// (k1 re/im, k2 re/im; NULL entries are not assembled).
int run_dense(int kind, const hz_params &p, const hz_dense_opts &o, const DeviceGrids *dg, int64_t n,
              hz::DevBuf &pbuf, hz::DevBuf &mbuf, double *dm[4], const bool want[4], long long *regcount)
{
    HZ_TRY(pbuf.ensure((size_t)HZ_DENSE_ROWS * (n > 0 ? n : 1) * sizeof(double)));
    const size_t nn = (size_t)n * (size_t)n;
    int cnt = 0;
    for (int q = 0; q < 4; q++) cnt += want[q] ? 1 : 0;
    HZ_TRY(mbuf.ensure((size_t)(cnt > 0 ? cnt : 1) * (nn > 0 ? nn : 1) * sizeof(double)));
    int used = 0;
    for (int q = 0; q < 4; q++) dm[q] = want[q] ? mbuf.as<double>() + (size_t)(used++) * nn : nullptr;
    hz::DevBuf ebuf;
    HZ_TRY(ebuf.ensure(sizeof(unsigned)));
    HZ_CHECK_CUDA(cudaMemset(ebuf.ptr, 0, sizeof(unsigned)));
    const double *g[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    if (dg)
        for (int q = 0; q < 6; q++) g[q] = dg->g[q];
    HZ_TRY(hz::dense_assemble_device(kind, p, o, g[0], g[1], g[2], g[3], g[4], g[5], n, pbuf.as<double>(), dm[0],
                                     dm[1], dm[2], dm[3], regcount, ebuf.as<unsigned>(), nullptr));
    unsigned e = 0;
    HZ_CHECK_CUDA(cudaMemcpy(&e, ebuf.ptr, sizeof(unsigned), cudaMemcpyDeviceToHost));
    if (e & hz::DEV_ERR_GRID) {
        hz::set_error("dense assembler: a projected point's interpolation cell lies outside the grid");
        return HZ_ERR_GRID;
    }
    return HZ_OK;
}

}  // namespace

extern "C" {
void hz_ref_get_config(hz_ref_config *c)
{
    if (c) *c = g_ref;
}
void hz_ref_set_config(const hz_ref_config *c)
{
    if (c) g_ref = *c;
}
}

int DoubleLayerKernel(int size, double epsilon, double ***level, double ***leveldx, double ***leveldy,
                      double ***leveldz, double ***levelmcurv, double ***levelgcurv, double *zxlist, double *zylist,
                      double *zzlist, double *zxstarlist, double *zystarlist, double *zzstarlist, double *dist,
                      double *gradx, double *grady, double *gradz, double *delta, double *Jacobian, double *regfactor,
                      double *regfactorimg, double *result, double **Kernel, double **Kernelimg, double wavenum)
{
    (void)wavenum;  // unused by the reference too (its kernel takes WAVE)
    const char *who = "DoubleLayerKernel";
    hz_params p;
    HZ_TRY(driver_params(p, who));
    hz_dense_opts o;
    hz_dense_opts_default(&o, HZ_DENSE_DOUBLE_LAYER, &p);
    o.epsilon = epsilon;
    o.onesided = g_ref.trad_onesided;
    DeviceGrids dg;
    double ***grids[6] = {level, leveldx, leveldy, leveldz, levelmcurv, levelgcurv};
    HZ_TRY(upload_grids(grids, SIZE, dg, who));
    hz::DevBuf pbuf, mbuf;
    double *dm[4];
    const bool want[4] = {Kernel != nullptr, Kernelimg != nullptr, false, false};
    HZ_TRY(run_dense(HZ_DENSE_DOUBLE_LAYER, p, o, &dg, size, pbuf, mbuf, dm, want, nullptr));
    const double *P = pbuf.as<double>();
    double *rows[15] = {zxlist, zylist, zzlist, zxstarlist, zystarlist, zzstarlist, dist, gradx, grady, gradz,
                        delta, Jacobian, regfactor, regfactorimg, result};
    const int idx[15] = {HZ_DP_ZX, HZ_DP_ZY, HZ_DP_ZZ, HZ_DP_XS, HZ_DP_YS, HZ_DP_ZS, HZ_DP_DIST, HZ_DP_GX,
                         HZ_DP_GY, HZ_DP_GZ, HZ_DP_DELTA, HZ_DP_JAC, HZ_DP_REG, HZ_DP_REGIMG, HZ_DP_RESULT};
    for (int q = 0; q < 15; q++) HZ_TRY(copy_row(rows[q], P, idx[q], size));
    HZ_TRY(copy_rows(Kernel, dm[0], size, who));
    HZ_TRY(copy_rows(Kernelimg, dm[1], size, who));
    return 0;
}

int new_HelmholtzKernelCombo(int size, double delta, double epsilon, double ***level, double ***leveldx,
                             double ***leveldy, double ***leveldz, double ***levelmcurv, double ***levelgcurv,
                             double *zxlist, double *zylist, double *zzlist, double *zxstarlist, double *zystarlist,
                             double *zzstarlist, double *dist, double *gradx, double *grady, double *gradz,
                             double *Jacobian, double *regfactor, double *regfactorimg, double *PolyW, double *SineW,
                             double *PolyResult, double *SineResult, double **PolyKernelH, double **PolyKernelHimg,
                             double **SineKernelH, double **SineKernelHimg, double wavenum, double eta)
{
    const char *who = "new_HelmholtzKernelCombo";
    hz_params p;
    HZ_TRY(driver_params(p, who));
    hz_dense_opts o;
    hz_dense_opts_default(&o, HZ_DENSE_COMBO, &p);
    o.delta0 = delta;
    o.epsilon = epsilon;
    o.wavenum = wavenum;
    o.eta = eta;
    o.poly = g_ref.poly;
    o.sine = g_ref.sine;
    o.onesided = g_ref.combo_onesided;
    o.combo_interior = g_ref.combo_interior;
    DeviceGrids dg;
    double ***grids[6] = {level, leveldx, leveldy, leveldz, levelmcurv, levelgcurv};
    HZ_TRY(upload_grids(grids, SIZE, dg, who));
    hz::DevBuf pbuf, mbuf;
    double *dm[4];
    const bool want[4] = {o.poly && PolyKernelH, o.poly && PolyKernelHimg, o.sine && SineKernelH,
                          o.sine && SineKernelHimg};
    long long regcount = 0;
    HZ_TRY(run_dense(HZ_DENSE_COMBO, p, o, &dg, size, pbuf, mbuf, dm, want, &regcount));
    const double *P = pbuf.as<double>();
    double *rows[13] = {zxlist, zylist, zzlist, zxstarlist, zystarlist, zzstarlist, dist, gradx, grady, gradz,
                        Jacobian, regfactor, regfactorimg};
    const int idx[13] = {HZ_DP_ZX, HZ_DP_ZY, HZ_DP_ZZ, HZ_DP_XS, HZ_DP_YS, HZ_DP_ZS, HZ_DP_DIST,
                         HZ_DP_GX, HZ_DP_GY, HZ_DP_GZ, HZ_DP_JAC, HZ_DP_REG, HZ_DP_REGIMG};
    for (int q = 0; q < 13; q++) HZ_TRY(copy_row(rows[q], P, idx[q], size));
    if (o.poly) {
        HZ_TRY(copy_row(PolyW, P, HZ_DP_POLYW, size));
        HZ_TRY(copy_row(PolyResult, P, HZ_DP_POLYRES, size));
        HZ_TRY(copy_rows(PolyKernelH, dm[0], size, who));
        HZ_TRY(copy_rows(PolyKernelHimg, dm[1], size, who));
    }
    if (o.sine) {
        HZ_TRY(copy_row(SineW, P, HZ_DP_SINEW, size));
        HZ_TRY(copy_row(SineResult, P, HZ_DP_SINERES, size));
        HZ_TRY(copy_rows(SineKernelH, dm[2], size, who));
        HZ_TRY(copy_rows(SineKernelHimg, dm[3], size, who));
    }
    return (int)regcount;
}

int new_HelmholtzKernel(int size, double delta, double epsilon, double *zxlist, double *zylist, double *zzlist,
                        double *zxstarlist, double *zystarlist, double *zzstarlist, double *dist, double *gradx,
                        double *grady, double *gradz, double *curv, double *Jacobian, double *PolyW, double *SineW,
                        double *PolyResult, double *SineResult, double **PolyKernelH, double **PolyKernelHimg,
                        double **SineKernelH, double **SineKernelHimg)
{
    const char *who = "new_HelmholtzKernel";
    hz_params p;
    HZ_TRY(driver_params(p, who));
    hz_dense_opts o;
    hz_dense_opts_default(&o, HZ_DENSE_SPHERE, &p);
    o.delta0 = delta;
    o.epsilon = epsilon;
    o.poly = g_ref.poly;
    o.sine = g_ref.sine;
    o.onesided = g_ref.combo_onesided;
    o.radius = g_ref.radius;
    for (int q = 0; q < 3; q++) o.center[q] = g_ref.center[q];
    hz::DevBuf pbuf, mbuf;
    double *dm[4];
    const bool want[4] = {o.poly && PolyKernelH, o.poly && PolyKernelHimg, o.sine && SineKernelH,
                          o.sine && SineKernelHimg};
    HZ_TRY(run_dense(HZ_DENSE_SPHERE, p, o, nullptr, size, pbuf, mbuf, dm, want, nullptr));
    const double *P = pbuf.as<double>();
    double *rows[12] = {zxlist, zylist, zzlist, zxstarlist, zystarlist, zzstarlist, dist, gradx, grady, gradz,
                        curv, Jacobian};
    const int idx[12] = {HZ_DP_ZX, HZ_DP_ZY, HZ_DP_ZZ, HZ_DP_XS, HZ_DP_YS, HZ_DP_ZS,
                         HZ_DP_DIST, HZ_DP_GX, HZ_DP_GY, HZ_DP_GZ, HZ_DP_CURV, HZ_DP_JAC};
    for (int q = 0; q < 12; q++) HZ_TRY(copy_row(rows[q], P, idx[q], size));
    if (o.poly) {
        HZ_TRY(copy_row(PolyW, P, HZ_DP_POLYW, size));
        HZ_TRY(copy_row(PolyResult, P, HZ_DP_POLYRES, size));
        HZ_TRY(copy_rows(PolyKernelH, dm[0], size, who));
        HZ_TRY(copy_rows(PolyKernelHimg, dm[1], size, who));
    }
    if (o.sine) {
        HZ_TRY(copy_row(SineW, P, HZ_DP_SINEW, size));
        HZ_TRY(copy_row(SineResult, P, HZ_DP_SINERES, size));
        HZ_TRY(copy_rows(SineKernelH, dm[2], size, who));
        HZ_TRY(copy_rows(SineKernelHimg, dm[3], size, who));
    }
    return 0;
}
