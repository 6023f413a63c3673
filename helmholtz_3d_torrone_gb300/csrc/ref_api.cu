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
    // BICGSTAB.h:12 DEFAULTACC
    return hz_dense_bicg((int64_t)n, are.data(), aim.data(), b, bimg, density, densityimg, 1e-7, maxit, HZ_HOST,
                         &info);
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
