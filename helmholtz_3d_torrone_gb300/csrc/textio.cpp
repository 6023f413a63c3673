// textio.cpp -- the reference driver's text file formats, so that a run of
// this library can start from, or hand over to, files of the reference:
//   distance<N>.txt      (N+1)^3 values in (i,j,k) order, read with "%lf"
//                        (large3Dexample2.c:405-424);
//   Rel_bN<N>k<k>.txt / Rel_bimgN<N>k<k>.txt   boundary data: a "%d" size
//                        line, then one "%.15lf" value per line
//                        (print_f, large3Dexample2.c:1236-1252,1333-1335);
//   Rel_DensityN<N>k<k>.txt / Rel_DensityimgN<N>k<k>.txt   density: "%.15lf "
//                        values, no header (large3Dexample2.c:3446-3474);
//   Rel_Result_N<N>k<k>.txt   the field check of NeumannTest (:1885-1896).
// Host-only code: no device work.
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstring>

#include "../../include/helmholtz_gb300.h"

namespace hz {
void set_error(const char *fmt, ...);
}

namespace {

struct File {
    FILE *f = nullptr;
    File(const char *path, const char *mode) { f = path ? fopen(path, mode) : nullptr; }
    ~File()
    {
        if (f) fclose(f);
    }
};

int open_error(const char *path)
{
    hz::set_error("cannot open %s: %s", path ? path : "(null)", strerror(errno));
    return HZ_ERR_ARG;
}

int read_values(FILE *f, const char *path, int64_t n, double *out)
{
    for (int64_t i = 0; i < n; i++) {
        if (fscanf(f, "%lf", &out[i]) != 1) {
            hz::set_error("%s: expected %lld values, found %lld", path, (long long)n, (long long)i);
            return HZ_ERR_ARG;
        }
        if (out[i] != out[i]) {
            hz::set_error("%s: value %lld is NaN", path, (long long)i);
            return HZ_ERR_NONFINITE;
        }
    }
    return HZ_OK;
}

}  // namespace

extern "C" {

int hz_reference_file_names(int N, double wave, char *b, char *bimg, char *dens, char *densimg, char *result,
                            char *distance, size_t cap)
{
    // (int)(N), (int)(WAVE) as in large3Dexample2.c:607-608,2990-2991,1635,407
    const int k = (int)wave;
    if (b) snprintf(b, cap, "Rel_bN%dk%d.txt", N, k);
    if (bimg) snprintf(bimg, cap, "Rel_bimgN%dk%d.txt", N, k);
    if (dens) snprintf(dens, cap, "Rel_DensityN%dk%d.txt", N, k);
    if (densimg) snprintf(densimg, cap, "Rel_DensityimgN%dk%d.txt", N, k);
    if (result) snprintf(result, cap, "Rel_Result_N%dk%d.txt", N, k);
    if (distance) snprintf(distance, cap, "distance%d.txt", N);
    return HZ_OK;
}

int hz_read_distance_file(const char *path, int N, double *d)
{
    if (N < 1 || !d) {
        hz::set_error("hz_read_distance_file: bad arguments");
        return HZ_ERR_ARG;
    }
    File f(path, "r");
    if (!f.f) return open_error(path);
    const int64_t S = (int64_t)N + 1;
    return read_values(f.f, path, S * S * S, d);
}

int hz_write_distance_file(const char *path, int N, const double *d)
{
    if (N < 1 || !d) {
        hz::set_error("hz_write_distance_file: bad arguments");
        return HZ_ERR_ARG;
    }
    File f(path, "w");
    if (!f.f) return open_error(path);
    const int64_t S = (int64_t)N + 1;
    for (int64_t i = 0; i < S * S; i++) {
        for (int64_t k = 0; k < S; k++) fprintf(f.f, "%.17g ", d[i * S + k]);
        fputc('\n', f.f);
    }
    return ferror(f.f) ? open_error(path) : HZ_OK;
}

int hz_write_rhs_files(const char *path_re, const char *path_im, int64_t n, const double *b_re, const double *b_im)
{
    const char *paths[2] = {path_re, path_im};
    const double *v[2] = {b_re, b_im};
    for (int c = 0; c < 2; c++) {
        if (!paths[c]) continue;
        File f(paths[c], "w");
        if (!f.f) return open_error(paths[c]);
        fprintf(f.f, "%d\n", (int)n);
        for (int64_t i = 0; i < n; i++) fprintf(f.f, "%.15lf\n", v[c][i]);
        if (ferror(f.f)) return open_error(paths[c]);
    }
    return HZ_OK;
}

int hz_read_rhs_files(const char *path_re, const char *path_im, int64_t n, double *b_re, double *b_im)
{
    const char *paths[2] = {path_re, path_im};
    double *v[2] = {b_re, b_im};
    for (int c = 0; c < 2; c++) {
        File f(paths[c], "r");
        if (!f.f) return open_error(paths[c]);
        int size = -1;
        // the size check of parallel_BiCGcomplex, large3Dexample2.c:3107-3113
        if (fscanf(f.f, "%d", &size) != 1 || size != (int)n) {
            hz::set_error("%s: size line %d does not match the tube size %lld", paths[c], size, (long long)n);
            return HZ_ERR_ARG;
        }
        const int rc = read_values(f.f, paths[c], n, v[c]);
        if (rc != HZ_OK) return rc;
    }
    return HZ_OK;
}

int hz_write_density_files(const char *path_re, const char *path_im, int64_t n, const double *x_re,
                           const double *x_im)
{
    const char *paths[2] = {path_re, path_im};
    const double *v[2] = {x_re, x_im};
    for (int c = 0; c < 2; c++) {
        if (!paths[c]) continue;
        File f(paths[c], "w");
        if (!f.f) return open_error(paths[c]);
        for (int64_t i = 0; i < n; i++) {
            if (v[c][i] != v[c][i]) {
                hz::set_error("density value %lld is NaN", (long long)i);
                return HZ_ERR_NONFINITE;
            }
            fprintf(f.f, "%.15lf ", v[c][i]);
        }
        if (ferror(f.f)) return open_error(paths[c]);
    }
    return HZ_OK;
}

int hz_read_density_files(const char *path_re, const char *path_im, int64_t n, double *x_re, double *x_im)
{
    const char *paths[2] = {path_re, path_im};
    double *v[2] = {x_re, x_im};
    for (int c = 0; c < 2; c++) {
        File f(paths[c], "r");
        if (!f.f) return open_error(paths[c]);
        const int rc = read_values(f.f, paths[c], n, v[c]);
        if (rc != HZ_OK) return rc;
    }
    return HZ_OK;
}

int hz_write_result_file(const char *path, double exact_re, double exact_im, double approx_re, double approx_im)
{
    File f(path, "w");
    if (!f.f) return open_error(path);
    const double en = sqrt(exact_re * exact_re + exact_im * exact_im);
    const double an = sqrt(approx_re * approx_re + approx_im * approx_im);
    fprintf(f.f, "Real: exact = %lf, trad_approxu = %lf, error %.2E\n", exact_re, approx_re,
            fabs(approx_re - exact_re) / fabs(exact_re));
    fprintf(f.f, "Imag: exact = %lf, trad_approxu = %lf, error %.2E\n", exact_im, approx_im,
            fabs(approx_im - exact_im) / fabs(exact_im));
    fprintf(f.f, "Norm: exact = %lf, trad_approxu = %lf, error %.2E\n", en, an, fabs(an - en) / fabs(en));
    return ferror(f.f) ? open_error(path) : HZ_OK;
}

}  // extern "C"
