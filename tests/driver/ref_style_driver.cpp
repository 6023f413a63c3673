// A driver written the way large3Dexample2.c drives the library (test
// infrastructure): it includes the reference's own headers, defines the
// globals the library reads (N, SIZE, H, HCUBED, WAVE; large3Dexample2.c:
// 46-58), allocates ragged grids (:378-403), fills the signed distance of a
// sphere (d > 0 inside), and calls the library's entry points by their C++
// names:
//   ASSIGN_GRADIENT                 (large3Dexample2.c:441)
//   BothCurvs, once per node        (:446-455)
//   DoubleLayerKernel               (HelmholtzKernel.c:613-761)
//   CompBiCG                        (BICGSTAB.c:5-339)
// The same source is linked once against the reference's objects and once
// against libhzgb300.so; the test compares what the two write.
//
// Usage: ref_style_driver N wave out.bin
// Output (doubles unless noted): int32 N, int32 size, then DX, DY, DZ,
// MCURV, GCURV ((N+1)^3 each, i-major), the 20 per-point lists in the order
// of DoubleLayerKernel's arguments (zx, zy, zz, zx*, zy*, zz*, dist, gradx,
// grady, gradz, delta, Jacobian, regfactor, regfactorimg, result; the rest
// zero), the size x size matrix (real, then imaginary), b, bimg, density,
// densityimg.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "BICGSTAB.h"
#include "HelmholtzKernel.h"
#include "distance_application3D.h"

int N = 20;
int SIZE = 21;
double H, HCUBED;
double WAVE = 15.0;
double G_DELTA;

static double ***grid(int S)
{
    double ***g = (double ***)malloc(S * sizeof(double **));
    for (int i = 0; i < S; i++) {
        g[i] = (double **)malloc(S * sizeof(double *));
        for (int j = 0; j < S; j++) g[i][j] = (double *)calloc(S, sizeof(double));
    }
    return g;
}

static void put(FILE *f, double ***g, int S)
{
    for (int i = 0; i < S; i++)
        for (int j = 0; j < S; j++) fwrite(g[i][j], sizeof(double), S, f);
}

int main(int argc, char **argv)
{
    if (argc < 4) {
        fprintf(stderr, "usage: %s N wave out.bin\n", argv[0]);
        return 2;
    }
    N = atoi(argv[1]);
    SIZE = N + 1;
    WAVE = atof(argv[2]);
    H = (INT_U - INT_L) / N;
    HCUBED = H * H * H;
    const double cx = 0.013, cy = 0.021, cz = 0.007, rad = 1.0;
    double ***dist = grid(SIZE), ***dx = grid(SIZE), ***dy = grid(SIZE), ***dz = grid(SIZE);
    double ***mc = grid(SIZE), ***gc = grid(SIZE);
    for (int i = 0; i < SIZE; i++)
        for (int j = 0; j < SIZE; j++)
            for (int k = 0; k < SIZE; k++) {
                const double x = INT_L + j * H, y = INT_L + i * H, z = INT_L + k * H;
                dist[i][j][k] = rad - sqrt((x - cx) * (x - cx) + (y - cy) * (y - cy) + (z - cz) * (z - cz));
            }
    if (ASSIGN_GRADIENT(N, H, dist, dx, dy, dz, 5) != 0) {
        fprintf(stderr, "ASSIGN_GRADIENT failed\n");
        return 1;
    }
    for (int i = 0; i < SIZE; i++)
        for (int j = 0; j < SIZE; j++)
            for (int k = 0; k < SIZE; k++) BothCurvs(dist, i, j, k, N, H, &mc[i][j][k], &gc[i][j][k]);
    const double epsilon = FACTOR * H;
    int size = 0;
    for (int i = 0; i < SIZE; i++)
        for (int j = 0; j < SIZE; j++)
            for (int k = 0; k < SIZE; k++)
                if (fabs(dist[i][j][k]) <= epsilon) size++;
    std::vector<std::vector<double>> lists(20, std::vector<double>(size, 0.0));
    double **K = (double **)malloc(size * sizeof(double *)), **Ki = (double **)malloc(size * sizeof(double *));
    for (int r = 0; r < size; r++) {
        K[r] = (double *)calloc(size, sizeof(double));
        Ki[r] = (double *)calloc(size, sizeof(double));
    }
    std::vector<double *> L(20);
    for (int r = 0; r < 20; r++) L[r] = lists[r].data();
    if (DoubleLayerKernel(size, epsilon, dist, dx, dy, dz, mc, gc, L[0], L[1], L[2], L[3], L[4], L[5], L[6], L[7],
                          L[8], L[9], L[10], L[11], L[12], L[13], L[14], K, Ki, WAVE) != 0) {
        fprintf(stderr, "DoubleLayerKernel failed\n");
        return 1;
    }
    // Dirichlet data of a point source at the sphere's centre at the
    // projected points: g = e^{ik r} / (4 pi r)
    std::vector<double> b(size), bimg(size), den(size, 0.0), denimg(size, 0.0);
    for (int p = 0; p < size; p++) {
        const double rx = L[3][p] - cx, ry = L[4][p] - cy, rz = L[5][p] - cz;
        const double r = sqrt(rx * rx + ry * ry + rz * rz);
        b[p] = cos(WAVE * r) / (4.0 * M_PI * r);
        bimg[p] = sin(WAVE * r) / (4.0 * M_PI * r);
    }
    if (CompBiCG(size, den.data(), denimg.data(), K, Ki, b.data(), bimg.data()) != 0) {
        fprintf(stderr, "CompBiCG failed\n");
        return 1;
    }
    FILE *f = fopen(argv[3], "wb");
    if (!f) return 1;
    const int hdr[2] = {N, size};
    fwrite(hdr, sizeof(int), 2, f);
    put(f, dx, SIZE);
    put(f, dy, SIZE);
    put(f, dz, SIZE);
    put(f, mc, SIZE);
    put(f, gc, SIZE);
    for (int r = 0; r < 20; r++) fwrite(L[r], sizeof(double), size, f);
    for (int r = 0; r < size; r++) fwrite(K[r], sizeof(double), size, f);
    for (int r = 0; r < size; r++) fwrite(Ki[r], sizeof(double), size, f);
    fwrite(b.data(), sizeof(double), size, f);
    fwrite(bimg.data(), sizeof(double), size, f);
    fwrite(den.data(), sizeof(double), size, f);
    fwrite(denimg.data(), sizeof(double), size, f);
    fclose(f);
    printf("size %d\n", size);
    return 0;
}
