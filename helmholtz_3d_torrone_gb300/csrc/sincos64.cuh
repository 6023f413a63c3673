// sincos64.cuh -- FP64 sin and cos of the pair sweeps' phases (x >= 0),
// after P. T. P. Tang, "Table-lookup algorithms for elementary functions and
// their error analysis" (1991): x = m (2 pi / 128) + r with |r| <= pi / 128,
// sin/cos(m 2 pi / 128) from a 128-entry table in shared memory, sin/cos(r)
// from their Taylor series (terms to r^7 and r^6; the first dropped terms,
// r^9/9! and r^8/8!, are below 1e-20 and 3.3e-18 at |r| = pi/128, about
// 0.03 ulp of 1), recombined by the angle-addition formulas.  Far shorter
// on GB300's FP64 pipe than a general sin/cos with its range reduction.
#pragma once

namespace hz {

constexpr int kSinTable = 128;

// tab[i] = (sin, cos)(2 pi i / 128), filled by the threads of one block; the
// caller synchronises the block before the first lookup.
__device__ __forceinline__ void fill_sin_table(double2 *tab)
{
    for (int i = threadIdx.x; i < kSinTable; i += blockDim.x) {
        double si, co;
        sincospi((double)i / (kSinTable / 2), &si, &co);
        tab[i] = make_double2(si, co);
    }
}

__device__ __forceinline__ void table_sincos(double x, const double2 *tab, double &s, double &c)
{
    // 2 pi / 128 split so that m * kStepHi is exact for m < 2^22
    const double kInvStep = 20.371832715762604;      // 128 / (2 pi)
    const double kStepHi = 0.049087385210441425;     // 2 pi / 128 rounded to 31 significant bits
    const double kStepLo = 1.899093908283185e-12;    // 2 pi / 128 - kStepHi
    // nearest integer m to x * 128/(2 pi) (below 2^51): add and remove 1.5 2^52;
    // the table index is the low word of the sum
    const double xm = fma(x, kInvStep, 6755399441055744.0);
    const double m = xm - 6755399441055744.0;
    double r = fma(-m, kStepHi, x);
    r = fma(-m, kStepLo, r);
    const double2 t = tab[__double2loint(xm) & (kSinTable - 1)];
    const double z = r * r;
    // sin r = r - r^3/3! + r^5/5! - r^7/7!,  cos r = 1 - r^2/2! + r^4/4! - r^6/6!
    const double ps = fma(fma(z, -1.0 / 5040.0, 1.0 / 120.0), z, -1.0 / 6.0);
    const double sr = fma(r * z, ps, r);
    const double cr = fma(fma(fma(z, -1.0 / 720.0, 1.0 / 24.0), z, -0.5), z, 1.0);
    s = fma(t.x, cr, t.y * sr);
    c = fma(t.y, cr, -(t.x * sr));
}

}  // namespace hz
