// sweep_multi.cu -- multi-right-hand-side pair sweeps: Q = A P for a block of
// RB density vectors with one kernel evaluation per point pair.
//
// Every pair's kernel value (distance, phase, sin/cos, projection) is
// computed once and multiplied into RB densities, so the per-RHS cost falls
// from a full pair evaluation to four fused multiply-adds.  Both precisions
// follow the single-vector sweeps (sweep_f32.cu, sweep_f64.cu) for the
// kernel arithmetic, tiling, TMA staging and the near-field rules (the FP32
// pass uses the same near-tile mask, head/tail target offsets and TwoSum
// cross-tile sums, with no FP64 instruction in its tile loop); the
// densities of a tile are staged as RB/2 rows of two complex values each.
#include "hz_internal.cuh"
#include "pair64.cuh"
#include "bulk_copy.cuh"
#include "krylov_multi.cuh"

namespace hz {
namespace {

constexpr double kPi = 3.14159265358979323846264338328;
// right-hand sides per kernel pass: a pass over RB columns evaluates each
// pair once and spends 4 FMAs per column on it
constexpr int kRBMax32 = 32;
constexpr int kRBMax64 = 16;

// ------------------------------------------------------------------ FP32
struct ArgsM32 {
    int64_t n, npad, mwords;
    int nr;  // right-hand sides in this pass (<= RB)
    float wave, tau2, guard_lo, guard_hi;
    double tau;
    const float4 *pos, *nrm;
    const float4 *dens;  // [RB/2][npad]: (p'_{2q} re, im, p'_{2q+1} re, im)
    const float4 *thi, *tlo, *ohi, *olo;
    const uint32_t *nearmask;
    const double4_32a *tpos, *pos64;
    const int *perm;
    const double *p_re, *p_im;  // [nr][n] (diagonal term)
    double *q_re, *q_im;        // [nr][n]
    unsigned *err;
};

// hi + lo += f without rounding loss (TwoSum, FP32 only)
__device__ __forceinline__ void two_sum_m(float &hi, float &lo, float f)
{
    const float s = hi + f;
    const float bp = s - hi;
    const float e = (hi - (s - bp)) + (f - bp);
    hi = s;
    lo += e;
}

template <int RB>
__global__ void prepm32_kernel(int64_t n, int64_t npad, int nr, const int *__restrict__ perm,
                               const double4_32a *__restrict__ tpos, const double *__restrict__ p_re,
                               const double *__restrict__ p_im, double scale, float4 *__restrict__ dens)
{
    for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < npad; s += (int64_t)gridDim.x * blockDim.x) {
        const int c = perm[s];
        const double ws = (c >= 0) ? tpos[s].w * scale : 0.0;
#pragma unroll
        for (int q = 0; q < RB / 2; q++) {
            float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
            if (c >= 0) {
                const int r0 = 2 * q, r1 = 2 * q + 1;
                if (r0 < nr) {
                    v.x = (float)(ws * p_re[(int64_t)r0 * n + c]);
                    v.y = (float)(ws * p_im[(int64_t)r0 * n + c]);
                }
                if (r1 < nr) {
                    v.z = (float)(ws * p_re[(int64_t)r1 * n + c]);
                    v.w = (float)(ws * p_im[(int64_t)r1 * n + c]);
                }
            }
            dens[(int64_t)q * npad + s] = v;
        }
    }
}

template <int RB, bool DIR, bool NEAR>
__device__ __forceinline__ void pairm32(const ArgsM32 &a, const float4 s_p, const float4 s_n, const float3 rel,
                                        const float3 tn, float treg, int64_t tslot, int64_t src_slot,
                                        const float4 *sd, int j, float (&acc)[2 * RB])
{
    const float dx = rel.x - s_p.x, dy = rel.y - s_p.y, dz = rel.z - s_p.z;
    const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
    bool near = false;
    if (NEAR) {
        near = r2 <= a.tau2;
        if (r2 > a.guard_lo && r2 < a.guard_hi) {
            const int c = a.perm[src_slot];
            if (c >= 0) {
                const double4_32a q = a.pos64[c];
                const double4_32a tp = a.tpos[tslot];
                const double x1 = tp.x - q.x, x2 = tp.y - q.y, x3 = tp.z - q.z;
                const double rr2 = x1 * x1 + x2 * x2 + x3 * x3;
                near = !(sqrt(rr2) > a.tau);
            }
        }
    }
    const float rinv = rsqrtf(r2);
    const float rho = r2 * rinv;
    float S, C;
    __sincosf(rho * a.wave, &S, &C);
    const float u1 = fmaf(C, rinv, a.wave * S);
    const float u2 = fmaf(a.wave, C, -S * rinv);
    const float rr = rinv * rinv;
    const float pA = DIR ? (dx * s_n.x + dy * s_n.y + dz * s_n.z) : (dx * tn.x + dy * tn.y + dz * tn.z);
    float vr = -u1 * rr * pA, vi = u2 * rr * pA;
    if (NEAR && near) {
        vr = DIR ? s_p.w : treg;
        vi = 0.f;
    }
#pragma unroll
    for (int q = 0; q < RB / 2; q++) {
        const float4 d = sd[q * kTile32 + j];
        acc[4 * q + 0] = fmaf(vr, d.x, fmaf(-vi, d.y, acc[4 * q + 0]));
        acc[4 * q + 1] = fmaf(vr, d.y, fmaf(vi, d.x, acc[4 * q + 1]));
        acc[4 * q + 2] = fmaf(vr, d.z, fmaf(-vi, d.w, acc[4 * q + 2]));
        acc[4 * q + 3] = fmaf(vr, d.w, fmaf(vi, d.z, acc[4 * q + 3]));
    }
}

constexpr int kNT32m = 256;
template <int RB>
constexpr size_t smem_m32() { return 2 * (2 + RB / 2) * kTile32 * sizeof(float4); }

template <int RB, bool DIR>
__global__ void __launch_bounds__(kNT32m, RB <= 8 ? 2 : 1) sweepm32_kernel(ArgsM32 a)
{
    constexpr int TS = kTile32;
    extern __shared__ __align__(128) float4 smem32[];
    __shared__ alignas(8) uint64_t bar[2];
    float4 *sp[2] = {smem32, smem32 + (2 + RB / 2) * TS};
    const int64_t slot = (int64_t)blockIdx.x * kNT32m + threadIdx.x;
    const float4 th = a.thi[slot], tl = a.tlo[slot];
    const float4 nn4 = a.nrm[slot];
    const float3 tn = make_float3(nn4.x, nn4.y, nn4.z);
    const float treg = a.pos[slot].w;
    // near-tile mask row of this block's target tile (kNT32m == kTile32)
    const uint32_t *mrow = a.nearmask + (slot / TS) * a.mwords;
    // cross-tile sums: FP32 head + tail (TwoSum)
    float acch[2 * RB], accl[2 * RB];
#pragma unroll
    for (int i = 0; i < 2 * RB; i++) acch[i] = accl[i] = 0.f;
    const int64_t ntiles = a.npad / TS;
    if (threadIdx.x == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        fence_barrier_init();
    }
    __syncthreads();
    auto issue = [&](int64_t tile, int buf) {
        const int64_t base = tile * TS;
        const uint32_t bytes = TS * sizeof(float4);
        mbar_arrive_expect_tx(&bar[buf], (2 + RB / 2) * bytes);
        bulk_g2s(sp[buf], a.pos + base, bytes, &bar[buf]);
        bulk_g2s(sp[buf] + TS, a.nrm + base, bytes, &bar[buf]);
#pragma unroll
        for (int q = 0; q < RB / 2; q++) bulk_g2s(sp[buf] + (2 + q) * TS, a.dens + q * a.npad + base, bytes, &bar[buf]);
    };
    if (threadIdx.x == 0) issue(0, 0);
    for (int64_t tile = 0; tile < ntiles; tile++) {
        const int buf = (int)(tile & 1);
        if (threadIdx.x == 0 && tile + 1 < ntiles) issue(tile + 1, buf ^ 1);
        const bool far = ((__ldg(mrow + (tile >> 5)) >> (tile & 31)) & 1u) == 0;
        const float4 oh = a.ohi[tile], ol = a.olo[tile];
        const float3 rel = make_float3((th.x - oh.x) + (tl.x - ol.x), (th.y - oh.y) + (tl.y - ol.y),
                                       (th.z - oh.z) + (tl.z - ol.z));
        const bool ok = mbar_wait_bounded(&bar[buf], (uint32_t)((tile >> 1) & 1), g_data_wait_limit);
        if (__syncthreads_or(!ok)) {
            if (threadIdx.x == 0) {
                atomicOr(a.err, DEV_ERR_WAIT);
                mbar_drain(&bar[buf], (uint32_t)((tile >> 1) & 1), &bar[buf ^ 1], (uint32_t)(((tile + 1) >> 1) & 1),
                           tile + 1 < ntiles);
            }
            return;
        }
        const float4 *P = sp[buf], *Nn = sp[buf] + TS, *D = sp[buf] + 2 * TS;
        float acc[2 * RB];
#pragma unroll
        for (int i = 0; i < 2 * RB; i++) acc[i] = 0.f;
        const int64_t base = tile * TS;
        if (far) {
            for (int j = 0; j < TS; j++)
                pairm32<RB, DIR, false>(a, P[j], Nn[j], rel, tn, treg, slot, base + j, D, j, acc);
        } else {
            for (int j = 0; j < TS; j++)
                pairm32<RB, DIR, true>(a, P[j], Nn[j], rel, tn, treg, slot, base + j, D, j, acc);
        }
#pragma unroll
        for (int i = 0; i < 2 * RB; i++) two_sum_m(acch[i], accl[i], acc[i]);
        __syncthreads();
    }
    const int c = a.perm[slot];
    if (c < 0) return;
#pragma unroll
    for (int r = 0; r < RB; r++) {
        if (r >= a.nr) break;
        const double vr = (double)acch[2 * r] + (double)accl[2 * r];
        const double vi = (double)acch[2 * r + 1] + (double)accl[2 * r + 1];
        if (!isfinite(vr) || !isfinite(vi)) atomicOr(a.err, DEV_ERR_NONFINITE);
        a.q_re[(int64_t)r * a.n + c] = vr + 0.5 * a.p_re[(int64_t)r * a.n + c];
        a.q_im[(int64_t)r * a.n + c] = vi + 0.5 * a.p_im[(int64_t)r * a.n + c];
    }
}

// ------------------------------------------------------------------ FP64
constexpr int kT64m = 128;  // sources per tile = threads per block

struct ArgsM64 {
    int64_t n;
    int nr;
    double wave, tau, tau2, sg;
    float kscale;     // k * 2048 / (2 pi), the phase table index in FP32
    long long tau2b;  // bit pattern of tau^2
    const double4_32a *pos, *nrm;
    const double4_32a *dens;  // [RB/2][n]: (w p_{2q}, w p_{2q+1})
    const double *p_re, *p_im;
    double *q_re, *q_im;
    unsigned *err;
};

template <int RB>
__global__ void prepm64_kernel(int64_t n, int nr, const double4_32a *__restrict__ nrm, const double *__restrict__ p_re,
                               const double *__restrict__ p_im, double4_32a *__restrict__ dens)
{
    for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < n; s += (int64_t)gridDim.x * blockDim.x) {
        const double w = nrm[s].w;
#pragma unroll
        for (int q = 0; q < RB / 2; q++) {
            const int r0 = 2 * q, r1 = 2 * q + 1;
            double4_32a v = make_double4_32a(0, 0, 0, 0);
            if (r0 < nr) {
                v.x = w * p_re[(int64_t)r0 * n + s];
                v.y = w * p_im[(int64_t)r0 * n + s];
            }
            if (r1 < nr) {
                v.z = w * p_re[(int64_t)r1 * n + s];
                v.w = w * p_im[(int64_t)r1 * n + s];
            }
            dens[(int64_t)q * n + s] = v;
        }
    }
}

template <int RB>
constexpr size_t smem_m64() { return 2 * (2 + RB / 2) * kT64m * sizeof(double4_32a); }

template <int RB, bool DIR>
__global__ void __launch_bounds__(kT64m) sweepm64_kernel(ArgsM64 a)
{
    constexpr int T = kT64m;
    extern __shared__ __align__(128) double4_32a smem64[];
    __shared__ alignas(8) uint64_t bar[2];
    __shared__ alignas(16) double2 tab[kPhaseTable];
    fill_phase_table(tab);
    double4_32a *sp[2] = {smem64, smem64 + (2 + RB / 2) * T};
    const double c4 = 1. / (4. * kPi);
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = t < a.n;
    double4_32a tp = make_double4_32a(0, 0, 0, 0), tn = make_double4_32a(0, 0, 0, 0);
    if (valid) {
        tp = a.pos[t];
        tn = a.nrm[t];
    }
    double acc[2 * RB];
#pragma unroll
    for (int i = 0; i < 2 * RB; i++) acc[i] = 0.0;
    const int64_t ntiles = (a.n + T - 1) / T;
    if (threadIdx.x == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        fence_barrier_init();
    }
    __syncthreads();
    auto issue = [&](int64_t tile, int buf) {
        const int64_t base = tile * T;
        const int64_t cnt = (a.n - base < T) ? (a.n - base) : T;
        const uint32_t bytes = (uint32_t)(cnt * sizeof(double4_32a));
        mbar_arrive_expect_tx(&bar[buf], (2 + RB / 2) * bytes);
        bulk_g2s(sp[buf], a.pos + base, bytes, &bar[buf]);
        bulk_g2s(sp[buf] + T, a.nrm + base, bytes, &bar[buf]);
#pragma unroll
        for (int q = 0; q < RB / 2; q++) bulk_g2s(sp[buf] + (2 + q) * T, a.dens + q * a.n + base, bytes, &bar[buf]);
    };
    if (threadIdx.x == 0 && ntiles > 0) issue(0, 0);
    for (int64_t tile = 0; tile < ntiles; tile++) {
        const int buf = (int)(tile & 1);
        if (threadIdx.x == 0 && tile + 1 < ntiles) issue(tile + 1, buf ^ 1);
        const bool ok = mbar_wait_bounded(&bar[buf], (uint32_t)((tile >> 1) & 1), g_data_wait_limit);
        if (__syncthreads_or(!ok)) {
            if (threadIdx.x == 0) {
                atomicOr(a.err, DEV_ERR_WAIT);
                mbar_drain(&bar[buf], (uint32_t)((tile >> 1) & 1), &bar[buf ^ 1], (uint32_t)(((tile + 1) >> 1) & 1),
                           tile + 1 < ntiles);
            }
            return;
        }
        const int64_t base = tile * T;
        const int cnt = (int)((a.n - base < T) ? (a.n - base) : T);
        const double4_32a *P = sp[buf], *Nn = sp[buf] + T, *D = sp[buf] + 2 * T;
        if (valid) {
            for (int j = 0; j < cnt; j++) {
                const double4_32a s_p = P[j], s_n = Nn[j];
                const double xmy1 = tp.x - s_p.x, xmy2 = tp.y - s_p.y, xmy3 = tp.z - s_p.z;
                const double r2 = fma(xmy3, xmy3, fma(xmy2, xmy2, xmy1 * xmy1));
                // near-field test as in sweep_f64.cu: bit patterns, the
                // reference's arithmetic within 8192 ulps of tau^2
                const long long rb = __double_as_longlong(r2);
                bool far = rb > a.tau2b;
                if ((unsigned long long)(rb - a.tau2b + 8192) <= 16384ull) {
                    const double r2ref = __dadd_rn(__dadd_rn(__dmul_rn(xmy1, xmy1), __dmul_rn(xmy2, xmy2)),
                                                   __dmul_rn(xmy3, xmy3));
                    far = __dsqrt_rn(r2ref) > a.tau;
                }
                double vr, vi;
                if (far) {
                    double ur, ui, y2;
                    far_factor64<false>(r2, a.wave, a.kscale, tab, ur, ui, y2);
                    const double in = DIR ? fma(xmy3, s_n.z, fma(xmy2, s_n.y, xmy1 * s_n.x))
                                          : fma(xmy3, tn.z, fma(xmy2, tn.y, xmy1 * tn.x));
                    const double f = (a.sg * c4) * (in * y2);
                    vr = ur * f;
                    vi = ui * f;
                } else {
                    vr = DIR ? s_p.w : tp.w;
                    vi = 0.0;
                }
#pragma unroll
                for (int q = 0; q < RB / 2; q++) {
                    const double4_32a d = D[q * T + j];
                    acc[4 * q + 0] += vr * d.x - vi * d.y;
                    acc[4 * q + 1] += vr * d.y + vi * d.x;
                    acc[4 * q + 2] += vr * d.z - vi * d.w;
                    acc[4 * q + 3] += vr * d.w + vi * d.z;
                }
            }
        }
        __syncthreads();
    }
    if (!valid) return;
#pragma unroll
    for (int r = 0; r < RB; r++) {
        if (r >= a.nr) break;
        const double vr = acc[2 * r], vi = acc[2 * r + 1];
        if (!isfinite(vr) || !isfinite(vi)) atomicOr(a.err, DEV_ERR_NONFINITE);
        a.q_re[(int64_t)r * a.n + t] = vr + 0.5 * a.p_re[(int64_t)r * a.n + t];
        a.q_im[(int64_t)r * a.n + t] = vi + 0.5 * a.p_im[(int64_t)r * a.n + t];
    }
}

int blocks_for(int64_t work)
{
    long long b = (work + 255) / 256;
    if (b > 4096) b = 4096;
    return (int)(b < 1 ? 1 : b);
}

// Block of the next pass for `left` remaining columns: the smallest compiled
// block that holds them all, else the largest (one pass over RB columns
// costs about c0 + c1 RB, so a wider block beats two narrower passes).
int pass_block(int precision, int left)
{
    const int top = (precision == HZ_PREC_F64) ? kRBMax64 : kRBMax32;
    for (int rb = 8; rb < top; rb *= 2)
        if (left <= rb) return rb;
    return top;
}

template <int RB>
int launch_m64(const SweepConst &c, const Rec64 &r64, int nr, const double *pr, const double *pi, double *qr,
               double *qi, void *scratch, cudaStream_t s)
{
    constexpr int smem = (int)smem_m64<RB>();
    if (!(c.wave * c.extent <= kMaxPhase64)) {
        set_error("FP64 multi-RHS sweep: k * domain diagonal = %g exceeds the phase reduction's range (%g)",
                  c.wave * c.extent, kMaxPhase64);
        return HZ_ERR_ARG;
    }
    HZ_CHECK_CUDA(cudaFuncSetAttribute(sweepm64_kernel<RB, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    HZ_CHECK_CUDA(cudaFuncSetAttribute(sweepm64_kernel<RB, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    double4_32a *dens = static_cast<double4_32a *>(scratch);
    prepm64_kernel<RB><<<blocks_for(c.n), 256, 0, s>>>(c.n, nr, r64.nrm, pr, pi, dens);
    HZ_CHECK_LAUNCH();
    ArgsM64 a;
    a.n = c.n;
    a.nr = nr;
    a.wave = c.wave;
    a.tau = c.tau;
    a.tau2 = c.tau * c.tau;
    a.tau2b = __builtin_bit_cast(long long, a.tau2);
    a.kscale = (float)(c.wave * (kPhaseTable / (2.0 * kPi)));
    a.sg = (c.interior == 1) ? -1.0 : 1.0;
    a.pos = r64.pos;
    a.nrm = r64.nrm;
    a.dens = dens;
    a.p_re = pr;
    a.p_im = pi;
    a.q_re = qr;
    a.q_im = qi;
    a.err = c.err;
    const unsigned blocks = (unsigned)((c.n + kT64m - 1) / kT64m);
    if (c.dirichlet) sweepm64_kernel<RB, true><<<blocks, kT64m, smem, s>>>(a);
    else sweepm64_kernel<RB, false><<<blocks, kT64m, smem, s>>>(a);
    HZ_CHECK_LAUNCH();
    return HZ_OK;
}

template <int RB>
int launch_m32(const SweepConst &c, const Rec32 &r32, const Rec64 &r64, int nr, const double *pr, const double *pi,
               double *qr, double *qi, void *scratch, cudaStream_t s)
{
    constexpr int smem = (int)smem_m32<RB>();
    HZ_CHECK_CUDA(cudaFuncSetAttribute(sweepm32_kernel<RB, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    HZ_CHECK_CUDA(cudaFuncSetAttribute(sweepm32_kernel<RB, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    float4 *dens = static_cast<float4 *>(scratch);
    const double scale = ((c.interior == 1) ? -1.0 : 1.0) / (4.0 * kPi);
    prepm32_kernel<RB><<<blocks_for(r32.npad), 256, 0, s>>>(c.n, r32.npad, nr, r32.perm, r32.tpos, pr, pi, scale,
                                                            dens);
    HZ_CHECK_LAUNCH();
    ArgsM32 a;
    a.n = c.n;
    a.npad = r32.npad;
    a.nr = nr;
    a.wave = (float)c.wave;
    a.tau = c.tau;
    a.mwords = r32.mwords;
    a.tau2 = (float)(c.tau * c.tau);
    a.guard_lo = (float)(c.tau * c.tau * (1.0 - 1e-4));
    a.guard_hi = (float)(c.tau * c.tau * (1.0 + 1e-4));
    a.pos = r32.pos;
    a.nrm = r32.nrm;
    a.dens = dens;
    a.thi = r32.thi;
    a.tlo = r32.tlo;
    a.ohi = r32.ohi;
    a.olo = r32.olo;
    a.nearmask = r32.nearmask;
    a.tpos = r32.tpos;
    a.pos64 = r64.pos;
    a.perm = r32.perm;
    a.p_re = pr;
    a.p_im = pi;
    a.q_re = qr;
    a.q_im = qi;
    a.err = c.err;
    const unsigned blocks = (unsigned)(r32.npad / kNT32m);
    if (c.dirichlet) sweepm32_kernel<RB, true><<<blocks, kNT32m, smem, s>>>(a);
    else sweepm32_kernel<RB, false><<<blocks, kNT32m, smem, s>>>(a);
    HZ_CHECK_LAUNCH();
    return HZ_OK;
}

}  // namespace

long long multi_rhs_passes(int precision, int nrhs)
{
    long long p = 0;
    for (int r0 = 0; r0 < nrhs; r0 += pass_block(precision, nrhs - r0)) p++;
    return p;
}

size_t multi_rhs_scratch_bytes(int64_t n, int64_t npad)
{
    const size_t a = (size_t)(kRBMax32 / 2) * (size_t)npad * sizeof(float4);
    const size_t b = (size_t)(kRBMax64 / 2) * (size_t)n * sizeof(double4_32a);
    return a > b ? a : b;
}

int sweep_multi(const SweepConst &c, const Rec32 &r32, const Rec64 &r64, int precision, int nrhs,
                const double *p_re, const double *p_im, double *q_re, double *q_im, void *scratch,
                cudaStream_t s)
{
    if (c.n <= 0 || nrhs <= 0) return HZ_OK;
    for (int r0 = 0; r0 < nrhs;) {
        const int rb = pass_block(precision, nrhs - r0);
        const int nr = (nrhs - r0 < rb) ? (nrhs - r0) : rb;
        const double *pr = p_re + (int64_t)r0 * c.n, *pi = p_im + (int64_t)r0 * c.n;
        double *qr = q_re + (int64_t)r0 * c.n, *qi = q_im + (int64_t)r0 * c.n;
        if (precision == HZ_PREC_F64) {
            if (rb == 8) HZ_TRY(launch_m64<8>(c, r64, nr, pr, pi, qr, qi, scratch, s));
            else HZ_TRY(launch_m64<16>(c, r64, nr, pr, pi, qr, qi, scratch, s));
        } else {
            if (rb == 8) HZ_TRY(launch_m32<8>(c, r32, r64, nr, pr, pi, qr, qi, scratch, s));
            else if (rb == 16) HZ_TRY(launch_m32<16>(c, r32, r64, nr, pr, pi, qr, qi, scratch, s));
            else HZ_TRY(launch_m32<32>(c, r32, r64, nr, pr, pi, qr, qi, scratch, s));
        }
        r0 += nr;
    }
    return HZ_OK;
}

HZ_DEFINE_WAIT_LIMIT_SETTER(set_wait_limit_multi)

}  // namespace hz
