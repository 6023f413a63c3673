// sweep_f32.cu -- FP32 matrix-free pair sweep (the bulk matvec of the
// mixed-precision solver): the same operator as sweep_f64.cu, evaluated on
// the FP32 and SFU pipes.
//
// Precision design:
//  * Sources are stored in a spatially blocked sweep order (8^3 node
//    blocks), so a tile of kTile32 consecutive sources is compact.  Each
//    tile has an FP64 origin o; sources hold FP32 offsets x_s - o.  Targets
//    and origins are held as FP32 head + tail pairs, and a target forms
//    x_t - o = (t_hi - o_hi) + (t_lo - o_lo): the head difference is rounded
//    to half an ulp of itself, so the offset of close pairs keeps FP32
//    relative precision with no FP64 instruction in the tile loop.
//  * The phase k*rho is reduced in revolutions with k/(2 pi) split into an
//    FP32 head and tail before the SFU's sin/cos (the MODE bit
//    SWEEP_PHASE_SPLIT, the operator's default), or passed to the SFU as one
//    FP32 product (hz_set_phase_mode(op, HZ_PHASE_DIRECT)).  rho itself
//    carries an FP32 rounding, so some phase error remains either way; the
//    FP32 product stays within 1e-7 of the FP64 product (2.9e-8 split,
//    4.6e-8 direct on the 256^3 torus at k = 20), and the split reduction
//    costs about 6 % of the throughput.
//  * The near-field test rho <= tau is decided in FP64 (with the FP64
//    sweep's own arithmetic) whenever the FP32 rho^2 lies within 1e-4 of
//    tau^2, so FP32 and FP64 operators classify every pair alike.
//  * Per tile the contributions are summed in FP32; across tiles into FP32
//    head + tail pairs by TwoSum (about 48 significant bits).
//
// Throughput design: the kernel is bound by instruction issue on the FP32
// pipe, and GB300 runs FP64 at 1/64 of the FP32 rate, so the tile loop
// holds no FP64 instruction at all.  A source tile whose bounding sphere is
// farther than tau (with a 1e-3 margin) from the bounding spheres of all of
// the block's target tiles holds no near pair; a bit mask built once per
// tube in FP64 says which, and such tiles run a loop without near-field
// tests or selects.  The factor sg/(4 pi) is folded into the densities (and
// divided out of the stored regularisation factors).  TMA bulk copies stage
// source tiles in shared memory, double-buffered on mbarriers with bounded
// waits.  Block shape and targets per thread come from a small table of
// compiled variants; the autotuner times them on the operator's own data.
#include "hz_internal.cuh"
#include "bulk_copy.cuh"

#include <cstring>
#include <vector>

namespace hz {
namespace {

constexpr double kPi = 3.14159265358979323846264338328;

// Internal MODE bit: reduce the phase in revolutions with a split k/(2 pi)
// (hz_set_phase_mode, HZ_PHASE_SPLIT) instead of passing k rho to the SFU.
constexpr int SWEEP_PHASE_SPLIT = 4;

struct Args32 {
    int64_t n, npad, mwords;
    float wave, kh, kl;  // k and k/(2 pi) = kh + kl (kh: 12 significant bits)
    float tau2, guard_lo, guard_hi;
    double tau;
    const float4 *pos, *nrm, *dens;
    const float4 *thi, *tlo, *ohi, *olo;
    const uint32_t *nearmask;
    const double4_32a *tpos;
    const int *perm;
    const double4_32a *pos64;  // tube order (for the near-field guard)
    const double *p_re, *p_im, *pt_re, *pt_im;
    double *q_re, *q_im, *qt_re, *qt_im;
    unsigned *err;
    // stream-K partition: CTA c takes work units [c U / P, (c+1) U / P) of
    // the U = blocks x tiles (target block, source tile) units
    int64_t units;
    int64_t nctas;
    double4_32a *partial;  // [P][2][slots per block]: (A re, A im, A^H re, A^H im)
};

// The CTA whose unit range holds work unit u: the largest c with
// floor(c U / P) <= u.
__device__ __forceinline__ int64_t cta_of_unit(int64_t u, int64_t units, int64_t nctas)
{
    return ((u + 1) * nctas - 1) / units;
}

// hi + lo += f without rounding loss (Knuth's TwoSum; FP32 only).
__device__ __forceinline__ void two_sum_acc(float &hi, float &lo, float f)
{
    const float s = hi + f;
    const float bp = s - hi;
    const float e = (hi - (s - bp)) + (f - bp);
    hi = s;
    lo += e;
}

// dens[s] = scale (w p, pt) at sweep slot s, FP32, scale = sg / (4 pi).
__global__ void prep32_kernel(int64_t npad, const int *__restrict__ perm, const double4_32a *__restrict__ tpos,
                              const double *__restrict__ p_re, const double *__restrict__ p_im,
                              const double *__restrict__ pt_re, const double *__restrict__ pt_im, double scale,
                              float4 *__restrict__ dens)
{
    for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < npad; s += (int64_t)gridDim.x * blockDim.x) {
        const int c = perm[s];
        float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
        if (c >= 0) {
            const double ws = tpos[s].w * scale;
            if (p_re) {
                v.x = (float)(ws * p_re[c]);
                v.y = (float)(ws * p_im[c]);
            }
            if (pt_re) {
                v.z = (float)(scale * pt_re[c]);
                v.w = (float)(scale * pt_im[c]);
            }
        }
        dens[s] = v;
    }
}

// One source against TG targets; NEAR selects the loop with near-field
// handling.  Accumulates into fA (A p) and fH (A^H pt).
template <int MODE, bool DIR, int NT, int TG, bool NEAR>
__device__ __forceinline__ void pair_block(const Args32 &a, const float4 s_p, const float4 s_n, const float4 s_d,
                                           const float3 (&rel)[TG], const float3 (&tn)[TG], const float (&treg)[TG],
                                           int64_t tslot0, int64_t src_slot, float (&fAr)[TG], float (&fAi)[TG],
                                           float (&fHr)[TG], float (&fHi)[TG])
{
#pragma unroll
    for (int g = 0; g < TG; g++) {
        const float dx = rel[g].x - s_p.x, dy = rel[g].y - s_p.y, dz = rel[g].z - s_p.z;
        const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
        bool near = false;
        if (NEAR) {
            near = r2 <= a.tau2;
            if (r2 > a.guard_lo && r2 < a.guard_hi) {
                // decide exactly as the FP64 sweep does
                const int c = a.perm[src_slot];
                if (c >= 0) {
                    const double4_32a q = a.pos64[c];
                    const double4_32a tp = a.tpos[tslot0 + (int64_t)g * NT];
                    const double x1 = tp.x - q.x, x2 = tp.y - q.y, x3 = tp.z - q.z;
                    near = !(sqrt(x1 * x1 + x2 * x2 + x3 * x3) > a.tau);
                }
            }
        }
        const float rinv = rsqrtf(r2);
        const float rho = r2 * rinv;
        float S, C;
        if (MODE & SWEEP_PHASE_SPLIT) {
            // revolutions rho k/(2 pi) less the nearest integer (|rho kh| <
            // 2^22: add and remove 1.5 2^23), exact to ~2^-24 before the SFU
            const float nn = fmaf(rho, a.kh, 12582912.f) - 12582912.f;
            float f = fmaf(rho, a.kh, -nn);
            f = fmaf(rho, a.kl, f);
            __sincosf(f * 6.28318530717958647692f, &S, &C);
        } else {
            __sincosf(rho * a.wave, &S, &C);
        }
        const float u1 = fmaf(C, rinv, a.wave * S);   // k sin + cos/rho
        const float u2 = fmaf(a.wave, C, -S * rinv);  // k cos - sin/rho
        const float rr = rinv * rinv;
        const float a1 = -u1 * rr, a2 = u2 * rr;
        const float pn = dx * s_n.x + dy * s_n.y + dz * s_n.z;        // (x_t-x_s).n_s
        const float pt = dx * tn[g].x + dy * tn[g].y + dz * tn[g].z;  // (x_t-x_s).n_t
        const float pA = DIR ? pn : pt, pH = DIR ? pt : pn;
        float vAr = a1 * pA, vAi = a2 * pA, vHr = -a1 * pH, vHi = a2 * pH;
        if (NEAR && near) {
            vAr = DIR ? s_p.w : treg[g];
            vHr = DIR ? treg[g] : s_p.w;
            vAi = 0.f;
            vHi = 0.f;
        }
        if (MODE & SWEEP_A) {
            fAr[g] = fmaf(vAr, s_d.x, fmaf(-vAi, s_d.y, fAr[g]));
            fAi[g] = fmaf(vAr, s_d.y, fmaf(vAi, s_d.x, fAi[g]));
        }
        if (MODE & SWEEP_AH) {
            fHr[g] = fmaf(vHr, s_d.z, fmaf(-vHi, s_d.w, fHr[g]));
            fHi[g] = fmaf(vHr, s_d.w, fmaf(vHi, s_d.z, fHi[g]));
        }
    }
}

// Final value of one target slot: q = sum + p/2 (A), qt = w sum + pt/2 (A^H).
template <int MODE>
__device__ __forceinline__ void write_slot(const Args32 &a, int64_t s, double ar, double ai, double hr, double hi)
{
    const int c = a.perm[s];
    if (c < 0) return;
    if (MODE & SWEEP_A) {
        if (!isfinite(ar) || !isfinite(ai)) atomicOr(a.err, DEV_ERR_NONFINITE);
        a.q_re[c] = ar + 0.5 * a.p_re[c];
        a.q_im[c] = ai + 0.5 * a.p_im[c];
    }
    if (MODE & SWEEP_AH) {
        const double w = a.tpos[s].w;
        const double r = w * hr, i = w * hi;
        if (!isfinite(r) || !isfinite(i)) atomicOr(a.err, DEV_ERR_NONFINITE);
        a.qt_re[c] = r + 0.5 * a.pt_re[c];
        a.qt_im[c] = i + 0.5 * a.pt_im[c];
    }
}

// Persistent stream-K sweep: every CTA walks its own contiguous range of
// (target block, source tile) units, so all CTAs carry the same number of
// tile pairs whatever the tube size.  A target block that lies wholly in
// one CTA's range is written out directly; the pieces of a block split
// between CTAs go to the partial buffer (slot 0: the CTA's first block,
// slot 1: its last) and sweep32_fixup adds them up in CTA order.
template <int MODE, bool DIR, int NT, int TG, int MINB>
__global__ void __launch_bounds__(NT, MINB) sweep32_kernel(Args32 a)
{
    constexpr int TS = kTile32;
    constexpr int SLOTS = NT * TG;   // target slots per block (a multiple of TS)
    constexpr int NTT = SLOTS / TS;  // target tiles per block
    __shared__ alignas(128) float4 sp[2][TS];
    __shared__ alignas(128) float4 sn[2][TS];
    __shared__ alignas(128) float4 sd[2][TS];
    __shared__ alignas(8) uint64_t bar[2];

    const int64_t ntiles = a.npad / TS;
    const int64_t u_begin = (int64_t)blockIdx.x * a.units / a.nctas;
    const int64_t u_end = ((int64_t)blockIdx.x + 1) * a.units / a.nctas;
    if (threadIdx.x == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        fence_barrier_init();
    }
    __syncthreads();
    if (u_begin >= u_end) return;
    auto issue = [&](int64_t u, int buf) {
        const int64_t base = (u % ntiles) * TS;
        const uint32_t bytes = TS * sizeof(float4);
        mbar_arrive_expect_tx(&bar[buf], 3 * bytes);
        bulk_g2s(&sp[buf][0], a.pos + base, bytes, &bar[buf]);
        bulk_g2s(&sn[buf][0], a.nrm + base, bytes, &bar[buf]);
        bulk_g2s(&sd[buf][0], a.dens + base, bytes, &bar[buf]);
    };
    if (threadIdx.x == 0) issue(u_begin, 0);
    int seg = 0;
    for (int64_t u = u_begin; u < u_end;) {
        const int64_t blk = u / ntiles;
        const int64_t seg_end = (u_end < (blk + 1) * ntiles) ? u_end : (blk + 1) * ntiles;
        const bool whole = (u == blk * ntiles) && (seg_end == (blk + 1) * ntiles);
        const int64_t slot0 = blk * SLOTS + threadIdx.x;
        float3 th[TG], tl[TG], tn[TG];
        float treg[TG];
        // cross-tile sums: FP32 head + tail (TwoSum), about 48 significant bits
        float hAr[TG], lAr[TG], hAi[TG], lAi[TG], hHr[TG], lHr[TG], hHi[TG], lHi[TG];
#pragma unroll
        for (int g = 0; g < TG; g++) {
            const int64_t s = slot0 + (int64_t)g * NT;
            const float4 h = a.thi[s], l = a.tlo[s], nn = a.nrm[s];
            th[g] = make_float3(h.x, h.y, h.z);
            tl[g] = make_float3(l.x, l.y, l.z);
            tn[g] = make_float3(nn.x, nn.y, nn.z);
            treg[g] = a.pos[s].w;
            hAr[g] = lAr[g] = hAi[g] = lAi[g] = hHr[g] = lHr[g] = hHi[g] = lHi[g] = 0.f;
        }
        // rows of the near-tile mask for this block's target tiles
        const uint32_t *mrow = a.nearmask + (blk * NTT) * a.mwords;
        for (; u < seg_end; u++) {
            const int64_t it = u - u_begin;
            const int buf = (int)(it & 1);
            if (threadIdx.x == 0 && u + 1 < u_end) issue(u + 1, buf ^ 1);
            const int64_t tile = u - blk * ntiles;
            uint32_t word = 0;
#pragma unroll
            for (int k = 0; k < NTT; k++) word |= __ldg(mrow + k * a.mwords + (tile >> 5));
            const bool far = ((word >> (tile & 31)) & 1u) == 0;
            // x_t - o: head difference (rounded once, to half an ulp of
            // itself) plus the tails
            const float4 oh = a.ohi[tile], ol = a.olo[tile];
            float3 rel[TG];
#pragma unroll
            for (int g = 0; g < TG; g++)
                rel[g] = make_float3((th[g].x - oh.x) + (tl[g].x - ol.x), (th[g].y - oh.y) + (tl[g].y - ol.y),
                                     (th[g].z - oh.z) + (tl[g].z - ol.z));
            const bool ok = mbar_wait_bounded(&bar[buf], (uint32_t)((it >> 1) & 1), g_data_wait_limit);
            if (__syncthreads_or(!ok)) {
                if (threadIdx.x == 0) {
                    atomicOr(a.err, DEV_ERR_WAIT);
                    mbar_drain(&bar[buf], (uint32_t)((it >> 1) & 1), &bar[buf ^ 1], (uint32_t)(((it + 1) >> 1) & 1),
                               u + 1 < u_end);
                }
                return;
            }
            float fAr[TG], fAi[TG], fHr[TG], fHi[TG];
#pragma unroll
            for (int g = 0; g < TG; g++) fAr[g] = fAi[g] = fHr[g] = fHi[g] = 0.f;
            const int64_t base = tile * TS;
            if (far) {
#pragma unroll 2
                for (int j = 0; j < TS; j++)
                    pair_block<MODE, DIR, NT, TG, false>(a, sp[buf][j], sn[buf][j], sd[buf][j], rel, tn, treg, slot0,
                                                         base + j, fAr, fAi, fHr, fHi);
            } else {
#pragma unroll 2
                for (int j = 0; j < TS; j++)
                    pair_block<MODE, DIR, NT, TG, true>(a, sp[buf][j], sn[buf][j], sd[buf][j], rel, tn, treg, slot0,
                                                        base + j, fAr, fAi, fHr, fHi);
            }
#pragma unroll
            for (int g = 0; g < TG; g++) {
                if (MODE & SWEEP_A) {
                    two_sum_acc(hAr[g], lAr[g], fAr[g]);
                    two_sum_acc(hAi[g], lAi[g], fAi[g]);
                }
                if (MODE & SWEEP_AH) {
                    two_sum_acc(hHr[g], lHr[g], fHr[g]);
                    two_sum_acc(hHi[g], lHi[g], fHi[g]);
                }
            }
            __syncthreads();
        }
#pragma unroll
        for (int g = 0; g < TG; g++) {
            const double ar = (double)hAr[g] + (double)lAr[g], ai = (double)hAi[g] + (double)lAi[g];
            const double hr = (double)hHr[g] + (double)lHr[g], hi = (double)hHi[g] + (double)lHi[g];
            if (whole) {
                write_slot<MODE>(a, slot0 + (int64_t)g * NT, ar, ai, hr, hi);
            } else {
                a.partial[((int64_t)blockIdx.x * 2 + seg) * SLOTS + threadIdx.x + g * NT] =
                    make_double4_32a(ar, ai, hr, hi);
            }
        }
        seg = 1;
    }
}

// Adds up, in CTA order, the pieces of every target block that the stream-K
// partition split between CTAs (one CTA per target block; blocks that one
// CTA covered whole return at once).
template <int MODE, int SLOTS>
__global__ void __launch_bounds__(256) sweep32_fixup(Args32 a)
{
    const int64_t blk = blockIdx.x;
    const int64_t ntiles = a.npad / kTile32;
    const int64_t c_lo = cta_of_unit(blk * ntiles, a.units, a.nctas);
    const int64_t c_hi = cta_of_unit((blk + 1) * ntiles - 1, a.units, a.nctas);
    if (c_lo == c_hi) return;
    for (int k = threadIdx.x; k < SLOTS; k += blockDim.x) {
        double ar = 0.0, ai = 0.0, hr = 0.0, hi = 0.0;
        for (int64_t c = c_lo; c <= c_hi; c++) {
            const int64_t first = (c * a.units / a.nctas) / ntiles;  // first block of CTA c
            const int sg = (first == blk) ? 0 : 1;
            const double4_32a v = a.partial[(c * 2 + sg) * SLOTS + k];
            ar += v.x;
            ai += v.y;
            hr += v.z;
            hi += v.w;
        }
        write_slot<MODE>(a, blk * SLOTS + k, ar, ai, hr, hi);
    }
}

// ------------------------------------------------------------ batches
// One operator of a batch: its sweep arguments (records, densities,
// constants) and its place in the batch's unit and block numbering.  The
// product vectors are columns of [R][stride] arrays passed to the launch.
struct BatchOp {
    Args32 a;
    int64_t unit0;   // first global (target block, source tile) unit
    int64_t block0;  // first global target block
    int64_t blocks, ntiles;
    int dir;
    int col;         // column of P and Q
    double scale;    // sg / (4 pi), folded into the densities
};

struct BatchVec {
    const double *p_re, *p_im;
    double *q_re, *q_im;
    int64_t stride;
};

// dens of every operator from its column of P (blockIdx.y = operator)
__global__ void batch_prep_kernel(const BatchOp *__restrict__ ops, BatchVec v)
{
    const BatchOp &o = ops[blockIdx.y];
    const double *pr = v.p_re + (int64_t)o.col * v.stride, *pi = v.p_im + (int64_t)o.col * v.stride;
    float4 *dens = const_cast<float4 *>(o.a.dens);
    for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < o.a.npad;
         s += (int64_t)gridDim.x * blockDim.x) {
        const int c = o.a.perm[s];
        float4 d = make_float4(0.f, 0.f, 0.f, 0.f);
        if (c >= 0) {
            const double ws = o.a.tpos[s].w * o.scale;
            d.x = (float)(ws * pr[c]);
            d.y = (float)(ws * pi[c]);
        }
        dens[s] = d;
    }
}

__device__ __forceinline__ int batch_op_of_unit(const BatchOp *ops, int nops, int64_t u, int from)
{
    int o = from;
    while (o + 1 < nops && u >= ops[o + 1].unit0) o++;
    return o;
}

__device__ __forceinline__ void batch_write(const Args32 &a, int64_t s, double ar, double ai, const double *p_re,
                                            const double *p_im, double *q_re, double *q_im)
{
    const int c = a.perm[s];
    if (c < 0) return;
    if (!isfinite(ar) || !isfinite(ai)) atomicOr(a.err, DEV_ERR_NONFINITE);
    q_re[c] = ar + 0.5 * p_re[c];
    q_im[c] = ai + 0.5 * p_im[c];
}

// The tiles of one segment (one target block of one operator) for the
// batched sweep: the same loop as sweep32_kernel with SWEEP_A.
template <bool DIR, int NT, int TG>
__device__ __forceinline__ bool batch_tiles(const Args32 &a, const BatchOp *ops, int nops, int o, int64_t &u,
                                            int64_t seg_end, int64_t u_begin, int64_t u_end, int64_t blk,
                                            int64_t slot0, const float3 (&th)[TG], const float3 (&tl)[TG],
                                            const float3 (&tn)[TG], const float (&treg)[TG], float (&hAr)[TG],
                                            float (&lAr)[TG], float (&hAi)[TG], float (&lAi)[TG],
                                            float4 (*sp)[kTile32], float4 (*sn)[kTile32], float4 (*sd)[kTile32],
                                            uint64_t *bar)
{
    constexpr int TS = kTile32;
    constexpr int NTT = NT * TG / TS;
    const int64_t ntiles = ops[o].ntiles, unit0 = ops[o].unit0;
    const uint32_t *mrow = a.nearmask + (blk * NTT) * a.mwords;
    for (; u < seg_end; u++) {
        const int64_t it = u - u_begin;
        const int buf = (int)(it & 1);
        if (threadIdx.x == 0 && u + 1 < u_end) {
            const int o2 = batch_op_of_unit(ops, nops, u + 1, o);
            const int64_t base = ((u + 1 - ops[o2].unit0) % ops[o2].ntiles) * TS;
            const uint32_t bytes = TS * sizeof(float4);
            mbar_arrive_expect_tx(&bar[buf ^ 1], 3 * bytes);
            bulk_g2s(&sp[buf ^ 1][0], ops[o2].a.pos + base, bytes, &bar[buf ^ 1]);
            bulk_g2s(&sn[buf ^ 1][0], ops[o2].a.nrm + base, bytes, &bar[buf ^ 1]);
            bulk_g2s(&sd[buf ^ 1][0], ops[o2].a.dens + base, bytes, &bar[buf ^ 1]);
        }
        const int64_t tile = u - unit0 - blk * ntiles;
        uint32_t word = 0;
#pragma unroll
        for (int k = 0; k < NTT; k++) word |= __ldg(mrow + k * a.mwords + (tile >> 5));
        const bool far = ((word >> (tile & 31)) & 1u) == 0;
        const float4 oh = a.ohi[tile], ol = a.olo[tile];
        float3 rel[TG];
#pragma unroll
        for (int g = 0; g < TG; g++)
            rel[g] = make_float3((th[g].x - oh.x) + (tl[g].x - ol.x), (th[g].y - oh.y) + (tl[g].y - ol.y),
                                 (th[g].z - oh.z) + (tl[g].z - ol.z));
        const bool ok = mbar_wait_bounded(&bar[buf], (uint32_t)((it >> 1) & 1), g_data_wait_limit);
        if (__syncthreads_or(!ok)) {
            if (threadIdx.x == 0) {
                atomicOr(a.err, DEV_ERR_WAIT);
                mbar_drain(&bar[buf], (uint32_t)((it >> 1) & 1), &bar[buf ^ 1], (uint32_t)(((it + 1) >> 1) & 1),
                           u + 1 < u_end);
            }
            return false;
        }
        float fAr[TG], fAi[TG], fHr[TG], fHi[TG];
#pragma unroll
        for (int g = 0; g < TG; g++) fAr[g] = fAi[g] = fHr[g] = fHi[g] = 0.f;
        const int64_t base = tile * TS;
        if (far) {
#pragma unroll 2
            for (int j = 0; j < TS; j++)
                pair_block<SWEEP_A, DIR, NT, TG, false>(a, sp[buf][j], sn[buf][j], sd[buf][j], rel, tn, treg, slot0,
                                                        base + j, fAr, fAi, fHr, fHi);
        } else {
#pragma unroll 2
            for (int j = 0; j < TS; j++)
                pair_block<SWEEP_A, DIR, NT, TG, true>(a, sp[buf][j], sn[buf][j], sd[buf][j], rel, tn, treg, slot0,
                                                       base + j, fAr, fAi, fHr, fHi);
        }
#pragma unroll
        for (int g = 0; g < TG; g++) {
            two_sum_acc(hAr[g], lAr[g], fAr[g]);
            two_sum_acc(hAi[g], lAi[g], fAi[g]);
        }
        __syncthreads();
    }
    return true;
}

// Q[r] = A_r P[r] for every operator r of a batch in one persistent launch:
// the stream-K partition of sweep32_kernel over the concatenated
// (operator, target block, source tile) units, so operators of different
// sizes share the GPU without a tail per operator.
template <int NT, int TG, int MINB>
__global__ void __launch_bounds__(NT, MINB) sweep32_batch_kernel(const BatchOp *__restrict__ ops, int nops,
                                                                 int64_t units, int64_t nctas,
                                                                 double4_32a *partial, BatchVec v)
{
    constexpr int TS = kTile32;
    constexpr int SLOTS = NT * TG;
    __shared__ alignas(128) float4 sp[2][TS];
    __shared__ alignas(128) float4 sn[2][TS];
    __shared__ alignas(128) float4 sd[2][TS];
    __shared__ alignas(8) uint64_t bar[2];
    const int64_t u_begin = (int64_t)blockIdx.x * units / nctas;
    const int64_t u_end = ((int64_t)blockIdx.x + 1) * units / nctas;
    if (threadIdx.x == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        fence_barrier_init();
    }
    __syncthreads();
    if (u_begin >= u_end) return;
    int o = batch_op_of_unit(ops, nops, u_begin, 0);
    if (threadIdx.x == 0) {
        const int64_t base = ((u_begin - ops[o].unit0) % ops[o].ntiles) * TS;
        const uint32_t bytes = TS * sizeof(float4);
        mbar_arrive_expect_tx(&bar[0], 3 * bytes);
        bulk_g2s(&sp[0][0], ops[o].a.pos + base, bytes, &bar[0]);
        bulk_g2s(&sn[0][0], ops[o].a.nrm + base, bytes, &bar[0]);
        bulk_g2s(&sd[0][0], ops[o].a.dens + base, bytes, &bar[0]);
    }
    int seg = 0;
    for (int64_t u = u_begin; u < u_end;) {
        o = batch_op_of_unit(ops, nops, u, o);
        const Args32 a = ops[o].a;
        const int64_t ntiles = ops[o].ntiles, unit0 = ops[o].unit0;
        const int64_t blk = (u - unit0) / ntiles;
        const int64_t blk_end = unit0 + (blk + 1) * ntiles;
        const int64_t seg_end = (u_end < blk_end) ? u_end : blk_end;
        const bool whole = (u == unit0 + blk * ntiles) && (seg_end == blk_end);
        const int64_t slot0 = blk * SLOTS + threadIdx.x;
        float3 th[TG], tl[TG], tn[TG];
        float treg[TG];
        float hAr[TG], lAr[TG], hAi[TG], lAi[TG];
#pragma unroll
        for (int g = 0; g < TG; g++) {
            const int64_t s = slot0 + (int64_t)g * NT;
            const float4 h = a.thi[s], l = a.tlo[s], nn = a.nrm[s];
            th[g] = make_float3(h.x, h.y, h.z);
            tl[g] = make_float3(l.x, l.y, l.z);
            tn[g] = make_float3(nn.x, nn.y, nn.z);
            treg[g] = a.pos[s].w;
            hAr[g] = lAr[g] = hAi[g] = lAi[g] = 0.f;
        }
        const bool ok = ops[o].dir
                            ? batch_tiles<true, NT, TG>(a, ops, nops, o, u, seg_end, u_begin, u_end, blk, slot0, th,
                                                        tl, tn, treg, hAr, lAr, hAi, lAi, sp, sn, sd, bar)
                            : batch_tiles<false, NT, TG>(a, ops, nops, o, u, seg_end, u_begin, u_end, blk, slot0, th,
                                                         tl, tn, treg, hAr, lAr, hAi, lAi, sp, sn, sd, bar);
        if (!ok) return;
        const int64_t off = (int64_t)ops[o].col * v.stride;
        const double *pr = v.p_re + off, *pi = v.p_im + off;
        double *qr = v.q_re + off, *qi = v.q_im + off;
#pragma unroll
        for (int g = 0; g < TG; g++) {
            const double ar = (double)hAr[g] + (double)lAr[g], ai = (double)hAi[g] + (double)lAi[g];
            if (whole)
                batch_write(a, slot0 + (int64_t)g * NT, ar, ai, pr, pi, qr, qi);
            else
                partial[((int64_t)blockIdx.x * 2 + seg) * SLOTS + threadIdx.x + g * NT] =
                    make_double4_32a(ar, ai, 0.0, 0.0);
        }
        seg = 1;
    }
}

// The batch's split blocks, summed in CTA order (one CTA per global block).
template <int SLOTS>
__global__ void __launch_bounds__(256) sweep32_batch_fixup(const BatchOp *__restrict__ ops, int nops, int64_t units,
                                                           int64_t nctas, const double4_32a *partial, BatchVec v)
{
    const int64_t gb = blockIdx.x;
    int o = 0;
    while (o + 1 < nops && gb >= ops[o + 1].block0) o++;
    const int64_t blk = gb - ops[o].block0, ntiles = ops[o].ntiles;
    const int64_t u0 = ops[o].unit0 + blk * ntiles;
    const int64_t c_lo = cta_of_unit(u0, units, nctas), c_hi = cta_of_unit(u0 + ntiles - 1, units, nctas);
    if (c_lo == c_hi) return;
    const Args32 &a = ops[o].a;
    for (int k = threadIdx.x; k < SLOTS; k += blockDim.x) {
        double ar = 0.0, ai = 0.0;
        for (int64_t c = c_lo; c <= c_hi; c++) {
            const int64_t ub = c * units / nctas;
            const int oc = batch_op_of_unit(ops, nops, ub, 0);
            const int64_t first = ops[oc].block0 + (ub - ops[oc].unit0) / ops[oc].ntiles;
            const int sg = (first == gb) ? 0 : 1;
            const double4_32a q = partial[(c * 2 + sg) * SLOTS + k];
            ar += q.x;
            ai += q.y;
        }
        const int64_t off = (int64_t)ops[o].col * v.stride;
        batch_write(a, blk * SLOTS + k, ar, ai, v.p_re + off, v.p_im + off, v.q_re + off, v.q_im + off);
    }
}

template <int NT, int TG, int MINB>
int64_t batch_resident_ctas()
{
    static int64_t cached = 0;
    if (cached == 0) {
        int dev = 0, sms = 152, per = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, sweep32_batch_kernel<NT, TG, MINB>, NT, 0) !=
                cudaSuccess ||
            per < 1) {
            cudaGetLastError();
            per = MINB;
        }
        cached = (int64_t)per * sms;
    }
    return cached;
}

template <int NT, int TG, int MINB>
int launch_batch(const BatchOp *ops_dev, int nops, int64_t units, int64_t blocks, double4_32a *partial,
                 size_t partial_bytes, const BatchVec &v, cudaStream_t s)
{
    constexpr int SLOTS = NT * TG;
    int64_t p = batch_resident_ctas<NT, TG, MINB>();
    if (p > units) p = units;
    if ((size_t)p * 2 * SLOTS * sizeof(double4_32a) > partial_bytes) p = partial_bytes / (2 * SLOTS * sizeof(double4_32a));
    if (p < 1) {
        set_error("batched FP32 sweep: partial buffer too small");
        return HZ_ERR_STATE;
    }
    sweep32_batch_kernel<NT, TG, MINB><<<(unsigned)p, NT, 0, s>>>(ops_dev, nops, units, p, partial, v);
    HZ_CHECK_LAUNCH();
    sweep32_batch_fixup<SLOTS><<<(unsigned)blocks, 256, 0, s>>>(ops_dev, nops, units, p, partial, v);
    HZ_CHECK_LAUNCH();
    return HZ_OK;
}

// Resident CTAs of one sweep instantiation on this device (cached).
template <int MODE, bool DIR, int NT, int TG, int MINB>
int64_t resident_ctas()
{
    static int64_t cached = 0;
    if (cached == 0) {
        int dev = 0, sms = 152, per = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, sweep32_kernel<MODE, DIR, NT, TG, MINB>, NT, 0) !=
                cudaSuccess ||
            per < 1) {
            cudaGetLastError();
            per = MINB;
        }
        cached = (int64_t)per * sms;
    }
    return cached;
}

// persistent: one CTA per resident slot (stream-K); otherwise one CTA per
// target block (the partition then never splits a block).
template <int MODE, bool DIR, int NT, int TG, int MINB>
int launch_streamk(Args32 a, bool persistent, size_t partial_bytes, cudaStream_t s)
{
    constexpr int SLOTS = NT * TG;
    const int64_t blocks = a.npad / SLOTS;
    a.units = blocks * (a.npad / kTile32);
    int64_t p = persistent ? resident_ctas<MODE, DIR, NT, TG, MINB>() : blocks;
    if (p > a.units) p = a.units;
    if (persistent && (size_t)p * 2 * SLOTS * sizeof(double4_32a) > partial_bytes)
        p = partial_bytes / (2 * SLOTS * sizeof(double4_32a));
    if (p < 1) {
        set_error("FP32 sweep: stream-K partial buffer too small");
        return HZ_ERR_STATE;
    }
    a.nctas = p;
    sweep32_kernel<MODE, DIR, NT, TG, MINB><<<(unsigned)p, NT, 0, s>>>(a);
    HZ_CHECK_LAUNCH();
    if (p != blocks) {
        sweep32_fixup<MODE, SLOTS><<<(unsigned)blocks, 256, 0, s>>>(a);
        HZ_CHECK_LAUNCH();
    }
    return HZ_OK;
}

// Compiled variants: (block size, targets per thread, minimum resident
// blocks) x (persistent stream-K grid, or one CTA per target block).  Every
// shape covers 256 or 512 sweep slots per block (npad is a multiple of 512).
constexpr int kShapes = 4;
template <int MODE, bool DIR>
int launch_cfg(int cfg, const Args32 &a, size_t pb, cudaStream_t s)
{
    const bool persistent = cfg < kShapes;
    switch (cfg % kShapes) {
    case 1: return launch_streamk<MODE, DIR, 128, 2, 4>(a, persistent, pb, s);
    case 2: return launch_streamk<MODE, DIR, 256, 1, 3>(a, persistent, pb, s);
    case 3: return launch_streamk<MODE, DIR, 128, 2, 6>(a, persistent, pb, s);
    default: return launch_streamk<MODE, DIR, 256, 2, 2>(a, persistent, pb, s);
    }
}

template <int MODE>
int launch32(int cfg, const Args32 &a, bool dir, size_t pb, cudaStream_t s)
{
    return dir ? launch_cfg<MODE, true>(cfg, a, pb, s) : launch_cfg<MODE, false>(cfg, a, pb, s);
}

}  // namespace

// Split k/(2 pi) into a head with 12 significant bits and an FP32 tail.
void split_wave(double wave, float &kh, float &kl)
{
    const double kc = wave / (2.0 * kPi);
    int e;
    frexp(kc, &e);
    const double q = ldexp(1.0, e - 12);
    const double head = nearbyint(kc / q) * q;
    kh = (float)head;
    kl = (float)(kc - head);
}

double sweep32_reg_scale(int interior) { return ((interior == 1) ? -1.0 : 1.0) * (4.0 * kPi); }

int sweep32_num_configs() { return 2 * kShapes; }

namespace {
template <int MODE, bool DIR, int NT, int TG, int MINB>
size_t partial_need()
{
    return (size_t)resident_ctas<MODE, DIR, NT, TG, MINB>() * 2 * NT * TG * sizeof(double4_32a);
}
template <int MODE, bool DIR>
size_t partial_need_all()
{
    size_t m = 0;
    const size_t v[kShapes] = {partial_need<MODE, DIR, 256, 2, 2>(), partial_need<MODE, DIR, 128, 2, 4>(),
                               partial_need<MODE, DIR, 256, 1, 3>(), partial_need<MODE, DIR, 128, 2, 6>()};
    for (size_t x : v) m = x > m ? x : m;
    return m;
}
}  // namespace

size_t sweep32_partial_bytes()
{
    constexpr int S = SWEEP_PHASE_SPLIT;
    const size_t v[12] = {partial_need_all<SWEEP_A, false>(),        partial_need_all<SWEEP_A, true>(),
                          partial_need_all<SWEEP_AH, false>(),       partial_need_all<SWEEP_AH, true>(),
                          partial_need_all<SWEEP_PAIR, false>(),     partial_need_all<SWEEP_PAIR, true>(),
                          partial_need_all<SWEEP_A | S, false>(),    partial_need_all<SWEEP_A | S, true>(),
                          partial_need_all<SWEEP_AH | S, false>(),   partial_need_all<SWEEP_AH | S, true>(),
                          partial_need_all<SWEEP_PAIR | S, false>(), partial_need_all<SWEEP_PAIR | S, true>()};
    size_t m = 0;
    for (size_t x : v) m = x > m ? x : m;
    return m;
}

// ---------------------------------------------------------------- batches
size_t batch32_desc_bytes(int R) { return (size_t)R * sizeof(BatchOp); }

int batch32_describe(const Batch32Item *items, int R, int cfg, void *desc_dev, int64_t &units, int64_t &blocks,
                     cudaStream_t s, const int *cols)
{
    static const int kSlots[kShapes] = {512, 256, 256, 256};  // NT * TG of shapes 0..3 (launch_cfg)
    const int slots = kSlots[cfg % kShapes];
    std::vector<BatchOp> h(R);
    units = 0;
    blocks = 0;
    for (int r = 0; r < R; r++) {
        const int col = cols ? cols[r] : r;
        const Batch32Item &it = items[col];
        BatchOp &b = h[r];
        memset(&b, 0, sizeof(b));
        b.col = col;
        Args32 &a = b.a;
        a.n = it.c.n;
        a.npad = it.r.npad;
        a.mwords = it.r.mwords;
        a.wave = (float)it.c.wave;
        a.tau = it.c.tau;
        a.tau2 = (float)(it.c.tau * it.c.tau);
        a.guard_lo = (float)(it.c.tau * it.c.tau * (1.0 - 1e-4));
        a.guard_hi = (float)(it.c.tau * it.c.tau * (1.0 + 1e-4));
        a.pos = it.r.pos;
        a.nrm = it.r.nrm;
        a.dens = it.dens;
        a.thi = it.r.thi;
        a.tlo = it.r.tlo;
        a.ohi = it.r.ohi;
        a.olo = it.r.olo;
        a.nearmask = it.r.nearmask;
        a.tpos = it.r.tpos;
        a.perm = it.r.perm;
        a.pos64 = it.pos64;
        a.err = it.c.err;
        if (it.r.npad % slots != 0) {
            set_error("batched FP32 sweep: operator %d has %lld slots, not a multiple of %d", col,
                      (long long)it.r.npad, slots);
            return HZ_ERR_STATE;
        }
        b.ntiles = it.r.npad / kTile32;
        b.blocks = it.r.npad / slots;
        b.unit0 = units;
        b.block0 = blocks;
        b.dir = it.c.dirichlet != 0;
        b.scale = ((it.c.interior == 1) ? -1.0 : 1.0) / (4.0 * kPi);
        units += b.blocks * b.ntiles;
        blocks += b.blocks;
    }
    HZ_CHECK_CUDA(cudaMemcpyAsync(desc_dev, h.data(), R * sizeof(BatchOp), cudaMemcpyHostToDevice, s));
    HZ_CHECK_CUDA(cudaStreamSynchronize(s));
    return HZ_OK;
}

size_t batch32_partial_bytes()
{
    const size_t v[kShapes] = {
        (size_t)batch_resident_ctas<256, 2, 2>() * 2 * 512 * sizeof(double4_32a),
        (size_t)batch_resident_ctas<128, 2, 4>() * 2 * 256 * sizeof(double4_32a),
        (size_t)batch_resident_ctas<256, 1, 3>() * 2 * 256 * sizeof(double4_32a),
        (size_t)batch_resident_ctas<128, 2, 6>() * 2 * 256 * sizeof(double4_32a)};
    size_t m = 0;
    for (size_t x : v) m = x > m ? x : m;
    return m;
}

int sweep_f32_batch(int cfg, const void *desc_dev, int R, int ncols, int64_t units, int64_t blocks,
                    double4_32a *partial, size_t partial_bytes, const double *p_re, const double *p_im,
                    double *q_re, double *q_im, int64_t stride, int64_t max_npad, cudaStream_t s, cudaEvent_t ev0,
                    cudaEvent_t ev1)
{
    // padded tails of the columns stay zero
    HZ_CHECK_CUDA(cudaMemsetAsync(q_re, 0, (size_t)ncols * stride * sizeof(double), s));
    HZ_CHECK_CUDA(cudaMemsetAsync(q_im, 0, (size_t)ncols * stride * sizeof(double), s));
    if (R <= 0 || units <= 0) return HZ_OK;
    const BatchOp *ops = static_cast<const BatchOp *>(desc_dev);
    BatchVec v{p_re, p_im, q_re, q_im, stride};
    long long bx = (max_npad + 255) / 256;
    if (bx > 256) bx = 256;
    batch_prep_kernel<<<dim3((unsigned)bx, (unsigned)R), 256, 0, s>>>(ops, v);
    HZ_CHECK_LAUNCH();
    if (ev0) HZ_CHECK_CUDA(record_timing_event(ev0, s));
    switch (cfg % kShapes) {
    case 1: HZ_TRY((launch_batch<128, 2, 4>(ops, R, units, blocks, partial, partial_bytes, v, s))); break;
    case 2: HZ_TRY((launch_batch<256, 1, 3>(ops, R, units, blocks, partial, partial_bytes, v, s))); break;
    case 3: HZ_TRY((launch_batch<128, 2, 6>(ops, R, units, blocks, partial, partial_bytes, v, s))); break;
    default: HZ_TRY((launch_batch<256, 2, 2>(ops, R, units, blocks, partial, partial_bytes, v, s))); break;
    }
    if (ev1) HZ_CHECK_CUDA(record_timing_event(ev1, s));
    return HZ_OK;
}

int sweep_f32(const SweepConst &c, const Rec32 &r, const double4_32a *pos64, int mode, const double *p_re,
              const double *p_im, const double *pt_re, const double *pt_im, double *q_re, double *q_im,
              double *qt_re, double *qt_im, float4 *dens, cudaStream_t s, cudaEvent_t ev0,
              cudaEvent_t ev1, int cfg)
{
    if (c.n <= 0) return HZ_OK;
    const bool useA = (mode & SWEEP_A) != 0, useH = (mode & SWEEP_AH) != 0;
    const double scale = ((c.interior == 1) ? -1.0 : 1.0) / (4.0 * kPi);
    {
        int dev = 0, sms = 152;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        long long b = (r.npad + 255) / 256;
        if (b > sms * 8) b = sms * 8;
        prep32_kernel<<<(unsigned)b, 256, 0, s>>>(r.npad, r.perm, r.tpos, useA ? p_re : nullptr,
                                                  useA ? p_im : nullptr, useH ? pt_re : nullptr,
                                                  useH ? pt_im : nullptr, scale, dens);
        HZ_CHECK_LAUNCH();
    }
    Args32 a;
    a.n = c.n;
    a.npad = r.npad;
    a.wave = (float)c.wave;
    a.tau = c.tau;
    a.mwords = r.mwords;
    a.thi = r.thi;
    a.tlo = r.tlo;
    a.ohi = r.ohi;
    a.olo = r.olo;
    a.nearmask = r.nearmask;
    a.tau2 = (float)(c.tau * c.tau);
    a.guard_lo = (float)(c.tau * c.tau * (1.0 - 1e-4));
    a.guard_hi = (float)(c.tau * c.tau * (1.0 + 1e-4));
    a.pos = r.pos;
    a.nrm = r.nrm;
    a.dens = dens;
    a.tpos = r.tpos;
    a.perm = r.perm;
    a.pos64 = pos64;
    a.p_re = p_re; a.p_im = p_im; a.pt_re = pt_re; a.pt_im = pt_im;
    a.q_re = q_re; a.q_im = q_im; a.qt_re = qt_re; a.qt_im = qt_im;
    a.err = c.err;
    if (ev0) HZ_CHECK_CUDA(record_timing_event(ev0, s));
    a.partial = r.partial;
    split_wave(c.wave, a.kh, a.kl);
    const bool dir = c.dirichlet != 0;
    constexpr int S = SWEEP_PHASE_SPLIT;
    if (c.phase_split) {
        if (mode == SWEEP_PAIR) HZ_TRY(launch32<SWEEP_PAIR | S>(cfg, a, dir, r.partial_bytes, s));
        else if (mode == SWEEP_A) HZ_TRY(launch32<SWEEP_A | S>(cfg, a, dir, r.partial_bytes, s));
        else HZ_TRY(launch32<SWEEP_AH | S>(cfg, a, dir, r.partial_bytes, s));
    } else {
        if (mode == SWEEP_PAIR) HZ_TRY(launch32<SWEEP_PAIR>(cfg, a, dir, r.partial_bytes, s));
        else if (mode == SWEEP_A) HZ_TRY(launch32<SWEEP_A>(cfg, a, dir, r.partial_bytes, s));
        else HZ_TRY(launch32<SWEEP_AH>(cfg, a, dir, r.partial_bytes, s));
    }
    if (ev1) HZ_CHECK_CUDA(record_timing_event(ev1, s));
    return HZ_OK;
}

HZ_DEFINE_WAIT_LIMIT_SETTER(set_wait_limit_f32)

}  // namespace hz
