// sweep_combo32.cu -- FP32 matrix-free products of the Combo formulation
// (new_HelmholtzKernelCombo, HelmholtzKernel.c:411-607): the bulk products of
// mixed-precision Combo solves, whose FP64 residuals come from combo.cu.
//
// Entry kappa_ij of target i and source j (combo.cu states the full sum):
//   kappa_ij = (eta parti + c4 D) + i (-eta part + c4 Dimg)
// with part + i parti the regularised single-layer gradient at x*_i (normal
// n_i, wave W; reg_i within tau) and D + i Dimg the hypersingular double
// layer between the offset point x*_i + |d_j| n_i and x*_j (wave k).  With
// c4 = 1/(4 pi) folded into the densities, kappa / c4 is
//   (eta parti' + Tr) + i (-eta part' + Ti),
//   part' = -(W S + C/r) sip / r^2,  parti' = (W C - S/r) sip / r^2,
//   sip = -(x_i - x_j).n_i,  part' = 4 pi reg_i within tau,
//   Tr = (1/y) [-cm1 e1 + cm2 (3 e1 / y - k^2 C2)],
//   Ti = (1/y) [ cm1 e2 - cm2 (3 e2 / y + k^2 S2)],
//   e1 = k S2 + C2 / y,  e2 = k C2 - S2 / y,  cm1 = n_i.n_j / y,
//   cm2 = (y.n_i)(y.n_j) / y^2,
// (S, C) = sin, cos (W r), (S2, C2) = sin, cos (k |y|): the reference's four
// terms t1..t4 (HelmholtzKernel.c:539-571) regrouped.
//
// The FP32 machinery is the classic sweep's (sweep_f32.cu): blocked sweep
// order, FP32 head + tail split target positions, phases straight into the
// SFU's sin/cos, the near-field test decided in FP64 inside a guard band
// around tau^2, a near-tile mask, TwoSum cross-tile sums and TMA bulk copies
// of source tiles on bounded mbarrier waits.  The
// per-source |d_j| rides in nrm32.w (the weight is in tpos.w).  A and A^H
// evaluate the offset point on different sides (x*_i + |d_j| n_i against
// x*_j + |d_i| n_j), so the two products are separate launches; one CTA
// holds one 256-slot target tile.
#include "hz_internal.cuh"
#include "bulk_copy.cuh"

namespace hz {
namespace {

constexpr double kPi = 3.14159265358979323846264338328;
constexpr int kCNT = 128;  // threads per CTA
constexpr int kCTG = 2;    // targets per thread: kCNT * kCTG = kTile32

struct Combo32Args {
    int64_t npad, mwords;
    float W;  // single-layer wave
    float K;  // hypersingular wave number
    float k2, eta;
    float tau2, guard_lo, guard_hi;
    double tau, eta64;
    const float4 *pos, *nrm, *dens;
    const float4 *thi, *tlo, *ohi, *olo;
    const uint32_t *nearmask;
    const double4_32a *tpos;
    const double4_32a *pos64;
    const int *perm;
    const double *p_re, *p_im;
    double *q_re, *q_im;
    unsigned *err;
};

__device__ __forceinline__ void two_sum_acc(float &hi, float &lo, float f)
{
    const float s = hi + f;
    const float bp = s - hi;
    const float e = (hi - (s - bp)) + (f - bp);
    hi = s;
    lo += e;
}

// One source slot against one target slot.  ADJ = false: kappa_ts (target t
// is row i); ADJ = true: conj(kappa_st) (the source slot is row i).
// m = x_t - x_s; s_n.w = |d_s|, td = |d_t|.
template <bool ADJ, bool NEAR>
__device__ __forceinline__ void combo_pair(const Combo32Args &a, const float4 s_p, const float4 s_n, const float4 s_d,
                                           const float3 rel, const float3 tn, float td, float treg, int64_t tslot,
                                           int64_t sslot, float &fr, float &fi)
{
    const float mx = rel.x - s_p.x, my = rel.y - s_p.y, mz = rel.z - s_p.z;
    const float r2 = fmaf(mx, mx, fmaf(my, my, mz * mz));
    bool near = false;
    if (NEAR) {
        near = r2 <= a.tau2;
        if (r2 > a.guard_lo && r2 < a.guard_hi) {
            // decide exactly as the FP64 Combo sweep does
            const int c = a.perm[sslot];
            if (c >= 0) {
                const double4_32a q = a.pos64[c];
                const double4_32a tp = a.tpos[tslot];
                const double x1 = tp.x - q.x, x2 = tp.y - q.y, x3 = tp.z - q.z;
                near = !(sqrt(x1 * x1 + x2 * x2 + x3 * x3) > a.tau);
            }
        }
    }
    // single-layer gradient at row i's point with row i's normal
    const float rinv = rsqrtf(r2);
    const float rho = r2 * rinv;
    float S, C;
    __sincosf(rho * a.W, &S, &C);
    const float u1 = fmaf(C, rinv, a.W * S);   // W sin + cos / r
    const float u2 = fmaf(a.W, C, -S * rinv);  // W cos - sin / r
    const float rr = rinv * rinv;
    const float sip = ADJ ? (mx * s_n.x + my * s_n.y + mz * s_n.z) : -(mx * tn.x + my * tn.y + mz * tn.z);
    float part = -u1 * rr * sip, parti = u2 * rr * sip;
    if (NEAR && near) {
        part = ADJ ? s_p.w : treg;
        parti = 0.f;
    }
    // hypersingular double layer: y = x*_i + |d_j| n_i - x*_j
    float3 na, nb, y;
    if (!ADJ) {
        na = tn;
        nb = make_float3(s_n.x, s_n.y, s_n.z);
        y = make_float3(fmaf(s_n.w, tn.x, mx), fmaf(s_n.w, tn.y, my), fmaf(s_n.w, tn.z, mz));
    } else {
        na = make_float3(s_n.x, s_n.y, s_n.z);
        nb = tn;
        y = make_float3(fmaf(td, s_n.x, -mx), fmaf(td, s_n.y, -my), fmaf(td, s_n.z, -mz));
    }
    // a floor on |y|^2 keeps padding slots (zero normals and densities) finite
    const float y2 = fmaxf(fmaf(y.x, y.x, fmaf(y.y, y.y, y.z * y.z)), 1e-20f);
    const float yinv = rsqrtf(y2);
    const float yn = y2 * yinv;
    float S2, C2;
    __sincosf(yn * a.K, &S2, &C2);
    const float ip1 = fmaf(na.x, nb.x, fmaf(na.y, nb.y, na.z * nb.z));
    const float ip2 = fmaf(y.x, na.x, fmaf(y.y, na.y, y.z * na.z));
    const float ip3 = fmaf(y.x, nb.x, fmaf(y.y, nb.y, y.z * nb.z));
    const float cm1 = ip1 * yinv;
    const float cm2 = ip2 * ip3 * (yinv * yinv);
    const float e1 = fmaf(C2, yinv, a.K * S2);
    const float e2 = fmaf(a.K, C2, -S2 * yinv);
    const float g3 = 3.f * yinv;
    const float Tr = yinv * fmaf(cm2, fmaf(g3, e1, -a.k2 * C2), -cm1 * e1);
    const float Ti = yinv * fmaf(-cm2, fmaf(g3, e2, a.k2 * S2), cm1 * e2);
    const float kr = fmaf(a.eta, parti, Tr);
    const float ki = fmaf(-a.eta, part, Ti);
    if (!ADJ) {
        fr = fmaf(kr, s_d.x, fmaf(-ki, s_d.y, fr));
        fi = fmaf(kr, s_d.y, fmaf(ki, s_d.x, fi));
    } else {
        fr = fmaf(kr, s_d.x, fmaf(ki, s_d.y, fr));
        fi = fmaf(kr, s_d.y, fmaf(-ki, s_d.x, fi));
    }
}

// A p (ADJ = false): q_t = sum_s kappa_ts r_s p_s + (i eta / 2) p_t;
// A^H p (ADJ = true): q_t = r_t sum_s conj(kappa_st) p_s - (i eta / 2) p_t.
template <bool ADJ>
__global__ void __launch_bounds__(kCNT) combo32_kernel(Combo32Args a)
{
    constexpr int TS = kTile32, NT = kCNT, TG = kCTG;
    static_assert(NT * TG == TS, "one target tile per CTA");
    __shared__ alignas(128) float4 sp[2][TS];
    __shared__ alignas(128) float4 sn[2][TS];
    __shared__ alignas(128) float4 sd[2][TS];
    __shared__ alignas(8) uint64_t bar[2];
    const int64_t ntiles = a.npad / TS;
    const int64_t blk = blockIdx.x;
    if (threadIdx.x == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        fence_barrier_init();
    }
    __syncthreads();
    auto issue = [&](int64_t tile, int buf) {
        const int64_t base = tile * TS;
        const uint32_t bytes = TS * sizeof(float4);
        mbar_arrive_expect_tx(&bar[buf], 3 * bytes);
        bulk_g2s(&sp[buf][0], a.pos + base, bytes, &bar[buf]);
        bulk_g2s(&sn[buf][0], a.nrm + base, bytes, &bar[buf]);
        bulk_g2s(&sd[buf][0], a.dens + base, bytes, &bar[buf]);
    };
    if (threadIdx.x == 0) issue(0, 0);
    const int64_t slot0 = blk * TS + threadIdx.x;
    float3 th[TG], tl[TG], tn[TG];
    float td[TG], treg[TG], hr[TG], lr[TG], hi[TG], li[TG];
#pragma unroll
    for (int g = 0; g < TG; g++) {
        const int64_t s = slot0 + (int64_t)g * NT;
        const float4 h = a.thi[s], l = a.tlo[s], nn = a.nrm[s];
        th[g] = make_float3(h.x, h.y, h.z);
        tl[g] = make_float3(l.x, l.y, l.z);
        tn[g] = make_float3(nn.x, nn.y, nn.z);
        td[g] = nn.w;
        treg[g] = a.pos[s].w;
        hr[g] = lr[g] = hi[g] = li[g] = 0.f;
    }
    const uint32_t *mrow = a.nearmask + blk * a.mwords;
    for (int64_t tile = 0; tile < ntiles; tile++) {
        const int buf = (int)(tile & 1);
        if (threadIdx.x == 0 && tile + 1 < ntiles) issue(tile + 1, buf ^ 1);
        const bool far = ((__ldg(mrow + (tile >> 5)) >> (tile & 31)) & 1u) == 0;
        const float4 oh = a.ohi[tile], ol = a.olo[tile];
        float3 rel[TG];
#pragma unroll
        for (int g = 0; g < TG; g++)
            rel[g] = make_float3((th[g].x - oh.x) + (tl[g].x - ol.x), (th[g].y - oh.y) + (tl[g].y - ol.y),
                                 (th[g].z - oh.z) + (tl[g].z - ol.z));
        const bool ok = mbar_wait_bounded(&bar[buf], (uint32_t)((tile >> 1) & 1), g_data_wait_limit);
        if (__syncthreads_or(!ok)) {
            if (threadIdx.x == 0) {
                atomicOr(a.err, DEV_ERR_WAIT);
                mbar_drain(&bar[buf], (uint32_t)((tile >> 1) & 1), &bar[buf ^ 1], (uint32_t)(((tile + 1) >> 1) & 1),
                           tile + 1 < ntiles);
            }
            return;
        }
        float fr[TG], fi[TG];
#pragma unroll
        for (int g = 0; g < TG; g++) fr[g] = fi[g] = 0.f;
        const int64_t base = tile * TS;
        if (far) {
#pragma unroll 2
            for (int j = 0; j < TS; j++) {
#pragma unroll
                for (int g = 0; g < TG; g++)
                    combo_pair<ADJ, false>(a, sp[buf][j], sn[buf][j], sd[buf][j], rel[g], tn[g], td[g], treg[g],
                                           slot0 + (int64_t)g * NT, base + j, fr[g], fi[g]);
            }
        } else {
#pragma unroll 2
            for (int j = 0; j < TS; j++) {
#pragma unroll
                for (int g = 0; g < TG; g++)
                    combo_pair<ADJ, true>(a, sp[buf][j], sn[buf][j], sd[buf][j], rel[g], tn[g], td[g], treg[g],
                                          slot0 + (int64_t)g * NT, base + j, fr[g], fi[g]);
            }
        }
#pragma unroll
        for (int g = 0; g < TG; g++) {
            two_sum_acc(hr[g], lr[g], fr[g]);
            two_sum_acc(hi[g], li[g], fi[g]);
        }
        __syncthreads();
    }
    const double he = 0.5 * a.eta64;
#pragma unroll
    for (int g = 0; g < TG; g++) {
        const int64_t s = slot0 + (int64_t)g * NT;
        const int c = a.perm[s];
        if (c < 0) continue;
        const double ar = (double)hr[g] + (double)lr[g], ai = (double)hi[g] + (double)li[g];
        const double pr = a.p_re[c], pi = a.p_im[c];
        double qr, qi;
        if (!ADJ) {
            qr = ar - he * pi;
            qi = ai + he * pr;
        } else {
            const double r = a.tpos[s].w;
            qr = r * ar + he * pi;
            qi = r * ai - he * pr;
        }
        if (!isfinite(qr) || !isfinite(qi)) atomicOr(a.err, DEV_ERR_NONFINITE);
        a.q_re[c] = qr;
        a.q_im[c] = qi;
    }
}

// Densities in sweep order: c4 r_s p_s (A) or c4 p_s (A^H); padding zero.
__global__ void combo32_prep_kernel(int64_t npad, const int *__restrict__ perm, const double4_32a *__restrict__ tpos,
                                    const double *__restrict__ p_re, const double *__restrict__ p_im, int adj,
                                    float4 *__restrict__ dens)
{
    const double c4 = 1.0 / (4.0 * kPi);
    for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < npad; s += (int64_t)gridDim.x * blockDim.x) {
        const int c = perm[s];
        float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
        if (c >= 0) {
            const double f = adj ? c4 : c4 * tpos[s].w;
            v.x = (float)(f * p_re[c]);
            v.y = (float)(f * p_im[c]);
        }
        dens[s] = v;
    }
}

// |d_s| of every slot into nrm32.w (padding: 0).
__global__ void combo32_dist_kernel(int64_t npad, const int *__restrict__ perm, const double *__restrict__ adist,
                                    float4 *__restrict__ nrm)
{
    for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < npad; s += (int64_t)gridDim.x * blockDim.x) {
        const int c = perm[s];
        nrm[s].w = c >= 0 ? (float)adist[c] : 0.f;
    }
}

unsigned prep_blocks(int64_t npad)
{
    long long b = (npad + 255) / 256;
    if (b > 4096) b = 4096;
    return (unsigned)(b < 1 ? 1 : b);
}

}  // namespace

int combo32_set_distances(const Rec32 &r, const double *adist, cudaStream_t s)
{
    if (r.npad <= 0) return HZ_OK;
    combo32_dist_kernel<<<prep_blocks(r.npad), 256, 0, s>>>(r.npad, r.perm, adist, r.nrm);
    HZ_CHECK_LAUNCH();
    return HZ_OK;
}

int sweep_combo32(const SweepConst &c, const Rec32 &r, const double4_32a *pos64, double wavenum, double eta, int mode,
                  const double *p_re, const double *p_im, const double *pt_re, const double *pt_im, double *q_re,
                  double *q_im, double *qt_re, double *qt_im, float4 *dens, cudaStream_t s, cudaEvent_t ev0,
                  cudaEvent_t ev1)
{
    if (c.n <= 0 || r.npad <= 0) return HZ_OK;
    if (r.npad % kTile32 != 0) {
        set_error("FP32 Combo sweep: %lld slots, not a multiple of %d", (long long)r.npad, kTile32);
        return HZ_ERR_STATE;
    }
    Combo32Args a;
    a.npad = r.npad;
    a.mwords = r.mwords;
    a.W = (float)c.wave;
    a.K = (float)wavenum;
    a.k2 = (float)(wavenum * wavenum);
    a.eta = (float)eta;
    a.eta64 = eta;
    a.tau = c.tau;
    a.tau2 = (float)(c.tau * c.tau);
    a.guard_lo = (float)(c.tau * c.tau * (1.0 - 1e-4));
    a.guard_hi = (float)(c.tau * c.tau * (1.0 + 1e-4));
    a.pos = r.pos;
    a.nrm = r.nrm;
    a.dens = dens;
    a.thi = r.thi;
    a.tlo = r.tlo;
    a.ohi = r.ohi;
    a.olo = r.olo;
    a.nearmask = r.nearmask;
    a.tpos = r.tpos;
    a.pos64 = pos64;
    a.perm = r.perm;
    a.err = c.err;
    const unsigned blocks = (unsigned)(r.npad / kTile32);
    if (ev0) HZ_CHECK_CUDA(record_timing_event(ev0, s));
    if (mode & SWEEP_A) {
        combo32_prep_kernel<<<prep_blocks(r.npad), 256, 0, s>>>(r.npad, r.perm, r.tpos, p_re, p_im, 0, dens);
        HZ_CHECK_LAUNCH();
        a.p_re = p_re;
        a.p_im = p_im;
        a.q_re = q_re;
        a.q_im = q_im;
        combo32_kernel<false><<<blocks, kCNT, 0, s>>>(a);
        HZ_CHECK_LAUNCH();
    }
    if (mode & SWEEP_AH) {
        combo32_prep_kernel<<<prep_blocks(r.npad), 256, 0, s>>>(r.npad, r.perm, r.tpos, pt_re, pt_im, 1, dens);
        HZ_CHECK_LAUNCH();
        a.p_re = pt_re;
        a.p_im = pt_im;
        a.q_re = qt_re;
        a.q_im = qt_im;
        combo32_kernel<true><<<blocks, kCNT, 0, s>>>(a);
        HZ_CHECK_LAUNCH();
    }
    if (ev1) HZ_CHECK_CUDA(record_timing_event(ev1, s));
    return HZ_OK;
}

HZ_DEFINE_WAIT_LIMIT_SETTER(set_wait_limit_combo32)

}  // namespace hz
