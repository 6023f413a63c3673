// tube.cu -- narrow-band tube, per-point arrays and sweep-order records.
//
// Built with -fmad=false so that the projection x* = z - d grad d, the
// Jacobian, the interpolated normals and the regularisation factors keep
// the reference's unfused arithmetic (large3Dexample2.c:4340-4452,
// interpolate3D.c:5-102,569-605); only delta_eps (CUDA cos vs. the C
// library's) can differ from the reference, by an ulp or so.
#include "hz_internal.cuh"
#include "interp.cuh"

namespace hz {
namespace {

constexpr int kScanThreads = 256;
constexpr int kScanItems = 4;
constexpr int kScanTile = kScanThreads * kScanItems;

// Node enumeration orders: lexicographic (the reference's tube order) and
// blocked (8^3 node blocks in lexicographic block order, lexicographic
// inside a block) for spatially compact sweep tiles.
struct LexOrder {
    long long S;
    __device__ long long size() const { return S * S * S; }
    __device__ long long node(long long q) const { return q; }
};
struct BlockOrder {
    long long S, NB;  // NB = ceil(S/8) blocks per axis
    __device__ long long size() const { return NB * NB * NB * 512; }
    __device__ long long node(long long q) const
    {
        const long long b = q >> 9;
        const int l = (int)(q & 511);
        const long long bk = b % NB, bj = (b / NB) % NB, bi = b / (NB * NB);
        const long long i = bi * 8 + (l >> 6), j = bj * 8 + ((l >> 3) & 7), k = bk * 8 + (l & 7);
        if (i >= S || j >= S || k >= S) return -1;
        return (i * S + j) * S + k;
    }
};

template <class Order>
__device__ __forceinline__ bool member(const Order &ord, long long q, const double *__restrict__ d,
                                       double eps, long long &node)
{
    if (q >= ord.size()) return false;
    node = ord.node(q);
    if (node < 0) return false;
    return fabs(__ldg(d + node)) <= eps;  // large3Dexample2.c:571
}

template <class Order>
__global__ void __launch_bounds__(kScanThreads) count_kernel(Order ord, const double *__restrict__ d,
                                                             double eps, int *__restrict__ counts)
{
    const long long base = (long long)blockIdx.x * kScanTile + threadIdx.x * kScanItems;
    int c = 0;
    for (int t = 0; t < kScanItems; t++) {
        long long node;
        c += member(ord, base + t, d, eps, node) ? 1 : 0;
    }
    __shared__ int red[kScanThreads / 32];
    for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
        int s = 0;
        for (int w = 0; w < kScanThreads / 32; w++) s += red[w];
        counts[blockIdx.x] = s;
    }
}

// Exclusive scan of nb block counts in one block; total in offsets[nb].
__global__ void __launch_bounds__(1024) scan_counts_kernel(const int *__restrict__ counts,
                                                           long long *__restrict__ offsets, long long nb)
{
    __shared__ long long carry;
    __shared__ long long warp_sums[32];
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (long long start = 0; start < nb; start += 1024) {
        const long long q = start + threadIdx.x;
        long long v = (q < nb) ? counts[q] : 0;
        long long x = v;
        for (int o = 1; o < 32; o <<= 1) {
            long long y = __shfl_up_sync(0xffffffffu, x, o);
            if ((threadIdx.x & 31) >= o) x += y;
        }
        if ((threadIdx.x & 31) == 31) warp_sums[threadIdx.x >> 5] = x;
        __syncthreads();
        if (threadIdx.x < 32) {
            long long w = warp_sums[threadIdx.x];
            for (int o = 1; o < 32; o <<= 1) {
                long long y = __shfl_up_sync(0xffffffffu, w, o);
                if (threadIdx.x >= o) w += y;
            }
            warp_sums[threadIdx.x] = w;
        }
        __syncthreads();
        const long long incl = x + ((threadIdx.x >= 32) ? warp_sums[(threadIdx.x >> 5) - 1] : 0);
        if (q < nb) offsets[q] = carry + incl - v;
        __syncthreads();
        if (threadIdx.x == 1023) carry += incl;
        __syncthreads();
    }
    if (threadIdx.x == 0) offsets[nb] = carry;
}

template <class Order>
__global__ void __launch_bounds__(kScanThreads) compact_kernel(Order ord, const double *__restrict__ d,
                                                               double eps, const long long *__restrict__ offsets,
                                                               int64_t *__restrict__ out)
{
    const long long base = (long long)blockIdx.x * kScanTile + threadIdx.x * kScanItems;
    long long nodes[kScanItems];
    int flags = 0, c = 0;
    for (int t = 0; t < kScanItems; t++) {
        long long node = -1;
        if (member(ord, base + t, d, eps, node)) {
            flags |= 1 << t;
            c++;
        }
        nodes[t] = node;
    }
    // block exclusive scan of c (thread order == enumeration order)
    __shared__ int warp_sums[kScanThreads / 32];
    int x = c;
    for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, x, o);
        if ((threadIdx.x & 31) >= o) x += y;
    }
    if ((threadIdx.x & 31) == 31) warp_sums[threadIdx.x >> 5] = x;
    __syncthreads();
    if (threadIdx.x == 0) {
        int s = 0;
        for (int w = 0; w < kScanThreads / 32; w++) {
            int t = warp_sums[w];
            warp_sums[w] = s;
            s += t;
        }
    }
    __syncthreads();
    long long pos = offsets[blockIdx.x] + warp_sums[threadIdx.x >> 5] + x - c;
    for (int t = 0; t < kScanItems; t++)
        if (flags & (1 << t)) out[pos++] = nodes[t];
}

template <class Order>
int ordered_compaction(const Order &ord, long long total, const double *d, double eps, DevBuf &out,
                       int64_t &n, DevBuf &scratch, cudaStream_t s)
{
    const long long nb = (total + kScanTile - 1) / kScanTile;
    HZ_TRY(scratch.ensure(nb * sizeof(int) + (nb + 1) * sizeof(long long) + 64));
    int *counts = scratch.as<int>();
    long long *offsets = reinterpret_cast<long long *>(
        (reinterpret_cast<uintptr_t>(counts + nb) + 15) & ~uintptr_t(15));
    count_kernel<<<(unsigned)nb, kScanThreads, 0, s>>>(ord, d, eps, counts);
    HZ_CHECK_LAUNCH();
    scan_counts_kernel<<<1, 1024, 0, s>>>(counts, offsets, nb);
    HZ_CHECK_LAUNCH();
    long long total_n = 0;
    HZ_CHECK_CUDA(cudaMemcpyAsync(&total_n, offsets + nb, sizeof(long long), cudaMemcpyDeviceToHost, s));
    HZ_CHECK_CUDA(cudaStreamSynchronize(s));
    n = total_n;
    HZ_TRY(out.ensure((size_t)(total_n > 0 ? total_n : 1) * sizeof(int64_t)));
    if (total_n > 0) {
        compact_kernel<<<(unsigned)nb, kScanThreads, 0, s>>>(ord, d, eps, offsets, out.as<int64_t>());
        HZ_CHECK_LAUNCH();
    }
    return HZ_OK;
}

// ------------------------------------------------------- per-point arrays
struct InitArgs {
    int N;
    double H, int_l, eps, tau, wave, HC;
    int interior;
    const double *d, *gx, *gy, *gz, *mc, *gc;
    int64_t n;
    const int64_t *idx;
    double *xs, *nrm, *delta, *jac, *reg, *w;
    double *dreg;  // d reg / d k (for wave-number gradients), may be NULL
    double4_32a *pos64, *nrm64;
    unsigned *err;
};

__global__ void __launch_bounds__(256) init_kernel(InitArgs a)
{
    const double PI = 3.14159265358979323846264338328;  // constants.h:5
    const long long S = a.N + 1;
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < a.n;
         c += (int64_t)gridDim.x * blockDim.x) {
        const long long o = a.idx[c];
        const int i = (int)(o / (S * S)), j = (int)((o / S) % S), k = (int)(o % S);
        const double H = a.H;
        const double zy = a.int_l + H * (double)(i);
        const double zx = a.int_l + H * (double)(j);
        const double zz = a.int_l + H * (double)(k);
        const double dd = a.d[o];
        // large3Dexample2.c:4369-4371
        const double tx = zx - dd * a.gx[o], ty = zy - dd * a.gy[o], tz = zz - dd * a.gz[o];
        // functions.c:366-374 (cosine delta; |dd| <= eps holds for tube members)
        const double delta = (fabs(dd) <= a.eps) ? (1.0 / (2.0 * a.eps)) * (1.0 + cos(PI * dd / a.eps)) : 0.0;
        // :4392
        const double jac = 1 + 2. * dd * a.mc[o] + dd * dd * a.gc[o];
        // interpolate3D.c:21-29 cell of x*, then trilinear gradient (:41-77)
        double nx = 0, ny = 0, nz = 0;
        unsigned bad = interp_gradient(a.N, H, a.int_l, tx, ty, tz, a.gx, a.gy, a.gz, nx, ny, nz);
        if (!(bad & DEV_ERR_GRID)) {
            // the driver normalises once more (:4408-4412)
            const double gn = sqrt(nx * nx + ny * ny + nz * nz);
            nx = nx / gn;
            ny = ny / gn;
            nz = nz / gn;
        }
        // interpolate3D.c:569-605 curvatures at x* (cell with a 1e-19 nudge)
        double cm = 0.0, cg = 0.0;
        bad |= interp_curvatures(a.N, H, a.int_l, tx, ty, tz, a.mc, a.gc, cm, cg);
        // :4427-4445 regularisation factor
        const double tau = a.tau;
        const double r1 = cm / (4. * PI * tau);
        const double r2 = -5. * tau * (2. * cm) * (4. * cm * cm - cg) / (512. * PI);
        const double r3 = -25. * tau * (2. * cm) * cg / (1536. * PI);
        const double r4 = a.wave * a.wave * tau * 2. * cm / (48. * PI);
        const double reg = (a.interior == 1) ? (r1 + r2 + r3 + r4) : -1. * (r1 + r2 + r3 + r4);
        // only r4 = k^2 tau 2H / (48 pi) depends on k
        if (a.dreg) {
            const double d4 = 2.0 * a.wave * tau * 2. * cm / (48. * PI);
            a.dreg[c] = (a.interior == 1) ? d4 : -d4;
        }
        const double w = a.HC * delta * jac;  // :4447
        if (!isfinite(w) || !isfinite(reg)) bad |= DEV_ERR_NONFINITE;
        a.xs[3 * c] = tx;
        a.xs[3 * c + 1] = ty;
        a.xs[3 * c + 2] = tz;
        a.nrm[3 * c] = nx;
        a.nrm[3 * c + 1] = ny;
        a.nrm[3 * c + 2] = nz;
        a.delta[c] = delta;
        a.jac[c] = jac;
        a.reg[c] = reg;
        a.w[c] = w;
        a.pos64[c] = make_double4_32a(tx, ty, tz, reg);
        a.nrm64[c] = make_double4_32a(nx, ny, nz, w);
        if (bad) atomicOr(a.err, bad);
    }
}

__global__ void mark_kernel(int64_t n, const int64_t *__restrict__ idx, int *__restrict__ pos_of_node,
                            double *__restrict__ flag)
{
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x) {
        pos_of_node[idx[c]] = (int)c;
        flag[idx[c]] = 0.0;
    }
}

__global__ void perm_kernel(int64_t n, int64_t npad, const int64_t *__restrict__ nodes,
                            const int *__restrict__ pos_of_node, int *__restrict__ perm)
{
    for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < npad; s += (int64_t)gridDim.x * blockDim.x)
        perm[s] = (s < n) ? pos_of_node[nodes[s]] : -1;
}

// One block per source tile: tile origin = centre of the tile's bounding
// box (FP64), then FP32 offsets from it.
__global__ void __launch_bounds__(kTile32) rec32_kernel(const int *__restrict__ perm,
                                                        const double4_32a *__restrict__ pos64,
                                                        const double4_32a *__restrict__ nrm64,
                                                        float4 *__restrict__ pos32, float4 *__restrict__ nrm32,
                                                        double4_32a *__restrict__ origin, double4_32a *__restrict__ tpos,
                                                        float4 *__restrict__ thi, float4 *__restrict__ tlo,
                                                        double reg_scale)
{
    const int64_t s = (int64_t)blockIdx.x * kTile32 + threadIdx.x;
    const int c = perm[s];
    double4_32a p = make_double4_32a(0, 0, 0, 0), q = make_double4_32a(0, 0, 0, 0);
    if (c >= 0) {
        p = pos64[c];
        q = nrm64[c];
    }
    __shared__ double lo[3][kTile32 / 32], hi[3][kTile32 / 32];
    double v[3] = {p.x, p.y, p.z};
    double mn[3], mx[3];
    for (int a = 0; a < 3; a++) {
        mn[a] = (c >= 0) ? v[a] : 1e300;
        mx[a] = (c >= 0) ? v[a] : -1e300;
        for (int o = 16; o > 0; o >>= 1) {
            mn[a] = fmin(mn[a], __shfl_xor_sync(0xffffffffu, mn[a], o));
            mx[a] = fmax(mx[a], __shfl_xor_sync(0xffffffffu, mx[a], o));
        }
        if ((threadIdx.x & 31) == 0) {
            lo[a][threadIdx.x >> 5] = mn[a];
            hi[a][threadIdx.x >> 5] = mx[a];
        }
    }
    __syncthreads();
    __shared__ double org[3], ext[3];
    if (threadIdx.x < 3) {
        double a0 = 1e300, a1 = -1e300;
        for (int w = 0; w < kTile32 / 32; w++) {
            a0 = fmin(a0, lo[threadIdx.x][w]);
            a1 = fmax(a1, hi[threadIdx.x][w]);
        }
        org[threadIdx.x] = (a0 <= a1) ? 0.5 * (a0 + a1) : 0.0;
        ext[threadIdx.x] = (a0 <= a1) ? 0.5 * (a1 - a0) : 0.0;
    }
    __syncthreads();
    // .w = radius of a sphere around the origin that holds every point of
    // the tile (half the bounding-box diagonal, rounded up a little)
    if (threadIdx.x == 0)
        origin[blockIdx.x] = make_double4_32a(org[0], org[1], org[2],
                                              sqrt(ext[0] * ext[0] + ext[1] * ext[1] + ext[2] * ext[2]) * (1.0 + 1e-12));
    if (c >= 0) {
        pos32[s] = make_float4((float)(p.x - org[0]), (float)(p.y - org[1]), (float)(p.z - org[2]),
                               (float)(p.w * reg_scale));
        nrm32[s] = make_float4((float)q.x, (float)q.y, (float)q.z, (float)q.w);
        tpos[s] = make_double4_32a(p.x, p.y, p.z, q.w);
    } else {
        pos32[s] = make_float4(0.f, 0.f, 0.f, 0.f);
        nrm32[s] = make_float4(0.f, 0.f, 0.f, 0.f);
        tpos[s] = make_double4_32a(org[0], org[1], org[2], 0.0);
        p = make_double4_32a(org[0], org[1], org[2], 0.0);
    }
    const float hx = (float)p.x, hy = (float)p.y, hz = (float)p.z;
    thi[s] = make_float4(hx, hy, hz, 0.f);
    tlo[s] = make_float4((float)(p.x - (double)hx), (float)(p.y - (double)hy), (float)(p.z - (double)hz), 0.f);
}

// Tile origins split into FP32 head + tail (x = hi + lo to about 2^-48 |x|).
__global__ void split_origin_kernel(int64_t ntiles, const double4_32a *__restrict__ origin, float4 *__restrict__ ohi,
                                    float4 *__restrict__ olo)
{
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= ntiles) return;
    const double4_32a o = origin[t];
    const float hx = (float)o.x, hy = (float)o.y, hz = (float)o.z;
    ohi[t] = make_float4(hx, hy, hz, 0.f);
    olo[t] = make_float4((float)(o.x - (double)hx), (float)(o.y - (double)hy), (float)(o.z - (double)hz), 0.f);
}

// Near-tile mask: bit s of row t is clear only when the bounding spheres of
// tiles t and s are more than tau_far apart, so that no pair between them
// has rho <= tau (tau_far carries a 1e-3 relative margin).
__global__ void nearmask_kernel(int64_t ntiles, int64_t mwords, const double4_32a *__restrict__ origin,
                                double tau_far, uint32_t *__restrict__ mask)
{
    const int64_t id = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (id >= ntiles * mwords) return;
    const int64_t t = id / mwords, w = id - t * mwords;
    const double4_32a o = origin[t];
    uint32_t bits = 0;
    for (int b = 0; b < 32; b++) {
        const int64_t q = w * 32 + b;
        if (q >= ntiles) break;
        const double4_32a u = origin[q];
        const double ex = u.x - o.x, ey = u.y - o.y, ez = u.z - o.z;
        const bool far = sqrt(ex * ex + ey * ey + ez * ez) - u.w - o.w > tau_far;
        if (!far) bits |= 1u << b;
    }
    mask[id] = bits;
}

int grid_blocks(long long work, int threads)
{
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    long long b = (work + threads - 1) / threads;
    const long long cap = (long long)sms * 32;
    if (b > cap) b = cap;
    if (b < 1) b = 1;
    return (int)b;
}

}  // namespace

int tube_build(int N, double eps, const double *d, DevBuf &idx, int64_t &n, DevBuf &scratch, cudaStream_t s)
{
    const long long S = N + 1;
    return ordered_compaction(LexOrder{S}, S * S * S, d, eps, idx, n, scratch, s);
}

int tube_init(const hz_params &p, const double *d, const double *gx, const double *gy, const double *gz,
              const double *mc, const double *gc, int64_t n, const int64_t *idx, double *xs, double *nrm,
              double *delta, double *jac, double *reg, double *w, double4_32a *pos64, double4_32a *nrm64,
              unsigned *err, cudaStream_t s, double *dreg)
{
    InitArgs a;
    a.dreg = dreg;
    a.N = p.N;
    a.H = (p.int_u - p.int_l) / p.N;
    a.int_l = p.int_l;
    a.eps = p.factor * a.H;
    a.tau = a.H * p.tau_factor;
    a.wave = p.wave;
    a.HC = a.H * a.H * a.H;
    a.interior = p.interior;
    a.d = d; a.gx = gx; a.gy = gy; a.gz = gz; a.mc = mc; a.gc = gc;
    a.n = n; a.idx = idx;
    a.xs = xs; a.nrm = nrm; a.delta = delta; a.jac = jac; a.reg = reg; a.w = w;
    a.pos64 = pos64; a.nrm64 = nrm64; a.err = err;
    if (n == 0) return HZ_OK;
    init_kernel<<<grid_blocks(n, 256), 256, 0, s>>>(a);
    HZ_CHECK_LAUNCH();
    return HZ_OK;
}

int sweep_order(int N, int64_t n, const int64_t *idx, int *perm, int64_t npad, DevBuf &scratch, cudaStream_t s)
{
    // Blocked enumeration of the tube nodes: mark members on a flag grid
    // (0 inside the tube, a large value outside), compact it in blocked
    // order, and map each node back to its lexicographic tube position.
    const long long S = N + 1;
    const long long NB = (S + 7) / 8;
    DevBuf map, nodes, flag;
    HZ_TRY(map.ensure((size_t)(S * S * S) * sizeof(int)));
    HZ_TRY(flag.ensure((size_t)(S * S * S) * sizeof(double)));
    HZ_CHECK_CUDA(cudaMemsetAsync(flag.ptr, 0x7f, (size_t)(S * S * S) * sizeof(double), s));
    if (n > 0) {
        mark_kernel<<<grid_blocks(n, 256), 256, 0, s>>>(n, idx, map.as<int>(), flag.as<double>());
        HZ_CHECK_LAUNCH();
    }
    int64_t n2 = 0;
    HZ_TRY(ordered_compaction(BlockOrder{S, NB}, NB * NB * NB * 512, flag.as<double>(), 0.5, nodes, n2, scratch, s));
    if (n2 != n) {
        set_error("sweep order: blocked enumeration found %lld of %lld tube nodes", (long long)n2, (long long)n);
        return HZ_ERR_STATE;
    }
    perm_kernel<<<grid_blocks(npad, 256), 256, 0, s>>>(n, npad, nodes.as<int64_t>(), map.as<int>(), perm);
    HZ_CHECK_LAUNCH();
    HZ_CHECK_CUDA(cudaStreamSynchronize(s));
    return HZ_OK;
}

int build_rec32(const Rec32 &r, const double4_32a *pos64, const double4_32a *nrm64, double reg_scale, double tau,
                cudaStream_t s)
{
    const int64_t ntiles = r.npad / kTile32;
    if (ntiles == 0) return HZ_OK;
    rec32_kernel<<<(unsigned)ntiles, kTile32, 0, s>>>(r.perm, pos64, nrm64, r.pos, r.nrm, r.origin, r.tpos, r.thi,
                                                      r.tlo, reg_scale);
    HZ_CHECK_LAUNCH();
    split_origin_kernel<<<(unsigned)((ntiles + 255) / 256), 256, 0, s>>>(ntiles, r.origin, r.ohi, r.olo);
    HZ_CHECK_LAUNCH();
    const int64_t cells = ntiles * r.mwords;
    nearmask_kernel<<<(unsigned)((cells + 255) / 256), 256, 0, s>>>(ntiles, r.mwords, r.origin, tau * (1.0 + 1e-3),
                                                                    r.nearmask);
    HZ_CHECK_LAUNCH();
    return HZ_OK;
}

}  // namespace hz
