// noalloc.cu -- an FP64 matrix-free product that allocates no memory.
//
// hz_matvec and the rest of the operator API stage the tube records and
// the weighted densities in device buffers that the operator allocates.  Some callers cannot
// allocate device memory at the point where they need a product: host
// applications that hand out all device memory from their own pools, plugin
// hosts that forbid allocation after start-up, and loops where the implicit
// synchronisation of cudaMalloc/cudaFree is not acceptable.  This entry point
// serves them: the caller passes device inputs and outputs, and the scratch
// (packed records, weighted densities, error word) lives in one file-scope
// __device__ array of fixed size, which every GPU that loads the library
// holds until the process exits.
#include "hz_internal.cuh"

#include <cmath>
#include <mutex>

namespace hz {
namespace {

constexpr int64_t kStaticMaxPoints = HZ_NOALLOC_MAX_POINTS;
constexpr size_t kRecBytes = sizeof(double4_32a) * (size_t)kStaticMaxPoints;
constexpr size_t kStaticBytes = 3 * kRecBytes + 256;  // pos, nrm, densities, error word

// The scratch.  In host code this name is only a stand-in for the symbol;
// its device address comes from cudaGetSymbolAddress.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kStaticBytes];

// Device addresses of the scratch, one per CUDA context: a __device__
// symbol's address belongs to the context that loaded the module, not to the
// device, so a context of the caller's own (cuCtxCreate / cuCtxSetCurrent) or
// a new primary context after cudaDeviceReset has its own copy.
constexpr int kMaxContexts = 64;
std::mutex g_mu;
struct CtxAddr {
    void *ctx;
    void *addr;
};
CtxAddr g_addr[kMaxContexts] = {};
int g_used = 0;

typedef int (*CtxGetCurrentFn)(void **);

// The driver's cuCtxGetCurrent, reached through the runtime so that the
// library needs no link against libcuda.
void *current_context()
{
    static CtxGetCurrentFn fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<CtxGetCurrentFn>(f);
        cudaGetLastError();
    });
    void *ctx = nullptr;
    if (!fn || fn(&ctx) != 0) return nullptr;
    return ctx;
}

// Device address of the scratch in the current context.  Outside stream
// capture the address is looked up again on every call (a host-side lookup,
// no device work), so a reset device or a switched context never sees a
// stale address; while `s` is capturing, the address cached for the current
// context by an earlier call is used, so the first call in a context must
// come before any capture.
int scratch_address(cudaStream_t s, void **out)
{
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    HZ_CHECK_CUDA(cudaStreamIsCapturing(s, &cap));
    void *ctx = current_context();
    std::lock_guard<std::mutex> lock(g_mu);
    int slot = -1;
    for (int i = 0; i < g_used; i++)
        if (g_addr[i].ctx == ctx) slot = i;
    if (cap != cudaStreamCaptureStatusNone) {
        if (slot < 0 || !g_addr[slot].addr) {
            set_error("hz_matvec_f64_noalloc: first call in this CUDA context made during stream capture");
            return HZ_ERR_STATE;
        }
        *out = g_addr[slot].addr;
        return HZ_OK;
    }
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
        set_error("hz_matvec_f64_noalloc: cudaGetSymbolAddress failed: %s", cudaGetErrorString(e));
        cudaGetLastError();
        return HZ_ERR_CUDA;
    }
    if (slot < 0) {
        slot = (g_used < kMaxContexts) ? g_used++ : (int)(((uintptr_t)ctx >> 4) % kMaxContexts);
        g_addr[slot].ctx = ctx;
    }
    g_addr[slot].addr = p;
    *out = p;
    return HZ_OK;
}

__global__ void pack_records_kernel(int64_t n, const double *__restrict__ xs, const double *__restrict__ nrm,
                                    const double *__restrict__ reg, const double *__restrict__ w,
                                    double4_32a *__restrict__ pos, double4_32a *__restrict__ nr)
{
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x) {
        pos[c] = make_double4_32a(xs[3 * c], xs[3 * c + 1], xs[3 * c + 2], reg[c]);
        nr[c] = make_double4_32a(nrm[3 * c], nrm[3 * c + 1], nrm[3 * c + 2], w[c]);
    }
}

}  // namespace
}  // namespace hz

using namespace hz;

extern "C" int hz_matvec_f64_noalloc(const hz_params *p, int64_t n, int adjoint, const double *xs,
                                     const double *nrm, const double *reg, const double *w, const double *p_re,
                                     const double *p_im, double *q_re, double *q_im, void *stream)
{
    if (!p || !(p->int_u > p->int_l) || p->N < 1 || !(p->tau_factor > 0) || !std::isfinite(p->wave)) {
        set_error("hz_matvec_f64_noalloc: bad parameters");
        return HZ_ERR_ARG;
    }
    if (n < 1 || n > kStaticMaxPoints) {
        set_error("hz_matvec_f64_noalloc: n = %lld is outside [1, %lld], the size of its static scratch",
                  (long long)n, (long long)kStaticMaxPoints);
        return HZ_ERR_ARG;
    }
    if (!xs || !nrm || !reg || !w || !p_re || !p_im || !q_re || !q_im) {
        set_error("hz_matvec_f64_noalloc: NULL pointer");
        return HZ_ERR_ARG;
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    void *base = nullptr;
    HZ_TRY(scratch_address(s, &base));
    unsigned char *b = static_cast<unsigned char *>(base);
    double4_32a *pos = reinterpret_cast<double4_32a *>(b);
    double4_32a *nr = reinterpret_cast<double4_32a *>(b + kRecBytes);
    double2 *dens = reinterpret_cast<double2 *>(b + 2 * kRecBytes);
    unsigned *err = reinterpret_cast<unsigned *>(b + 3 * kRecBytes);
    // the array keeps the previous call's contents: records and densities
    // are rewritten for c < n below, the error word must start at zero
    HZ_CHECK_CUDA(cudaMemsetAsync(err, 0, sizeof(unsigned), s));
    {
        long long blocks = (n + 255) / 256;
        if (blocks > 1024) blocks = 1024;
        pack_records_kernel<<<(unsigned)blocks, 256, 0, s>>>(n, xs, nrm, reg, w, pos, nr);
        HZ_CHECK_LAUNCH();
    }
    SweepConst c;
    c.n = n;
    c.wave = p->wave;
    c.tau = ((p->int_u - p->int_l) / p->N) * p->tau_factor;
    c.dirichlet = p->dirichlet;
    c.interior = p->interior;
    c.err = err;
    c.extent = 1.7320508075688772 * (p->int_u - p->int_l);
    Rec64 r;
    r.pos = pos;
    r.nrm = nr;
    if (adjoint)
        HZ_TRY(sweep_f64(c, r, SWEEP_AH, nullptr, nullptr, p_re, p_im, nullptr, nullptr, q_re, q_im, dens, s));
    else
        HZ_TRY(sweep_f64(c, r, SWEEP_A, p_re, p_im, nullptr, nullptr, q_re, q_im, nullptr, nullptr, dens, s));
    unsigned e = 0;
    HZ_CHECK_CUDA(cudaMemcpyAsync(&e, err, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
    HZ_CHECK_CUDA(cudaStreamSynchronize(s));
    if (e & DEV_ERR_WAIT) {
        set_error("hz_matvec_f64_noalloc: a bounded device wait gave up");
        return HZ_ERR_DEVICE_WAIT;
    }
    if (e & DEV_ERR_NONFINITE) {
        set_error("hz_matvec_f64_noalloc: non-finite value");
        return HZ_ERR_NONFINITE;
    }
    return HZ_OK;
}
