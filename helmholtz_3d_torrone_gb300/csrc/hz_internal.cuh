// hz_internal.cuh -- shared declarations of the GB300 IBIM Helmholtz library.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <cstddef>
#include <vector>

#include "../../include/helmholtz_gb300.h"

namespace hz {

// ---------------------------------------------------------------- errors
void set_error(const char *fmt, ...);
// Host-or-device staging for the C ABI (capi.cu): copy count doubles from
// src (host memory when where == HZ_HOST, device otherwise) to device dst,
// and back; stage_out ignores a NULL dst.
int stage_in(double *dst, const double *src, size_t count, int where, cudaStream_t s);
int stage_out(double *dst, const double *src, size_t count, int where, cudaStream_t s);
int where_ok(int where);
void note_launch(int count = 1);

#define HZ_CHECK_CUDA(call)                                                                      \
    do {                                                                                         \
        cudaError_t e_ = (call);                                                                 \
        if (e_ != cudaSuccess) {                                                                 \
            ::hz::set_error("%s:%d %s: %s", __FILE__, __LINE__, #call, cudaGetErrorString(e_));  \
            return HZ_ERR_CUDA;                                                                  \
        }                                                                                        \
    } while (0)

#define HZ_CHECK_LAUNCH()                                                                        \
    do {                                                                                         \
        ::hz::note_launch();                                                                     \
        cudaError_t e_ = cudaGetLastError();                                                     \
        if (e_ != cudaSuccess) {                                                                 \
            ::hz::set_error("%s:%d launch: %s", __FILE__, __LINE__, cudaGetErrorString(e_));    \
            return HZ_ERR_CUDA;                                                                  \
        }                                                                                        \
    } while (0)

#define HZ_TRY(expr)                                                                             \
    do {                                                                                         \
        int rc_ = (expr);                                                                        \
        if (rc_ != HZ_OK) return rc_;                                                            \
    } while (0)

// Bits of the device-side error word.
enum : unsigned {
    DEV_ERR_GRID = 1u,      // interpolation cell outside the grid
    DEV_ERR_NONFINITE = 2u, // non-finite value produced
    DEV_ERR_WAIT = 4u,      // a bounded wait on an mbarrier gave up
    DEV_ERR_NORMAL = 8u,    // interpolated gradient norm far from 1 (reference warns)
};

// Spin limit of every mbarrier wait (polls); far above any real wait.
constexpr long long kWaitLimit = 1ll << 24;

// ----------------------------------------------------------- device memory
struct DevBuf {
    void *ptr = nullptr;
    size_t bytes = 0;
    DevBuf() = default;
    DevBuf(const DevBuf &) = delete;
    DevBuf &operator=(const DevBuf &) = delete;
    ~DevBuf() { release(); }
    int ensure(size_t nbytes);  // grow-only
    void release();
    template <class T> T *as() const { return static_cast<T *>(ptr); }
};

// ------------------------------------------------------------ sweep types
// Source/target record of the FP64 sweep (lexicographic tube order).
struct Rec64 {
    double4_32a *pos;  // x*, y*, z*, reg
    double4_32a *nrm;  // nx, ny, nz, w
    const double4_32a *posk = nullptr;  // k x*, k y*, k z*, reg (optional: the scaled FP64 sweep)
};

// Tile geometry of the FP32 sweep.
constexpr int kTile32 = 256;  // sources per shared-memory tile
constexpr int kThreads32 = 256;
constexpr int kTgt32 = 2;     // targets per thread
constexpr int kTile64 = 128;
constexpr int kThreads64 = 128;

// Sweep-order (spatially blocked) FP32 records.  perm[s] is the tube index
// of sweep slot s; slots >= n are padding with zero weight.
// Record a timing event on s.  Inside a stream capture the record becomes an
// external event node (replayed with the graph); outside it is a plain record.
inline cudaError_t record_timing_event(cudaEvent_t ev, cudaStream_t s)
{
    cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
    const cudaError_t e = cudaStreamIsCapturing(s, &st);
    if (e != cudaSuccess) return e;
    if (st == cudaStreamCaptureStatusActive) return cudaEventRecordWithFlags(ev, s, cudaEventRecordExternal);
    return cudaEventRecord(ev, s);
}

struct Rec32 {
    int64_t npad;        // multiple of kTile32 and of kThreads32*kTgt32
    int *perm;           // npad entries, -1 for padding
    float4 *pos;         // x-o, y-o, z-o relative to the slot's tile origin; .w = reg
    float4 *nrm;         // nx, ny, nz, w
    double4_32a *origin;     // per tile: origin (x, y, z) and bounding radius .w
    double4_32a *tpos;       // per slot FP64 position (x, y, z), .w = w (targets)
    float4 *thi, *tlo;       // per slot position split into FP32 head + tail (x = hi + lo)
    float4 *ohi, *olo;       // per tile origin split into FP32 head + tail
    uint32_t *nearmask;      // [target tile][mwords]: bit s set unless source tile s is
                             // farther than tau from every point of the target tile
    int64_t mwords;          // 32-bit words per mask row: ceil(tiles / 32)
    double4_32a *partial;    // stream-K scratch: pieces of target blocks split between CTAs
    size_t partial_bytes;
};

struct SweepConst {
    int64_t n;
    double wave;
    double tau;
    int dirichlet;
    int interior;
    unsigned *err;  // device error word
    int phase_split = 0;  // FP32 sweep: phase reduced with a split k/(2 pi) (HZ_PHASE_SPLIT)
    double extent = 0.0;  // largest point distance: the domain's diagonal sqrt(3) (int_u - int_l)
};

// sweep modes
enum { SWEEP_A = 1, SWEEP_AH = 2, SWEEP_PAIR = 3 };

// CUDA events around pair-sweep kernel launches, read back after the host
// synchronises (also inside captured graphs, whose event-record nodes
// re-record the same events on every replay).
struct SweepTimer {
    static constexpr int kSlots = 8;
    bool on = false;
    cudaEvent_t start[kSlots] = {}, stop[kSlots] = {};
    int next = 0;         // slots recorded since the last harvest
    int graph_slots = 0;  // slots recorded by the captured iteration graph
    double total_ms = 0.0;
    long long launches = 0;
    int slot();           // next slot, or -1 when timing is off / full
    void harvest(int count);
};

// dense.cu: the dense assemblers of HelmholtzKernel.c, all pointers on the
// device (pts [HZ_DENSE_ROWS][n], matrices n x n row-major, may be NULL).
int dense_assemble_device(int kind, const hz_params &p, const hz_dense_opts &o, const double *d, const double *gx,
                          const double *gy, const double *gz, const double *mc, const double *gc, int64_t n_expected,
                          double *pts, double *k1re, double *k1im, double *k2re, double *k2im,
                          long long *regcount, unsigned *err, cudaStream_t s);
int dense_count_device(int kind, const hz_params &p, const hz_dense_opts &o, const double *d, int64_t &n,
                       cudaStream_t s);
// selection (lexicographic node indices in idx) and per-point rows only
int dense_points_device(int kind, const hz_params &p, const hz_dense_opts &o, const double *d, const double *gx,
                        const double *gy, const double *gz, const double *mc, const double *gc, DevBuf &idx,
                        int64_t &n, DevBuf &pts, unsigned *err, cudaStream_t s);
// combo.cu: the Combo formulation as a matrix-free FP64 operator
int combo_pack(int64_t n, const double *pts, int sine, double *xs, double *nrm, double *delta, double *jac,
               double *reg, double *w, double *adist, double4_32a *pos64, double4_32a *nrm64, cudaStream_t s);
int sweep_combo64(int64_t n, double wave, double wavenum, double eta, double tau, const double4_32a *pos,
                  const double4_32a *nrm, const double *adist, int mode, const double *p_re, const double *p_im,
                  const double *pt_re, const double *pt_im, double *q_re, double *q_im, double *qt_re, double *qt_im,
                  cudaStream_t s, cudaEvent_t ev0, cudaEvent_t ev1);
int launch_eval_combo(int64_t n, const double4_32a *pos, const double4_32a *nrm, const double *s_re,
                      const double *s_im, int64_t m, const double *rx, double wave, double tau, double eta,
                      double *u_re, double *u_im, cudaStream_t s);
// shape_grad.cu: dJ/dphi given sigma, lambda and the receiver residuals
int shape_gradient_device(const hz_params &p, double H, double eps, double tau, int64_t n, const int64_t *idx,
                          const double *d, const double *gx, const double *gy, const double *gz, const double *mc,
                          const double *gc, const double *xs, const double *w, const double4_32a *pos,
                          const double4_32a *nrm, const double *s_re, const double *s_im, const double *l_re,
                          const double *l_im, int64_t m, const double *rx, const double *r_re, const double *r_im,
                          const double *src, double *work, double *phib, cudaStream_t s);
size_t shape_gradient_work_bytes(int64_t n, int N);
// stencils.cu
int launch_grid_stencils(int N, double H, const double *d, double *gx, double *gy, double *gz,
                         double *mc, double *gc, int order, cudaStream_t s);
// reverse of the grid stencils by local central differences (stencils.cu):
// phib += the adjoints of gx, gy, gz, mc, gc pulled back to the grid values
int launch_stencil_adjoint(int N, double H, const double *d, const double *gxb, const double *gyb, const double *gzb,
                           const double *mcb, const double *gcb, double *phib, int order, double h, cudaStream_t s);
// reinitialisation (stencils.cu): iters TVD-RK2 steps of dt = cfl*H, in place
int launch_reinit(int N, double H, double *phi, double *tmp1, double *tmp2, const double *phi0, int iters,
                  double cfl, int order, cudaStream_t s);
// tube.cu
int tube_build(int N, double eps, const double *d, DevBuf &idx, int64_t &n, DevBuf &scratch,
               cudaStream_t s);
int tube_init(const hz_params &p, const double *d, const double *gx, const double *gy,
              const double *gz, const double *mc, const double *gc, int64_t n, const int64_t *idx,
              double *xs, double *nrm, double *delta, double *jac, double *reg, double *w,
              double4_32a *pos64, double4_32a *nrm64, unsigned *err, cudaStream_t s,
              double *dreg = nullptr);
int sweep_order(int N, int64_t n, const int64_t *idx, int *perm, int64_t npad, DevBuf &scratch,
                cudaStream_t s);
// reg_scale multiplies the regularisation factor stored in pos32.w (the
// FP32 sweep folds sg/(4 pi) into its densities and divides it out here).
// Fill every array of r (npad, perm and the pointers set by the caller):
// FP32 records, tile origins, split positions and the near-tile mask for
// the regularisation radius tau.
int build_rec32(const Rec32 &r, const double4_32a *pos64, const double4_32a *nrm64, double reg_scale, double tau,
                cudaStream_t s);
// sweep_f64.cu
// Data-wait poll limit of each sweep translation unit, on the current device.
int set_wait_limit_f32(long long polls);
int set_wait_limit_combo32(long long polls);
int set_wait_limit_f64(long long polls);
int set_wait_limit_multi(long long polls);

int sweep_f64(const SweepConst &c, const Rec64 &r, int mode, const double *p_re, const double *p_im,
              const double *pt_re, const double *pt_im, double *q_re, double *q_im, double *qt_re,
              double *qt_im, double2 *scratch, cudaStream_t s, cudaEvent_t ev0 = nullptr,
              cudaEvent_t ev1 = nullptr);
// posk[i] = (k x, k y, k z, reg) of pos[i]: the FP64 sweep's scaled records.
int scale_records64(int64_t n, double k, const double4_32a *pos, double4_32a *posk, cudaStream_t s);
// sweep_f32.cu
int sweep_f32(const SweepConst &c, const Rec32 &r, const double4_32a *pos64, int mode,
              const double *p_re, const double *p_im, const double *pt_re, const double *pt_im,
              double *q_re, double *q_im, double *qt_re, double *qt_im, float4 *dens,
              cudaStream_t s, cudaEvent_t ev0 = nullptr, cudaEvent_t ev1 = nullptr, int cfg = 0);
// 1 / (sg / 4 pi): the factor applied to regularisation factors in pos32.w
double sweep32_reg_scale(int interior);
// number of compiled FP32 sweep variants (block shape x targets per thread)
int sweep32_num_configs();
// Batched FP32 products (sweep_f32.cu): Q[r] = A_r P[r] for the described
// operators of a batch in one persistent launch; P, Q are [ncols][stride]
// column arrays and each described operator owns one column.
struct Batch32Item {
    SweepConst c;
    Rec32 r;
    const double4_32a *pos64;
    float4 *dens;
};
size_t batch32_desc_bytes(int R);
// Describes nops operators: items[cols[i]] owning column cols[i] (cols NULL:
// items[i], column i).
int batch32_describe(const Batch32Item *items, int nops, int cfg, void *desc_dev, int64_t &units, int64_t &blocks,
                     cudaStream_t s, const int *cols = nullptr);
size_t batch32_partial_bytes();
// Columns of described operators get their product; every column's padded
// tail (and every column of an operator not described) is zeroed.
int sweep_f32_batch(int cfg, const void *desc_dev, int nops, int ncols, int64_t units, int64_t blocks,
                    double4_32a *partial, size_t partial_bytes, const double *p_re, const double *p_im,
                    double *q_re, double *q_im, int64_t stride, int64_t max_npad, cudaStream_t s, cudaEvent_t ev0,
                    cudaEvent_t ev1);
// bytes of stream-K scratch that every FP32 sweep variant fits in
size_t sweep32_partial_bytes();
// FP32 products of the Combo formulation (sweep_combo32.cu) on the blocked
// records of the annulus points; combo32_set_distances stores |d| of every
// slot in r.nrm[].w once per build.
int combo32_set_distances(const Rec32 &r, const double *adist, cudaStream_t s);
int sweep_combo32(const SweepConst &c, const Rec32 &r, const double4_32a *pos64, double wavenum, double eta, int mode,
                  const double *p_re, const double *p_im, const double *pt_re, const double *pt_im, double *q_re,
                  double *q_im, double *qt_re, double *qt_im, float4 *dens, cudaStream_t s,
                  cudaEvent_t ev0 = nullptr, cudaEvent_t ev1 = nullptr);

}  // namespace hz

struct hz_solver_state;

// The operator handle.
struct hz_operator {
    hz_params p{};
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t own_stream = nullptr;
    double H = 0, eps = 0, tau = 0;
    // grids
    hz::DevBuf d, gx, gy, gz, mc, gc;
    bool have_distance = false, built = false;
    // tube
    int64_t n = 0;
    hz::DevBuf idx, xs, nrm, delta, jac, reg, w, dreg;
    hz::DevBuf pos64, nrm64;
    hz::DevBuf posk64;  // pos64 with the coordinates scaled by k (FP64 sweep)
    // FP32 sweep records
    hz::Rec32 r32{};
    hz::DevBuf perm, pos32, nrm32, origin32, tpos32, split32, nearmask32, partial32;
    // scratch and error word
    hz::DevBuf scratch, err;
    hz::DevBuf io;  // staging for host <-> device vectors
    hz::DevBuf dens32;
    hz_solver_state *solver = nullptr;  // Krylov workspaces (capi.cu)
    hz::SweepTimer timer;
    int sweep_cfg = 0;  // FP32 sweep variant of the fused A p + A^H pt pass (hz_autotune)
    int sweep_cfg_a = -1;  // variant of the single-product passes (A p or A^H p); -1: sweep_cfg
    int phase_mode = HZ_PHASE_SPLIT; // HZ_PHASE_SPLIT (default) or HZ_PHASE_DIRECT (hz_set_phase_mode)
    // Combo formulation (hz_set_combo): annulus points, FP64 products only
    int combo = 0;
    hz_dense_opts combo_opts{};
    hz::DevBuf adist, cpts;  // |d| per point; per-point rows of the selection
};

namespace hz {
int check_device_error(hz_operator *op, const char *where);
hz::SweepConst sweep_const(const hz_operator *op);
hz::Rec64 rec64(hz_operator *op);

// Inner tolerance of a refinement step that starts from the FP64 relative
// residual res: the factor by which the residual still has to fall, with a
// margin of 4, clamped to [opts.inner_tol, 0.5].  The first step (res = 1)
// solves to max(inner_tol, tol / 4); a step that only has to close a small
// gap stops after a few iterations instead of repeating a full solve.
inline double refine_inner_tol(const hz_solve_opts &o, double res)
{
    double t = (res > 0) ? o.tol / (4.0 * res) : 0.5;
    if (t > 0.5) t = 0.5;
    return t > o.inner_tol ? t : o.inner_tol;
}
}  // namespace hz
