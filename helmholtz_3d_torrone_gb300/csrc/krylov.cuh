// krylov.cuh -- device Krylov solvers over an abstract linear operator.
#pragma once

#include <vector>

#include "hz_internal.cuh"

namespace hz {

// Apply q = A p (SWEEP_A), qt = A^H pt (SWEEP_AH) or both (SWEEP_PAIR).
struct LinOp {
    virtual ~LinOp() = default;
    virtual int apply(int mode, const double *p_re, const double *p_im, const double *pt_re,
                      const double *pt_im, double *q_re, double *q_im, double *qt_re, double *qt_im,
                      cudaStream_t s) = 0;
    // hooks for per-kernel timing around graph capture and after each
    // synchronised iteration (graph: the iteration ran as a graph replay)
    virtual void capture_begin() {}
    virtual void capture_end() {}
    virtual void iteration_done(bool graph) { (void)graph; }
    // identity of the operator a captured iteration graph was built for
    virtual uint64_t key() const = 0;
};

// The adjoint of an operator: A^H p and (A^H)^H pt = A pt, by swapping the
// roles of the two products of the wrapped operator.
struct AdjointOp final : LinOp {
    LinOp &base;
    explicit AdjointOp(LinOp &b) : base(b) {}
    int apply(int mode, const double *p_re, const double *p_im, const double *pt_re, const double *pt_im,
              double *q_re, double *q_im, double *qt_re, double *qt_im, cudaStream_t s) override
    {
        const int m = ((mode & SWEEP_A) ? SWEEP_AH : 0) | ((mode & SWEEP_AH) ? SWEEP_A : 0);
        return base.apply(m, pt_re, pt_im, p_re, p_im, qt_re, qt_im, q_re, q_im, s);
    }
    void capture_begin() override { base.capture_begin(); }
    void capture_end() override { base.capture_end(); }
    void iteration_done(bool graph) override { base.iteration_done(graph); }
    uint64_t key() const override { return base.key() ^ 0x8000000000000000ull; }
};

struct KrylovScalars {
    double rho_re, rho_im;      // BiCG: <r, rt>; BiCGSTAB: <r, rh>
    double alpha_re, alpha_im;
    double beta_re, beta_im;
    double omega_re, omega_im;
    double normb, err, preerr;
    int status;                 // 0 ok, 1 zero right-hand side, 2 breakdown
};

class Krylov {
  public:
    enum { X = 0, R, RT, P, PT, Q, QT, XB, kVecs };  // XB: best iterate of a solve with a stall limit
    // BiCGSTAB reuses slots: RH = RT (shadow), V = PT, Q = t
    enum { RH = RT, V = PT };
    ~Krylov();
    int reserve(int64_t n);
    // Solve A x = b with x0 = 0; b on the device.  Solution in re(X)/im(X).
    // stall > 0: also stop once the residual has not reached a new minimum for
    // max(stall, iterations to the last minimum) iterations (used by inner
    // solves of the FP32 operator, whose rounding of the densities bounds
    // the attainable residual near 1e-7; a plateau may last as long as the
    // progress before it),
    // and return the iterate with the smallest residual seen (BiCG's
    // residual can swing by orders of magnitude between iterations).
    int solve(LinOp &A, int method, const double *b_re, const double *b_im, double tol, int maxit,
              bool stagnation, bool use_graph, cudaStream_t s, int &iters, double &resid, int &status,
              int stall = 0);
    double *re(int v);
    double *im(int v);
    void invalidate_graph() { graph_key = 0; }
    std::vector<double> history;  // relative residual after each iteration of the last solve

  private:
    int bicg_iteration(LinOp &A, cudaStream_t s);
    int stab_iteration(LinOp &A, cudaStream_t s);
    int keep_best(cudaStream_t s);
    int64_t n = 0;
    DevBuf vecs, partial, scal;
    double *host_err = nullptr;
    cudaGraphExec_t graph_exec = nullptr;
    uint64_t graph_key = 0;
    int graph_key_method = -1;
    cudaStream_t graph_stream = nullptr;
};

int vec_axpy(int64_t n, double a, const double *e_re, const double *e_im, double *x_re, double *x_im,
             cudaStream_t s);
int vec_sub(int64_t n, const double *b_re, const double *b_im, const double *q_re, const double *q_im,
            double *r_re, double *r_im, cudaStream_t s);
int vec_scale(int64_t n, double a, const double *x_re, const double *x_im, double *y_re, double *y_im,
              cudaStream_t s);
int vec_norm(int64_t n, const double *x_re, const double *x_im, double *dev_partial, double *dev_out,
             double &host_out, cudaStream_t s);
size_t vec_partial_bytes();

// Restarted GMRES(m) for A x = b (x0 = 0, b and x on the device), FP64
// vectors; work/small grow as needed.  Stops at ||b - A x|| / ||b|| < tol
// (the recurrence's residual), after maxit iterations, or (stall > 0) after
// `stall` iterations without a new minimum.  products counts A products.
int gmres_solve(LinOp &A, int64_t n, int m, const double *b_re, const double *b_im, double *x_re, double *x_im,
                double tol, int maxit, int stall, DevBuf &work, DevBuf &small, cudaStream_t s, int &iters,
                double &resid, int &products);

}  // namespace hz
