// krylov.cuh -- device Krylov solvers over an abstract linear operator.
#pragma once

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
    enum { X = 0, R, RT, P, PT, Q, QT, kVecs };
    // BiCGSTAB reuses slots: RH = RT (shadow), V = PT, Q = t
    enum { RH = RT, V = PT };
    ~Krylov();
    int reserve(int64_t n);
    // Solve A x = b with x0 = 0; b on the device.  Solution in re(X)/im(X).
    int solve(LinOp &A, int method, const double *b_re, const double *b_im, double tol, int maxit,
              bool stagnation, bool use_graph, cudaStream_t s, int &iters, double &resid, int &status);
    double *re(int v);
    double *im(int v);
    void invalidate_graph()
    {
        graph_key_op = nullptr;
    }

  private:
    int bicg_iteration(LinOp &A, cudaStream_t s);
    int stab_iteration(LinOp &A, cudaStream_t s);
    int64_t n = 0;
    DevBuf vecs, partial, scal;
    double *host_err = nullptr;
    cudaGraphExec_t graph_exec = nullptr;
    const LinOp *graph_key_op = nullptr;
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

}  // namespace hz
