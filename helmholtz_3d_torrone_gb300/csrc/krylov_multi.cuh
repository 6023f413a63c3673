// krylov_multi.cuh -- lockstep BiCGSTAB over R right-hand sides.
#pragma once

#include <vector>

#include "hz_internal.cuh"

namespace hz {

// Q = A P for R column vectors stored one after the other ([R][n]).
struct MultiOp {
    virtual ~MultiOp() = default;
    virtual int apply(int R, const double *p_re, const double *p_im, double *q_re, double *q_im,
                      cudaStream_t s) = 0;
    // nonzero: apply only enqueues kernels and copies on s (no allocation, no
    // synchronisation), so a solver iteration around it can be captured in a
    // CUDA graph; the value identifies the operator the graph was built for
    virtual uint64_t key() const { return 0; }
    // The solver calls this with the columns still iterating, before its
    // first iteration and whenever a column stops: an operator may then skip
    // the others (their products are not read).  A change of what apply
    // enqueues must change key().
    virtual int restrict_to(const std::vector<int> &cols, cudaStream_t s)
    {
        (void)cols;
        (void)s;
        return HZ_OK;
    }
};

class KrylovMulti {
  public:
    enum { X = 0, RV, RH, P, V, T, XB, kVecs };  // XB: best iterates (stall > 0)
    ~KrylovMulti();
    int reserve(int64_t n, int R);
    // Solve A X = B column by column (x0 = 0); B on the device, [R][n].
    // col_iters (optional): the iterations each column took part in.
    // stall > 0: a column also stops once its residual has not reached a new
    // minimum for `stall` iterations, and ends on its best iterate.
    int solve(MultiOp &A, const double *b_re, const double *b_im, double tol, int maxit, bool stagnation,
              cudaStream_t s, int &iters, std::vector<double> &resid, int stall = 0,
              std::vector<int> *col_iters = nullptr);
    double *re(int v);
    double *im(int v);

  private:
    int iteration(MultiOp &A, double tol, bool stagnation, int stall, cudaStream_t s);
    int64_t n = 0;
    int R = 0;
    DevBuf vecs, partial, scal;
    double *host = nullptr;
    cudaGraphExec_t graph_exec = nullptr;
    uint64_t graph_key = 0;
    cudaStream_t graph_stream = nullptr;
    double graph_tol = 0.0;
    int graph_flags = 0;
};

// gmres_multi.cu: lockstep restarted GMRES(m) over R right-hand sides ([R][n]
// device arrays); x = 0 start; stall as in KrylovMulti::solve.  resid gets
// each column's final residual estimate, col_iters its iterations.
size_t gmres_multi_work_bytes(int64_t n, int R, int m);
int gmres_multi_solve(MultiOp &A, int64_t n, int R, int m, const double *b_re, const double *b_im, double *x_re,
                      double *x_im, double tol, int maxit, int stall, DevBuf &work, DevBuf &small, cudaStream_t s,
                      int &iters, std::vector<double> &resid, std::vector<int> *col_iters = nullptr);

// sweep_multi.cu
// kernel passes (one evaluation of every pair each) for nrhs columns
long long multi_rhs_passes(int precision, int nrhs);
size_t multi_rhs_scratch_bytes(int64_t n, int64_t npad);
int sweep_multi(const SweepConst &c, const Rec32 &r32, const Rec64 &r64, int precision, int nrhs,
                const double *p_re, const double *p_im, double *q_re, double *q_im, void *scratch,
                cudaStream_t s);

}  // namespace hz
