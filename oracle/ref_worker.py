"""The reference's FP64 C solve in a child process (TEST INFRASTRUCTURE ONLY).

The reference keeps its tube arrays in function statics (omp_get_Ccomp,
large3Dexample2.c:4249-4277), so one process serves one (N, k, distance
grid) configuration.  RefWorker starts a child with the spawn method (safe
after CUDA is initialised in the parent), which runs the reference build
(oracle/_ref/libref_<variant>.so): ASSIGN_GRADIENT, the BothCurvs loop, the
tube (large3Dexample2.c:548-597), the per-point set-up (:4340-4452) and the
dense matrix of omp_get_Ccomp entries (:4463-4564); it then answers
right-hand sides with CompBiCG (BICGSTAB.c:5-339, DEFAULTACC 1e-13 in this
build).  Used by the tests to check the GPU's adjoint gradients against
central differences of the reference's own solve.
"""
import multiprocessing as mp
import os

import numpy as np


def _serve(conn, variant, N, wave, d, want_matrix, threads, chunk):
    os.environ["OMP_NUM_THREADS"] = str(threads)
    import oracle as O
    devnull = os.open(os.devnull, os.O_WRONLY)
    os.dup2(devnull, 1)  # the reference prints progress on stdout
    ref = O.Reference(variant)
    ref.setup(N, wave, d)
    idx = ref.tube()
    n = len(idx)
    tp = ref.tube_points(n)
    are, aim = ref.dense(n, nthreads=threads)
    info = dict(idx=idx, n=n, **tp)
    if want_matrix:
        info["A"] = are + 1j * aim
    conn.send(info)
    while True:
        msg = conn.recv()
        if msg is None:
            break
        conn.send(ref.compbicg(are, aim, msg, chunk))
    conn.close()


class RefWorker:
    """One reference configuration in a child process: .tube has the
    reference's tube (idx, xs, nrm, delta, jac, reg, w, and the dense matrix
    as A with matrix=True); .solve(b) runs CompBiCG on it (omp_CompBiCG with
    that OpenMP chunk when omp_chunk > 0)."""

    def __init__(self, variant, N, wave, d, matrix=False, timeout=900, threads=None, omp_chunk=0):
        ctx = mp.get_context("spawn")
        self.timeout = timeout
        threads = threads or (os.cpu_count() or 1)
        self.conn, child = ctx.Pipe()
        self.proc = ctx.Process(target=_serve, args=(child, variant, N, wave, np.ascontiguousarray(d), matrix,
                                                     threads, omp_chunk), daemon=True)
        self.proc.start()
        child.close()
        self.tube = self._recv()

    def _recv(self):
        if not self.conn.poll(self.timeout):
            self.close()
            raise TimeoutError("reference worker gave no answer in %d s" % self.timeout)
        try:
            return self.conn.recv()
        except EOFError:
            raise RuntimeError("reference worker exited (exit code %s)" % self.proc.exitcode)

    def solve(self, b):
        self.conn.send(np.ascontiguousarray(b, dtype=np.complex128))
        return self._recv()

    def close(self):
        try:
            self.conn.send(None)
        except (BrokenPipeError, OSError):
            pass
        self.proc.join(10)
        if self.proc.is_alive():
            self.proc.kill()
            self.proc.join()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def solve_many(variant, N, wave, grids, b_of_tube, processes=None):
    """Reference solves of several distance grids, one child process per grid
    (up to `processes` at a time, one thread each): b_of_tube(tube) gives
    each grid's right-hand side from its reference tube.  Returns
    [(tube, x)] in order."""
    processes = processes or max(1, min(16, os.cpu_count() or 1))
    out = [None] * len(grids)
    pending = list(enumerate(grids))
    while pending:
        batch, pending = pending[:processes], pending[processes:]
        workers = [(i, RefWorker(variant, N, wave, d, threads=1)) for i, d in batch]
        try:
            for i, w in workers:
                out[i] = (w.tube, w.solve(b_of_tube(w.tube)))
        finally:
            for _, w in workers:
                w.close()
    return out
