"""GB300 (sm_103a) implementation of the implicit-boundary-integral Helmholtz
hot path of moorhsum/Helmholtz-3D-torrone.

The compute lives in the CUDA library ``libhzgb300.so`` behind the C ABI of
``include/helmholtz_gb300.h``; this module is a thin ctypes binding of that
ABI.  There is no CPU fallback: every call fails loudly when the library or
a CUDA device is missing.

Arrays follow the reference's conventions: grids are (N+1)^3 float64 arrays
indexed [i, j, k] with i = y, j = x, k = z (large3Dexample2.c:428-437);
complex vectors are numpy complex128 here and split into real/imaginary
parts at the boundary (the reference's density / densityimg pairs).
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libhzgb300.so")

HZ_OK = 0
HZ_HOST, HZ_DEVICE = 0, 1
PREC_F64, PREC_F32, PREC_F32_REFINED = 0, 1, 2
BICG, BICGSTAB, GMRES = 0, 1, 2
SINGLE_LAYER, DOUBLE_LAYER, COMBO_LAYER = 0, 1, 2
PHASE_DIRECT, PHASE_SPLIT = 0, 1
RHS_POINT_DIRICHLET, RHS_POINT_NEUMANN, RHS_MONOPOLE_NEUMANN, RHS_MONOPOLE_DIRICHLET = 0, 1, 2, 3
NOALLOC_MAX_POINTS = 32768  # HZ_NOALLOC_MAX_POINTS

ERRORS = {-1: "HZ_ERR_ARG", -2: "HZ_ERR_CUDA", -3: "HZ_ERR_STATE", -4: "HZ_ERR_GRID",
          -5: "HZ_ERR_NONFINITE", -6: "HZ_ERR_BREAKDOWN", -7: "HZ_ERR_DEVICE_WAIT"}
globals().update({name: code for code, name in ERRORS.items()})


class HzError(RuntimeError):
    """A failed C call: .code is the HZ_ERR_* status, the message hz_last_error()."""
    def __init__(self, code, msg):
        super().__init__("%s (%d): %s" % (ERRORS.get(code, "?"), code, msg))
        self.code = code


class Params(C.Structure):
    """hz_params: grid size N over [int_l, int_u]^3, wave number, tube factor
    (eps = factor H), near-field factor (tau = tau_factor H), formulation
    (dirichlet, interior) and WENO order; build one with params()."""
    _fields_ = [("N", C.c_int), ("int_l", C.c_double), ("int_u", C.c_double), ("wave", C.c_double),
                ("factor", C.c_double), ("tau_factor", C.c_double), ("dirichlet", C.c_int),
                ("interior", C.c_int), ("weno_order", C.c_int)]

    @property
    def H(self):
        """Grid spacing (int_u - int_l) / N (large3Dexample2.c:174)."""
        return (self.int_u - self.int_l) / self.N

    @property
    def eps(self):
        """Tube half-width factor * H."""
        return self.factor * self.H


class SolveOpts(C.Structure):
    """hz_solve_opts: method (BICG, BICGSTAB, GMRES), precision (PREC_F64,
    PREC_F32, PREC_F32_REFINED), tolerance, iteration limits, inner
    tolerance and refinement steps of PREC_F32_REFINED, stagnation stop,
    GMRES restart length; build one with solve_opts()."""
    _fields_ = [("method", C.c_int), ("precision", C.c_int), ("tol", C.c_double), ("maxit", C.c_int),
                ("inner_tol", C.c_double), ("max_outer", C.c_int), ("stagnation", C.c_int), ("restart", C.c_int)]


class DenseOpts(C.Structure):
    """hz_dense_opts: switches and arguments of the dense assemblers."""
    _fields_ = [("delta0", C.c_double), ("epsilon", C.c_double), ("wavenum", C.c_double), ("eta", C.c_double),
                ("poly", C.c_int), ("sine", C.c_int), ("onesided", C.c_int), ("combo_interior", C.c_int),
                ("radius", C.c_double), ("center", C.c_double * 3)]


class RefConfig(C.Structure):
    """hz_ref_config: the compile-time switches the reference-signature
    dense assemblers read (include/helmholtz_ref_api.h)."""
    _fields_ = [("int_l", C.c_double), ("int_u", C.c_double), ("tau_factor", C.c_double), ("interior", C.c_int),
                ("poly", C.c_int), ("sine", C.c_int), ("trad_onesided", C.c_int), ("combo_onesided", C.c_int),
                ("combo_interior", C.c_int), ("radius", C.c_double), ("center", C.c_double * 3),
                ("bicg_acc", C.c_double)]


MAX_STEPS = 8  # HZ_MAX_STEPS


class SolveInfo(C.Structure):
    """hz_solve_info: iterations (inner ones for refined solves), refinement
    steps, final relative residual (FP64 for refined solves), seconds, pair
    evaluations, status, whether the final residual is below tol, and per
    refinement step its inner iterations, inner tolerance and FP64 residual."""
    _fields_ = [("iterations", C.c_int), ("outer", C.c_int), ("resid", C.c_double), ("resid_f64", C.c_double),
                ("seconds", C.c_double), ("pair_evals", C.c_int64), ("status", C.c_int), ("converged", C.c_int),
                ("steps", C.c_int), ("step_iters", C.c_int * MAX_STEPS),
                ("step_inner_tol", C.c_double * MAX_STEPS), ("step_resid", C.c_double * MAX_STEPS)]

    def as_dict(self):
        """The fields as a dict (the per-step arrays cut to the steps taken)."""
        out = {}
        for f, _ in self._fields_:
            v = getattr(self, f)
            out[f] = list(v)[:self.steps] if f.startswith("step_") else v
        return out


_lib = None
_dp = C.POINTER(C.c_double)
_vp = C.c_void_p

# Every symbol of include/helmholtz_gb300.h with its ctypes signature.
SIGNATURES = {
    "hz_last_error": ([], C.c_char_p),
    "hz_params_default": ([C.POINTER(Params), C.c_int, C.c_double], None),
    "hz_create": ([C.POINTER(Params), C.POINTER(C.c_void_p)], C.c_int),
    "hz_destroy": ([_vp], None),
    "hz_set_stream": ([_vp, _vp], C.c_int),
    "hz_get_stream": ([_vp], _vp),
    "hz_set_distance": ([_vp, _vp, C.c_int], C.c_int),
    "hz_set_combo": ([_vp, _vp], C.c_int),
    "hz_shape_gradient": ([_vp, C.POINTER(SolveOpts), _vp, C.c_int64, _vp, _vp, _vp, C.POINTER(C.c_double), _vp,
                           C.c_int, C.POINTER(SolveInfo)], C.c_int),
    "hz_batch_create": ([C.POINTER(_vp), C.c_int, C.POINTER(_vp)], C.c_int),
    "hz_batch_destroy": ([_vp], None),
    "hz_batch_autotune": ([_vp, C.POINTER(C.c_int), C.POINTER(C.c_double)], C.c_int),
    "hz_batch_set_variant": ([_vp, C.c_int], C.c_int),
    "hz_batch_matvec": ([_vp, C.c_int, C.POINTER(_vp), C.POINTER(_vp), C.POINTER(_vp), C.POINTER(_vp), C.c_int],
                        C.c_int),
    "hz_batch_solve": ([_vp, C.POINTER(SolveOpts)] + [C.POINTER(_vp)] * 4 + [C.c_int, C.POINTER(SolveInfo), _vp],
                       C.c_int),
    "hz_build": ([_vp, C.POINTER(C.c_int64)], C.c_int),
    "hz_tube_size": ([_vp], C.c_int64),
    "hz_sweep_timing": ([_vp, C.c_int, _dp, C.POINTER(C.c_int64)], C.c_int),
    "hz_autotune": ([_vp, C.POINTER(C.c_int), _dp], C.c_int),
    "hz_set_sweep_config": ([_vp, C.c_int], C.c_int),
    "hz_set_phase_mode": ([_vp, C.c_int], C.c_int),
    "hz_get_grids": ([_vp, _vp, _vp, _vp, _vp, _vp, C.c_int], C.c_int),
    "hz_get_tube": ([_vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, C.c_int], C.c_int),
    "hz_matvec": ([_vp, C.c_int, C.c_int, _vp, _vp, _vp, _vp, C.c_int], C.c_int),
    "hz_matvec_pair": ([_vp, C.c_int, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, C.c_int], C.c_int),
    "hz_matvec_multi": ([_vp, C.c_int, C.c_int, _vp, _vp, _vp, _vp, C.c_int], C.c_int),
    "hz_solve": ([_vp, C.POINTER(SolveOpts), _vp, _vp, _vp, _vp, C.c_int, C.POINTER(SolveInfo)], C.c_int),
    "hz_residual_history": ([_vp, _vp, C.c_int, C.POINTER(C.c_int)], C.c_int),
    "hz_solve_opts_default": ([C.POINTER(SolveOpts)], None),
    "hz_solve_multi": ([_vp, C.POINTER(SolveOpts), C.c_int, _vp, _vp, _vp, _vp, C.c_int, C.POINTER(SolveInfo),
                        _vp], C.c_int),
    "hz_rhs_plane_waves": ([_vp, C.c_int, _vp, C.c_int, _vp, _vp, C.c_int], C.c_int),
    "hz_rhs_point_source": ([_vp, _vp, C.c_int, _vp, _vp, C.c_int], C.c_int),
    "hz_misfit_gradient": ([_vp, C.POINTER(SolveOpts), _vp, _vp, C.c_int, C.c_int64, _vp, _vp, _vp, _dp, _vp, _vp,
                            _dp, _vp, C.c_int, C.POINTER(SolveInfo)], C.c_int),
    "hz_eval": ([_vp, C.c_int, C.c_int64, _vp, _vp, _vp, _vp, _vp, C.c_int], C.c_int),
    "hz_assign_gradient": ([C.c_int, C.c_double, _vp, _vp, _vp, _vp, C.c_int, C.c_int], C.c_int),
    "hz_assign_curvatures": ([C.c_int, C.c_double, _vp, _vp, _vp, C.c_int], C.c_int),
    "hz_reinitialize": ([C.c_int, C.c_double, _vp, C.c_int, C.c_double, C.c_int, C.c_int], C.c_int),
    "hz_dense_bicg": ([C.c_int64, _vp, _vp, _vp, _vp, _vp, _vp, C.c_double, C.c_int, C.c_int,
                       C.POINTER(SolveInfo)], C.c_int),
    "hz_dense_opts_default": ([C.POINTER(DenseOpts), C.c_int, C.POINTER(Params)], None),
    "hz_dense_count": ([C.c_int, C.POINTER(Params), C.POINTER(DenseOpts), _vp, C.c_int, C.POINTER(C.c_int64)],
                       C.c_int),
    "hz_dense_assemble": ([C.c_int, C.POINTER(Params), C.POINTER(DenseOpts)] + [_vp] * 6 +
                          [C.c_int64] + [_vp] * 5 + [C.POINTER(C.c_int64), C.c_int], C.c_int),
    "hz_ref_get_config": ([C.POINTER(RefConfig)], None),
    "hz_ref_set_config": ([C.POINTER(RefConfig)], None),
    "hz_kernel_launches": ([], C.c_int64),
    "hz_set_wait_limit": ([C.c_longlong], C.c_int),
    "hz_measure_fma_peaks": ([_dp, _dp], C.c_int),
    "hz_eval_slice": ([_vp, C.c_int, C.c_int, C.c_double, C.c_int, C.c_double, C.c_double, C.c_double, _vp, _vp,
                       _vp, _vp, C.c_int], C.c_int),
    "hz_reference_file_names": ([C.c_int, C.c_double, C.c_char_p, C.c_char_p, C.c_char_p, C.c_char_p, C.c_char_p,
                                 C.c_char_p, C.c_size_t], C.c_int),
    "hz_read_distance_file": ([C.c_char_p, C.c_int, _vp], C.c_int),
    "hz_write_distance_file": ([C.c_char_p, C.c_int, _vp], C.c_int),
    "hz_write_rhs_files": ([C.c_char_p, C.c_char_p, C.c_int64, _vp, _vp], C.c_int),
    "hz_read_rhs_files": ([C.c_char_p, C.c_char_p, C.c_int64, _vp, _vp], C.c_int),
    "hz_write_density_files": ([C.c_char_p, C.c_char_p, C.c_int64, _vp, _vp], C.c_int),
    "hz_read_density_files": ([C.c_char_p, C.c_char_p, C.c_int64, _vp, _vp], C.c_int),
    "hz_write_result_file": ([C.c_char_p, C.c_double, C.c_double, C.c_double, C.c_double], C.c_int),
    "hz_matvec_f64_noalloc": ([C.POINTER(Params), C.c_int64, C.c_int, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp,
                               _vp], C.c_int),
}


def load(path=LIB_PATH):
    """Load libhzgb300.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError("libhzgb300.so is not built; run __graft_entry__.build() "
                           "or python helmholtz_3d_torrone_gb300/_build.py")
    L = C.CDLL(path)
    for name, (args, res) in SIGNATURES.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = res
    _lib = L
    return L


def _check(rc):
    if rc != HZ_OK:
        raise HzError(rc, load().hz_last_error().decode())


def _ptr(a):
    """Address of a numpy array (host) or of a torch tensor / int (device)."""
    if a is None:
        return None
    if isinstance(a, int):
        return a
    if hasattr(a, "data_ptr"):
        return a.data_ptr()
    return a.ctypes.data


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def params(N, wave, int_l=-2.0, int_u=2.0, factor=2.0, tau_factor=2.0, dirichlet=0, interior=0, weno_order=5):
    """Problem parameters; defaults are the reference's compile-time values."""
    return Params(N, int_l, int_u, wave, factor, tau_factor, dirichlet, interior, weno_order)


def solve_opts(method=BICG, precision=PREC_F64, tol=1e-7, maxit=2000, inner_tol=1e-5, max_outer=20,
               stagnation=1, restart=40):
    """SolveOpts with the C defaults (hz_solve_opts_default) unless given."""
    return SolveOpts(method, precision, tol, maxit, inner_tol, max_outer, stagnation, restart)


def kernel_launches():
    """Kernels this library has launched so far (graph replays counted by
    their nodes)."""
    return int(load().hz_kernel_launches())


def set_wait_limit(polls=-1):
    """Poll limit of the pair sweeps' data waits on the current device
    (negative: the default).  A short limit makes the waits give up, which
    the sweeps report as HZ_ERR_DEVICE_WAIT."""
    _check(load().hz_set_wait_limit(int(polls)))


def measure_fma_peaks():
    """(FP32, FP64) FMA throughput of the current GPU in TFLOP/s."""
    a, b = C.c_double(), C.c_double()
    _check(load().hz_measure_fma_peaks(C.byref(a), C.byref(b)))
    return a.value, b.value


class Operator:
    """Device-resident tube operator (one per surface and wave number)."""

    def __init__(self, p):
        L = load()
        self.p = p
        h = C.c_void_p()
        _check(L.hz_create(C.byref(p), C.byref(h)))
        self.h = h
        self.n = None

    def close(self):
        """Release the device memory (also on garbage collection)."""
        if getattr(self, "h", None):
            load().hz_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def set_stream(self, stream_handle):
        """Run the operator's work on this CUDA stream (a cudaStream_t as int)."""
        _check(load().hz_set_stream(self.h, stream_handle))

    def shape_gradient(self, src, receivers, target, opts=None, **kw):
        """(J, dJ/dphi on the grid, info) for point-source Dirichlet data."""
        opts = opts if opts is not None else solve_opts(**kw)
        rx = _f64(receivers).reshape(-1, 3)
        tr, ti = _f64(np.asarray(target).real), _f64(np.asarray(target).imag)
        S = self.p.N + 1
        g = np.zeros((S, S, S))
        J = C.c_double()
        info = SolveInfo()
        _check(load().hz_shape_gradient(self.h, C.byref(opts), _ptr(_f64(src)), rx.shape[0], _ptr(rx), _ptr(tr),
                                        _ptr(ti), C.byref(J), _ptr(g), HZ_HOST, C.byref(info)))
        return J.value, g, info.as_dict()

    def set_combo(self, opts):
        """Switch to the Combo formulation (before build); opts a DenseOpts
        (see dense_opts(DENSE_COMBO, p)), None switches back."""
        self._combo_opts = opts
        _check(load().hz_set_combo(self.h, None if opts is None else C.byref(opts)))

    def set_distance(self, d, where=HZ_HOST):
        """The signed-distance grid, (N+1)^3 values, node (i, j, k) at [i, j, k]."""
        if where == HZ_HOST:
            d = _f64(d)
            S = self.p.N + 1
            if d.size != S ** 3:
                raise ValueError("distance grid must have (N+1)^3 = %d values" % S ** 3)
        _check(load().hz_set_distance(self.h, _ptr(d), where))

    def build(self):
        """Stencil grids, tube, projected points, weights and sweep records;
        returns the tube size n."""
        n = C.c_int64()
        _check(load().hz_build(self.h, C.byref(n)))
        self.n = n.value
        return self.n

    def autotune(self):
        """Pick the fastest FP32 sweep variant for this tube: (variant, ms)."""
        cfg, ms = C.c_int(), C.c_double()
        _check(load().hz_autotune(self.h, C.byref(cfg), C.byref(ms)))
        return cfg.value, ms.value

    def set_sweep_config(self, cfg):
        """Force FP32 sweep variant cfg (0 .. 7) instead of the autotuned one."""
        _check(load().hz_set_sweep_config(self.h, cfg))

    def set_phase_mode(self, mode):
        """PHASE_SPLIT (default) or PHASE_DIRECT for the FP32 pair sweep."""
        _check(load().hz_set_phase_mode(self.h, mode))

    def sweep_timing(self, enable=-1):
        """Enable (1) / disable (0) per-sweep CUDA-event timing, or read (-1):
        returns (total device ms, launches) accumulated so far."""
        ms, k = C.c_double(), C.c_int64()
        _check(load().hz_sweep_timing(self.h, enable, C.byref(ms), C.byref(k)))
        return ms.value, k.value

    def grids(self):
        """[gx, gy, gz, mean curvature, Gaussian curvature] on the grid."""
        S = self.p.N + 1
        g = [np.empty((S, S, S)) for _ in range(5)]
        _check(load().hz_get_grids(self.h, *[_ptr(a) for a in g], HZ_HOST))
        return g

    def tube(self):
        """Tube points in the reference's order: node idx, x*, normals, delta,
        Jacobian, regularisation factor and weight."""
        n = self.n
        idx = np.empty(n, dtype=np.int64)
        xs, nrm = np.empty((n, 3)), np.empty((n, 3))
        delta, jac, reg, w = (np.empty(n) for _ in range(4))
        _check(load().hz_get_tube(self.h, _ptr(idx), _ptr(xs), _ptr(nrm), _ptr(delta), _ptr(jac), _ptr(reg),
                                  _ptr(w), HZ_HOST))
        return dict(idx=idx, xs=xs, nrm=nrm, delta=delta, jac=jac, reg=reg, w=w)

    def matvec(self, v, precision=PREC_F64, adjoint=False):
        """A v (or A^H v) in FP64 or FP32."""
        vr, vi = _f64(v.real), _f64(v.imag)
        qr, qi = np.empty(self.n), np.empty(self.n)
        _check(load().hz_matvec(self.h, precision, int(adjoint), _ptr(vr), _ptr(vi), _ptr(qr), _ptr(qi), HZ_HOST))
        return qr + 1j * qi

    def matvec_pair(self, v, vt, precision=PREC_F64):
        """(A v, A^H vt) in one fused pass over the pairs."""
        a = [_f64(v.real), _f64(v.imag), _f64(vt.real), _f64(vt.imag)]
        q = [np.empty(self.n) for _ in range(4)]
        _check(load().hz_matvec_pair(self.h, precision, *[_ptr(x) for x in a], *[_ptr(x) for x in q], HZ_HOST))
        return q[0] + 1j * q[1], q[2] + 1j * q[3]

    def matvec_multi(self, V, precision=PREC_F32):
        """A V for every row of V ([nrhs][n]), one pair evaluation per pass
        over a block of rows."""
        V = np.atleast_2d(V)
        nrhs = V.shape[0]
        vr, vi = _f64(V.real), _f64(V.imag)
        qr, qi = np.empty_like(vr), np.empty_like(vi)
        _check(load().hz_matvec_multi(self.h, precision, nrhs, _ptr(vr), _ptr(vi), _ptr(qr), _ptr(qi), HZ_HOST))
        return qr + 1j * qi

    def solve(self, b, opts=None, **kw):
        """Solve A x = b; returns (x, info dict).  opts: SolveOpts, else
        solve_opts(**kw)."""
        opts = opts if opts is not None else solve_opts(**kw)
        br, bi = _f64(b.real), _f64(b.imag)
        xr, xi = np.empty(self.n), np.empty(self.n)
        info = SolveInfo()
        rc = load().hz_solve(self.h, C.byref(opts), _ptr(br), _ptr(bi), _ptr(xr), _ptr(xi), HZ_HOST, C.byref(info))
        _check(rc)
        return xr + 1j * xi, info.as_dict()

    def residual_history(self):
        """Relative residual after each Krylov iteration of the last solve
        (BiCG/BiCGSTAB; inner FP32 solves one after another when refined)."""
        cnt = C.c_int()
        _check(load().hz_residual_history(self.h, None, 0, C.byref(cnt)))
        out = np.empty(cnt.value)
        if cnt.value:
            _check(load().hz_residual_history(self.h, _ptr(out), cnt.value, C.byref(cnt)))
        return out

    def solve_multi(self, B, opts=None, **kw):
        """Solve for every row of B ([nrhs][n] complex); returns X, info, resid."""
        opts = opts if opts is not None else solve_opts(**kw)
        B = np.atleast_2d(B)
        nrhs = B.shape[0]
        br, bi = _f64(B.real), _f64(B.imag)
        xr, xi = np.empty_like(br), np.empty_like(bi)
        info = SolveInfo()
        res = np.empty(nrhs)
        _check(load().hz_solve_multi(self.h, C.byref(opts), nrhs, _ptr(br), _ptr(bi), _ptr(xr), _ptr(xi), HZ_HOST,
                                     C.byref(info), _ptr(res)))
        return xr + 1j * xi, info.as_dict(), res

    def rhs_plane_waves(self, dirs, kind=RHS_POINT_DIRICHLET):
        """Boundary data of incident plane waves e^{ik d.x}, one row per
        direction in dirs."""
        d = _f64(dirs).reshape(-1, 3)
        m = d.shape[0]
        br, bi = np.empty((m, self.n)), np.empty((m, self.n))
        _check(load().hz_rhs_plane_waves(self.h, m, _ptr(d), kind, _ptr(br), _ptr(bi), HZ_HOST))
        return br + 1j * bi

    def evaluate_slice(self, sigma, axis=2, c=0.0, n2=64, lo=None, h2=None, layer=DOUBLE_LAYER, mask=0.0):
        """Field on the plane axis = c (headless n2 x n2 buffer, row-major)."""
        lo = self.p.int_l if lo is None else lo
        h2 = (self.p.int_u - self.p.int_l) / (n2 - 1) if h2 is None else h2
        sr, si = _f64(sigma.real), _f64(sigma.imag)
        ur, ui = np.empty(n2 * n2), np.empty(n2 * n2)
        _check(load().hz_eval_slice(self.h, layer, axis, c, n2, lo, h2, mask, _ptr(sr), _ptr(si), _ptr(ur), _ptr(ui),
                                    HZ_HOST))
        return (ur + 1j * ui).reshape(n2, n2)

    def misfit_gradient(self, b, receivers, target, layer=None, opts=None, **kw):
        """J = sum |u(x_m) - t_m|^2 and its adjoint gradients.

        Returns (J, g, dJ_dk, dJ_dw, info) where g = dJ/dRe(b) + i dJ/dIm(b)."""
        opts = opts if opts is not None else solve_opts(**kw)
        layer = (DOUBLE_LAYER if self.p.dirichlet else SINGLE_LAYER) if layer is None else layer
        br, bi = _f64(b.real), _f64(b.imag)
        rx = _f64(receivers).reshape(-1, 3)
        tr, ti = _f64(np.real(target)), _f64(np.imag(target))
        J, dk = C.c_double(), C.c_double()
        gr, gi, gw = np.empty(self.n), np.empty(self.n), np.empty(self.n)
        info = SolveInfo()
        _check(load().hz_misfit_gradient(self.h, C.byref(opts), _ptr(br), _ptr(bi), layer, rx.shape[0], _ptr(rx),
                                         _ptr(tr), _ptr(ti), C.byref(J), _ptr(gr), _ptr(gi), C.byref(dk), _ptr(gw),
                                         HZ_HOST, C.byref(info)))
        return J.value, gr + 1j * gi, dk.value, gw, info.as_dict()

    def rhs_point_source(self, src, kind):
        """Boundary data of a point source at src (RHS_* kind)."""
        s = _f64(src)
        br, bi = np.empty(self.n), np.empty(self.n)
        _check(load().hz_rhs_point_source(self.h, _ptr(s), kind, _ptr(br), _ptr(bi), HZ_HOST))
        return br + 1j * bi

    def evaluate(self, receivers, sigma, layer):
        """Field of the density sigma at receivers ([m][3]) for the layer
        (SINGLE_LAYER, DOUBLE_LAYER or COMBO_LAYER)."""
        rx = _f64(receivers).reshape(-1, 3)
        m = rx.shape[0]
        sr, si = _f64(sigma.real), _f64(sigma.imag)
        ur, ui = np.empty(m), np.empty(m)
        _check(load().hz_eval(self.h, layer, m, _ptr(rx), _ptr(sr), _ptr(si), _ptr(ur), _ptr(ui), HZ_HOST))
        return ur + 1j * ui


def assign_gradient(d, N, H, weno_order=5):
    """Device replacement of ASSIGN_GRADIENT (distance_application3D.c:56-140)."""
    d = _f64(d)
    g = [np.empty_like(d) for _ in range(3)]
    _check(load().hz_assign_gradient(N, H, _ptr(d), *[_ptr(a) for a in g], weno_order, HZ_HOST))
    return g


def assign_curvatures(d, N, H):
    """Device replacement of the BothCurvs loop (large3Dexample2.c:446-455)."""
    d = _f64(d)
    m, g = np.empty_like(d), np.empty_like(d)
    _check(load().hz_assign_curvatures(N, H, _ptr(d), _ptr(m), _ptr(g), HZ_HOST))
    return m, g


def reinitialize(phi, N, H, iters, cfl=0.5, weno_order=5):
    """Device reinitialisation of a level set toward the signed distance."""
    out = np.array(phi, dtype=np.float64, copy=True, order="C")
    _check(load().hz_reinitialize(N, H, _ptr(out), iters, cfl, weno_order, HZ_HOST))
    return out


def dense_bicg(A, b, tol=1e-7, maxit=1000):
    """Device replacement of CompBiCG (BICGSTAB.c:5-339) on a dense matrix."""
    are, aim = _f64(A.real), _f64(A.imag)
    br, bi = _f64(b.real), _f64(b.imag)
    n = are.shape[0]
    xr, xi = np.empty(n), np.empty(n)
    info = SolveInfo()
    _check(load().hz_dense_bicg(n, _ptr(are), _ptr(aim), _ptr(br), _ptr(bi), _ptr(xr), _ptr(xi), tol, maxit,
                                HZ_HOST, C.byref(info)))
    return xr + 1j * xi, info.as_dict()


# ------------------------------------------------------------------ batches
class Batch:
    """Independent built operators solved together (hz_batch_*): one
    persistent FP32 launch per product over all of them."""

    def __init__(self, ops):
        self.ops = list(ops)
        arr = (_vp * len(self.ops))(*[o.h for o in self.ops])
        h = _vp()
        _check(load().hz_batch_create(arr, len(self.ops), C.byref(h)))
        self.h = h

    def close(self):
        """Destroy the batch (the operators stay)."""
        if self.h:
            load().hz_batch_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def autotune(self):
        """Time the batch sweep shapes on this batch and keep the fastest:
        (shape, ms per product)."""
        cfg, ms = C.c_int(), C.c_double()
        _check(load().hz_batch_autotune(self.h, C.byref(cfg), C.byref(ms)))
        return cfg.value, ms.value

    def set_variant(self, v):
        """Force batch sweep shape v (0 .. 3)."""
        _check(load().hz_batch_set_variant(self.h, v))

    @staticmethod
    def _ptrs(arrs):
        return (_vp * len(arrs))(*[a.ctypes.data for a in arrs])

    def matvec(self, vs, precision=PREC_F32):
        """A_r v_r for every operator r of the batch."""
        pr = [_f64(v.real) for v in vs]
        pi = [_f64(v.imag) for v in vs]
        qr = [np.empty(o.n) for o in self.ops]
        qi = [np.empty(o.n) for o in self.ops]
        _check(load().hz_batch_matvec(self.h, precision, self._ptrs(pr), self._ptrs(pi), self._ptrs(qr),
                                      self._ptrs(qi), HZ_HOST))
        return [a + 1j * b for a, b in zip(qr, qi)]

    def solve(self, bs, opts=None, **kw):
        """Solve every A_r x_r = b_r together; returns (xs, info dict,
        residuals)."""
        opts = opts if opts is not None else solve_opts(**kw)
        br = [_f64(b.real) for b in bs]
        bi = [_f64(b.imag) for b in bs]
        xr = [np.empty(o.n) for o in self.ops]
        xi = [np.empty(o.n) for o in self.ops]
        info = SolveInfo()
        res = np.empty(len(self.ops))
        _check(load().hz_batch_solve(self.h, C.byref(opts), self._ptrs(br), self._ptrs(bi), self._ptrs(xr),
                                     self._ptrs(xi), HZ_HOST, C.byref(info), _ptr(res)))
        return [a + 1j * b for a, b in zip(xr, xi)], info.as_dict(), res


# ------------------------------------------------------------ dense assemblers
DENSE_DOUBLE_LAYER, DENSE_COMBO, DENSE_SPHERE = 0, 1, 2
DENSE_ROWS = ["zx", "zy", "zz", "xs", "ys", "zs", "dist", "gx", "gy", "gz", "delta", "jac", "curv", "reg",
              "regimg", "polyw", "sinew", "polyres", "sineres", "result"]


def dense_opts(kind, p, **kw):
    """hz_dense_opts with the reference's defaults for kind, then kw."""
    o = DenseOpts()
    load().hz_dense_opts_default(C.byref(o), kind, C.byref(p))
    for k, v in kw.items():
        if k == "center":
            o.center[:] = list(v)
        else:
            setattr(o, k, v)
    return o


def dense_assemble(kind, p, o, d=None, grids=None, matrices=True):
    """Assemble one of the dense operators of HelmholtzKernel.c on the GPU.

    Returns (pts [20][n], K1, K2, regcount): K1 the double-layer or PolyWeight
    matrix, K2 the SineWeight matrix (None when not assembled)."""
    L = load()
    dd = None if d is None else _f64(d)
    n = C.c_int64()
    _check(L.hz_dense_count(kind, C.byref(p), C.byref(o), None if dd is None else _ptr(dd), HZ_HOST, C.byref(n)))
    n = n.value
    g = [None] * 5 if grids is None else [_f64(x) for x in grids]
    pts = np.zeros((len(DENSE_ROWS), n))
    want1 = matrices and (kind == DENSE_DOUBLE_LAYER or o.poly)
    want2 = matrices and kind != DENSE_DOUBLE_LAYER and o.sine
    m1 = [np.empty((n, n)), np.empty((n, n))] if want1 else [None, None]
    m2 = [np.empty((n, n)), np.empty((n, n))] if want2 else [None, None]
    rc = C.c_int64()
    ptr = lambda a: None if a is None else _ptr(a)
    _check(L.hz_dense_assemble(kind, C.byref(p), C.byref(o), ptr(dd), *[ptr(x) for x in g], n, _ptr(pts),
                               ptr(m1[0]), ptr(m1[1]), ptr(m2[0]), ptr(m2[1]), C.byref(rc), HZ_HOST))
    K1 = None if m1[0] is None else m1[0] + 1j * m1[1]
    K2 = None if m2[0] is None else m2[0] + 1j * m2[1]
    return pts, K1, K2, rc.value


def ref_config(**kw):
    """Read (and with kw, update) the switches of the reference-signature
    dense assemblers; returns the configuration in force."""
    c = RefConfig()
    load().hz_ref_get_config(C.byref(c))
    if kw:
        for k, v in kw.items():
            if k == "center":
                c.center[:] = list(v)
            else:
                setattr(c, k, v)
        load().hz_ref_set_config(C.byref(c))
    return c


# ------------------------------------------------------------------ text files
def reference_file_names(N, wave):
    """Names the reference driver uses for distance, boundary data, density
    and result files (large3Dexample2.c:407,607-608,2990-2991,1635)."""
    bufs = [C.create_string_buffer(256) for _ in range(6)]
    _check(load().hz_reference_file_names(N, wave, *bufs, 256))
    keys = ["b", "bimg", "density", "densityimg", "result", "distance"]
    return {k: b.value.decode() for k, b in zip(keys, bufs)}


def read_distance_file(path, N):
    """A distance<N>.txt grid in the reference's format ((N+1)^3 values)."""
    d = np.empty((N + 1,) * 3)
    _check(load().hz_read_distance_file(path.encode(), N, _ptr(d)))
    return d


def write_distance_file(path, N, d):
    """Write a grid in the reference's distance-file format."""
    d = _f64(d)
    _check(load().hz_write_distance_file(path.encode(), N, _ptr(d)))


def write_rhs_files(path_re, path_im, b):
    """Boundary data in the reference's b / bimg file format."""
    br, bi = _f64(b.real), _f64(b.imag)
    _check(load().hz_write_rhs_files(path_re.encode(), path_im.encode(), len(br), _ptr(br), _ptr(bi)))


def read_rhs_files(path_re, path_im, n):
    """Read n complex boundary values from the reference's b / bimg files."""
    br, bi = np.empty(n), np.empty(n)
    _check(load().hz_read_rhs_files(path_re.encode(), path_im.encode(), n, _ptr(br), _ptr(bi)))
    return br + 1j * bi


def write_density_files(path_re, path_im, x):
    """A density in the reference's density / densityimg file format."""
    xr, xi = _f64(x.real), _f64(x.imag)
    _check(load().hz_write_density_files(path_re.encode(), path_im.encode(), len(xr), _ptr(xr), _ptr(xi)))


def read_density_files(path_re, path_im, n):
    """Read n complex density values from the reference's density files."""
    xr, xi = np.empty(n), np.empty(n)
    _check(load().hz_read_density_files(path_re.encode(), path_im.encode(), n, _ptr(xr), _ptr(xi)))
    return xr + 1j * xi


def write_result_file(path, exact, approx):
    """Append one line of the reference's Rel_Result log (exact and computed field)."""
    _check(load().hz_write_result_file(path.encode(), exact.real, exact.imag, approx.real, approx.imag))


def misfit_function(op, receivers, target, layer=None, **solve_kw):
    """A torch.autograd.Function over (Re b, Im b) for gradcheck of the
    adjoint gradient against finite differences of the forward solve (used
    by the tests only; the product entry point is Operator.misfit_gradient)."""
    import torch

    class _Misfit(torch.autograd.Function):
        @staticmethod
        def forward(ctx, b_re, b_im):
            b = b_re.detach().cpu().numpy() + 1j * b_im.detach().cpu().numpy()
            J, g, _, _, _ = op.misfit_gradient(b, receivers, target, layer=layer, **solve_kw)
            ctx.save_for_backward(torch.from_numpy(g.real.copy()), torch.from_numpy(g.imag.copy()))
            return torch.tensor(J, dtype=torch.float64)

        @staticmethod
        def backward(ctx, grad_out):
            gr, gi = ctx.saved_tensors
            return grad_out * gr, grad_out * gi

    return _Misfit.apply
