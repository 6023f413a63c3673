"""Test oracle for the IBIM Helmholtz hot path (TEST INFRASTRUCTURE ONLY).

Two checkers live here, both CPU-only:

* ``Oracle`` -- ctypes binding of ``ibim_oracle.c``, a C restatement of the
  reference's algorithm (moorhsum/Helmholtz-3D-torrone) written for this
  project.  Built by ``make -C oracle``.
* ``Reference`` -- ctypes binding of the reference's own C code, patched and
  compiled by ``oracle/build_ref.py`` into ``oracle/_ref/libref_<variant>.so``.
  Each instance runs in the process that loads it and holds one
  configuration (the reference keeps its tube arrays in function statics).

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline and
reference legs use this package.  The product never imports it.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_LIB = os.path.join(HERE, "_build", "libibim_oracle.so")
REF_DIR = os.path.join(HERE, "_ref")

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int64)
_i32p = C.POINTER(C.c_int)


def build_oracle():
    subprocess.run(["make", "-s", "-C", HERE], check=True)


def _d(a):
    return a.ctypes.data_as(_dp)


def _i(a):
    return a.ctypes.data_as(_ip)


class Params(C.Structure):
    _fields_ = [("N", C.c_int), ("int_l", C.c_double), ("int_u", C.c_double), ("wave", C.c_double),
                ("factor", C.c_double), ("tau_factor", C.c_double), ("dirichlet", C.c_int),
                ("interior", C.c_int)]

    @property
    def H(self):
        return (self.int_u - self.int_l) / self.N

    @property
    def eps(self):
        return self.factor * self.H


def make_params(N, wave, int_l=-1.0, int_u=1.0, factor=3.0, tau_factor=2.0, dirichlet=1, interior=0):
    return Params(N, int_l, int_u, wave, factor, tau_factor, dirichlet, interior)


class DenseOpts(C.Structure):
    """Options of the dense assemblers (or_dense_opts)."""
    _fields_ = [("delta0", C.c_double), ("epsilon", C.c_double), ("wavenum", C.c_double), ("eta", C.c_double),
                ("poly", C.c_int), ("sine", C.c_int), ("onesided", C.c_int), ("combo_interior", C.c_int),
                ("radius", C.c_double), ("cx", C.c_double), ("cy", C.c_double), ("cz", C.c_double)]


# rows of the per-point arrays of the dense assemblers (or_dense_points)
DENSE_ROWS = ["zx", "zy", "zz", "xs", "ys", "zs", "dist", "gx", "gy", "gz", "delta", "jac", "curv", "reg",
              "regimg", "polyw", "sinew", "polyres", "sineres", "result"]
DENSE_DOUBLE_LAYER, DENSE_COMBO, DENSE_SPHERE = 0, 1, 2


class Oracle:
    """ctypes wrapper over ibim_oracle.c (every call is FP64 on the CPU)."""

    def __init__(self, path=ORACLE_LIB):
        if not os.path.exists(path):
            build_oracle()
        L = C.CDLL(path)
        self.L = L
        P = C.POINTER(Params)
        L.or_weno.argtypes = [_dp, _dp, _dp, C.c_double, C.c_int]
        L.or_gradient.argtypes = [C.c_int, C.c_double, _dp, _dp, _dp, _dp, C.c_int]
        L.or_curvatures.argtypes = [C.c_int, C.c_double, _dp, _dp, _dp]
        L.or_tube.argtypes = [C.c_int, _dp, C.c_double, _ip]
        L.or_tube.restype = C.c_int64
        L.or_tube_init.argtypes = [P, _dp, _dp, _dp, _dp, _dp, _dp, C.c_int64, _ip] + [_dp] * 6
        L.or_tube_init.restype = C.c_int
        L.or_entry.argtypes = [P, _dp, _dp, _dp, _dp, C.c_int64, C.c_int64, _dp, _dp]
        L.or_dense_rows.argtypes = [P, C.c_int64, _dp, _dp, _dp, _dp, C.c_int64, C.c_int64, _dp, _dp]
        L.or_matvec.argtypes = [P, C.c_int64, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp, C.c_int,
                                C.c_int64, C.c_int64, C.c_int]
        L.or_bicg.argtypes = [P, C.c_int64, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp, C.c_double,
                              C.c_int, C.c_int, _dp]
        L.or_bicg.restype = C.c_int
        L.or_bicg_dense.argtypes = [C.c_int64, _dp, _dp, _dp, _dp, _dp, _dp, C.c_double, C.c_int, _dp]
        L.or_bicg_dense.restype = C.c_int
        L.or_eval.argtypes = [P, C.c_int64, _dp, _dp, _dp, _dp, _dp, C.c_int64, _dp, _dp, _dp,
                              C.c_int, C.c_int]
        L.or_point_source_rhs.argtypes = [P, C.c_int64, _dp, _dp, _dp, C.c_int, _dp, _dp]
        L.or_reinit.argtypes = [C.c_int, C.c_double, _dp, C.c_int, C.c_double, C.c_int]
        L.or_godunov.argtypes = [C.c_double] * 7
        L.or_godunov.restype = C.c_double
        D = C.POINTER(DenseOpts)
        L.or_dense_points.argtypes = [C.c_int, P, D] + [_dp] * 6 + [C.c_int64, _dp]
        L.or_dense_points.restype = C.c_int64
        L.or_dense_matrix.argtypes = [C.c_int, P, D, C.c_int64, _dp, _dp, _dp, _dp, _dp]
        L.or_dense_matrix.restype = C.c_int64
        L.or_poly_weight.argtypes = [C.c_double, C.c_double]
        L.or_poly_weight.restype = C.c_double
        L.or_sine_weight.argtypes = [C.c_double, C.c_double]
        L.or_sine_weight.restype = C.c_double

    def weno(self, fi, dx, order=5):
        fi = np.ascontiguousarray(fi, dtype=np.float64)
        p, n = C.c_double(), C.c_double()
        self.L.or_weno(C.byref(p), C.byref(n), _d(fi), dx, order)
        return p.value, n.value

    def godunov(self, signage, a, b, c, d, e, f):
        return self.L.or_godunov(signage, a, b, c, d, e, f)

    def gradient(self, N, H, d, order=5):
        d = np.ascontiguousarray(d, dtype=np.float64)
        g = [np.empty_like(d) for _ in range(3)]
        self.L.or_gradient(N, H, _d(d), _d(g[0]), _d(g[1]), _d(g[2]), order)
        return g

    def reinit(self, N, H, phi, iters, cfl=0.5, order=5):
        out = np.array(phi, dtype=np.float64, copy=True, order="C")
        self.L.or_reinit(N, H, _d(out), iters, cfl, order)
        return out

    def curvatures(self, N, H, d):
        d = np.ascontiguousarray(d, dtype=np.float64)
        m, g = np.empty_like(d), np.empty_like(d)
        self.L.or_curvatures(N, H, _d(d), _d(m), _d(g))
        return m, g

    def tube(self, N, d, eps):
        d = np.ascontiguousarray(d, dtype=np.float64)
        n = self.L.or_tube(N, _d(d), eps, None)
        idx = np.empty(n, dtype=np.int64)
        self.L.or_tube(N, _d(d), eps, _i(idx))
        return idx

    def tube_init(self, p, d, grads, mc, gc, idx):
        n = len(idx)
        xs, nrm = np.empty((n, 3)), np.empty((n, 3))
        delta, jac, reg, w = (np.empty(n) for _ in range(4))
        bad = self.L.or_tube_init(C.byref(p), _d(d), _d(grads[0]), _d(grads[1]), _d(grads[2]),
                                  _d(mc), _d(gc), n, _i(idx), _d(xs), _d(nrm), _d(delta), _d(jac),
                                  _d(reg), _d(w))
        return dict(xs=xs, nrm=nrm, delta=delta, jac=jac, reg=reg, w=w, bad=bad)

    def dense(self, p, tp, r0=0, r1=None):
        n = len(tp["w"])
        r1 = n if r1 is None else r1
        are = np.empty((r1 - r0, n))
        aim = np.empty((r1 - r0, n))
        self.L.or_dense_rows(C.byref(p), n, _d(tp["xs"]), _d(tp["nrm"]), _d(tp["reg"]), _d(tp["w"]),
                             r0, r1, _d(are), _d(aim))
        return are, aim

    def matvec(self, p, tp, v, adjoint=False, r0=0, r1=None, nthreads=os.cpu_count() or 1):
        n = len(tp["w"])
        r1 = n if r1 is None else r1
        vr = np.ascontiguousarray(v.real, dtype=np.float64)
        vi = np.ascontiguousarray(v.imag, dtype=np.float64)
        qr, qi = np.empty(r1 - r0), np.empty(r1 - r0)
        self.L.or_matvec(C.byref(p), n, _d(tp["xs"]), _d(tp["nrm"]), _d(tp["reg"]), _d(tp["w"]),
                         _d(vr), _d(vi), _d(qr), _d(qi), int(adjoint), r0, r1, nthreads)
        return qr + 1j * qi

    def bicg(self, p, tp, b, acc=1e-13, maxit=2000, nthreads=os.cpu_count() or 1):
        n = len(tp["w"])
        br = np.ascontiguousarray(b.real, dtype=np.float64)
        bi = np.ascontiguousarray(b.imag, dtype=np.float64)
        xr, xi = np.empty(n), np.empty(n)
        res = C.c_double()
        it = self.L.or_bicg(C.byref(p), n, _d(tp["xs"]), _d(tp["nrm"]), _d(tp["reg"]), _d(tp["w"]),
                            _d(br), _d(bi), _d(xr), _d(xi), acc, maxit, nthreads, C.byref(res))
        return xr + 1j * xi, it, res.value

    def bicg_dense(self, are, aim, b, acc=1e-13, maxit=2000):
        n = are.shape[0]
        are = np.ascontiguousarray(are)
        aim = np.ascontiguousarray(aim)
        br = np.ascontiguousarray(b.real, dtype=np.float64)
        bi = np.ascontiguousarray(b.imag, dtype=np.float64)
        xr, xi = np.empty(n), np.empty(n)
        res = C.c_double()
        it = self.L.or_bicg_dense(n, _d(are), _d(aim), _d(br), _d(bi), _d(xr), _d(xi), acc, maxit,
                                  C.byref(res))
        return xr + 1j * xi, it, res.value

    def evaluate(self, p, tp, sigma, receivers, double_layer, nthreads=os.cpu_count() or 1):
        n = len(tp["w"])
        rx = np.ascontiguousarray(receivers, dtype=np.float64)
        m = rx.shape[0]
        sr = np.ascontiguousarray(sigma.real)
        si = np.ascontiguousarray(sigma.imag)
        ur, ui = np.empty(m), np.empty(m)
        self.L.or_eval(C.byref(p), n, _d(tp["xs"]), _d(tp["nrm"]), _d(tp["w"]), _d(sr), _d(si), m,
                       _d(rx), _d(ur), _d(ui), int(double_layer), nthreads)
        return ur + 1j * ui

    def rhs(self, p, tp, src, kind):
        n = len(tp["w"])
        s = np.ascontiguousarray(src, dtype=np.float64)
        br, bi = np.empty(n), np.empty(n)
        self.L.or_point_source_rhs(C.byref(p), n, _d(tp["xs"]), _d(tp["nrm"]), _d(s), kind, _d(br), _d(bi))
        return br + 1j * bi

    def dense_points(self, kind, p, o, d=None, grids=None):
        """Per-point arrays of a dense assembler: dict of DENSE_ROWS."""
        if grids is None:
            args = [None] * 6 if d is None else [_d(np.ascontiguousarray(d))] + [None] * 5
        else:
            args = [_d(np.ascontiguousarray(d))] + [_d(np.ascontiguousarray(g)) for g in grids]
        n = self.L.or_dense_points(kind, C.byref(p), C.byref(o), *args, 0, None)
        if n < 0:
            raise ValueError("interpolation cell outside the grid at point %d" % (-n - 1))
        pts = np.zeros((len(DENSE_ROWS), n))
        self.L.or_dense_points(kind, C.byref(p), C.byref(o), *args, n, _d(pts))
        return {k: pts[i] for i, k in enumerate(DENSE_ROWS)}, pts

    def dense_matrix(self, kind, p, o, pts):
        """(K1, K2, regcount): K1 the double-layer or PolyWeight matrix, K2 the
        SineWeight matrix (None when not assembled)."""
        n = pts.shape[1]
        pts = np.ascontiguousarray(pts)
        k1 = [np.zeros((n, n)), np.zeros((n, n))]
        k2 = [np.zeros((n, n)), np.zeros((n, n))] if kind != DENSE_DOUBLE_LAYER and o.sine else [None, None]
        if kind != DENSE_DOUBLE_LAYER and not o.poly:
            k1 = [None, None]
        ptr = lambda a: None if a is None else _d(a)
        rc = self.L.or_dense_matrix(kind, C.byref(p), C.byref(o), n, _d(pts), ptr(k1[0]), ptr(k1[1]),
                                    ptr(k2[0]), ptr(k2[1]))
        K1 = None if k1[0] is None else k1[0] + 1j * k1[1]
        K2 = None if k2[0] is None else k2[0] + 1j * k2[1]
        return K1, K2, int(rc)

    def pipeline(self, p, d):
        """Grids -> tube -> per-point arrays, all on the CPU."""
        N, H = p.N, p.H
        grads = self.gradient(N, H, d)
        mc, gc = self.curvatures(N, H, d)
        idx = self.tube(N, d, p.eps)
        tp = self.tube_init(p, d, grads, mc, gc, idx)
        tp.update(idx=idx, grads=grads, mc=mc, gc=gc)
        return tp


class Reference:
    """ctypes wrapper over the patched reference build (one config per process)."""

    def __init__(self, variant):
        path = os.path.join(REF_DIR, "libref_%s.so" % variant)
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        L = C.CDLL(path)
        self.L = L
        L.ref_config.argtypes = [_dp]
        L.ref_setup.argtypes = [C.c_int, C.c_double, _dp]
        L.ref_grids.argtypes = [_dp] * 5
        L.ref_h.restype = C.c_double
        L.ref_eps.restype = C.c_double
        L.ref_weno.argtypes = [_dp, _dp, _dp, C.c_double, C.c_int]
        L.ref_godunov.argtypes = [C.c_double] * 7
        L.ref_godunov.restype = C.c_double
        L.ref_tube.argtypes = [C.c_double, _ip]
        L.ref_tube.restype = C.c_int64
        L.ref_tube_points.argtypes = [C.c_double, C.c_int64] + [_dp] * 6
        L.ref_tube_points.restype = C.c_int
        L.ref_entries.argtypes = [C.c_int, C.c_int64, _i32p, _i32p, _dp, _dp]
        L.ref_dense_rows.argtypes = [C.c_int, C.c_int, C.c_int, _dp, _dp, C.c_int]
        L.ref_compbicg.argtypes = [C.c_int, _dp, _dp, _dp, _dp, _dp, _dp, C.c_int]
        L.ref_rows_matvec.argtypes = [C.c_int, C.c_int, C.c_int, _dp, _dp, _dp, _dp, C.c_int]
        L.ref_double_layer.argtypes = [C.c_int, C.c_double, _dp, _dp, _dp]
        L.ref_combo.argtypes = [C.c_int, C.c_double, C.c_double, C.c_double, C.c_double] + [_dp] * 5
        L.ref_combo.restype = C.c_int
        L.ref_sphere_kernel.argtypes = [C.c_int, C.c_double, C.c_double] + [_dp] * 5
        L.ref_dense_flags.argtypes = [_i32p]
        L.ref_sphere.argtypes = [_dp]
        cfg = np.zeros(6)
        L.ref_config(_d(cfg))
        self.int_l, self.int_u, self.factor, self.tau_factor = cfg[:4]
        self.dirichlet, self.interior = int(cfg[4]), int(cfg[5])
        self.N = None

    def params(self, N, wave):
        return Params(N, self.int_l, self.int_u, wave, self.factor, self.tau_factor, self.dirichlet,
                      self.interior)

    def setup(self, N, wave, d):
        d = np.ascontiguousarray(d, dtype=np.float64)
        self.N, self.wave = N, wave
        self.L.ref_setup(N, wave, _d(d))

    def grids(self):
        S = self.N + 1
        g = [np.empty((S, S, S)) for _ in range(5)]
        self.L.ref_grids(*[_d(a) for a in g])
        return g

    def weno(self, fi, dx, order=5):
        fi = np.ascontiguousarray(fi, dtype=np.float64)
        p, n = C.c_double(), C.c_double()
        self.L.ref_weno(C.byref(p), C.byref(n), _d(fi), dx, order)
        return p.value, n.value

    def godunov(self, signage, a, b, c, d, e, f):
        return self.L.ref_godunov(signage, a, b, c, d, e, f)

    def tube(self):
        eps = self.L.ref_eps()
        n = self.L.ref_tube(eps, None)
        idx = np.empty(n, dtype=np.int64)
        self.L.ref_tube(eps, _i(idx))
        return idx

    def tube_points(self, n):
        xs, nrm = np.empty((n, 3)), np.empty((n, 3))
        delta, jac, reg, w = (np.empty(n) for _ in range(4))
        flagged = self.L.ref_tube_points(self.L.ref_eps(), n, _d(xs), _d(nrm), _d(delta), _d(jac),
                                         _d(reg), _d(w))
        return dict(xs=xs, nrm=nrm, delta=delta, jac=jac, reg=reg, w=w, flagged=flagged)

    def entries(self, n, pi, pj):
        pi = np.ascontiguousarray(pi, dtype=np.int32)
        pj = np.ascontiguousarray(pj, dtype=np.int32)
        re, im = np.empty(len(pi)), np.empty(len(pi))
        self.L.ref_entries(n, len(pi), pi.ctypes.data_as(_i32p), pj.ctypes.data_as(_i32p), _d(re), _d(im))
        return re + 1j * im

    def dense(self, n, r0=0, r1=None, nthreads=os.cpu_count() or 1):
        r1 = n if r1 is None else r1
        are, aim = np.empty((r1 - r0, n)), np.empty((r1 - r0, n))
        self.L.ref_dense_rows(n, r0, r1, _d(are), _d(aim), nthreads)
        return are, aim

    def dense_flags(self):
        """POLY_TEST, SINE_TEST, TRAD_ONESIDED, COMBO_ONESIDED, COMBO_INTERIOR,
        INTERIOR_MODE the reference library was compiled with, and its frame.h
        sphere (radius, centre)."""
        f = np.zeros(6, dtype=np.int32)
        self.L.ref_dense_flags(f.ctypes.data_as(_i32p))
        sph = np.zeros(4)
        self.L.ref_sphere(_d(sph))
        return dict(poly=int(f[0]), sine=int(f[1]), trad_onesided=int(f[2]), combo_onesided=int(f[3]),
                    combo_interior=int(f[4]), interior=int(f[5]), radius=sph[0], center=tuple(sph[1:]))

    def double_layer(self, n, epsilon=None):
        """DoubleLayerKernel: (per-point rows (20 x n), dense complex matrix)."""
        epsilon = self.ref_eps() if epsilon is None else epsilon
        pts = np.zeros((20, n))
        are, aim = np.empty((n, n)), np.empty((n, n))
        self.L.ref_double_layer(n, epsilon, _d(pts), _d(are), _d(aim))
        return pts, are + 1j * aim

    def ref_eps(self):
        return self.L.ref_eps()

    def combo(self, n, delta0, epsilon, wavenum, eta):
        """new_HelmholtzKernelCombo: (rows (20 x n), PolyK, SineK, regcount)."""
        pts = np.zeros((20, n))
        m = [np.zeros((n, n)) for _ in range(4)]
        rc = self.L.ref_combo(n, delta0, epsilon, wavenum, eta, _d(pts), *[_d(a) for a in m])
        return pts, m[0] + 1j * m[1], m[2] + 1j * m[3], rc

    def sphere_kernel(self, n, delta0, epsilon):
        """new_HelmholtzKernel on the frame.h sphere: (rows, PolyK, SineK)."""
        pts = np.zeros((20, n))
        m = [np.zeros((n, n)) for _ in range(4)]
        self.L.ref_sphere_kernel(n, delta0, epsilon, _d(pts), *[_d(a) for a in m])
        return pts, m[0] + 1j * m[1], m[2] + 1j * m[3]

    def rows_matvec(self, n, v, r0, r1, nthreads=os.cpu_count() or 1):
        vr = np.ascontiguousarray(v.real)
        vi = np.ascontiguousarray(v.imag)
        qr, qi = np.empty(r1 - r0), np.empty(r1 - r0)
        self.L.ref_rows_matvec(n, r0, r1, _d(vr), _d(vi), _d(qr), _d(qi), nthreads)
        return qr + 1j * qi

    def compbicg(self, are, aim, b, chunk=0):
        """The reference's CompBiCG (chunk <= 0) or omp_CompBiCG (chunk > 0)."""
        n = are.shape[0]
        br = np.ascontiguousarray(b.real)
        bi = np.ascontiguousarray(b.imag)
        xr, xi = np.empty(n), np.empty(n)
        self.L.ref_compbicg(n, _d(np.ascontiguousarray(are)), _d(np.ascontiguousarray(aim)), _d(br), _d(bi),
                            _d(xr), _d(xi), int(chunk))
        return xr + 1j * xi
