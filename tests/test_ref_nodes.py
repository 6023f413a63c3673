"""The reference's per-node entry points exported by libhzgb300.so (host code,
no GPU): weno, WENO_DX/DY/DZ (weno.h:26-31) and BothCurvs, MeanCurv,
GaussianCurv (distance_application3D.h:9-11).  Each is called through its
C++ (mangled) name on every node of a small grid and compared bit for bit
with the same function of the reference build (oracle/_ref, compiled from
the reference sources by oracle/build_ref.py)."""
import ctypes as C
import os

import numpy as np
import pytest

from conftest import ROOT

REF_SO = os.path.join(ROOT, "oracle", "_ref", "libref_neumann.so")

SYMS = {
    "weno": "_Z4wenoPdS_S_di",
    "WENO_DX": "_Z7WENO_DXPPPdiiiidS_S_i",
    "WENO_DY": "_Z7WENO_DYPPPdiiiidS_S_i",
    "WENO_DZ": "_Z7WENO_DZPPPdiiiidS_S_i",
    "BothCurvs": "_Z9BothCurvsPPPdiiiidS_S_",
    "MeanCurv": "_Z8MeanCurvPPPdiiiid",
    "GaussianCurv": "_Z12GaussianCurvPPPdiiiid",
}

_dp = C.POINTER(C.c_double)
_ppp = C.POINTER(C.POINTER(_dp))


def bind(path):
    L = C.CDLL(path)
    f = {}
    for name, sym in SYMS.items():
        fn = getattr(L, sym)
        if name == "weno":
            fn.argtypes = [_dp, _dp, _dp, C.c_double, C.c_int]
            fn.restype = None
        elif name.startswith("WENO_D"):
            fn.argtypes = [_ppp, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, _dp, _dp, C.c_int]
            fn.restype = None
        elif name == "BothCurvs":
            fn.argtypes = [_ppp, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, _dp, _dp]
            fn.restype = C.c_int
        else:
            fn.argtypes = [_ppp, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double]
            fn.restype = C.c_double
        f[name] = fn
    return L, f


def ragged(a):
    """double*** view of a contiguous (S, S, S) array (rows point into a)."""
    S = a.shape[0]
    rows = [(_dp * S)(*[a[i, j].ctypes.data_as(_dp) for j in range(S)]) for i in range(S)]
    top = (C.POINTER(_dp) * S)(*[C.cast(r, C.POINTER(_dp)) for r in rows])
    return C.cast(top, _ppp), rows, top


@pytest.fixture(scope="module")
def libs(hz):
    if not os.path.exists(REF_SO):
        pytest.skip("reference build oracle/_ref not present")
    return bind(hz.LIB_PATH)[1], bind(REF_SO)[1]


def grid(N, seed):
    from helmholtz_3d_torrone_gb300 import geometry as G
    d = G.sphere(N, radius=1.0, center=(0.013, 0.021, 0.007), int_l=-2.0, int_u=2.0)
    # a small seeded ripple, so that limiter branches and ties vary
    rng = np.random.default_rng(seed)
    return np.ascontiguousarray(d + 0.01 * rng.standard_normal(d.shape))


def test_weno_kernel_bit_exact(libs):
    ours, ref = libs
    rng = np.random.default_rng(1)
    for order in (5, 3):
        for _ in range(2000):
            fi = np.ascontiguousarray(rng.standard_normal(7) * rng.choice([1e-3, 1.0, 1e3]))
            a, b, c, d = (C.c_double() for _ in range(4))
            ours["weno"](C.byref(a), C.byref(b), fi.ctypes.data_as(_dp), 0.1, order)
            ref["weno"](C.byref(c), C.byref(d), fi.ctypes.data_as(_dp), 0.1, order)
            assert (a.value, b.value) == (c.value, d.value)


def test_weno_lines_and_curvatures_bit_exact(libs):
    ours, ref = libs
    N = 12
    H = 4.0 / N
    d = grid(N, 7)
    g, _rows, _top = ragged(d)
    S = N + 1
    for i in range(S):
        for j in range(S):
            for k in range(S):
                for name in ("WENO_DX", "WENO_DY", "WENO_DZ"):
                    for order in (5, 3, 4):  # 4: neither order, outputs untouched
                        a, b = C.c_double(-7.0), C.c_double(-7.0)
                        c, e = C.c_double(-7.0), C.c_double(-7.0)
                        ours[name](g, i, j, k, N, H, C.byref(a), C.byref(b), order)
                        ref[name](g, i, j, k, N, H, C.byref(c), C.byref(e), order)
                        assert (a.value, b.value) == (c.value, e.value), (name, order, i, j, k)
                m1, g1, m2, g2 = (C.c_double() for _ in range(4))
                assert ours["BothCurvs"](g, i, j, k, N, H, C.byref(m1), C.byref(g1)) == 0
                ref["BothCurvs"](g, i, j, k, N, H, C.byref(m2), C.byref(g2))
                assert (m1.value, g1.value) == (m2.value, g2.value), (i, j, k)
                assert ours["MeanCurv"](g, i, j, k, N, H) == ref["MeanCurv"](g, i, j, k, N, H)
                assert ours["GaussianCurv"](g, i, j, k, N, H) == ref["GaussianCurv"](g, i, j, k, N, H)
