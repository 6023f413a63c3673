"""Dense assemblers of HelmholtzKernel.c on the GPU, against the reference.

* hz_dense_assemble (C ABI) for DoubleLayerKernel, new_HelmholtzKernelCombo
  and new_HelmholtzKernel against the golden fixture made from the compiled
  reference (ref_neumann_dense_n16): geometry rows (nodes, x*, distances,
  normals, Jacobian, curvature, regularisation) bit-exact; rows through
  cos/exp/pow (delta_eps, PolyWeight/SineWeight and the weighted results)
  1e-14 relative; sampled matrix entries and the seeded products K v 1e-12
  relative (CUDA's cos/sin against the C library's, through finite
  differences); Combo's regcount exact.
* The full GPU matrices against the oracle's: 1e-12 relative.
* The reference-signature drop-ins (C++ linkage, ragged arrays, the
  driver's globals N, SIZE, H, HCUBED, WAVE) give the same arrays as the
  C ABI.
"""
import ctypes as C
import json
import subprocess

import numpy as np
import pytest

from conftest import golden, rel_err

pytestmark = pytest.mark.gpu

EXACT = {"zx", "zy", "zz", "xs", "ys", "zs", "dist", "gx", "gy", "gz", "jac", "curv", "reg", "regimg"}
ROWS = {
    "dl": ["zx", "zy", "zz", "xs", "ys", "zs", "dist", "gx", "gy", "gz", "delta", "jac", "reg", "regimg", "result"],
    "combo": ["zx", "zy", "zz", "xs", "ys", "zs", "dist", "gx", "gy", "gz", "jac", "reg", "regimg", "sinew",
              "sineres"],
    "sphere": ["zx", "zy", "zz", "xs", "ys", "zs", "dist", "gx", "gy", "gz", "jac", "curv", "sinew", "sineres"],
}
KIND = {"dl": 0, "combo": 1, "sphere": 2}


@pytest.fixture(scope="module")
def case(hz):
    g = golden("ref_neumann_dense_n16")
    m = json.loads(str(g["meta"]))
    p = hz.params(m["N"], m["wave"], int_l=m["int_l"], int_u=m["int_u"], factor=m["factor"],
                  tau_factor=m["tau_factor"], dirichlet=m["dirichlet"], interior=m["interior"])
    return g, m, p


def opts(hz, m, p, tag):
    f = m["flags"]
    if tag == "dl":
        return hz.dense_opts(0, p, epsilon=m["epsilon"], poly=f["poly"], sine=f["sine"], onesided=f["trad_onesided"])
    return hz.dense_opts(KIND[tag], p, delta0=m["delta0"], epsilon=m["epsilon0"], wavenum=m["wave"], eta=m["eta"],
                         poly=f["poly"], sine=f["sine"], onesided=f["combo_onesided"],
                         combo_interior=f["combo_interior"], radius=f["radius"], center=f["center"])


@pytest.fixture(scope="module")
def assembled(hz, case):
    g, m, p = case
    out = {}
    for tag in ("dl", "combo", "sphere"):
        o = opts(hz, m, p, tag)
        d = None if tag == "sphere" else g["d"]
        out[tag] = hz.dense_assemble(KIND[tag], p, o, d)
    return out


def matrix_of(tag, m, res):
    pts, K1, K2, rc = res
    return K1 if tag == "dl" else (K2 if m["flags"]["sine"] else K1)


@pytest.mark.parametrize("tag", ["dl", "combo", "sphere"])
def test_dense_vs_reference_fixture(hz, case, assembled, tag):
    g, m, p = case
    pts, K1, K2, rc = assembled[tag]
    ref = g[tag + "_pts"]
    assert pts.shape == ref.shape
    for name in ROWS[tag]:
        i = hz.DENSE_ROWS.index(name)
        if name in EXACT:
            assert np.array_equal(pts[i].view(np.uint64), ref[i].view(np.uint64)), name
        else:
            assert rel_err(pts[i], ref[i]) <= 1e-14, name
    K = matrix_of(tag, m, assembled[tag])
    assert rel_err(K[g[tag + "_pi"], g[tag + "_pj"]], g[tag + "_entries"]) <= 1e-12
    assert rel_err(K @ g[tag + "_v"], g[tag + "_Kv"]) <= 1e-12
    if tag == "combo":
        assert rc == m["regcount"]


@pytest.mark.parametrize("tag", ["dl", "combo", "sphere"])
def test_dense_full_matrix_vs_oracle(hz, oracle, case, assembled, tag):
    import oracle as O
    g, m, p = case
    f = m["flags"]
    po = O.Params(m["N"], m["int_l"], m["int_u"], m["wave"], m["factor"], m["tau_factor"], m["dirichlet"],
                  m["interior"])
    if tag == "dl":
        o = O.DenseOpts(0.0, m["epsilon"], m["wave"], m["eta"], f["poly"], f["sine"], f["trad_onesided"],
                        f["combo_interior"], f["radius"], *f["center"])
    else:
        o = O.DenseOpts(m["delta0"], m["epsilon0"], m["wave"], m["eta"], f["poly"], f["sine"], f["combo_onesided"],
                        f["combo_interior"], f["radius"], *f["center"])
    pts = assembled[tag][0]
    K1, K2, rc = oracle.dense_matrix(KIND[tag], po, o, pts)
    Ko = K1 if tag == "dl" else (K2 if f["sine"] else K1)
    assert rel_err(matrix_of(tag, m, assembled[tag]), Ko) <= 1e-12
    if tag == "combo":
        assert rc == assembled[tag][3]


def test_dense_count_mismatch_is_an_error(hz, case):
    g, m, p = case
    o = opts(hz, m, p, "dl")
    n = C.c_int64()
    hz._check(hz.load().hz_dense_count(0, C.byref(p), C.byref(o), hz._ptr(hz._f64(g["d"])), hz.HZ_HOST,
                                       C.byref(n)))
    rc = hz.load().hz_dense_assemble(0, C.byref(p), C.byref(o), hz._ptr(hz._f64(g["d"])), None, None, None, None,
                                     None, n.value + 1, None, None, None, None, None, None, hz.HZ_HOST)
    assert rc == -1


# --------------------------------------------------------------- drop-ins
_dp = C.POINTER(C.c_double)


def ragged3(a, keep):
    S = a.shape[0]
    planes = []
    for i in range(S):
        rows = (_dp * S)(*[a[i, j].ctypes.data_as(_dp) for j in range(S)])
        keep.append(rows)
        planes.append(C.cast(rows, C.POINTER(_dp)))
    top = (C.POINTER(_dp) * S)(*planes)
    keep.append(top)
    return C.cast(top, C.POINTER(C.POINTER(_dp)))


def ragged2(a, keep):
    rows = (_dp * a.shape[0])(*[a[i].ctypes.data_as(_dp) for i in range(a.shape[0])])
    keep.append(rows)
    return C.cast(rows, C.POINTER(_dp))


def mangled(lib_path, name):
    out = subprocess.run(["nm", "-D", "--defined-only", lib_path], capture_output=True, text=True, check=True).stdout
    for line in out.splitlines():
        s = line.split()[-1]
        if s.startswith("_Z%d%s" % (len(name), name)):
            return s
    raise KeyError(name)


def set_driver_globals(lib, m):
    N = m["N"]
    H = (m["int_u"] - m["int_l"]) / N
    C.c_int.in_dll(lib, "N").value = N
    C.c_int.in_dll(lib, "SIZE").value = N + 1
    C.c_double.in_dll(lib, "H").value = H
    C.c_double.in_dll(lib, "HCUBED").value = H * H * H
    C.c_double.in_dll(lib, "WAVE").value = m["wave"]


def test_reference_signature_double_layer_and_combo(hz, case, assembled):
    g, m, p = case
    L = hz.load()
    set_driver_globals(L, m)
    hz.ref_config(int_l=m["int_l"], int_u=m["int_u"], tau_factor=m["tau_factor"], interior=m["interior"])
    N = m["N"]
    H = (m["int_u"] - m["int_l"]) / N
    d = np.ascontiguousarray(g["d"])
    gx, gy, gz = (np.empty_like(d) for _ in range(3))
    mc, gc = np.empty_like(d), np.empty_like(d)
    hz._check(L.hz_assign_gradient(N, H, hz._ptr(d), hz._ptr(gx), hz._ptr(gy), hz._ptr(gz), 5, hz.HZ_HOST))
    hz._check(L.hz_assign_curvatures(N, H, hz._ptr(d), hz._ptr(mc), hz._ptr(gc), hz.HZ_HOST))
    keep = []
    grids = [ragged3(a, keep) for a in (d, gx, gy, gz, mc, gc)]
    # DoubleLayerKernel
    n = assembled["dl"][0].shape[1]
    lists = [np.zeros(n) for _ in range(15)]
    K, Ki = np.zeros((n, n)), np.zeros((n, n))
    f = getattr(L, mangled(hz.LIB_PATH, "DoubleLayerKernel"))
    f.restype = C.c_int
    rc = f(C.c_int(n), C.c_double(m["epsilon"]), *grids, *[x.ctypes.data_as(_dp) for x in lists],
           ragged2(K, keep), ragged2(Ki, keep), C.c_double(m["wave"]))
    assert rc == 0, hz.load().hz_last_error()
    pts = assembled["dl"][0]
    order = ["zx", "zy", "zz", "xs", "ys", "zs", "dist", "gx", "gy", "gz", "delta", "jac", "reg", "regimg", "result"]
    for name, arr in zip(order, lists):
        assert np.array_equal(arr, pts[hz.DENSE_ROWS.index(name)]), name
    assert np.array_equal(K + 1j * Ki, assembled["dl"][1])
    # new_HelmholtzKernelCombo
    n = assembled["combo"][0].shape[1]
    lists = [np.zeros(n) for _ in range(17)]
    mats = [np.zeros((n, n)) for _ in range(4)]
    f = getattr(L, mangled(hz.LIB_PATH, "new_HelmholtzKernelCombo"))
    f.restype = C.c_int
    rc = f(C.c_int(n), C.c_double(m["delta0"]), C.c_double(m["epsilon0"]), *grids,
           *[x.ctypes.data_as(_dp) for x in lists], *[ragged2(a, keep) for a in mats], C.c_double(m["wave"]),
           C.c_double(m["eta"]))
    assert rc == m["regcount"], hz.load().hz_last_error()
    pts = assembled["combo"][0]
    order = ["zx", "zy", "zz", "xs", "ys", "zs", "dist", "gx", "gy", "gz", "jac", "reg", "regimg", "polyw", "sinew",
             "polyres", "sineres"]
    for name, arr in zip(order, lists):
        if name.startswith("poly") and not m["flags"]["poly"]:
            continue
        assert np.array_equal(arr, pts[hz.DENSE_ROWS.index(name)]), name
    if m["flags"]["sine"]:
        assert np.array_equal(mats[2] + 1j * mats[3], assembled["combo"][2])
