"""The oracle's dense assemblers against the reference's (golden fixture
ref_neumann_dense_n16, made by tests/golden/make_golden.py from the compiled
reference): DoubleLayerKernel (HelmholtzKernel.c:613-761),
new_HelmholtzKernelCombo (:173-610) and new_HelmholtzKernel (:3-169).

Tolerances: geometry rows (nodes, x*, dist, normals, Jacobian,
regularisation, curvature) bit-exact; rows and entries that go through libm
transcendentals (delta_eps, PolyWeight/SineWeight, the kernel's cos/sin)
1e-14 relative, so that another libm build still passes; the seeded
products K v 1e-13.
"""
import json

import numpy as np
import pytest

from conftest import golden, rel_err

EXACT_ROWS = {"zx", "zy", "zz", "xs", "ys", "zs", "dist", "gx", "gy", "gz", "jac", "curv", "reg", "regimg"}
ROWS_OF = {
    "dl": ["zx", "zy", "zz", "xs", "ys", "zs", "dist", "gx", "gy", "gz", "delta", "jac", "reg", "regimg", "result"],
    "combo": ["zx", "zy", "zz", "xs", "ys", "zs", "dist", "gx", "gy", "gz", "jac", "reg", "regimg", "sinew",
              "sineres"],
    "sphere": ["zx", "zy", "zz", "xs", "ys", "zs", "dist", "gx", "gy", "gz", "jac", "curv", "sinew", "sineres"],
}


@pytest.fixture(scope="module")
def dense_case(oracle):
    import oracle as O
    g = golden("ref_neumann_dense_n16")
    m = json.loads(str(g["meta"]))
    p = O.Params(m["N"], m["int_l"], m["int_u"], m["wave"], m["factor"], m["tau_factor"], m["dirichlet"],
                 m["interior"])
    grads = oracle.gradient(m["N"], p.H, g["d"])
    mc, gc = oracle.curvatures(m["N"], p.H, g["d"])
    return g, m, p, [grads[0], grads[1], grads[2], mc, gc]


def opts_for(O, m, tag):
    f = m["flags"]
    if tag == "dl":
        return O.DenseOpts(0.0, m["epsilon"], m["wave"], m["eta"], f["poly"], f["sine"], f["trad_onesided"],
                           f["combo_interior"], f["radius"], *f["center"])
    return O.DenseOpts(m["delta0"], m["epsilon0"], m["wave"], m["eta"], f["poly"], f["sine"], f["combo_onesided"],
                       f["combo_interior"], f["radius"], *f["center"])


@pytest.mark.parametrize("tag,kind", [("dl", 0), ("combo", 1), ("sphere", 2)])
def test_dense_oracle_vs_reference(oracle, dense_case, tag, kind):
    import oracle as O
    g, m, p, grids = dense_case
    o = opts_for(O, m, tag)
    d = None if tag == "sphere" else g["d"]
    rows, pts = oracle.dense_points(kind, p, o, d, None if tag == "sphere" else grids)
    ref = g[tag + "_pts"]
    assert pts.shape == ref.shape
    for name in ROWS_OF[tag]:
        i = O.DENSE_ROWS.index(name)
        if name in EXACT_ROWS:
            assert np.array_equal(pts[i].view(np.uint64), ref[i].view(np.uint64)), name
        else:
            assert rel_err(pts[i], ref[i]) <= 1e-14, name
    K1, K2, regcount = oracle.dense_matrix(kind, p, o, pts)
    K = K1 if tag == "dl" else (K2 if m["flags"]["sine"] else K1)
    assert rel_err(K[g[tag + "_pi"], g[tag + "_pj"]], g[tag + "_entries"]) <= 1e-14
    assert rel_err(K @ g[tag + "_v"], g[tag + "_Kv"]) <= 1e-13
    if tag == "combo":
        assert regcount == m["regcount"]


def test_weight_functions(oracle):
    """PolyWeight / SineWeight vanish outside (tau, 1) and are smooth inside."""
    L = oracle.L
    for w in (L.or_poly_weight, L.or_sine_weight):
        assert w(0.05, 0.1) == 0.0 and w(1.0, 0.1) == 0.0 and w(1.5, 0.1) == 0.0
        t = np.linspace(0.11, 0.99, 200)
        v = np.array([w(x, 0.1) for x in t])
        assert np.all(np.isfinite(v)) and np.max(np.abs(np.diff(v))) < 0.2 * np.max(np.abs(v))
