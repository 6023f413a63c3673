"""The CPU oracle against golden vectors produced by the reference's own C code
(tests/golden/make_golden.py).  This pins the oracle: every GPU parity test
compares against it."""
import json

import numpy as np
import pytest

from conftest import golden, rel_err

CASES = ["ref_neumann_sphere_n16", "ref_neumann_sphere_n24", "ref_dirichlet_sphere_n20",
         "ref_dirichlet_torus_n32"]


def params_of(g):
    import oracle as O
    m = json.loads(str(g["meta"]))
    return O.Params(m["N"], m["int_l"], m["int_u"], m["wave"], m["factor"], m["tau_factor"], m["dirichlet"],
                    m["interior"]), m


@pytest.mark.parametrize("case", CASES)
def test_grids_tube_points_bitexact(oracle, case):
    g = golden(case)
    p, m = params_of(g)
    tp = oracle.pipeline(p, g["d"])
    for key, ours in [("gx", tp["grads"][0]), ("gy", tp["grads"][1]), ("gz", tp["grads"][2]), ("mc", tp["mc"]),
                      ("gc", tp["gc"])]:
        assert np.array_equal(ours.view(np.uint64), g[key].view(np.uint64)), key
    assert np.array_equal(tp["idx"], g["idx"])
    assert tp["bad"] == 0
    for key in ["xs", "nrm", "delta", "jac", "reg", "w"]:
        assert np.array_equal(tp[key], g[key]), key


@pytest.mark.parametrize("case", CASES)
def test_entries_and_products(oracle, case):
    g = golden(case)
    p, m = params_of(g)
    tp = {k: g[k] for k in ["xs", "nrm", "reg", "w"]}
    n = m["n"]
    import ctypes as C
    re, im = C.c_double(), C.c_double()
    ent = []
    for a, b in zip(g["pi"], g["pj"]):
        oracle.L.or_entry(C.byref(p), tp["xs"].ctypes.data_as(C.POINTER(C.c_double)),
                          tp["nrm"].ctypes.data_as(C.POINTER(C.c_double)),
                          tp["reg"].ctypes.data_as(C.POINTER(C.c_double)),
                          tp["w"].ctypes.data_as(C.POINTER(C.c_double)), int(a), int(b), C.byref(re), C.byref(im))
        ent.append(re.value + 1j * im.value)
    assert np.array_equal(np.array(ent), g["entries"])
    q = oracle.matvec(p, tp, g["p"])
    qh = oracle.matvec(p, tp, g["p"], adjoint=True)
    # numpy's dense product and the oracle's sequential sums differ in order only
    assert rel_err(q, g["Ap"]) < 1e-13
    assert rel_err(qh, g["AHp"]) < 1e-13
    assert n == len(g["w"])


@pytest.mark.parametrize("case", CASES)
def test_bicg_matches_reference_compbicg(oracle, case):
    g = golden(case)
    p, m = params_of(g)
    tp = {k: g[k] for k in ["xs", "nrm", "reg", "w"]}
    b = oracle.rhs(p, tp, np.zeros(3), m["rhs_kind"])
    assert np.array_equal(b, g["b"])
    x, it, res = oracle.bicg(p, tp, b, acc=1e-13)
    assert res < 1e-12
    assert rel_err(x, g["x"]) < 1e-10


def test_weno_bitexact(oracle):
    g = golden("ref_neumann_sphere_n16")
    fi = g["weno_in"]
    out = [oracle.weno(f, 0.1, 5) for f in fi] + [oracle.weno(f[:5], 0.1, 3) for f in fi]
    assert np.array_equal(np.array(out), g["weno_out"])


def test_godunov_bitexact(oracle):
    """The oracle's Godunov upwind |grad phi| (the reinitialisation's
    Hamiltonian) equals the reference's finite_difference3D.c:5-27 bit for
    bit on the seeded fixture (zeros, both signs, signage -1 / 0 / +1)."""
    g = golden("ref_godunov")
    out = np.array([oracle.godunov(s, *row) for s, row in zip(g["signage"], g["derivs"])])
    assert np.array_equal(out, g["out"])
    assert np.count_nonzero(g["out"]) > 0.5 * g["out"].size
