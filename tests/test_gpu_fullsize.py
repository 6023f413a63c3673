"""The benchmark's full size: the torus R = 0.6, r = 0.25 on 256^3 over
[-1,1]^3, tube 3h (n = 581,420), k = 20, and the ellipsoid (0.7, 0.5, 0.4)
on 256^3 at k = 20 and k = 40.

* The grid stages equal the reference's on the torus: the reference build
  ran ASSIGN_GRADIENT, the BothCurvs loop, the tube selection and the
  per-point set-up at 256^3 (tests/golden/make_golden.py), and its outputs
  are pinned by SHA-256 digests: WENO gradient and curvature grids, tube
  index list, x*, normals, Jacobian and regularisation factor bit for bit;
  delta and w (they hold cos()) to 1e-15 on a strided sample.
* The tube index list is the lexicographic list of nodes with
  |phi| <= 3h, bit for bit (the reference's rule, large3Dexample2.c:548-597;
  at 256^3 h and 3h are exact binary fractions, so numpy's comparison is
  the same comparison).
* The FP32 product is within 1e-6 (relative 2-norm) of the FP64 product on
  the torus (k = 20) and on the reinitialised ellipsoid (k = 20, 40), with
  the phase passed to the SFU directly and split-k reduced.
* The FP32 fused sweep is linear: A(p + 2i q) = A p + 2i A q to FP32
  rounding (2e-6 of the norms).
* The fused sweep's two products are adjoint: <A p, w> = <p, A^H w> to
  FP32 rounding (1e-5 relative).
"""
import hashlib
import json
import os

import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu

N, K = 256, 20.0


@pytest.fixture(scope="module")
def full(hz):
    from helmholtz_3d_torrone_gb300 import geometry as G
    d = G.torus(N, R=0.6, r=0.25, int_l=-1.0, int_u=1.0)
    p = hz.params(N, K, int_l=-1.0, int_u=1.0, factor=3.0, tau_factor=2.0, dirichlet=1)
    op = hz.Operator(p)
    op.set_distance(d)
    op.build()
    yield op, d
    op.close()


def test_tube_index_list_full_size(full):
    op, d = full
    eps = 3.0 * (2.0 / N)
    expect = np.flatnonzero(np.abs(d).ravel() <= eps)
    assert op.n == expect.size == 581420
    assert np.array_equal(op.tube()["idx"], expect)


def test_fp32_sweep_linear_and_adjoint_full_size(hz, full):
    op, d = full
    rng = np.random.default_rng(256)
    p = rng.standard_normal(op.n) + 1j * rng.standard_normal(op.n)
    q = rng.standard_normal(op.n) + 1j * rng.standard_normal(op.n)
    w = rng.standard_normal(op.n) + 1j * rng.standard_normal(op.n)
    Ap, AHw = op.matvec_pair(p, w, precision=hz.PREC_F32)
    Aq = op.matvec(q, precision=hz.PREC_F32)
    Apq = op.matvec(p + 2j * q, precision=hz.PREC_F32)
    scale = np.linalg.norm(Ap) + 2 * np.linalg.norm(Aq)
    assert np.linalg.norm(Apq - (Ap + 2j * Aq)) <= 2e-6 * scale
    lhs, rhs = np.vdot(w, Ap), np.vdot(AHw, p)
    assert abs(lhs - rhs) <= 1e-5 * max(abs(lhs), np.linalg.norm(Ap) * np.linalg.norm(w) * 1e-3)


def _sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def test_grid_stages_match_reference_digests_full_size(full):
    op, d = full
    g = golden("ref_dirichlet_torus_n256_digest")
    m = json.loads(str(g["meta"]))
    sha = m["sha256"]
    assert _sha(d) == sha["d"], "the regenerated torus distance grid differs from the reference run's input"
    for name, arr in zip(("gx", "gy", "gz", "mc", "gc"), op.grids()):
        assert _sha(arr) == sha[name], name
    t = op.tube()
    assert op.n == m["n"]
    assert _sha(t["idx"].astype(np.int64)) == sha["idx"]
    for name in ("xs", "nrm", "jac", "reg"):
        assert _sha(t[name]) == sha[name], name
    st = m["stride"]
    for name in ("delta", "w"):
        ref = g[name]
        assert np.max(np.abs(t[name][::st] - ref)) <= 1e-15 * np.max(np.abs(ref)), name


def _product_errors(hz, op, seed):
    rng = np.random.default_rng(seed)
    v = rng.standard_normal(op.n) + 1j * rng.standard_normal(op.n)
    q64 = op.matvec(v, precision=hz.PREC_F64)
    out = {}
    for mode, name in ((hz.PHASE_DIRECT, "direct"), (hz.PHASE_SPLIT, "split")):
        op.set_phase_mode(mode)
        q32 = op.matvec(v, precision=hz.PREC_F32)
        out[name] = float(np.linalg.norm(q32 - q64) / np.linalg.norm(q64))
        out[name + "_max"] = float(np.max(np.abs(q32 - q64)) / np.max(np.abs(q64)))
    op.set_phase_mode(hz.PHASE_SPLIT)  # back to the default
    return out


def _record(key, value):
    """Append a measured figure to the JSON file named by HZ_TEST_RECORD, if set."""
    path = os.environ.get("HZ_TEST_RECORD")
    if not path:
        return
    data = json.load(open(path)) if os.path.exists(path) else {}
    data[key] = value
    json.dump(data, open(path, "w"), indent=1)


def test_fp32_vs_fp64_product_torus_full_size(hz, full):
    op, d = full
    err = _product_errors(hz, op, 20)
    _record("fp32_vs_fp64_torus256_k20", err)
    assert err["direct"] < 1e-6 and err["split"] < 1e-6, err


@pytest.mark.parametrize("wave", [20.0, 40.0])
def test_fp32_vs_fp64_product_ellipsoid_full_size(hz, wave):
    from helmholtz_3d_torrone_gb300 import geometry as G
    H = 2.0 / N
    d = hz.reinitialize(G.ellipsoid_levelset(N), N, H, 60)
    p = hz.params(N, wave, int_l=-1.0, int_u=1.0, factor=3.0, tau_factor=2.0, dirichlet=1)
    with hz.Operator(p) as op:
        op.set_distance(d)
        op.build()
        err = _product_errors(hz, op, int(wave))
    _record("fp32_vs_fp64_ellipsoid256_k%d" % int(wave), dict(err, n=op.n))
    assert err["direct"] < 1e-6 and err["split"] < 1e-6, err
