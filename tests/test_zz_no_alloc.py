"""The allocation-free FP64 product hz_matvec_f64_noalloc, called through the
C ABI, against the operator's own FP64 product hz_matvec.

It exists for callers that cannot allocate device memory when they need a
product (memory handed out by the application's own pools, plugin hosts that
forbid allocation after start-up, loops that cannot take cudaMalloc's
implicit synchronisation); its scratch is a fixed __device__ array.  This
file is collected last so a run that stops at its first failure has run
every other test before it.  Tolerance: 1e-12 relative, as for the other
FP64 product tests.
"""
import ctypes as C
import json

import numpy as np
import pytest

from conftest import golden, rel_err

pytestmark = pytest.mark.gpu


def test_noalloc_matches_operator_product_twice(hz):
    torch = pytest.importorskip("torch")
    g = golden("ref_dirichlet_sphere_n20")
    m = json.loads(str(g["meta"]))
    p = hz.params(m["N"], m["wave"], int_l=m["int_l"], int_u=m["int_u"], factor=m["factor"],
                  tau_factor=m["tau_factor"], dirichlet=m["dirichlet"], interior=m["interior"])
    L = hz.load()
    with hz.Operator(p) as op:
        op.set_distance(g["d"])
        n = op.build()
        t = op.tube()
        dev = torch.device("cuda", 0)

        def to_dev(a):
            return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).to(dev)

        xs, nrm, reg, w = to_dev(t["xs"].ravel()), to_dev(t["nrm"].ravel()), to_dev(t["reg"]), to_dev(t["w"])
        rng = np.random.default_rng(11)
        for call in range(2):  # two calls in a row share (and must fully rewrite) the static scratch
            v = rng.standard_normal(n) + 1j * rng.standard_normal(n)
            for adjoint in (0, 1):
                expect = op.matvec(v, precision=hz.PREC_F64, adjoint=bool(adjoint))
                pr, pi = to_dev(v.real), to_dev(v.imag)
                qr = torch.empty(n, dtype=torch.float64, device=dev)
                qi = torch.empty(n, dtype=torch.float64, device=dev)
                torch.cuda.synchronize()
                rc = L.hz_matvec_f64_noalloc(C.byref(p), n, adjoint, xs.data_ptr(), nrm.data_ptr(), reg.data_ptr(),
                                             w.data_ptr(), pr.data_ptr(), pi.data_ptr(), qr.data_ptr(),
                                             qi.data_ptr(), None)
                assert rc == 0, L.hz_last_error().decode()
                got = qr.cpu().numpy() + 1j * qi.cpu().numpy()
                assert rel_err(got, expect) < 1e-12, (call, adjoint)
        # sizes beyond the static scratch are refused before any GPU work
        rc = L.hz_matvec_f64_noalloc(C.byref(p), hz.NOALLOC_MAX_POINTS + 1, 0, xs.data_ptr(), nrm.data_ptr(),
                                     reg.data_ptr(), w.data_ptr(), pr.data_ptr(), pi.data_ptr(), qr.data_ptr(),
                                     qi.data_ptr(), None)
        assert rc == -1
        assert b"static scratch" in L.hz_last_error()
