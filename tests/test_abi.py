"""The C-ABI library loads and exports every entry point declared in include/*.h
(no compute: runs without a GPU)."""
import os
import re
import subprocess

import pytest

from conftest import ROOT


def declared(header, extern_c_only=True):
    text = open(os.path.join(ROOT, "include", header)).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    text = re.sub(r"//[^\n]*", "", text)
    names = re.findall(r"\b([A-Za-z_]\w*)\s*\(", text)
    skip = {"if", "for", "while", "return", "sizeof", "defined"}
    return sorted({n for n in names if n not in skip and not n.isupper() or n.startswith("hz_")})


def exported(lib):
    out = subprocess.run(["nm", "-D", "--defined-only", lib], capture_output=True, text=True, check=True).stdout
    return {line.split()[-1] for line in out.splitlines() if line.strip()}


def test_c_abi_symbols_exported(hz):
    names = [n for n in declared("helmholtz_gb300.h") if n.startswith("hz_")]
    assert len(names) >= 20
    syms = exported(hz.LIB_PATH)
    missing = [n for n in names if n not in syms]
    assert not missing, missing
    # and ctypes sees the same set with signatures
    for n in names:
        assert n in hz.SIGNATURES, n


def test_reference_compat_symbols_exported(hz):
    hdr = os.path.join(ROOT, "include", "helmholtz_ref_api.h")
    if not os.path.exists(hdr):
        pytest.skip("no reference-compatibility header")
    syms = exported(hz.LIB_PATH)
    demangled = subprocess.run(["nm", "-DC", "--defined-only", hz.LIB_PATH], capture_output=True, text=True,
                               check=True).stdout
    text = open(hdr).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    text = re.sub(r"//[^\n]*", "", text)
    funcs = re.findall(r"^\s*(?:HZ_API\s+)?(?:int|void|double)\s+([A-Za-z_]\w*)\s*\(", text, flags=re.M)
    assert funcs
    for f in funcs:
        assert re.search(r"\b%s\(" % re.escape(f), demangled) or f in syms, f
    # link compatibility: the mangled names equal those of the reference's own
    # objects (built by oracle/build_ref.py from the reference sources)
    objdir = os.path.join(ROOT, "oracle", "_ref", "obj_neumann")
    if os.path.isdir(objdir):
        ref_syms = set()
        for o in os.listdir(objdir):
            out = subprocess.run(["nm", "--defined-only", os.path.join(objdir, o)], capture_output=True, text=True,
                                 check=True).stdout
            ref_syms |= {line.split()[-1] for line in out.splitlines() if line.strip()}
        for f in funcs:
            if f.startswith("hz_"):  # extern "C" helpers of the drop-ins
                assert f in syms, f
                continue
            ours = [s for s in syms if re.fullmatch(r"_Z%d%s\w+" % (len(f), re.escape(f)), s)]
            assert ours, f
            if any(re.fullmatch(r"_Z%d%s\w+" % (len(f), re.escape(f)), s) for s in ref_syms):
                assert set(ours) <= ref_syms, (f, ours)


def test_errors_without_device(hz):
    """Without a GPU the library reports an error instead of falling back."""
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    p = hz.params(16, 2.0)
    with pytest.raises(hz.HzError) as e:
        hz.Operator(p)
    assert e.value.code == -2


def test_bad_params_rejected(hz):
    p = hz.params(4, 2.0)  # N below the supported minimum
    with pytest.raises(hz.HzError) as e:
        hz.Operator(p)
    assert e.value.code == -1


def test_null_handles_and_bad_arguments(hz):
    """The C entry points answer a NULL handle or a bad argument with
    HZ_ERR_ARG and a message, before touching a device (the reference would
    exit(0) or read out of bounds)."""
    import ctypes as C
    L = hz.load()
    opts = hz.solve_opts()
    info = hz.SolveInfo()
    cases = {
        "hz_set_phase_mode": lambda: L.hz_set_phase_mode(None, hz.PHASE_SPLIT),
        "hz_set_combo": lambda: L.hz_set_combo(None, None),
        "hz_matvec_multi": lambda: L.hz_matvec_multi(None, hz.PREC_F32, 1, None, None, None, None, hz.HZ_HOST),
        "hz_solve_multi": lambda: L.hz_solve_multi(None, C.byref(opts), 1, None, None, None, None, hz.HZ_HOST,
                                                   C.byref(info), None),
        "hz_batch_create": lambda: L.hz_batch_create(None, 0, C.byref(C.c_void_p())),
        "hz_batch_solve": lambda: L.hz_batch_solve(None, C.byref(opts), None, None, None, None, hz.HZ_HOST,
                                                   C.byref(info), None),
        "hz_residual_history": lambda: L.hz_residual_history(None, None, 0, C.byref(C.c_int())),
    }
    for name, call in cases.items():
        rc = call()
        assert rc == -1, (name, rc)
        assert L.hz_last_error().decode(), name
