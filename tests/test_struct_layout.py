"""The ctypes mirrors of the C ABI's structures (helmholtz_3d_torrone_gb300)
have the layout the C compiler gives the declarations in include/*.h: size
and every field's offset, checked by compiling a small C program against
the headers (CPU only)."""
import ctypes as C
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CASES = {
    "hz_params": ("Params", "helmholtz_gb300.h"),
    "hz_solve_opts": ("SolveOpts", "helmholtz_gb300.h"),
    "hz_solve_info": ("SolveInfo", "helmholtz_gb300.h"),
    "hz_dense_opts": ("DenseOpts", "helmholtz_gb300.h"),
    "hz_ref_config": ("RefConfig", "helmholtz_ref_api.h"),
}


def test_struct_layouts_match_headers(hz, tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "helmholtz_gb300.h"',
             '#include "helmholtz_ref_api.h"', "int main(void) {"]
    for cname, (pyname, _) in CASES.items():
        cls = getattr(hz, pyname)
        lines.append('printf("%s size %%zu\\n", sizeof(%s));' % (cname, cname))
        for f, _ in cls._fields_:
            lines.append('printf("%s.%s %%zu\\n", offsetof(%s, %s));' % (cname, f, cname, f))
    lines += ["return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run([cc, "-x", "c++" if cc.endswith("g++") else "c", "-I", os.path.join(ROOT, "include"), str(src),
                    "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")
    got = dict(l.rsplit(" ", 1) for l in out if l)
    for cname, (pyname, _) in CASES.items():
        cls = getattr(hz, pyname)
        assert int(got[cname + " size"]) == C.sizeof(cls), cname
        for f, _ in cls._fields_:
            assert int(got["%s.%s" % (cname, f)]) == getattr(cls, f).offset, (cname, f)
