"""The ctypes mirrors of the C-ABI structs (mbsolve_gb300/capi_types.py)
have the headers' layout: a C program compiled from include/*.h prints
sizeof and offsetof of every field the Python side declares (an unknown
field name fails to compile). CPU only."""
import ctypes as C
import os
import shutil
import subprocess

import pytest

from mbsolve_gb300 import capi_types as T

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
STRUCTS = ["mbg_qm", "mbg_material", "mbg_region", "mbg_device", "mbg_source",
           "mbg_record", "mbg_scenario", "mbg_grid", "mbg_tuning",
           "mbg_gemm_segment", "mbg_gemm_desc", "mbg_fno_layer_desc"]


@pytest.mark.skipif(shutil.which("gcc") is None, reason="no C compiler")
def test_ctypes_layout_matches_headers(tmp_path):
    lines = ["#include <stdio.h>", "#include <stddef.h>",
             '#include "mbsolve_gb300.h"', '#include "mbsolve_fno.h"',
             "int main(void) {"]
    want = {}
    for name in STRUCTS:
        cls = getattr(T, name)
        lines.append('printf("%s %%zu\\n", sizeof(%s));' % (name, name))
        want[name] = C.sizeof(cls)
        for f in cls._fields_:
            key = "%s.%s" % (name, f[0])
            lines.append('printf("%s %%zu\\n", offsetof(%s, %s));'
                         % (key, name, f[0]))
            want[key] = getattr(cls, f[0]).offset
    lines += ["return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c99", "-I", os.path.join(ROOT, "include"),
                    str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True,
                         text=True).stdout
    got = dict((k, int(v)) for k, v in (l.split() for l in out.splitlines()))
    assert got == want
