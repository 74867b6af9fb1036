"""The ctypes mirrors of the C ABI's structures (utr_public_gb300/__init__.py)
against include/msk.h and include/msk_utr.h: gcc compiles a program that
prints sizeof and every field's offsetof, and each must equal the ctypes
layout.  A field added to a header but not to its mirror (or in another
place) shifts every later field the library reads."""
import ctypes as C
import os
import shutil
import subprocess

import pytest

import utr_public_gb300 as msk

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

MIRRORS = [(msk.Series, "msk_series"), (msk.Utr, "msk_utr"), (msk.Stack, "msk_stack"),
           (msk.SpecimenDesc, "msk_specimen"), (msk.Plane, "msk_plane"),
           (msk.KernelStat, "msk_kernel_stat")]


def c_layout(tmp_path):
    lines = ["#include <stddef.h>", "#include <stdio.h>", '#include "msk.h"',
             '#include "msk_utr.h"', "int main(void) {"]
    for cls, cname in MIRRORS:
        lines.append('printf("%s sizeof %%zu\\n", sizeof(%s));' % (cname, cname))
        for f in cls._fields_:
            lines.append('printf("%s %s %%zu\\n", offsetof(%s, %s));'
                         % (cname, f[0], cname, f[0]))
    lines += ["return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c99", "-I", os.path.join(ROOT, "include"), str(src), "-o",
                    str(exe)], check=True, capture_output=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    return {(a, b): int(c) for a, b, c in (l.split() for l in out.splitlines())}


@pytest.mark.skipif(shutil.which("gcc") is None, reason="needs gcc")
def test_ctypes_mirrors_match_headers(tmp_path):
    lay = c_layout(tmp_path)
    for cls, cname in MIRRORS:
        assert C.sizeof(cls) == lay[(cname, "sizeof")], cname
        for f in cls._fields_:
            assert getattr(cls, f[0]).offset == lay[(cname, f[0])], (cname, f[0])


def test_plane_arrays():
    off, arr, total = msk._plane_arrays([[(1, 2, 3, 4)], [], [(5, 6, 7, 8), (9, 10, 11, 12)]], 3)
    assert list(off) == [0, 1, 1, 3] and total == 3
    assert [(p.defocus, p.rotation, p.astig, p.astig_angle) for p in arr] == \
        [(1, 2, 3, 4), (5, 6, 7, 8), (9, 10, 11, 12)]
