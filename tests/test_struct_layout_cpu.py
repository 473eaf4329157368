"""The argument blocks of the C ABI (include/magic_sht.h) against their
ctypes mirrors in magic_gb300._lib: a small C program compiled with the host
compiler prints sizeof and the offset of every field the mirror names; each
must agree (a field added to one side only shifts every later pointer)."""
import ctypes
import os
import shutil
import subprocess

import pytest

from magic_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

MIRRORS = {
    "magic_sht_desc": _lib.Desc,
    "magic_sht_grid_space_args": _lib.GridSpaceArgs,
    "magic_sht_lm_space_args": _lib.LmSpaceArgs,
    "magic_sht_tuning": _lib.Tuning,
    "magic_sht_nl_opts": _lib.NlOpts,
    "magic_sht_nl_grids": _lib.NlGrids,
    "magic_sht_nl_out": _lib.NlOut,
    "magic_sht_td_args": _lib.TdArgs,
    "magic_sht_td_opts": _lib.TdOpts,
    "magic_sht_td_in": _lib.TdIn,
    "magic_sht_td_out": _lib.TdOut,
    "magic_sht_courant_args": _lib.CourantArgs,
    "magic_sht_rigid_args": _lib.RigidArgs,
    "magic_sht_job": _lib.Job,
}


def test_ctypes_mirrors_match_the_header(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no host C compiler")
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "magic_sht.h"', "int main(void) {"]
    for cname, py in MIRRORS.items():
        lines.append('printf("%s sizeof %%zu\\n", sizeof(%s));' % (cname, cname))
        for f, _ in py._fields_:
            lines.append('printf("%s %s %%zu\\n", offsetof(%s, %s));' % (cname, f, cname, f))
    lines += ["return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run([cc, "-std=c11", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    got = {}
    for line in subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.splitlines():
        c, f, v = line.split()
        got[(c, f)] = int(v)
    for cname, py in MIRRORS.items():
        assert got[(cname, "sizeof")] == ctypes.sizeof(py), cname
        for f, _ in py._fields_:
            assert got[(cname, f)] == getattr(py, f).offset, (cname, f)
