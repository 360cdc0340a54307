"""The C ABI header is plain C, and the ctypes mirror in _native.py has its layout.

Compiles a small C program against include/gnlse.h with the host C compiler and
compares sizeof / offsetof of every descriptor field with the ctypes structures
(no GPU, no CUDA headers: gnlse.h includes only stdint.h)."""

import ctypes as ct
import os
import shutil
import subprocess

import pytest

from pyofsschanged_gb300 import _native as nat

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
STRUCTS = {"gnlse_grid_desc": nat.GridDesc, "gnlse_instance_desc": nat.InstanceDesc,
           "gnlse_stats": nat.Stats}

pytestmark = pytest.mark.skipif(shutil.which("gcc") is None, reason="no host C compiler")


@pytest.mark.parametrize("header", ["gnlse.h", "sno.h"])
def test_headers_are_plain_c(header):
    subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", "-fsyntax-only", "-x", "c",
                    os.path.join(ROOT, "include", header)], check=True)


def test_ctypes_layout_matches_header(tmp_path):
    lines = ['#include <stddef.h>', '#include <stdio.h>', '#include "gnlse.h"', "int main(void) {"]
    for cname, py in STRUCTS.items():
        lines.append(f'  printf("{cname} sizeof %zu\\n", sizeof({cname}));')
        for field, _ in py._fields_:
            lines.append(f'  printf("{cname} {field} %zu\\n", offsetof({cname}, {field}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c99", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)],
                   check=True)
    got = {}
    for ln in subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.splitlines():
        cname, field, value = ln.split()
        got[(cname, field)] = int(value)
    for cname, py in STRUCTS.items():
        assert got[(cname, "sizeof")] == ct.sizeof(py), cname
        for field, _ in py._fields_:
            assert got[(cname, field)] == getattr(py, field).offset, (cname, field)
