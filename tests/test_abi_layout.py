"""The ctypes mirrors of the C-ABI's structs (mambatracer_gb300/_lib.py) have the
sizes and field offsets that include/mambatracer.h gives them: a C program built
against the header prints them. Needs gcc, no GPU."""
import ctypes as C
import os
import shutil
import subprocess

import pytest

from mambatracer_gb300 import _lib

HEADER_DIR = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include")
MIRRORS = {
    "mt_render_config": _lib.RenderConfig,
    "mt_batch_frame": _lib.BatchFrame,
    "mt_server_config": _lib.ServerConfig,
    "mt_tuning": _lib.Tuning,
    "mt_served_stats": _lib.ServedStats,
}


def test_struct_layouts_match_the_header(tmp_path):
    if not shutil.which("gcc"):
        pytest.skip("gcc not found")
    lines = ['#include <stddef.h>', '#include <stdio.h>', '#include "mambatracer.h"', "int main(void) {"]
    for cname, py in MIRRORS.items():
        lines.append(f'  printf("{cname} size %zu\\n", sizeof({cname}));')
        for field, _ in py._fields_:
            lines.append(f'  printf("{cname} {field} %zu\\n", offsetof({cname}, {field}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c11", "-I", HEADER_DIR, str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    got = {tuple(l.split()[:2]): int(l.split()[2]) for l in out if l}
    for cname, py in MIRRORS.items():
        assert got[(cname, "size")] == C.sizeof(py), cname
        for field, _ in py._fields_:
            assert got[(cname, field)] == getattr(py, field).offset, (cname, field)
