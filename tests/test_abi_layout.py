"""The ctypes mirror of every public struct in include/mhdproj.h has the C
layout: a C program compiled against the header prints each struct's size
and every field's offset, and the Python structures must agree (no GPU)."""
import ctypes as C
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PAIRS = {
    "mhdproj_grid": "Grid",
    "mhdproj_options": "Options",
    "mhdproj_stats": "Stats",
    "mhdproj_diagnostics": "Diagnostics",
    "mhdproj_step_params": "StepParams",
    "mhdproj_kernel_time": "KernelTime",
    "mhdproj_em_config": "EmConfig",
    "mhdproj_em_diagnostics": "EmDiagnostics",
}


def _c_layout(tmp_path, mhdproj):
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "mhdproj.h"', 'int main(void) {']
    for cname, pyname in PAIRS.items():
        py = getattr(mhdproj, pyname)
        lines.append(f'    printf("{cname} size %zu\\n", sizeof({cname}));')
        for field, _ in py._fields_:
            lines.append(f'    printf("{cname} {field} %zu\\n", offsetof({cname}, {field}));')
    lines += ['    return 0;', '}']
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run([shutil.which("gcc") or "gcc", "-std=c11", "-I", os.path.join(ROOT, "include"), str(src), "-o",
                    str(exe)], check=True, capture_output=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    return {tuple(line.split()[:2]): int(line.split()[2]) for line in out.splitlines()}


@pytest.mark.skipif(shutil.which("gcc") is None, reason="needs gcc")
def test_ctypes_structs_match_the_header(tmp_path):
    import mhdproj

    layout = _c_layout(tmp_path, mhdproj)
    for cname, pyname in PAIRS.items():
        py = getattr(mhdproj, pyname)
        assert layout[(cname, "size")] == C.sizeof(py), cname
        for field, _ in py._fields_:
            assert layout[(cname, field)] == getattr(py, field).offset, (cname, field)
