"""The ctypes structures of lokigpu.capi against include/loki_gpu.h.

The C ABI passes plain structs by pointer; a field added to the header but not
to the binding (or in another order) would shift every later field silently.
A small C program compiled against the header prints each struct's size and
every field's offset, and the ctypes classes must agree field by field.
"""
import ctypes
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

# C struct name -> capi class name
STRUCTS = {
    "lgpu_config": "Config",
    "lgpu_process": "Process",
    "lgpu_gas": "Gas",
    "lgpu_conditions": "Conditions",
    "lgpu_result": "Result",
    "lgpu_step_report": "StepReport",
    "lgpu_timing": "Timing",
    "lgpu_batch_report": "BatchReport",
    "lgpu_job": "Job",
    "lgpu_job_status": "JobStatus",
    "lgpu_server_report": "ServerReport",
}


def _c_layout(tmp_path, capi):
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "loki_gpu.h"', "int main(void) {"]
    for cname, pyname in STRUCTS.items():
        cls = getattr(capi, pyname)
        lines.append(f'  printf("{cname} size %zu\\n", sizeof({cname}));')
        for field in cls._fields_:
            f = field[0]
            lines.append(f'  printf("{cname} {f} %zu\\n", offsetof({cname}, {f}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.check_call(["gcc", "-std=c11", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)])
    out = subprocess.check_output([str(exe)], text=True)
    layout = {}
    for line in out.splitlines():
        cname, what, value = line.split()
        layout[(cname, what)] = int(value)
    return layout


@pytest.mark.skipif(shutil.which("gcc") is None, reason="needs gcc")
def test_ctypes_structures_match_header(tmp_path):
    from lokigpu import capi

    layout = _c_layout(tmp_path, capi)
    mismatches = []
    for cname, pyname in STRUCTS.items():
        cls = getattr(capi, pyname)
        if ctypes.sizeof(cls) != layout[(cname, "size")]:
            mismatches.append(f"{cname}: size {layout[(cname, 'size')]} in C, {ctypes.sizeof(cls)} in ctypes")
        for field in cls._fields_:
            f = field[0]
            off = getattr(cls, f).offset
            if off != layout[(cname, f)]:
                mismatches.append(f"{cname}.{f}: offset {layout[(cname, f)]} in C, {off} in ctypes")
    assert not mismatches, "\n".join(mismatches)
