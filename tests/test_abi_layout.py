"""The Python mirror's structures have the C header's layout (no GPU needed).

A small C program built against include/ifluids.h prints sizeof and the
offsetof of every field the ctypes mirror declares; the mirror must agree on
each, so a field added to one side only (or reordered) fails here instead of
corrupting arguments at run time."""
import ctypes as C
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PAIRS = [("Params", "ifl_params"), ("Timing", "ifl_timing"), ("_CBody", "ifl_body"),
         ("PcgStats", "ifl_pcg_stats"), ("StepStats", "ifl_step_stats"), ("Inflow", "ifl_inflow"),
         ("BatchOptions", "ifl_batch_options"), ("BatchInfo", "ifl_batch_info"),
         ("ServerParams", "ifl_server_params"), ("Request", "ifl_request"), ("Completion", "ifl_completion"),
         ("ServerInfo", "ifl_server_info")]


def test_ctypes_mirror_matches_the_header(ifl, tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "ifluids.h"', "int main(void) {"]
    for py, c in PAIRS:
        lines.append(f'printf("{py} size %zu\\n", sizeof({c}));')
        for f in getattr(ifl, py)._fields_:
            lines.append(f'printf("{py} {f[0]} %zu\\n", offsetof({c}, {f[0]}));')
    lines.append("return 0; }")
    src, exe = tmp_path / "layout.c", tmp_path / "layout"
    src.write_text("\n".join(lines))
    subprocess.run([cc, "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    seen = 0
    for line in out.splitlines():
        py, field, value = line.split()
        cls = getattr(ifl, py)
        got = C.sizeof(cls) if field == "size" else getattr(cls, field).offset
        assert got == int(value), (py, field, got, int(value))
        seen += 1
    assert seen > len(PAIRS) * 2
