"""The ctypes mirrors of the C-ABI structs have the header's layout: a C
program built from include/ves2d_gb300.h prints sizeof and offsetof of every
field, compared with the ctypes classes of ves2dpy_gb300._native (no GPU)."""
import ctypes
import os
import shutil
import subprocess

import pytest

from ves2dpy_gb300 import _native as nat

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

STRUCTS = {
    "ves_near_lists": nat.NearLists,
    "ves_step_params": nat.StepParams,
    "ves_step_result": nat.StepResult,
    "ves_net_block": nat.NetBlock,
    "ves_mlarm_norms": nat.MlarmNorms,
    "ves_mlarm_params": nat.MlarmParams,
    "ves_mlarm_result": nat.MlarmResult,
    "ves_mlarm_trace": nat.MlarmTrace,
    "ves_stats": nat.Stats,
}


def _c_layout(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "ves2d_gb300.h"', "int main(void) {"]
    for cname, cls in STRUCTS.items():
        lines.append(f'  printf("{cname} sizeof %zu\\n", sizeof({cname}));')
        for fname, _ in cls._fields_:
            lines.append(f'  printf("{cname} {fname} %zu\\n", offsetof({cname}, {fname}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run([cc, "-std=c99", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True,
                   capture_output=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    table = {}
    for line in out.splitlines():
        cname, field, value = line.split()
        table[(cname, field)] = int(value)
    return table


def test_ctypes_structs_match_the_header(tmp_path):
    table = _c_layout(tmp_path)
    for cname, cls in STRUCTS.items():
        assert ctypes.sizeof(cls) == table[(cname, "sizeof")], (cname, ctypes.sizeof(cls), table[(cname, "sizeof")])
        for fname, _ in cls._fields_:
            assert getattr(cls, fname).offset == table[(cname, fname)], (cname, fname)
