"""The ctypes structures of the Python host against the C-ABI header: size and field offsets of
every struct in include/cyclix_gpu.h, computed by the C compiler (gcc, sizeof / offsetof) and by
ctypes.  A mismatch would pass garbage parameters to the library without any error."""
import ctypes as C
import shutil
import subprocess
from pathlib import Path

import pytest

from cyclix_msparc_gb300 import _lib

ROOT = Path(__file__).resolve().parents[1]
STRUCTS = ["cx_grid", "cx_rc_image", "cx_atom", "cx_block", "cx_eig_params", "cx_scf_params", "cx_scf_result",
           "cx_scf_step_info"]


@pytest.fixture(scope="module")
def c_layout(tmp_path_factory):
    if shutil.which("gcc") is None:
        pytest.skip("gcc not available")
    d = tmp_path_factory.mktemp("abi")
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "cyclix_gpu.h"', "int main(void) {"]
    for s in STRUCTS:
        py = getattr(_lib, s)
        lines.append(f'  printf("{s} size %zu\\n", sizeof({s}));')
        for name, _ in py._fields_:
            lines.append(f'  printf("{s} {name} %zu\\n", offsetof({s}, {name}));')
    lines += ["  return 0;", "}"]
    src = d / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = d / "layout"
    subprocess.run(["gcc", "-std=c11", "-I", str(ROOT / "include"), str(src), "-o", str(exe)], check=True,
                   capture_output=True, text=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    table = {}
    for ln in out.splitlines():
        s, key, val = ln.split()
        table[(s, key)] = int(val)
    return table


@pytest.mark.parametrize("name", STRUCTS)
def test_struct_layout_matches_header(c_layout, name):
    py = getattr(_lib, name)
    assert C.sizeof(py) == c_layout[(name, "size")], (name, C.sizeof(py), c_layout[(name, "size")])
    for field, _ in py._fields_:
        assert getattr(py, field).offset == c_layout[(name, field)], (name, field)
