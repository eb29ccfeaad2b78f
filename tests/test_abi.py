"""The C-ABI library builds for sm_103a, loads, and exports every function ``include/cyclix_gpu.h``
declares (no compute call is made: this runs without a GPU)."""
import ctypes
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
HEADER = ROOT / "include" / "cyclix_gpu.h"


def declared_functions():
    text = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?[a-z_0-9]+\s*\**\s+(cx_[a-z_0-9]+)\s*\(", text, flags=re.M)
    return sorted(set(names))


@pytest.fixture(scope="module")
def lib():
    from cyclix_msparc_gb300 import _lib
    return _lib.load(build_if_missing=True)


def test_header_declares_entry_points():
    names = declared_functions()
    for must in ("cx_create", "cx_destroy", "cx_hpsi", "cx_chebyshev_filter", "cx_eigsolver", "cx_poisson", "cx_scf",
                 "cx_hpsi_noalloc", "cx_last_error"):
        assert must in names


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_covers_header(lib):
    from cyclix_msparc_gb300 import _lib
    assert sorted(_lib.EXPORTS) == declared_functions()


def test_version_string(lib):
    assert lib.cx_version().decode().startswith("cyclix_gpu")


def test_null_handle_is_rejected(lib):
    # argument checks run before any CUDA call
    assert lib.cx_hpsi(None, 0, 1, None, None, 0) == 1      # CX_ERR_ARG
    assert lib.cx_eigsolver(None, 1, 4, 4, None, None, None, None) == 1
    assert lib.cx_destroy(None) == 0
