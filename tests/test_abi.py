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


def _grid(**kw):
    import numpy as np
    from cyclix_msparc_gb300 import _lib
    from cyclix_msparc_gb300.cychel import fd_weights
    w1, w2 = fd_weights(6)
    keep = [np.ascontiguousarray(w1), np.ascontiguousarray(w2), np.ones(16 * 8 * 10)]
    args = dict(Nx=16, Ny=8, Nz=10, FDn=6, cell_typ=3, BCx=1, BCy=0, BCz=0, dx=0.25, dy=0.06, dz=0.2, xin=4.0, twist=0.0,
                L1=3.75, L2=0.52, L3=2.0)
    args.update(kw)
    g = _lib.cx_grid(**args)
    g.w1 = _lib.dptr(keep[0])
    g.w2 = _lib.dptr(keep[1])
    g.W = _lib.dptr(keep[2])
    return g, keep


@pytest.mark.parametrize("bad,msg", [
    (dict(FDn=0), "FDn"),
    (dict(cell_typ=2), "cell_typ"),
    (dict(BCx=0), "Dirichlet"),
    (dict(Ny=6), "Ny, Nz > FDn"),
    (dict(cell_typ=5, twist=0.0), "twist"),
])
def test_create_rejects_bad_grids_without_cuda(lib, bad, msg):
    # argument checks come before any CUDA call, so they run on a machine without a GPU
    import ctypes as C
    g, keep = _grid(**bad)
    h = C.c_void_p()
    st = lib.cx_create(C.byref(g), 0, None, 1, C.byref(h))
    assert st == 1 and not h.value
    assert msg in lib.cx_last_error(None).decode()


def test_create_rejects_bad_spin_and_atoms(lib):
    import ctypes as C
    g, keep = _grid()
    h = C.c_void_p()
    assert lib.cx_create(C.byref(g), 0, None, 3, C.byref(h)) == 1
    assert "nspin" in lib.cx_last_error(None).decode()
    assert lib.cx_create(C.byref(g), 2, None, 1, C.byref(h)) == 1
    assert "atoms" in lib.cx_last_error(None).decode()
    assert lib.cx_create(None, 0, None, 1, C.byref(h)) == 1


def test_create_rejects_more_projector_columns_than_the_kernels_hold(lib):
    # a psp8 atom with two projectors per l (l <= 1) has 8 columns; the kernels hold 4
    import ctypes as C
    import numpy as np
    from cyclix_msparc_gb300 import _lib as L
    g, keep = _grid()
    gam = np.ones(8)
    atoms = (L.cx_atom * 1)()
    atoms[0].angnum = 8
    atoms[0].n_image_rc = 0
    atoms[0].gamma_Jl = gam.ctypes.data_as(C.POINTER(C.c_double))
    h = C.c_void_p()
    assert lib.cx_create(C.byref(g), 1, atoms, 1, C.byref(h)) == 1
    msg = lib.cx_last_error(None).decode()
    assert "angnum must be 0..4" in msg and "got 8" in msg
