"""Host <-> device transfers of psi in the complex64 path: from page-locked host memory the
conversion kernels read and write the caller's complex128 array directly (no staging copy); the
result must equal the staged transfer of pageable memory bit for bit (both round complex128 to
complex64 once, and widen back exactly)."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_page_locked_and_pageable_transfers_agree(small_cyclic):
    from cyclix_msparc_gb300.msparc import CyclixGPU
    from cyclix_msparc_gb300.workloads import WORKLOADS, block_layout
    S = small_cyclic
    g = CyclixGPU(S, block_layout(WORKLOADS["cyclic-40x12x20-ns48-m20"], S), "mixed")
    try:
        rng = np.random.default_rng(3)
        X = np.asfortranarray(rng.standard_normal((S.N, 48)) + 1j * rng.standard_normal((S.N, 48)))
        g.set_psi(0, X)
        pageable = g.get_psi(0)
        assert np.array_equal(pageable, X.astype(np.complex64).astype(np.complex128))
        Xp = np.asfortranarray(X.copy())
        out = np.empty_like(Xp, order="F")
        assert g.lib.cx_host_register(Xp.ctypes.data_as(C.c_void_p), Xp.nbytes) == 0
        assert g.lib.cx_host_register(out.ctypes.data_as(C.c_void_p), out.nbytes) == 0
        try:
            from cyclix_msparc_gb300._lib import check, cptr
            check(g.lib, g.h, g.lib.cx_set_psi(g.h, 0, cptr(Xp)))
            check(g.lib, g.h, g.lib.cx_get_psi(g.h, 0, cptr(out)))
        finally:
            g.lib.cx_host_unregister(Xp.ctypes.data_as(C.c_void_p))
            g.lib.cx_host_unregister(out.ctypes.data_as(C.c_void_p))
        assert np.array_equal(out, pageable)
    finally:
        g.close()
