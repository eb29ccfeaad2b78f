"""cx_hpsi_noalloc: H*psi on caller-owned device buffers with no device allocation.

Callers whose device memory belongs to another allocator (a framework's caching allocator,
a MEX session that must leave nothing allocated) cannot let the library call cudaMalloc; this
entry point uses a fixed device array of the library for its projector scratch instead.  The
test owns the device buffers (allocated through PyTorch, as such a caller would) and checks two
calls in a row against the allocating entry point cx_hpsi, with the H*psi tolerances used by
the other GPU tests (1e-12 relative for complex128, 2e-6 for complex64), and that the second call
leaves the device's free memory unchanged.  This file is collected
last so that a run that stops at the first failure has already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _rand(N, n, seed):
    rng = np.random.default_rng(seed)
    return np.asfortranarray(rng.standard_normal((N, n)) + 1j * rng.standard_normal((N, n)))


def _to_device(torch, X, prec):
    # column-major complex block -> contiguous interleaved device buffer of the precision
    flat = np.ascontiguousarray(X.reshape(-1, order="F"))
    host = flat.view(np.float64) if prec == "fp64" else flat.astype(np.complex64).view(np.float32)
    return torch.from_numpy(host.copy()).cuda()


def _from_device(Yd, N, n, prec):
    a = Yd.cpu().numpy()
    c = a.view(np.complex128) if prec == "fp64" else a.view(np.complex64).astype(np.complex128)
    return c.reshape((N, n), order="F")


@pytest.mark.parametrize("prec,tol", [("fp64", 1e-12), ("mixed", 2e-6)])
def test_hpsi_noalloc_matches_hpsi(small_cyclic, prec, tol):
    torch = pytest.importorskip("torch")
    from cyclix_msparc_gb300 import _lib
    from cyclix_msparc_gb300.msparc import CyclixGPU
    from cyclix_msparc_gb300.workloads import block_layout, WORKLOADS
    S = small_cyclic
    g = CyclixGPU(S, block_layout(WORKLOADS["cyclic-40x12x20-ns48-m20"], S), prec)
    try:
        for call, ncol in enumerate((6, 3)):                      # two calls in a row
            X = _rand(S.N, ncol, 40 + call)
            ref = g.hpsi(0, X, prec)
            Xd = _to_device(torch, X, prec)
            Yd = torch.empty_like(Xd)
            torch.cuda.synchronize()
            free0 = torch.cuda.mem_get_info()[0]
            st = g.lib.cx_hpsi_noalloc(g.h, 0, ncol, C.c_void_p(Xd.data_ptr()), C.c_void_p(Yd.data_ptr()), _lib.PREC[prec])
            assert st == _lib.CX_OK, g.lib.cx_last_error(g.h).decode()
            torch.cuda.synchronize()
            if call == 1:
                # the second call (its kernels were loaded by the first) leaves the free device memory unchanged
                assert torch.cuda.mem_get_info()[0] == free0
            got = _from_device(Yd, S.N, ncol, prec)
            err = np.max(np.abs(got - ref)) / np.max(np.abs(ref))
            assert err < tol, (call, err)
    finally:
        g.close()


def test_hpsi_noalloc_rejects_oversized_calls(small_cyclic):
    torch = pytest.importorskip("torch")
    from cyclix_msparc_gb300 import _lib
    from cyclix_msparc_gb300.msparc import CyclixGPU
    from cyclix_msparc_gb300.workloads import block_layout, WORKLOADS
    S = small_cyclic
    g = CyclixGPU(S, block_layout(WORKLOADS["cyclic-40x12x20-ns48-m20"], S), "fp64")
    try:
        x = torch.zeros(2, dtype=torch.float64, device="cuda")
        y = torch.zeros(2, dtype=torch.float64, device="cuda")
        # 60000 columns need far more than the fixed scratch: refused on the host, nothing launched
        st = g.lib.cx_hpsi_noalloc(g.h, 0, 60000, C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()), _lib.CX_PREC_FP64)
        assert st == _lib.CX_ERR_ARG
        assert b"static scratch" in g.lib.cx_last_error(g.h)
    finally:
        g.close()
