"""GPU against the oracle at the full sizes of the benchmarked workloads.

The oracle's H*psi and Chebyshev filter are vectorised sparse products, so a few columns at the
full grids take seconds on the CPU.  For the scaled-up cyclic cell (96 x 24 x 64), the batched
cell (16 nu blocks, 64 x 16 x 48), the helical cell (80 x 32 x 40, eta / nu / spin blocks) and the
384-atom SCF cell (128 x 48 x 96, two theta tiles with TMA halos), three columns of the first,
middle and last Bloch block (with the workload's Bloch vector and spin) go through the C-ABI
and through the oracle (src/h_nonlocal_vector_mult.m:1-43, src/chebyshev_filter.m:24-42):
  * H*psi: max |GPU - oracle| / max |oracle| <= 1e-12 (complex128), <= 2e-6 (complex64);
  * degree-6 Chebyshev filter: <= 1e-11 (complex128), <= 1e-5 (complex64);
  * linearity of H*psi: H(a x + b y) = a H x + b H y to 1e-12 relative (complex128);
  * the batched eigensolver (16 Bloch blocks of uneven Ns) gives the same lowest eigenvalues in
    mixed precision as in FP64 after two steps from a random start: <= 1e-3 Ha on the lowest half
    of each block (the two trajectories are not converged yet; converged results are compared
    through the SCF energy).
"""
import numpy as np
import pytest

from cyclix_msparc_gb300.workloads import WORKLOADS, block_layout, initial_psi, make_system
from oracle import cychel_ops as O

pytestmark = pytest.mark.gpu

CASES = {
    "cyclic-96x24x64-ns256-m24": "one block, theta tile of 24 rows, 77 atoms",
    "cyclic-batched-16nu-64x16x48-ns96to320-m24": "one theta tile of 16 rows, 16 nu blocks",
    "helical-80x32x40-96k2s-ns192-m24": "helical, 32 theta rows in one tile (3 rows per thread), eta / nu / spin blocks",
    "scf-128x48x96-384at-8k-ns1024": "two theta tiles of 24 rows with TMA halos, 384 atoms",
}


def _rand(N, n, seed):
    rng = np.random.default_rng(seed)
    return np.asfortranarray(rng.standard_normal((N, n)) + 1j * rng.standard_normal((N, n)))


def _relerr(a, b):
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


@pytest.fixture(scope="module", params=list(CASES))
def fullsize(request):
    wl = WORKLOADS[request.param]
    S = make_system(wl)
    if S.Veff is None:
        # the SCF workload carries no potential: use the initial electrostatics-like field
        S.Veff = np.repeat((-S.rho_at)[:, None], S.nspin, axis=1)
    bl = block_layout(wl, S)
    pick = sorted({0, len(bl) // 2, len(bl) - 1})
    blocks = [(bl[i][0], bl[i][1], 4) for i in pick]
    return wl, S, blocks


def test_fullsize_matches_oracle(fullsize):
    from cyclix_msparc_gb300.msparc import CyclixGPU
    wl, S, blocks = fullsize
    g64 = CyclixGPU(S, blocks, "fp64")
    g32 = CyclixGPU(S, blocks, "mixed")
    try:
        for b, (k, spin, _) in enumerate(blocks):
            H = O.Hamiltonian(S, k, S.Veff[:, spin])
            X = _rand(S.N, 3, 100 + b)
            ref = H(X)
            assert _relerr(g64.hpsi(b, X), ref) <= 1e-12, (wl.name, b)
            assert _relerr(g32.hpsi(b, X), ref) <= 2e-6, (wl.name, b)
            fref = O.chebyshev_filter(X, 6, 10.0, 3000.0, -5.0, H)
            assert _relerr(g64.filter(b, X, 6, 10.0, 3000.0, -5.0), fref) <= 1e-11, (wl.name, b)
            assert _relerr(g32.filter(b, X, 6, 10.0, 3000.0, -5.0), fref) <= 1e-5, (wl.name, b)
        # linearity (complex128)
        x, y = _rand(S.N, 1, 7), _rand(S.N, 1, 8)
        a, c = 0.3 - 1.1j, 2.0 + 0.5j
        lhs = g64.hpsi(0, a * x + c * y)
        rhs = a * g64.hpsi(0, x) + c * g64.hpsi(0, y)
        assert np.max(np.abs(lhs - rhs)) <= 1e-12 * np.max(np.abs(rhs))
    finally:
        g64.close()
        g32.close()


def test_fullsize_batched_eigensolver_mixed_vs_fp64():
    from cyclix_msparc_gb300.msparc import CyclixGPU
    wl = WORKLOADS["cyclic-batched-16nu-64x16x48-ns96to320-m24"]
    S = make_system(wl)
    bl = block_layout(wl, S)
    nblk = len(bl)
    out = {}
    for prec in ("fp64", "mixed"):
        g = CyclixGPU(S, bl, prec)
        try:
            for b, (_, _, n) in enumerate(bl):
                g.set_psi(b, initial_psi(S.N, n, 500 + b))
            EV = np.zeros(sum(n for (_, _, n) in bl))
            a0, bup, lc = np.zeros(nblk), np.zeros(nblk), np.zeros(nblk)
            for count in (1, 2):
                g.eigsolve(count, wl.npl, EV, a0, bup, lc)
            out[prec] = EV.copy()
        finally:
            g.close()
    off = 0
    for (_, _, n) in bl:
        lo = n // 2
        err = np.max(np.abs(out["mixed"][off:off + lo] - out["fp64"][off:off + lo]))
        assert err <= 1e-3, (n, err)
        off += n
