"""GPU against the committed golden fixtures (oracle outputs on seeded inputs), through the C-ABI.

Tolerances:
  * H*psi and the degree-6 filter: max |GPU - golden| / max |golden| <= 1e-12 (complex128),
    <= 2e-6 (complex64);
  * three eigSolver steps (count 2..4): <= 1e-9 Ha per eigenvalue (complex128);
  * Poisson (AAR, tol 1e-10): the GPU potential agrees with the golden one to 1e-8 relative.
"""
import json
from pathlib import Path

import numpy as np
import pytest

import golden.make_golden as G
from cyclix_msparc_gb300.workloads import block_layout, initial_psi, make_system

pytestmark = pytest.mark.gpu
GOLD = Path(__file__).resolve().parent / "golden"


def _gpu(name, prec):
    from cyclix_msparc_gb300.msparc import CyclixGPU
    wl = G.tiny_cases()[name]
    S = make_system(wl)
    bl = block_layout(wl, S)
    return S, bl, CyclixGPU(S, bl, prec)


@pytest.mark.parametrize("prec,tol", [("fp64", 1e-12), ("mixed", 2e-6)])
@pytest.mark.parametrize("name", ["cyclic", "helical"])
def test_operators_vs_golden(name, prec, tol):
    ref = np.load(GOLD / f"operators_{name}.npz")
    S, bl, g = _gpu(name, prec)
    try:
        for b in range(len(bl)):
            X = G.seeded_block(S.N, 2, 21 + b)
            Y = g.hpsi(b, X)
            assert np.max(np.abs(Y - ref[f"hpsi_{b}"])) <= tol * np.max(np.abs(ref[f"hpsi_{b}"]))
            F = G.FILTER
            Y = g.filter(b, X, F["m"], F["cut"], F["bup"], F["a0"])
            assert np.max(np.abs(Y - ref[f"filter_{b}"])) <= tol * np.max(np.abs(ref[f"filter_{b}"]))
    finally:
        g.close()


@pytest.mark.parametrize("name", ["cyclic", "helical"])
def test_eigsolver_vs_golden(name):
    ref = json.loads((GOLD / f"eig_{name}.json").read_text())
    S, bl, g = _gpu(name, "fp64")
    S.npl = 6
    try:
        nb = len(bl)
        for b, (_, _, n) in enumerate(bl):
            g.set_psi(b, initial_psi(S.N, n, 31 + b))
        EV = np.concatenate([np.array(rb["ev0"]) for rb in ref["blocks"]])
        a0 = np.array([rb["a0"] for rb in ref["blocks"]])
        bup = np.array([rb["bup"] for rb in ref["blocks"]])
        lc = np.zeros(nb)
        for step, count in enumerate((2, 3, 4)):
            g.eigsolve(count, 6, EV, a0, bup, lc)
            off = 0
            for b, (_, _, n) in enumerate(bl):
                want = np.array(ref["blocks"][b]["steps"][step])
                assert np.max(np.abs(EV[off:off + n] - want)) < 1e-9, (b, count)
                off += n
    finally:
        g.close()


def test_poisson_vs_golden():
    ref = np.load(GOLD / "poisson_cyclic.npz")
    S, bl, g = _gpu("cyclic", "fp64")
    try:
        rng = np.random.default_rng(41)
        rho = rng.standard_normal(S.N)
        rho -= np.sum(rho * S.W) / np.sum(S.W)
        phi, it, rr, ok = g.poisson(-4 * np.pi * rho, None, 1e-10, 1000)
        assert ok and rr <= 1e-10
        assert np.max(np.abs(phi - ref["phi"])) <= 1e-8 * np.max(np.abs(ref["phi"]))
    finally:
        g.close()
