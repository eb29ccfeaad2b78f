"""GPU exchange-correlation potential (cx_xc, src/exchangeCorrelationPotential.m, nspin = 1) against
the oracle fixtures tests/golden/xc_*.npz: LDA_PW, LDA_PZ and GGA_PBE on the 24 x 12 x 20 cyclic
and 24 x 12 x 16 helical (twist 0.05 rad/bohr) grids, on a seeded density with 1 % of its points at
or below the 1e-14 clip.

Tolerance: Vxc and e_xc within 1e-11 of the fixture, relative to the field's largest magnitude
(FP64 throughout; the oracle sums its sparse gradient products in another order)."""
from pathlib import Path

import numpy as np
import pytest

from cyclix_msparc_gb300.workloads import WORKLOADS, block_layout, make_system
from kat_systems import xc_density

pytestmark = pytest.mark.gpu
GOLD = Path(__file__).resolve().parent / "golden"
GRIDS = [("scf-small-24x12x20-12at-2k-ns40", "xc_cyclic.npz"), ("scf-small-helical-24x12x16-8at-2k-ns28", "xc_helical.npz")]


@pytest.fixture(scope="module", params=GRIDS, ids=["cyclic", "helical"])
def grid(request):
    from cyclix_msparc_gb300.msparc import CyclixGPU
    name, fixture = request.param
    wl = WORKLOADS[name]
    S = make_system(wl)
    g = CyclixGPU(S, block_layout(wl, S), "fp64")
    yield S, g, np.load(GOLD / fixture)
    g.close()


@pytest.mark.parametrize("xc", ["LDA_PW", "LDA_PZ", "GGA_PBE"])
def test_xc_matches_oracle(grid, xc):
    S, g, ref = grid
    rho = xc_density(S, 17)
    V, e = g.xc(rho, xc)
    Vr, er = ref["V_" + xc], ref["e_" + xc]
    assert np.max(np.abs(V - Vr)) < 1e-11 * np.max(np.abs(Vr))
    assert np.max(np.abs(e - er)) < 1e-11 * np.max(np.abs(er))


def test_exchange_correlation_wrapper(grid):
    """The MATLAB-named wrapper sets S.Vxc and S.e_xc from S.rho for S's functional."""
    from cyclix_msparc_gb300 import msparc
    S, g, ref = grid
    S.gpu = g
    S.rho = xc_density(S, 17)
    S.extra["xc"] = "GGA_PBE"
    try:
        msparc.exchangeCorrelationPotential(S)
    finally:
        S.extra.pop("xc")
    assert np.max(np.abs(S.Vxc - ref["V_GGA_PBE"])) < 1e-11 * np.max(np.abs(ref["V_GGA_PBE"]))


def test_xc_rejects_unknown_functional(grid):
    """An unknown functional is refused by the wrapper and, as a code, by the library (no CUDA work)."""
    from cyclix_msparc_gb300 import _lib
    S, g, _ = grid
    with pytest.raises(_lib.CxError):
        g.xc(np.ones(S.N), "GGA_RPBE")
    rho, V, e = np.ones(S.N), np.zeros(S.N), np.zeros(S.N)
    assert g.lib.cx_xc(g.h, 5, _lib.dptr(rho), _lib.dptr(V), _lib.dptr(e)) == _lib.CX_ERR_ARG
