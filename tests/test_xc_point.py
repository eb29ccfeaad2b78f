"""The exchange-correlation arithmetic of the GPU kernels, compiled for the host, against the oracle.

``cyclix_msparc_gb300/csrc/cx_xc_point.h`` holds the per-point code that the SCF kernels run
(LDA_PW, LDA_PZ, the PBE energy with its dual-number derivatives, and the two GGA passes over the
Cyclix gradient stencils).  Compiled by g++ into a small shared library, it must reproduce:
  * the oracle's point functions (oracle/scf.py: lda_pw_potential, lda_pz_potential, _pbe_parts)
    on densities from 1e-14 to 30 and reduced gradients over 32 decades;
  * the oracle's Vxc and e_xc fixtures (tests/golden/xc_*.npz, src/exchangeCorrelationPotential.m)
    on the 24 x 12 x 20 cyclic and 24 x 12 x 16 helical grids, clipped points included.
Tolerances: relative 1e-12 on values; df/dsigma, a difference of exchange and correlation terms
that cancel, absolutely 1e-15 on its natural scale rho^(-4/3); Vxc and e_xc 1e-11 relative to
their largest magnitude (the oracle sums the sparse-matrix products in another order)."""
import ctypes as C
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

from cyclix_msparc_gb300.workloads import WORKLOADS, make_system
from kat_systems import xc_density

ROOT = Path(__file__).resolve().parents[1]
GOLD = Path(__file__).resolve().parent / "golden"

SHIM = r"""
#include "cx_xc_point.h"
using namespace cx::xc;
extern "C" {
void pw(const double* r, int n, double* v, double* e) { for (int i = 0; i < n; ++i) lda_pw(r[i], v[i], e[i]); }
void pz(const double* r, int n, double* v, double* e) { for (int i = 0; i < n; ++i) lda_pz(r[i], v[i], e[i]); }
void pbe_pts(const double* r, const double* s, int n, double* f, double* fr, double* fs) {
  for (int i = 0; i < n; ++i) pbe(r[i], s[i], f[i], fr[i], fs[i]);
}
void gga(const double* rho, const int* dims, const double* geo, const double* w1, double* vxc, double* erho, double* q) {
  GgaGrid g{};
  g.Nx = dims[0]; g.Ny = dims[1]; g.Nz = dims[2]; g.FDn = dims[3];
  g.xin = geo[0]; g.dx = geo[1]; g.dy = geo[2]; g.dz = geo[3]; g.twist = geo[4];
  for (int k = 1; k <= g.FDn; ++k) { g.gr[k] = w1[k] / g.dx; g.gt[k] = w1[k] / g.dy; g.gz[k] = w1[k] / g.dz; }
  const int N = g.Nx * g.Ny * g.Nz;
  for (int p = 0; p < N; ++p) gga_pass1_point(rho, g, p, vxc, erho, q);
  for (int p = 0; p < N; ++p) gga_pass2_point(q, g, p, vxc);
}
}
"""


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    d = tmp_path_factory.mktemp("xc")
    (d / "shim.cpp").write_text(SHIM)
    so = d / "shim.so"
    subprocess.run(["g++", "-O2", "-std=c++17", "-shared", "-fPIC", "-I", str(ROOT / "cyclix_msparc_gb300" / "csrc"),
                    str(d / "shim.cpp"), "-o", str(so)], check=True, capture_output=True, text=True)
    return C.CDLL(str(so))


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def _points(n=20000, seed=1):
    rng = np.random.default_rng(seed)
    rho = np.concatenate([10 ** rng.uniform(-14, 1.5, n), [1e-14, 1.0, 0.5]])
    sig = np.concatenate([10 ** rng.uniform(-30, 2, n), [0.0, 0.0, 1e-3]]) * rho ** (8 / 3) * 10 ** rng.uniform(-2, 2, n + 3)
    return rho, sig


def test_lda_point_functions_match_oracle(lib):
    from oracle.scf import lda_pw_potential, lda_pz_energy, lda_pz_potential
    rho, _ = _points()
    n = rho.size
    v, e = np.zeros(n), np.zeros(n)
    lib.pw(_p(rho), n, _p(v), _p(e))
    vo = lda_pw_potential(rho)
    assert np.max(np.abs(v - vo) / np.abs(vo)) < 1e-12
    lib.pz(_p(rho), n, _p(v), _p(e))
    vo = lda_pz_potential(rho)
    assert np.max(np.abs(v - vo) / np.abs(vo)) < 1e-12
    eo = np.array([lda_pz_energy(np.array([r]), np.array([1.0])) for r in rho[:2000]])
    assert np.max(np.abs(e[:2000] - eo) / np.abs(eo)) < 1e-12


def test_pbe_point_function_and_derivatives_match_oracle(lib):
    from oracle.scf import _pbe_parts
    rho, sig = _points()
    n = rho.size
    f, fr, fs = np.zeros(n), np.zeros(n), np.zeros(n)
    lib.pbe_pts(_p(rho), _p(sig), n, _p(f), _p(fr), _p(fs))
    fo, fro, fso = _pbe_parts(rho, sig)
    assert np.max(np.abs(f - fo) / np.abs(fo)) < 1e-12
    assert np.max(np.abs(fr - fro) / np.abs(fro)) < 1e-12
    assert np.max(np.abs(fs - fso) / rho ** (-4 / 3)) < 1e-15


@pytest.mark.parametrize("name,fixture", [("scf-small-24x12x20-12at-2k-ns40", "xc_cyclic.npz"),
                                          ("scf-small-helical-24x12x16-8at-2k-ns28", "xc_helical.npz")],
                         ids=["cyclic", "helical"])
def test_gga_passes_match_oracle_fixture(lib, name, fixture):
    """Both GGA passes of the GPU kernels over a whole grid: Vxc and e_xc = f / rho_c."""
    S = make_system(WORKLOADS[name])
    rho = xc_density(S, 17)
    ref = np.load(GOLD / fixture)
    N = S.N
    dims = np.array([S.Nx, S.Ny, S.Nz, S.FDn], dtype=np.int32)
    geo = np.array([S.xin, S.dx, S.dy, S.dz, S.twist], dtype=np.float64)
    w1 = np.ascontiguousarray(S.w1, dtype=np.float64)
    vxc, erho, q = np.zeros(N), np.zeros(N), np.zeros(3 * N)
    lib.gga(_p(rho), _p(dims), _p(geo), _p(w1), _p(vxc), _p(erho), _p(q))
    rc = np.maximum(rho, 1e-14)
    V, e = ref["V_GGA_PBE"], ref["e_GGA_PBE"]
    assert np.max(np.abs(vxc - V)) < 1e-11 * np.max(np.abs(V))
    assert np.max(np.abs(erho / rc - e)) < 1e-11 * np.max(np.abs(e))
