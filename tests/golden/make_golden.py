"""Generate the golden fixtures of this directory with the CPU oracle.

    python tests/golden/make_golden.py            # all fixtures
    python tests/golden/make_golden.py scf_small  # one

The reference is MATLAB and cannot run on these machines, so the fixtures are outputs of the
oracle (``oracle/``), itself pinned by the known-answer tests of ``tests/test_oracle_kat.py``.
They freeze the oracle's answers on seeded inputs so that the GPU tests compare against fixed
numbers and any change of the oracle shows up as a fixture mismatch.

Inputs are regenerated from seeds (``numpy.random.default_rng``, platform independent); only
the outputs are stored.
"""
from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
for p in (ROOT, ROOT / "tests"):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))

from cyclix_msparc_gb300.workloads import WORKLOADS, block_layout, initial_psi, make_system  # noqa: E402
from kat_systems import tiny_cyclic_workload, tiny_helical_workload, xc_density  # noqa: E402
from oracle import cychel_ops as O  # noqa: E402

# filter parameters of the fixtures: degree, cutoff, upper bound, lower bound
FILTER = dict(m=6, cut=8.0, bup=160.0, a0=-6.0)


def seeded_block(N: int, n: int, seed: int) -> np.ndarray:
    rng = np.random.default_rng(seed)
    return np.asfortranarray(rng.standard_normal((N, n)) + 1j * rng.standard_normal((N, n)))


def tiny_cases():
    return {"cyclic": tiny_cyclic_workload(), "helical": tiny_helical_workload()}


def operator_case(name: str) -> dict:
    """H*X and the degree-6 filter of X for every block of a tiny cell, X = seeded_block(N, 2, 21 + b)."""
    wl = tiny_cases()[name]
    S = make_system(wl)
    out = {}
    for b, (k, spin, _) in enumerate(block_layout(wl, S)):
        H = O.Hamiltonian(S, k, S.Veff[:, spin])
        X = seeded_block(S.N, 2, 21 + b)
        out[f"hpsi_{b}"] = H(X)
        out[f"filter_{b}"] = O.chebyshev_filter(X, FILTER["m"], FILTER["cut"], FILTER["bup"], FILTER["a0"], H)
    return out


def eig_case(name: str) -> dict:
    """Three eigSolver steps (count 2..4, npl 6) per block from initial_psi(N, Ns, 31 + b), with the
    bounds a0 = lambda_min - 0.1, bup = 1.01 lambda_max of the dense spectrum and the previous
    eigenvalues of the first step set to the lowest dense ones + 0.5 (cutoff = their max + 0.1)."""
    import scipy.linalg as sla
    wl = tiny_cases()[name]
    S = make_system(wl)
    res = {"blocks": []}
    for b, (k, spin, n) in enumerate(block_layout(wl, S)):
        H = O.Hamiltonian(S, k, S.Veff[:, spin])
        lam = np.sort(np.real(sla.eigvals(H.dense())))
        bounds = (float(lam[0] - 0.1), float(1.01 * lam[-1]), 0.0)
        psi = initial_psi(S.N, n, 31 + b)
        ev0 = lam[:n] + 0.5
        ev = ev0.copy()
        steps = []
        for count in (2, 3, 4):
            psi, ev, bounds = O.eig_solver_block(S, H, psi, count, bounds, ev, rhoTrigger=4)
            steps.append(ev.tolist())
        res["blocks"].append(dict(a0=float(lam[0] - 0.1), bup=float(1.01 * lam[-1]), ev0=ev0.tolist(), steps=steps,
                                  dense_lowest=lam[:n].tolist()))
    return res


def poisson_case() -> dict:
    """AAR Poisson solve (tol 1e-10) on the tiny cyclic cell for f = -4 pi (seeded zero-mean field)."""
    from oracle.scf import PoissonOperator
    S = make_system(tiny_cyclic_workload())
    rng = np.random.default_rng(41)
    rho = rng.standard_normal(S.N)
    rho -= np.sum(rho * S.W) / np.sum(S.W)
    f = -4 * np.pi * rho
    phi, relres, it = PoissonOperator(S).solve(f, None, 1e-10)
    return dict(phi=phi, relres=relres, iters=it)


def xc_case(name: str) -> dict:
    """Vxc and e_xc of LDA_PW, LDA_PZ and GGA_PBE (src/exchangeCorrelationPotential.m, nspin = 1)
    on xc_density(S, 17) of a workload's grid; e_xc per particle at the clipped density."""
    from oracle.scf import XC_RHOTOL, cyclix_gradients, gga_pbe, lda_pw_potential, lda_pz_potential, _pz_corr
    S = make_system(WORKLOADS[name])
    rho = xc_density(S, 17)
    rc = np.where(rho < XC_RHOTOL, XC_RHOTOL, rho)
    out = {}
    out["V_LDA_PW"] = lda_pw_potential(rho)
    rs = (0.75 / (np.pi * rc)) ** (1 / 3)
    A, a1 = 0.031091, 0.21370
    b1, b2, b3, b4 = 7.5957, 3.5876, 1.6382, 0.49294
    ec = -2 * A * (1 + a1 * rs) * np.log(1 + 1 / (2 * A * (b1 * rs ** 0.5 + b2 * rs + b3 * rs ** 1.5 + b4 * rs * rs)))
    C2 = 0.73855876638202
    out["e_LDA_PW"] = ec - C2 * rc ** (1 / 3)
    out["V_LDA_PZ"] = lda_pz_potential(rho)
    out["e_LDA_PZ"] = _pz_corr(rc)[0] - C2 * rc ** (1 / 3)
    V, e = gga_pbe(rho, cyclix_gradients(S))
    out["V_GGA_PBE"], out["e_GGA_PBE"] = V, e
    return out


def scf_small(name: str = "scf-small-24x12x20-12at-2k-ns40", fermi_dirac: bool = False, xc: str = "LDA_PW") -> dict:
    """The oracle SCF (src/scf.m) on a small cell, tol 1e-6, psi = initial_psi(N, Ns, 7 + b);
    Gaussian smearing, or Fermi-Dirac at the same smearing width; exchange-correlation xc."""
    wl = WORKLOADS[name]
    S = make_system(wl)
    if fermi_dirac:
        S.elec_T_type = 0
    S.extra["xc"] = xc
    bl = block_layout(wl, S)
    psis = [initial_psi(S.N, n, 7 + i) for i, (_, _, n) in enumerate(bl)]
    from oracle.scf import scf
    r = scf(S, psis, bl, scf_tol=1e-6)
    return dict(workload=wl.name, smearing="fermi-dirac" if fermi_dirac else "gaussian", xc=xc, scf_tol=1e-6, n_atm=S.n_atm,
                Etotal=r["Etotal"], E_per_atom=r["Etotal"] / S.n_atm,
                lambda_f=r["lambda_f"], n_scf=r["n_scf"], history=[list(h) for h in r["history"]],
                EigVal=[ev.tolist() for ev in r["EigVal"]])


def write_all(which=None):
    jobs = {
        "operators_cyclic": lambda: np.savez_compressed(HERE / "operators_cyclic.npz", **operator_case("cyclic")),
        "operators_helical": lambda: np.savez_compressed(HERE / "operators_helical.npz", **operator_case("helical")),
        "eig_cyclic": lambda: (HERE / "eig_cyclic.json").write_text(json.dumps(eig_case("cyclic"), indent=1)),
        "eig_helical": lambda: (HERE / "eig_helical.json").write_text(json.dumps(eig_case("helical"), indent=1)),
        "poisson_cyclic": lambda: np.savez_compressed(HERE / "poisson_cyclic.npz", **poisson_case()),
        "scf_small": lambda: (HERE / "scf_small.json").write_text(json.dumps(scf_small(), indent=1)),
        "scf_small_helical": lambda: (HERE / "scf_small_helical.json").write_text(
            json.dumps(scf_small("scf-small-helical-24x12x16-8at-2k-ns28"), indent=1)),
        "scf_small_fd": lambda: (HERE / "scf_small_fd.json").write_text(
            json.dumps(scf_small(fermi_dirac=True), indent=1)),
        "scf_small_gga": lambda: (HERE / "scf_small_gga.json").write_text(
            json.dumps(scf_small(xc="GGA_PBE"), indent=1)),
        "scf_small_helical_gga": lambda: (HERE / "scf_small_helical_gga.json").write_text(
            json.dumps(scf_small("scf-small-helical-24x12x16-8at-2k-ns28", xc="GGA_PBE"), indent=1)),
        "scf_small_pz": lambda: (HERE / "scf_small_pz.json").write_text(
            json.dumps(scf_small(xc="LDA_PZ"), indent=1)),
        "xc_cyclic": lambda: np.savez_compressed(HERE / "xc_cyclic.npz", **xc_case("scf-small-24x12x20-12at-2k-ns40")),
        "xc_helical": lambda: np.savez_compressed(HERE / "xc_helical.npz",
                                                  **xc_case("scf-small-helical-24x12x16-8at-2k-ns28")),
    }
    for k, fn in jobs.items():
        if which is None or k in which:
            fn()
            print("wrote", k)


if __name__ == "__main__":
    write_all(sys.argv[1:] or None)
