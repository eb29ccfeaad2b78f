"""Write the set-up of two of the reference's own Cyclix decks as compact fixtures, so that the
GPU SCF can be checked against the free energy the reference printed for them on a machine that
does not hold the reference tree.

For each deck the psp8 set-up of ``cyclix_msparc_gb300.deck.load_deck`` (grid, quadrature weights,
pseudocharges b, atomic density guess, self and correction energy, Bloch points and weights, the
psp8 projectors in the S.Atom(J).rcImage layout) is saved as ``deck_<name>.npz`` next to this
script, with the free energy per atom of the deck's ``.out`` file and the tolerances of its run.
Nothing of the reference's files is copied: the arrays are this library's set-up of the deck.

    CYCLIX_REFERENCE=<reference project root> python tests/golden/make_deck_fixtures.py [name ...]
    python tests/golden/make_deck_fixtures.py --oracle GGA_wrong_SG15   # tight oracle SCF of a saved deck
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [ROOT, os.path.join(ROOT, "tests")]

DECKS = {"CNT_chiral": "tests/Cyclix/CNT_chiral/C.inpt", "CNT_ABINITmatch": "tests/Cyclix/CNT_ABINITmatch/C.inpt",
         "GGA_wrong_SG15": "GGA_wrong_SG15/C.inpt"}


def save(name, rel, root):
    from cyclix_msparc_gb300.deck import load_deck
    from golden.pin_decks import out_values, ran_with
    inpt = os.path.join(root, rel)
    d = load_deck(inpt, overrides=ran_with(inpt))
    S = d.S
    ref = out_values(os.path.splitext(inpt)[0] + ".out")
    arrays = dict(
        grid=np.array([S.Nx, S.Ny, S.Nz, S.FDn, S.cell_typ, S.BCx, S.BCy, S.BCz], dtype=np.int64),
        geom=np.array([S.dx, S.dy, S.dz, S.xin, S.twist, S.L1, S.L2, S.L3]),
        w1=S.w1, w2=S.w2, W=S.W, Atoms=S.Atoms, kptgrid=S.kptgrid, wkpt=S.wkpt,
        b=S.b, rho_at=S.rho_at,
        scalars=np.array([S.Nev, S.npl, S.NegCharge, S.Eself, S.E_corr, S.bet, S.elec_T_type, S.occfac, S.n_atm,
                          d.scf_tol, d.poisson_tol, ref["free_energy_per_atom"]]),
        atom_angnum=np.array([A.angnum for A in S.Atom], dtype=np.int64),
        atom_gamma=np.concatenate([A.gamma_Jl for A in S.Atom]),
        atom_nimg=np.array([A.n_image_rc for A in S.Atom], dtype=np.int64),
        img_coords=np.array([img.coordinates for A in S.Atom for img in A.rcImage]),
        img_nnodes=np.array([img.rc_pos.size for A in S.Atom for img in A.rcImage], dtype=np.int64),
        img_pos=np.concatenate([img.rc_pos for A in S.Atom for img in A.rcImage]).astype(np.int32),
        img_chi=np.concatenate([img.Chi_mat.reshape(-1, order="F") for A in S.Atom for img in A.rcImage]),
        xc=np.array(S.extra.get("xc", "LDA_PW")),
        # the local-potential part of the set-up, for the force tests: per atom type the valence
        # charge, the psp8 radial grid with its local potential and isolated-atom density, and the
        # pseudocharge box half-widths; per atom its type
        atom_type=np.asarray(S.extra["atom_type"], dtype=np.int64),
        psp_Z=np.array([P.Z for P in d.psps]), rb=np.array([list(r) for r in d.rb]),
        **{f"psp{t}_{k}": getattr(P, k) for t, P in enumerate(d.psps) for k in ("r", "Vloc", "rho_iso")},
    )
    path = os.path.join(HERE, f"deck_{name}.npz")
    np.savez_compressed(path, **arrays)
    print(f"{name}: N = {S.N}, {S.tnkpt} Bloch points, Nev {S.Nev}, npl {S.npl}; printed free energy "
          f"{ref['free_energy_per_atom']:.10f} Ha/atom -> {path} ({os.path.getsize(path) / 1e6:.2f} MB)")


def load(name):
    """Rebuild the CyclixS of a saved deck: (S, scf_tol, poisson_tol, printed free energy per atom)."""
    from cyclix_msparc_gb300.cychel import AtomNL, CyclixS, RcImage
    z = np.load(os.path.join(HERE, f"deck_{name}.npz"))
    Nx, Ny, Nz, FDn, cell_typ, BCx, BCy, BCz = (int(v) for v in z["grid"])
    dx, dy, dz, xin, twist, L1, L2, L3 = (float(v) for v in z["geom"])
    Nev, npl, NegCharge, Eself, E_corr, bet, elec_T_type, occfac, n_atm, scf_tol, poisson_tol, e_ref = z["scalars"]
    S = CyclixS(Nx=Nx, Ny=Ny, Nz=Nz, FDn=FDn, cell_typ=cell_typ, BCx=BCx, BCy=BCy, BCz=BCz, dx=dx, dy=dy, dz=dz, xin=xin,
                twist=twist, L1=L1, L2=L2, L3=L3, w1=z["w1"], w2=z["w2"], W=z["W"], Atoms=z["Atoms"], Atom=[],
                kptgrid=z["kptgrid"], wkpt=z["wkpt"], nspin=1, Nev=int(Nev), npl=int(npl))
    atoms, gi, ii, ni, ci = [], 0, 0, 0, 0
    for J in range(len(z["atom_angnum"])):
        ang = int(z["atom_angnum"][J])
        imgs = []
        for _ in range(int(z["atom_nimg"][J])):
            nn = int(z["img_nnodes"][ii])
            pos = z["img_pos"][ni:ni + nn].astype(np.int64)
            chi = z["img_chi"][ci:ci + nn * ang].reshape((nn, ang), order="F")
            imgs.append(RcImage(z["img_coords"][ii].copy(), pos, chi))
            ii += 1
            ni += nn
            ci += nn * ang
        atoms.append(AtomNL(ang, z["atom_gamma"][gi:gi + ang].copy(), imgs))
        gi += ang
    S.Atom = atoms
    S.b, S.rho_at = z["b"], z["rho_at"]
    S.NegCharge, S.Eself, S.E_corr, S.bet = float(NegCharge), float(Eself), float(E_corr), float(bet)
    S.elec_T_type, S.occfac, S.n_atm = int(elec_T_type), float(occfac), int(n_atm)
    S.extra.update(deck=name, xc=str(z["xc"]) if "xc" in z.files else "LDA_PW")
    return S, float(scf_tol), float(poisson_tol), float(e_ref)


def load_force_deck(name):
    """A deck object for the force code (``forces.local_force_setup``, oracle/forces.py) rebuilt from a
    saved set-up that holds the local-potential tables: S, psps (valence charge, radial grid, local
    potential, isolated-atom density per type), rb, and the pseudocharge set-up (b, b_ref, V_c, ...)
    recomputed from them.  Returns (deck, scf_tol, poisson_tol, printed free energy per atom)."""
    from types import SimpleNamespace
    from cyclix_msparc_gb300.deck import pseudocharges
    S, scf_tol, poisson_tol, e_ref = load(name)
    z = np.load(os.path.join(HERE, f"deck_{name}.npz"))
    psps = [SimpleNamespace(Z=float(Z), r=z[f"psp{t}_r"], Vloc=z[f"psp{t}_Vloc"], rho_iso=z[f"psp{t}_rho_iso"])
            for t, Z in enumerate(z["psp_Z"])]
    rb = [tuple(float(v) for v in r) for r in z["rb"]]
    S.extra["atom_type"] = z["atom_type"].astype(int)
    pc = pseudocharges(S, psps, S.extra["atom_type"], rb)
    return SimpleNamespace(S=S, psps=psps, rb=rb, pseudo=pc), scf_tol, poisson_tol, e_ref


def oracle_reference(name, scf_tol=1e-8, poisson_tol=1e-10, max_scf=60):
    """The oracle SCF (oracle/scf.py) on the saved set-up of a deck, from the initial psi the GPU
    deck tests use (initial_psi(N, Nev, 700 + b)), converged tightly so that the fixed point does not
    depend on the Poisson solver's stopping point; written to deck_<name>_oracle.json."""
    import json
    import time
    from cyclix_msparc_gb300.workloads import initial_psi
    from oracle.scf import scf
    S, _, _, e_ref = load(name)
    blocks = [(S.kptgrid[k].copy(), 0, S.Nev) for k in range(S.tnkpt)]
    psis = [initial_psi(S.N, S.Nev, 700 + b) for b in range(len(blocks))]
    t = time.time()
    r = scf(S, psis, blocks, scf_tol=scf_tol, poisson_tol=poisson_tol, max_scf=max_scf,
            log=lambda c, e, err: print(f"{name} oracle SCF {c}: {e:.12f} Ha/atom, error {err:.3e}", flush=True))
    out = dict(deck=name, xc=S.extra["xc"], scf_tol=scf_tol, poisson_tol=poisson_tol, n_scf=r["n_scf"],
               free_energy_per_atom=r["Etotal"] / S.n_atm, lambda_f=r["lambda_f"], printed_free_energy_per_atom=e_ref,
               history=[list(h) for h in r["history"]], wall_s=round(time.time() - t, 1))
    path = os.path.join(HERE, f"deck_{name}_oracle.json")
    with open(path, "w") as f:
        json.dump(out, f, indent=1)
    print(f"{name}: oracle {out['free_energy_per_atom']:.12f} Ha/atom after {out['n_scf']} steps -> {path}")


if __name__ == "__main__":
    args = [a for a in sys.argv[1:] if not a.startswith("--")]
    if "--oracle" in sys.argv:
        for name in args:
            oracle_reference(name)
        sys.exit(0)
    root = os.environ.get("CYCLIX_REFERENCE", "")
    if not root:
        sys.exit("set CYCLIX_REFERENCE to the reference project root")
    for name, rel in DECKS.items():
        if not args or name in args:
            save(name, rel, root)
