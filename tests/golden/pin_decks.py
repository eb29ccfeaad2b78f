"""Pin the oracle end to end on the reference's own Cyclix decks.

For each deck, the reference's input files (.inpt, .ion, .psp8) are loaded by
``cyclix_msparc_gb300.deck`` and the oracle SCF (oracle/scf.py) runs from the atomic density
guess.  The free energy per atom, the self and correction energy and the pseudocharge radii are
compared with the numbers the reference printed into the deck's .out file, and, where the deck's
.static file holds them, the drift-free atomic forces (oracle/forces.py).  The result is
written to ``deck_pins.json`` next to this script; tests/test_decks.py checks the record and
re-derives the fast quantities (radii, self and correction energy) from the deck files.

Run from the repository root, where the reference tree is readable:

    python tests/golden/pin_decks.py [deck ...]        # default: LDA_CNT/C.inpt
    python tests/golden/pin_decks.py tests/Cyclix/CNT_chiral/C.inpt     # helical, Fermi-Dirac

Decks are paths relative to the reference project root, taken from ``--root DIR`` or the
CYCLIX_REFERENCE environment variable.  A deck takes ~1 min per SCF step on one core (LDA_CNT: 111,320 grid points,
8 Bloch points, 15 states, degree 35).  ``--gpu fp64|mixed`` runs the same SCF through the GPU
library (``CyclixGPU.scf``) instead of the oracle and records it under ``<deck>@gpu-<prec>``.
"""
import json
import os
import re
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [ROOT, os.path.join(ROOT, "tests")]

# root of the reference project (the directory holding src/ and tests/)
REFERENCE = os.environ.get("CYCLIX_REFERENCE", "")


def out_values(out_path):
    """Numbers the reference printed: free energy per atom, self and correction energy, radii, SCF count."""
    txt = open(out_path).read()

    def num(pat):
        m = re.search(pat + r"\s*:\s*([-+0-9.Ee]+)", txt)
        return float(m.group(1)) if m else None
    radii = re.search(r"Pseudocharge radii of atom type 1\s*:\s*([0-9.]+)\s+([0-9.]+)\s+([0-9.]+)", txt)
    nscf = re.search(r"Total number of SCF:\s*(\d+)", txt)
    last_err = re.findall(r"^\d+\s+[-+0-9.Ee]+\s+([0-9.Ee+-]+)\s+[0-9.]+\s*$", txt, re.M)
    static = os.path.splitext(out_path)[0] + ".static"
    forces = None
    if os.path.exists(static):
        st = open(static).read().split("Atomic forces (Ha/Bohr):")
        if len(st) > 1:
            rows = []
            for ln in st[1].strip().splitlines():
                parts = ln.split()
                if len(parts) != 3:
                    break
                try:
                    rows.append([float(v) for v in parts])
                except ValueError:
                    break
            forces = rows or None
    return dict(forces=forces, free_energy_per_atom=num(r"Free energy per atom"),
                self_and_correction=num(r"Self and correction energy"),
                fermi_level=num(r"Fermi level"),
                radii=[float(radii.group(i)) for i in (1, 2, 3)] if radii else None,
                n_scf=int(nscf.group(1)) if nscf else None,
                last_scf_error=float(last_err[-1]) if last_err else None)


PRINTED = ["CELL", "FD_GRID", "TWIST_ANGLE", "TOL_PSEUDOCHARGE", "TOL_SCF", "KPOINT_GRID", "NSTATES", "CHEB_DEGREE"]


def ran_with(inpt_path):
    """The .inpt keywords whose values in the .out's input-parameter block differ (beyond the 6
    digits the .out prints), and the pseudopotential files the run read where the .ion now names
    others: the parameters that run actually used.  Keywords the .inpt leaves out are derived
    defaults, which the loader derives as well."""
    from cyclix_msparc_gb300.deck import read_inpt, read_ion
    txt = open(os.path.splitext(inpt_path)[0] + ".out").read()
    head = txt.split("Initialization")[0]
    cur = read_inpt(inpt_path)
    ov = {}
    # the pseudopotential files the run read (one line per atom type)
    used = re.findall(r"^Pseudopotential\s*:\s*(\S+)", txt, re.M)
    files = [T.psp_file for T in read_ion(os.path.splitext(inpt_path)[0] + ".ion")]
    if used and len(used) == len(files) and [os.path.basename(u) for u in used] != [os.path.basename(f) for f in files]:
        ov["PSEUDO_POT"] = [os.path.basename(u) for u in used]
    for k in PRINTED:
        m = re.search(r"^" + k + r":\s*(.*)$", head, re.M)
        if not m or k not in cur:
            continue
        vals = m.group(1).split()
        same = len(cur[k]) >= len(vals) and all(
            abs(float(a) - float(b)) <= 5e-7 * max(1.0, abs(float(a))) for a, b in zip(cur[k], vals))
        if not same:
            ov[k] = vals
    return ov


def _gpu_scf(S, blocks, psis, prec, scf_tol, poisson_tol, max_scf, log):
    from cyclix_msparc_gb300.msparc import CyclixGPU
    g = CyclixGPU(S, blocks, prec)
    try:
        for b, p in enumerate(psis):
            g.set_psi(b, p)
        res, EV, rho, V, hist = g.scf(S, scf_tol=scf_tol, poisson_tol=poisson_tol, max_scf=max_scf)
    finally:
        g.close()
    for it, (e, err) in enumerate(hist, 1):
        log(it, e, err)
    return dict(Etotal=res.Etotal, lambda_f=res.lambda_f, n_scf=res.n_scf)


def pin(deck_rel, scf_tol=1e-6, max_scf=60, root=REFERENCE, gpu=None):
    from cyclix_msparc_gb300.deck import load_deck
    from cyclix_msparc_gb300.workloads import initial_psi
    inpt = os.path.join(root, deck_rel)
    out = os.path.splitext(inpt)[0] + ".out"
    ref = out_values(out)
    t0 = time.time()
    overrides = ran_with(inpt)
    d = load_deck(inpt, overrides=overrides)
    S = d.S
    scf_tol = min(scf_tol, d.scf_tol)
    blocks = [(S.kptgrid[k].copy(), 0, S.Nev) for k in range(S.tnkpt)]
    psis = [initial_psi(S.N, S.Nev, 700 + k) for k in range(S.tnkpt)]
    hist = []

    def log(it, e, err):
        hist.append((it, float(e), float(err)))
        print(f"  SCF {it:3d}  E = {e:.10f} Ha/atom  err = {err:.3e}  ({time.time() - t0:.0f} s)", flush=True)
    forces = None
    if gpu:
        res = _gpu_scf(S, blocks, psis, gpu, scf_tol, d.poisson_tol, max_scf, log)
    else:
        from oracle import scf as OS
        from oracle.forces import atomic_forces
        res = OS.scf(S, psis, blocks, scf_tol=scf_tol, poisson_tol=d.poisson_tol, max_scf=max_scf, log=log)
        if ref.get("forces") is not None:
            F, _ = atomic_forces(d, res["psis"], res["occ"], res["phi"])
            forces = F.tolist()
    E = res["Etotal"] / S.n_atm
    # the energy when the oracle's SCF error first fell to the reference's final error
    e_at_ref = next((e for (_, e, err) in hist if err <= ref["last_scf_error"]), None) if ref["last_scf_error"] else None
    rec = dict(deck=deck_rel, solver=f"gpu-{gpu}" if gpu else "oracle", overrides=overrides, grid=[S.Nx, S.Ny, S.Nz], n_atm=S.n_atm, n_kpt=S.tnkpt, Nev=S.Nev,
               npl=S.npl, smearing="fermi-dirac" if S.elec_T_type == 0 else "gaussian", twist=S.twist,
               reference=ref,
               oracle=dict(free_energy_per_atom=E, self_and_correction=S.E_corr - S.Eself,
                           radii=[round(v, 6) for v in d.rb[0]], lambda_f=float(res["lambda_f"]),
                           n_scf=res["n_scf"], scf_tol=scf_tol, energy_at_reference_error=e_at_ref,
                           history=hist, wall_s=round(time.time() - t0, 1)),
               diff_free_energy_per_atom=E - ref["free_energy_per_atom"],
               forces=forces,
               max_diff_force=(float(np.max(np.abs(np.array(forces) - np.array(ref["forces"]))))
                               if forces is not None else None),
               diff_self_and_correction=(S.E_corr - S.Eself) - ref["self_and_correction"])
    return rec


def main():
    import argparse
    ap = argparse.ArgumentParser()
    ap.add_argument("decks", nargs="*", default=["LDA_CNT/C.inpt"])
    ap.add_argument("--root", default=REFERENCE, help="directory holding the decks (reference project root)")
    ap.add_argument("--gpu", choices=["fp64", "mixed"], help="run the SCF through the GPU library")
    ap.add_argument("--out", default=os.path.join(HERE, "deck_pins.json"))
    args = ap.parse_args()
    if not args.root:
        ap.error("name the reference project root with --root or CYCLIX_REFERENCE")
    path = args.out
    for dk in args.decks:
        print(f"deck {dk}", flush=True)
        rec = pin(dk, root=args.root, gpu=args.gpu)
        print(f"  free energy per atom: oracle {rec['oracle']['free_energy_per_atom']:.10f}  "
              f"reference {rec['reference']['free_energy_per_atom']:.10f}  "
              f"diff {rec['diff_free_energy_per_atom']:.2e}", flush=True)
        # merge with the records other runs wrote meanwhile
        recs = json.load(open(path)) if os.path.exists(path) else {}
        recs[dk + (f"@gpu-{args.gpu}" if args.gpu else "")] = rec
        with open(path, "w") as f:
            json.dump(recs, f, indent=1)


if __name__ == "__main__":
    main()
