"""Cyclix input decks (``.inpt`` / ``.ion`` / ``.psp8``) turned into the struct-``S`` fields of the
CheFSI path: grid, Bloch points, pseudocharges, self and correction energies, the atomic density
guess and the Kleinman-Bylander projectors of the pseudopotential files.

This is the host-side setup the reference runs before its SCF (paths relative to the reference
project root ``Cyclix_MS_200220/``):

* ``read_psp8``: src/readPseudopot.m:15-97 (ONCVPSP psp8, local part forced to ``lloc = 4``);
* ``read_inpt`` / ``read_ion``: the keywords of src/read_inpt.m and src/read_ion.m that cyclic
  and helical decks use, with the defaults of src/initialization.m (``Nev``: :508-514, ``npl``:
  :488-506 and :856-869, smearing: :265-273, tolerances: :548-560);
* ``pseudocharge_radii``: ``Calculate_rb`` (src/initialization.m:47-134);
* ``pseudocharges``: src/calculate_b_guessRho_Eself.m:17-216 with the Cyclix pseudocharge
  Laplacian of Cychel/pseudochargeDensity_atom_cychel.m:1-34;
* ``projectors``: src/calculate_nloc_projector.m:23-287 (psp8 branch, Cyclix image rotation);
* ``load_deck``: the chain above, as src/initialization.m:13-42 orders it.

Everything is vectorised NumPy/SciPy; nothing here touches a GPU.  ``interp1(..., 'spline')``
is MATLAB's not-a-knot cubic spline, which is ``scipy.interpolate.CubicSpline``'s default.
"""
from __future__ import annotations

import math
import os
from dataclasses import dataclass, field

import numpy as np
from scipy.interpolate import CubicSpline

from .cychel import (AtomNL, CyclixS, RcImage, clipped_box, cyclix_kpoints, fd_weights, image_reaches_cell,
                     intg_weights, noncart2cart, periodic_images, real_ylm, rot_z)

HARTREE_EV = 27.211386245988        # src/initialization.m:947 (Cst)
RC_REF = 0.5                        # reference pseudopotential cut-off, src/initialization.m:971


# ------------------------------------------------------------------------------------------------
# pseudopotential files
# ------------------------------------------------------------------------------------------------
@dataclass
class Psp8:
    """One psp8 file as src/readPseudopot.m keeps it (``S.Atm(ityp)``)."""
    Z: float                         # valence charge (zion)
    r: np.ndarray                    # (mmax,) radial grid
    Vloc: np.ndarray                 # (mmax,) local potential
    lmax: int
    lloc: int                        # forced to 4 (src/readPseudopot.m:29)
    nproj: np.ndarray                # (lmax+1,) projectors per l
    proj: list                       # per l: (mmax, nproj_l) projectors divided by r, or None
    gamma: list                      # per l: (nproj_l,) KB energies
    rho_iso: np.ndarray              # (mmax,) isolated-atom valence density / (4 pi)
    rc: float                        # largest r_core of the header line


def read_psp8(path: str) -> Psp8:
    """Parse a psp8 file in the order src/readPseudopot.m:22-82 reads it."""
    with open(path) as f:
        lines = f.read().splitlines()
    head = lines[0].split()
    Z = float(lines[1].split()[1])
    hdr = lines[2].split()
    lmax, mmax = int(hdr[2]), int(hdr[4])
    lloc = 4
    fchrg = float(lines[3].split()[1])
    if fchrg != 0.0:
        raise ValueError(f"{path}: model core charge (fchrg = {fchrg}) is not read by the reference's psp8 reader")
    nproj = np.array([int(v) for v in lines[4].split()[:lmax + 1]])
    tok = " ".join(lines[6:]).split()
    pos = 0

    def take(n):
        nonlocal pos
        out = np.array([float(t.replace("D", "E")) for t in tok[pos:pos + n]])
        pos += n
        return out

    proj, gamma = [None] * (lmax + 1), [None] * (lmax + 1)
    r = Vloc = None
    for l in range(lmax + 1):
        take(1)                                        # the l of the block
        if l != lloc:
            gamma[l] = take(int(nproj[l]))
            A = take((2 + int(nproj[l])) * mmax).reshape(mmax, 2 + int(nproj[l]))
            r = A[:, 1].copy()
            P = A[:, 2:].copy()
            P[1:] = P[1:] / r[1:, None]
            P[0] = P[1]
            proj[l] = P
        else:
            A = take(3 * mmax).reshape(mmax, 3)
            r, Vloc = A[:, 1].copy(), A[:, 2].copy()
    if lloc > lmax:
        take(1)
        A = take(3 * mmax).reshape(mmax, 3)
        r, Vloc = A[:, 1].copy(), A[:, 2].copy()
    A = take(5 * mmax).reshape(mmax, 5)
    rho_iso = A[:, 2] / (4 * math.pi)
    # r_core values follow the first three words of the first line
    rc = max(float(v) for v in head[3:3 + lmax + 1])
    return Psp8(Z, r, Vloc, lmax, lloc, nproj, proj, gamma, rho_iso, rc)


# ------------------------------------------------------------------------------------------------
# input files
# ------------------------------------------------------------------------------------------------
def read_inpt(path: str) -> dict:
    """``KEY: values`` lines of an .inpt file (values as lists of strings)."""
    out = {}
    with open(path) as f:
        for ln in f:
            ln = ln.split("#")[0].strip()
            if ":" not in ln:
                continue
            k, v = ln.split(":", 1)
            out[k.strip().upper()] = v.split()
    return out


@dataclass
class AtomType:
    typ: str
    psp_file: str
    coords: np.ndarray               # (n, 3) as written
    frac: bool


def read_ion(path: str) -> list:
    """Atom types of an .ion file (ATOM_TYPE, PSEUDO_POT, N_TYPE_ATOM, COORD / COORD_FRAC)."""
    with open(path) as f:
        lines = [ln.split("#")[0].strip() for ln in f]
    types, i = [], 0
    cur = None
    while i < len(lines):
        ln = lines[i]
        key = ln.split(":")[0].strip().upper() if ":" in ln else ""
        val = ln.split(":", 1)[1].split() if ":" in ln else []
        if key == "ATOM_TYPE":
            cur = dict(typ=val[0], psp=None, n=0)
            types.append(cur)
        elif key == "PSEUDO_POT":
            cur["psp"] = val[0]
        elif key == "N_TYPE_ATOM":
            cur["n"] = int(val[0])
        elif key in ("COORD", "COORD_FRAC"):
            rows = []
            while len(rows) < cur["n"]:
                i += 1
                if lines[i]:
                    rows.append([float(v) for v in lines[i].split()[:3]])
            cur["coords"] = np.array(rows)
            cur["frac"] = key == "COORD_FRAC"
        i += 1
    return [AtomType(t["typ"], t["psp"], t["coords"], t["frac"]) for t in types]


def cheb_degree_from_mesh(h: float) -> int:
    """``Mesh2ChebDegree`` (src/initialization.m:856-869): cubic fit of the degree in h."""
    if h > 0.7:
        return 14
    p3, p2, p1, p0 = -700.0 / 3.0, 1240.0 / 3.0, -773.0 / 3.0, 1078.0 / 15.0
    return int(_mround(((p3 * h + p2) * h + p1) * h + p0))


def default_scf_tol(inp: dict, Nelectron: float, n_atm: int) -> float:
    """SCF tolerance when the deck gives none (src/initialization.m:516-546): a fit in
    log10(electrons per atom) to a target force accuracy (ACCURACY level, SCF_FORCE_ACC, default
    1e-3 Ha/bohr) or energy accuracy (SCF_ENERGY_ACC)."""
    levels = {"minimal": 0, "low": 1, "medium": 2, "high": 3, "extreme": 4}
    lg = math.log10(Nelectron / n_atm)
    force = energy = -1.0
    if "ACCURACY" in inp:
        force = 10.0 ** (levels[inp["ACCURACY"][0].lower()] + 1)     # as written in the reference
    elif "SCF_FORCE_ACC" in inp:
        force = float(inp["SCF_FORCE_ACC"][0])
    elif "SCF_ENERGY_ACC" in inp:
        energy = float(inp["SCF_ENERGY_ACC"][0])
    if force < 0 and energy < 0:
        force = 1e-3
    if force > 0:
        return 10.0 ** ((math.log10(force) - (-0.33145 + 1.1761 * lg)) / 1.03)
    return 10.0 ** ((math.log10(energy) - (-0.25440 + lg)) / 2.02)


def _mround(x: float) -> float:
    # MATLAB's round: half away from zero
    return math.copysign(math.floor(abs(x) + 0.5), x)


# ------------------------------------------------------------------------------------------------
# grid helpers
# ------------------------------------------------------------------------------------------------
def _cart(S, r, t, z):
    ang = t + S.twist * z
    return r * np.cos(ang), r * np.sin(ang), z


def _distance_box(S, xx, yy, zz, x0, y0, z0):
    """Cartesian distances from (x0, y0, z0) to the nodes of the ndgrid box xx x yy x zz
    (Cychel/calculateDistance_cychel.m:1-6); arrays are indexed [i, j, k]."""
    R, T, Zg = np.meshgrid(xx, yy, zz, indexing="ij")
    X, Y, Zc = _cart(S, R, T, Zg)
    ax, ay, az = _cart(S, x0, y0, z0)
    return np.sqrt((X - ax) ** 2 + (Y - ay) ** 2 + (Zc - az) ** 2)


def _pseudocharge_lap(S, V: np.ndarray, x_first: float) -> np.ndarray:
    """The Cyclix Laplacian of ``V`` on the interior of a box with FDn-wide margins
    (Cychel/pseudochargeDensity_atom_cychel.m:1-34): radial second and first derivative with
    1/r, theta with 1/r^2 (+ tau^2 on a helical cell), z, and the helical cross term."""
    n = S.FDn
    nx, ny, nz = V.shape
    c1, c2, c3 = 1.0 / S.dx ** 2, 1.0 / S.dy ** 2, 1.0 / S.dz ** 2
    c4 = S.twist ** 2 / S.dy ** 2
    c5 = -2.0 * S.twist / (S.dy * S.dz)
    c6 = 1.0 / S.dx
    rr = (x_first + np.arange(n, nx - n) * S.dx)[:, None, None]
    I, J, K = slice(n, nx - n), slice(n, ny - n), slice(n, nz - n)
    w1, w2 = S.w1, S.w2
    ct = c2 / (rr * rr) + c4
    b = w2[0] * (c1 + c2 / (rr * rr) + c3 + c4) * V[I, J, K]
    for p in range(1, n + 1):
        Ip, Im = slice(n + p, nx - n + p), slice(n - p, nx - n - p)
        Jp, Jm = slice(n + p, ny - n + p), slice(n - p, ny - n - p)
        Kp, Km = slice(n + p, nz - n + p), slice(n - p, nz - n - p)
        b = b + (c1 * w2[p] + c6 * w1[p] / rr) * V[Ip, J, K] + (c1 * w2[p] - c6 * w1[p] / rr) * V[Im, J, K]
        b = b + ct * w2[p] * (V[I, Jp, K] + V[I, Jm, K]) + c3 * w2[p] * (V[I, J, Kp] + V[I, J, Km])
        if S.twist != 0.0:
            for q in range(1, n + 1):
                Kq, Kmq = slice(n + q, nz - n + q), slice(n - q, nz - n - q)
                b = b + c5 * w1[p] * w1[q] * (V[I, Jp, Kq] - V[I, Jp, Kmq] - V[I, Jm, Kq] + V[I, Jm, Kmq])
    return b


def _v_local(psp: Psp8, dd: np.ndarray) -> np.ndarray:
    """V_J at distance dd: spline of r*Vloc, -Z beyond the grid, divided by dd; Vloc(1) inside
    the first grid interval (src/calculate_b_guessRho_Eself.m:113-120)."""
    V = np.empty_like(dd)
    far = dd > psp.r[-1]
    V[far] = -psp.Z
    V[~far] = CubicSpline(psp.r, psp.r * psp.Vloc)(dd[~far])
    with np.errstate(divide="ignore", invalid="ignore"):
        V = V / dd
    V[dd < psp.r[1]] = psp.Vloc[0]
    return V


def _v_ref(Z: float, dd: np.ndarray, rc: float = RC_REF) -> np.ndarray:
    """Reference potential: -Z/r outside rc, a degree-7 polynomial inside
    (src/calculate_b_guessRho_Eself.m:122-128)."""
    V = np.empty_like(dd)
    out = dd >= rc
    V[out] = -Z / dd[out]
    d = dd[~out]
    V[~out] = -Z * (9 * d ** 7 - 30 * rc * d ** 6 + 28 * rc * rc * d ** 5 - 14 * rc ** 5 * d ** 2 + 12 * rc ** 7) / (5 * rc ** 8)
    return V


def _rho_iso(psp: Psp8, dd: np.ndarray) -> np.ndarray:
    rho = CubicSpline(psp.r, psp.rho_iso)(dd)
    rho[dd > psp.r[-1]] = 0.0
    return rho


# ------------------------------------------------------------------------------------------------
# pseudocharge radii, pseudocharges, self energy and correction
# ------------------------------------------------------------------------------------------------
def pseudocharge_radii(S, psp: Psp8, xmax_at: float, xvac: float, tol: float) -> tuple:
    """``Calculate_rb`` (src/initialization.m:47-134) for a Cyclix cell: grow (rb_x, rb_z) by
    min(dx, dz) and set rb_y = acos(1 - rb_z^2 / (2 r_max^2)) + tau rb_z / 2 until the pseudocharge
    of one atom at the largest radius integrates to -Z within ``tol`` over the rb box
    (half-space in z, doubled)."""
    def f_rby(y):
        return math.acos(1.0 - y * y / (2 * xmax_at * xmax_at)) + S.twist * y * 0.5
    n = S.FDn
    up_x, up_y, up_z = xvac, f_rby(12.0), 12.0
    is_, ie = -math.ceil(up_x / S.dx), math.ceil(up_x / S.dx)
    js, je = -math.ceil(up_y / S.dy), math.ceil(up_y / S.dy)
    ks, ke = 0, math.ceil(up_z / S.dz)
    xx = xmax_at + np.arange(is_ - n, ie + n + 1) * S.dx
    yy = np.arange(js - n, je + n + 1) * S.dy
    zz = np.arange(ks - n, ke + n + 1) * S.dz
    Nx, Ny, Nz = ie - is_ + 1, je - js + 1, ke - ks + 1
    dd = _distance_box(S, xx, yy, zz, xmax_at, 0.0, 0.0)
    # weights of the box, Dirichlet ends in all three directions
    W = intg_weights(Nx, Ny, Nz, 1, 1, float(xx[n]), S.dx, S.dy, S.dz).reshape(Nx, Ny, Nz, order="F")
    b = -_pseudocharge_lap(S, _v_local(psp, dd), float(xx[0])) / (4 * math.pi)
    rbx = math.ceil(psp.rc / S.dx - 1e-12) * S.dx
    rby = math.ceil(f_rby(psp.rc) / S.dy - 1e-12) * S.dy
    rbz = math.ceil(psp.rc / S.dz - 1e-12) * S.dz
    ds = min(S.dx, S.dz)
    err, count = 100.0, 1
    while err > tol and count <= 300 and rbx <= up_x and rby <= up_y and rbz <= up_z:
        rbx += ds
        rbz += ds
        rby = f_rby(rbz)
        # b and W are indexed from the interior box; the reference's ranges are offset by FDn
        ii = np.arange(-is_ - math.floor(rbx / S.dx), -is_ + math.floor(rbx / S.dx) + 1)
        jj = np.arange(-js - math.floor(rby / S.dy), -js + math.floor(rby / S.dy) + 1)
        kk = np.arange(0, math.floor(rbz / S.dz) + 1)
        sub = np.ix_(ii, jj, kk)
        err = abs(2.0 * float(np.sum(W[sub] * b[sub])) + psp.Z)
        count += 1
    if not (rbx <= up_x and rby <= up_y and rbz <= up_z):
        raise ValueError("pseudocharge radius exceeds the vacuum: increase the cell's radial extent")
    return rbx, rby, rbz


_images = periodic_images        # image enumeration and box clipping shared with the synthetic systems
_box = clipped_box


def pseudocharges(S, psps: list, atom_type: np.ndarray, rbs: list) -> dict:
    """b, b_ref, rho_at (scaled to the electron count), Eself, Eself_ref, V_c, E_corr, PosCharge
    and NegCharge (src/calculate_b_guessRho_Eself.m:17-216, nspin = 1)."""
    n = S.FDn
    b = np.zeros(S.N)
    b_ref = np.zeros(S.N)
    rho_at = np.zeros(S.N)
    V_c = np.zeros(S.N)
    Eself = Eself_ref = 0.0
    Wg = S.W
    for J in range(S.Atoms.shape[0]):
        psp, rb = psps[atom_type[J]], rbs[atom_type[J]]
        x0, y0, z0 = S.Atoms[J]
        for (x0i, y0i, z0i) in _images(S, x0, y0, z0, rb[1], rb[2]):
            (is_, ie), (js, je), (ks, ke) = _box(S, x0i, y0i, z0i, rb)
            if ie < is_ or je < js or ke < ks:
                continue
            xx = S.xin + np.arange(is_ - n - 1, ie + n) * S.dx
            yy = np.arange(js - n - 1, je + n) * S.dy
            zz = np.arange(ks - n - 1, ke + n) * S.dz
            dd = _distance_box(S, xx, yy, zz, x0i, y0i, z0i)
            V = _v_local(psp, dd)
            Vr = _v_ref(psp.Z, dd)
            rho = _rho_iso(psp, dd)
            bJ = _pseudocharge_lap(S, V, float(xx[0]))
            bJr = _pseudocharge_lap(S, Vr, float(xx[0]))
            I, Jj, K = np.meshgrid(np.arange(is_, ie + 1), np.arange(js, je + 1), np.arange(ks, ke + 1), indexing="ij")
            row = ((K - 1) * S.Nx * S.Ny + (Jj - 1) * S.Nx + I - 1).reshape(-1, order="F")
            inner = (slice(n, -n), slice(n, -n), slice(n, -n))
            Vi, Vri = V[inner].reshape(-1, order="F"), Vr[inner].reshape(-1, order="F")
            bJf, bJrf = bJ.reshape(-1, order="F"), bJr.reshape(-1, order="F")
            np.add.at(b, row, bJf)
            np.add.at(b_ref, row, bJrf)
            np.add.at(rho_at, row, rho[inner].reshape(-1, order="F"))
            np.add.at(V_c, row, Vri - Vi)
            Eself += 0.5 * float(np.sum(bJf * Vi * Wg[row]))
            Eself_ref += 0.5 * float(np.sum(bJrf * Vri * Wg[row]))
    s = -1.0 / (4 * math.pi)
    b *= s
    b_ref *= s
    Eself *= s
    Eself_ref *= s
    PosCharge = abs(float(Wg @ b))
    NegCharge = -PosCharge
    rho_at *= abs(NegCharge / float(Wg @ rho_at))
    E_corr = 0.5 * float(np.sum((b_ref + b) * V_c * Wg)) + Eself - Eself_ref
    return dict(b=b, b_ref=b_ref, rho_at=rho_at, V_c=V_c, Eself=Eself, Eself_ref=Eself_ref, E_corr=E_corr,
                PosCharge=PosCharge, NegCharge=NegCharge)


# ------------------------------------------------------------------------------------------------
# nonlocal projectors
# ------------------------------------------------------------------------------------------------
def _rot_pow(R: np.ndarray, p: int) -> np.ndarray:
    return np.linalg.matrix_power(R, p) if p >= 0 else np.linalg.matrix_power(R.T, -p)


def projectors(S, psps: list, atom_type: np.ndarray, rbs: list) -> list:
    """``S.Atom(J)`` of the psp8 projectors (src/calculate_nloc_projector.m:23-287): images from the
    rb box, nodes of the ball |x - R_img| <= rc, the displacement rotated back to the atom's own
    frame by RotM1^fac1 RotM2^fac2 (:174-184), columns ordered (l, projector, m) with
    Chi = UdV_l,p(d) Y_lm (:224-238) and gamma_Jl the matching KB energies (:256-269)."""
    RotM1 = rot_z(S.L2)
    RotM2 = rot_z(S.twist * S.L3)
    out = []
    for J in range(S.Atoms.shape[0]):
        psp, rb = psps[atom_type[J]], rbs[atom_type[J]]
        x0, y0, z0 = S.Atoms[J]
        cols = [(l, p, m) for l in range(psp.lmax + 1) if l != psp.lloc for p in range(int(psp.nproj[l]))
                for m in range(-l, l + 1)]
        splines = {(l, p): CubicSpline(psp.r, psp.proj[l][:, p]) for (l, p, _) in cols}
        images = []
        for (x0i, y0i, z0i) in _images(S, x0, y0, z0, rb[1], rb[2]):
            if not image_reaches_cell(S, x0i, y0i, z0i, rb):
                continue
            (is_, ie), (js, je), (ks, ke) = _box(S, x0i, y0i, z0i, rb)
            if ie < is_ or je < js or ke < ks:
                continue
            I, Jj, K = np.meshgrid(np.arange(is_, ie + 1), np.arange(js, je + 1), np.arange(ks, ke + 1), indexing="ij")
            I, Jj, K = (a.reshape(-1, order="F") for a in (I, Jj, K))
            node = noncart2cart(S, np.stack([S.xin + (I - 1) * S.dx, (Jj - 1) * S.dy, (K - 1) * S.dz], axis=1))
            atm = noncart2cart(S, np.array([[x0i, y0i, z0i]]))[0]
            disp = node - atm
            dd = np.sqrt((disp ** 2).sum(axis=1))
            inb = dd <= psp.rc
            if not inb.any():
                continue
            disp, dd = disp[inb], dd[inb]
            fac1 = int(round((y0 - y0i) / S.L2))
            fac2 = int(round((z0 - z0i) / S.L3))
            P = (_rot_pow(RotM1, fac1) @ _rot_pow(RotM2, fac2) @ disp.T).T
            chi = np.empty((dd.shape[0], len(cols)))
            centre = dd == 0.0
            with np.errstate(divide="ignore", invalid="ignore"):
                for c, (l, p, m) in enumerate(cols):
                    chi[:, c] = splines[(l, p)](dd) * real_ylm(l, m, P[:, 0], P[:, 1], P[:, 2])
                    if l > 0:
                        # a node exactly on the atom: Y_lm has no direction there (the reference's
                        # x/|x| gives 0/0); the projector u_l(r) Y_lm is continuous and 0 at r = 0
                        chi[centre, c] = 0.0
            if not np.all(np.isfinite(chi)):
                raise ValueError(f"atom {J + 1}: non-finite projector values")
            pos = ((K - 1) * S.Nx * S.Ny + (Jj - 1) * S.Nx + I)[inb].astype(np.int64)
            images.append(RcImage(np.array([x0i, y0i, z0i]), pos, chi))
        gam = np.array([psp.gamma[l][p] for (l, p, _) in cols])
        out.append(AtomNL(len(cols), gam, images))
    return out


# ------------------------------------------------------------------------------------------------
# the whole deck
# ------------------------------------------------------------------------------------------------
@dataclass
class Deck:
    S: CyclixS
    inpt: dict
    types: list
    psps: list
    rb: list                         # per type (rb_x, rb_y, rb_z)
    scf_tol: float
    poisson_tol: float
    Nelectron: float
    pseudo: dict = field(default_factory=dict)


def load_deck(inpt_path: str, for_scf: bool = True, overrides: dict | None = None) -> Deck:
    """Read ``<name>.inpt``, ``<name>.ion`` and the psp8 files of a cyclic or helical deck and build
    ``S`` with the fields the CheFSI path and the SCF need (src/initialization.m:13-42,
    src/calculate_b_guessRho_Eself.m, src/calculate_nloc_projector.m).

    With ``for_scf`` the deck must be one the SCF path runs (LDA_PW, no spin polarisation);
    without it only the grid, pseudocharges and projectors are built, which do not depend on
    those settings.  ``overrides`` replaces .inpt keywords (``{"FD_GRID": ["120",
    "61", "8"]}``), as editing the file would."""
    base = os.path.splitext(inpt_path)[0]
    root = os.path.dirname(inpt_path)
    inp = read_inpt(inpt_path)
    inp.update({k.upper(): [str(x) for x in v] for k, v in (overrides or {}).items()})
    types = read_ion(base + ".ion")
    if "PSEUDO_POT" in inp:                      # one file per atom type, in .ion order
        for T, f in zip(types, inp["PSEUDO_POT"]):
            T.psp_file = f
    L1, L2, L3 = (float(v) for v in inp["CELL"][:3])
    if "BC" in inp:
        bc = [c.upper() for c in inp["BC"][:3]]
        if bc[0] != "D" or bc[1] != "C" or bc[2] not in ("P", "H"):
            raise ValueError(f"BC {' '.join(bc)}: only cyclic (D C P) and helical (D C H) cells are supported")
        BC = 7 if bc[2] == "H" else 5
    else:
        BC = int(float(inp["BOUNDARY_CONDITION"][0]))
    if BC not in (5, 7):
        raise ValueError(f"boundary condition {BC}: only cyclic (5) and helical (7) cells are supported")
    cell_typ, BCx, BCy, BCz = (3, 1, 0, 0) if BC == 5 else (5, 1, 0, 0)
    twist = float(inp["TWIST_ANGLE"][0]) if "TWIST_ANGLE" in inp else 0.0
    if cell_typ == 3:
        twist = 0.0
    xc = inp.get("EXCHANGE_CORRELATION", ["LDA_PW"])[0]
    if for_scf and xc not in ("LDA_PW", "LDA_PZ", "GGA_PBE"):
        raise ValueError(f"exchange-correlation {xc}: the SCF paths implement LDA_PW (and the oracle LDA_PZ, GGA_PBE)")
    if for_scf and "SPIN_TYP" in inp and int(inp["SPIN_TYP"][0]) != 0:
        raise ValueError("spin-polarised decks are not supported by the SCF path")
    Nx0, Ny0, Nz0 = (int(v) for v in inp["FD_GRID"][:3])
    dx, dy, dz = L1 / Nx0, L2 / Ny0, L3 / Nz0
    Nx, Ny, Nz = Nx0 + BCx, Ny0 + BCy, Nz0 + BCz
    FDn = int(inp.get("FD_ORDER", ["12"])[0]) // 2
    w1, w2 = fd_weights(FDn)
    # atoms in (r, theta, z) (src/read_ion.m:144-158; Cartesian input through the Cyclix transform)
    coords, atom_type = [], []
    for t, T in enumerate(types):
        c = T.coords.copy()
        if T.frac:
            c = c * np.array([L1, L2, L3])
        else:
            c = np.stack([np.hypot(c[:, 0], c[:, 1]), np.arctan2(c[:, 1], c[:, 0]) - twist * c[:, 2], c[:, 2]], axis=1)
        coords.append(c)
        atom_type += [t] * c.shape[0]
    Atoms = np.concatenate(coords)
    atom_type = np.array(atom_type)
    xmin_at, xmax_at = float(Atoms[:, 0].min()), float(Atoms[:, 0].max())
    xvac = (L1 - (xmax_at - xmin_at)) / 2
    xin = xmin_at - xvac
    W = intg_weights(Nx, Ny, Nz, BCy, BCz, xin, dx, dy, dz)
    nkpt = [int(v) for v in inp.get("KPOINT_GRID", ["1", "1", "1"])[:3]]
    shift = [float(v) for v in inp.get("KPOINT_SHIFT", ["0", "0", "0"])[:3]]
    kpt, wkpt = cyclix_kpoints(nkpt, L1, L2, L3, kptshift=shift, time_reversal=True)
    psps = [read_psp8(os.path.join(root, T.psp_file)) for T in types]
    Nelectron = float(sum(psps[t].Z for t in atom_type))
    # defaults of src/initialization.m
    xout = xmax_at + xvac
    h_eff = math.sqrt(3.0 / (1 / dx ** 2 + 1 / (((xin + xout) / 2) * dy) ** 2 + 1 / dz ** 2))
    npl = int(inp["CHEB_DEGREE"][0]) if "CHEB_DEGREE" in inp else cheb_degree_from_mesh(h_eff)
    Nev = int(inp["NSTATES"][0]) if "NSTATES" in inp else int(_mround(math.floor(Nelectron / 2) * 1.2 + 5))
    scf_tol = float(inp["TOL_SCF"][0]) if "TOL_SCF" in inp else default_scf_tol(inp, Nelectron, len(atom_type))
    poisson_tol = float(inp["TOL_POISSON"][0]) if "TOL_POISSON" in inp else 0.01 * scf_tol
    pc_tol = float(inp["TOL_PSEUDOCHARGE"][0]) if "TOL_PSEUDOCHARGE" in inp else 0.01 * scf_tol
    elec_T_type = 1
    if "ELEC_TEMP_TYPE" in inp:
        t = inp["ELEC_TEMP_TYPE"][0].lower()
        elec_T_type = 0 if t in ("fd", "fermi-dirac", "0") else 1
    if "SMEARING" in inp:
        bet = 1.0 / float(inp["SMEARING"][0])
    elif "ELEC_TEMP" in inp:
        bet = 1.0 / (3.1668115634556e-6 * float(inp["ELEC_TEMP"][0]))
    else:
        bet = HARTREE_EV / 0.2
    S = CyclixS(Nx=Nx, Ny=Ny, Nz=Nz, FDn=FDn, cell_typ=cell_typ, BCx=BCx, BCy=BCy, BCz=BCz, dx=dx, dy=dy, dz=dz,
                xin=xin, twist=twist, L1=L1, L2=L2, L3=L3, w1=w1, w2=w2, W=W, Atoms=Atoms, Atom=[],
                kptgrid=kpt, wkpt=wkpt, nspin=1, Nev=Nev, npl=npl)
    rbs = [pseudocharge_radii(S, p, xmax_at, xvac, pc_tol) for p in psps]
    pc = pseudocharges(S, psps, atom_type, rbs)
    S.Atom = projectors(S, psps, atom_type, rbs)
    S.b, S.rho_at, S.NegCharge = pc["b"], pc["rho_at"], pc["NegCharge"]
    S.Eself, S.E_corr = pc["Eself"], pc["E_corr"]
    S.bet, S.elec_T_type, S.occfac, S.n_atm = bet, elec_T_type, 2.0, int(Atoms.shape[0])
    S.extra.update(deck=os.path.basename(base), atom_type=atom_type, xvac=xvac, xc=xc)
    return Deck(S, inp, types, psps, rbs, scf_tol, poisson_tol, Nelectron, pc)
