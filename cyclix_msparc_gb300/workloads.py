"""Seeded synthetic Cyclix systems with the shapes of the benchmarked workloads.

There is no public dataset for this path; every input is generated here from a
seed: atom sites in a tube shell, a local potential made of Gaussians, and
Gaussian Kleinman-Bylander projectors laid out exactly like the reference's
``S.Atom(J).rcImage(img)`` records (src/calculate_nloc_projector.m:23-287,
Cyclix image rotation at :178-184).  The full-SCF workload adds Gaussian
pseudocharges ``b`` (the reference builds ``b`` from psp8 files in
src/calculate_b_guessRho_Eself.m; that reader is outside this path).

Geometry choices that the workload descriptions leave open (recorded here so
that a run can be reproduced):

* radial domain ``r in [3, 11]`` bohr with ``Nr`` nodes including the
  Dirichlet end node, atoms in the shell ``r in [5, 7]``;
* ``dz = 0.2`` bohr, so ``L3 = 0.2 * Nz`` (periodic z);
* cyclic wedge ``L2 = 2 pi / n_cyc`` with ``n_cyc`` equal to the number of
  distinct cyclic wavenumbers the workload uses (12 when it uses one);
* FD order 12 (``FDn = 6``); projector cut-off ``rc = 1.2`` bohr with a
  Gaussian radial part of width ``rc / 3``; ``gamma = +-1`` Ha (seeded).
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

from .cychel import (AtomNL, CyclixS, RcImage, cell_type, clipped_box, fd_weights, image_reaches_cell,
                     intg_weights, noncart2cart, periodic_images, real_ylm, rot_z)


@dataclass(frozen=True)
class Workload:
    name: str
    Nr: int
    Nt: int
    Nz: int
    Ns: tuple                 # states per block (uneven allowed)
    kpts: tuple               # ((k1, nu, eta), ...) per block, before spin
    nspin: int
    npl: int
    n_atm: int
    n_cyc: int
    twist: float = 0.0
    xin: float = 3.0
    L1: float = 8.0
    dz: float = 0.2
    rc: float = 1.2
    scf: bool = False
    seed: int = 0
    zval: float = 4.0         # valence charge of each Gaussian pseudocharge (SCF workloads)

    @property
    def N(self) -> int:
        return self.Nr * self.Nt * self.Nz

    @property
    def nblocks(self) -> int:
        return len(self.Ns)


def _eta_grid(n: int, L3: float) -> list:
    # Monkhorst-Pack grid along z in the reference's convention, scaled by 2pi/L3
    s = -((n - 1) // 2)
    g = (np.arange(s, s + n) / n)
    eps = np.finfo(float).eps
    g = np.mod(g + 0.5 - eps, 1.0) - 0.5 + eps
    return list((2 * np.pi / L3) * g)


def _make_workloads() -> dict:
    w = {}
    # one cyclic block, small (runs on the CPU oracle in seconds)
    w["cyclic-40x12x20-ns48-m20"] = Workload(
        "cyclic-40x12x20-ns48-m20", 40, 12, 20, (48,), ((0.0, 1.0, 0.0),), 1, 20, 24, 12)
    # the same operator scaled up: one block of 256 states
    w["cyclic-96x24x64-ns256-m24"] = Workload(
        "cyclic-96x24x64-ns256-m24", 96, 24, 64, (256,), ((0.0, 1.0, 0.0),), 1, 24, 77, 12)
    # 16 cyclic wavenumbers nu = 0..15 with uneven block sizes in [96, 320]
    ns3 = tuple(int(v) for v in np.random.default_rng(0).integers(96, 321, 16))
    w["cyclic-batched-16nu-64x16x48-ns96to320-m24"] = Workload(
        "cyclic-batched-16nu-64x16x48-ns96to320-m24", 64, 16, 48, ns3,
        tuple((0.0, float(nu), 0.0) for nu in range(16)), 1, 24, 96, 16)
    # the same cell, atoms and projectors as an SCF cell (Gaussian pseudocharges of valence 1, so
    # the 48 occupied states per block fit the smallest block of 99 states)
    w["scf-batched-16nu-64x16x48-96at-ns96to320-m24"] = Workload(
        "scf-batched-16nu-64x16x48-96at-ns96to320-m24", 64, 16, 48, ns3,
        tuple((0.0, float(nu), 0.0) for nu in range(16)), 1, 24, 96, 16, scf=True, zval=1.0)
    # helical twist 0.05 rad/bohr, 24 eta x 4 nu, two spin channels
    L3h = 0.2 * 40
    etas = _eta_grid(24, L3h)
    k4 = tuple((0.0, float(nu), eta) for nu in range(4) for eta in etas)
    w["helical-80x32x40-96k2s-ns192-m24"] = Workload(
        "helical-80x32x40-96k2s-ns192-m24", 80, 32, 40, (192,) * (len(k4) * 2), k4, 2, 24, 48, 4, twist=0.05)
    # full SCF: 384 atoms, 8 cyclic wavenumbers, uneven Ns up to 1024
    w["scf-128x48x96-384at-8k-ns1024"] = Workload(
        "scf-128x48x96-384at-8k-ns1024", 128, 48, 96, tuple(1024 - 16 * b for b in range(8)),
        tuple((0.0, float(nu), 0.0) for nu in range(8)), 1, 24, 384, 8, scf=True)
    # small SCF used by the tests (same construction, CPU-oracle sized)
    w["scf-small-24x12x20-12at-2k-ns40"] = Workload(
        "scf-small-24x12x20-12at-2k-ns40", 24, 12, 20, (40, 36),
        ((0.0, 0.0, 0.0), (0.0, 1.0, 0.0)), 1, 16, 12, 12, scf=True)
    # small helical SCF used by the tests (twist 0.05 rad/bohr, one nu = 0 and one nu = 1, eta block)
    w["scf-small-helical-24x12x16-8at-2k-ns28"] = Workload(
        "scf-small-helical-24x12x16-8at-2k-ns28", 24, 12, 16, (28, 24),
        ((0.0, 0.0, 0.0), (0.0, 1.0, 0.6)), 1, 16, 8, 12, twist=0.05, dz=0.25, scf=True)
    return w


WORKLOADS = _make_workloads()


def _grid_fields(wl: Workload):
    cell_typ, BCx, BCy, BCz = cell_type(wl.twist != 0.0)
    L1, L2, L3 = wl.L1, 2 * np.pi / wl.n_cyc, wl.dz * wl.Nz
    Nx, Ny, Nz = wl.Nr, wl.Nt, wl.Nz
    dx = L1 / (Nx - BCx)
    dy = L2 / (Ny - BCy)
    dz = L3 / (Nz - BCz)
    return cell_typ, BCx, BCy, BCz, L1, L2, L3, Nx, Ny, Nz, dx, dy, dz


def make_atoms(wl: Workload, rng) -> np.ndarray:
    """Atom sites (r, theta, z): r ~ U[5,7], theta ~ U[0,L2), z ~ U[0,L3)."""
    L2 = 2 * np.pi / wl.n_cyc
    L3 = wl.dz * wl.Nz
    r = rng.uniform(5.0, 7.0, wl.n_atm)
    t = rng.uniform(0.0, L2, wl.n_atm)
    z = rng.uniform(0.0, L3, wl.n_atm)
    return np.stack([r, t, z], axis=1)


def _radial(l: int, d: np.ndarray, sig: float) -> np.ndarray:
    # Gaussian radial projector, normalised so that int (f_l Y_lm)^2 d^3x = 1
    if l == 0:
        A = math.sqrt(4.0 / (sig ** 3 * math.sqrt(math.pi)))
        return A * np.exp(-0.5 * (d / sig) ** 2)
    A = math.sqrt(8.0 / (3.0 * math.sqrt(math.pi) * sig ** 3))
    return A * (d / sig) * np.exp(-0.5 * (d / sig) ** 2)


def nloc_projectors(S: CyclixS, rc: float, gammas: np.ndarray, lmax: int = 1) -> list:
    """Gaussian KB projectors in the reference's per-image layout.

    Follows src/calculate_nloc_projector.m:50-287 with the Cyclix branch: image
    counts per periodic direction (:58-72), image positions (:78-81), the
    bounding box of each image clipped to the cell (:110-122), the ball test
    ``dd <= rc`` on Cartesian distances (:156-169, Cychel/calculateDistance_cychel.m),
    the rotation of the displacement by ``RotM1^fac1 * RotM2^fac2`` (:178-184)
    and ``Chi(:, lm) = UdV_l(d) * Y_lm`` in (l, m) order (:206-215).  The
    theta half-width used for the bounding box is ``asin(rc / r0) + |tau| rc``
    (the reference uses the larger pseudocharge radius ``rb_y``; the ball test
    makes the two equivalent).
    """
    sig = rc / 3.0
    RotM1 = rot_z(S.L2)
    RotM2 = rot_z(S.twist * S.L3)
    atoms = []
    angnum = (lmax + 1) ** 2
    for J in range(S.Atoms.shape[0]):
        x0, y0, z0 = S.Atoms[J]
        rcx = rc
        rcy = math.asin(min(1.0, rc / max(x0 - rc, 1e-12))) + abs(S.twist) * rc
        rcz = rc
        rb = (rcx, rcy, rcz)
        images = []
        for (x0i, y0i, z0i) in periodic_images(S, x0, y0, z0, rcy, rcz):
            if not image_reaches_cell(S, x0i, y0i, z0i, rb):
                continue
            (ii_s, ii_e), (jj_s, jj_e), (kk_s, kk_e) = clipped_box(S, x0i, y0i, z0i, rb)
            if ii_e < ii_s or jj_e < jj_s or kk_e < kk_s:
                continue
            ii = np.arange(ii_s, ii_e + 1)
            jj = np.arange(jj_s, jj_e + 1)
            kk = np.arange(kk_s, kk_e + 1)
            I3, J3, K3 = np.meshgrid(ii, jj, kk, indexing="ij")
            I3 = I3.reshape(-1, order="F")
            J3 = J3.reshape(-1, order="F")
            K3 = K3.reshape(-1, order="F")
            XX = S.xin + (I3 - 1) * S.dx
            YY = (J3 - 1) * S.dy
            ZZ = (K3 - 1) * S.dz
            pos = (K3 - 1) * S.Nx * S.Ny + (J3 - 1) * S.Nx + I3
            node_c = noncart2cart(S, np.stack([XX, YY, ZZ], axis=1))
            atm_c = noncart2cart(S, np.array([[x0i, y0i, z0i]]))[0]
            disp = node_c - atm_c
            dd = np.sqrt((disp ** 2).sum(axis=1))
            inb = dd <= rc
            if not inb.any():
                continue
            disp = disp[inb]
            dd = dd[inb]
            fac1 = int(round((y0 - y0i) / S.L2))
            fac2 = int(round((z0 - z0i) / S.L3))
            ROT = np.linalg.matrix_power(RotM1, fac1) @ np.linalg.matrix_power(RotM2, fac2) \
                if fac1 >= 0 and fac2 >= 0 else _rot_pow(RotM1, fac1) @ _rot_pow(RotM2, fac2)
            P = (ROT @ disp.T).T
            chi = np.zeros((dd.shape[0], angnum))
            col = 0
            for l in range(lmax + 1):
                f = _radial(l, dd, sig)
                for m in range(-l, l + 1):
                    chi[:, col] = f * real_ylm(l, m, P[:, 0], P[:, 1], P[:, 2])
                    col += 1
            images.append(RcImage(np.array([x0i, y0i, z0i]), pos[inb].astype(np.int64), chi))
        g = np.concatenate([np.full(2 * l + 1, gammas[J, l]) for l in range(lmax + 1)])
        atoms.append(AtomNL(angnum, g, images))
    return atoms


def _rot_pow(R: np.ndarray, p: int) -> np.ndarray:
    if p >= 0:
        return np.linalg.matrix_power(R, p)
    return np.linalg.matrix_power(R.T, -p)


def _gaussian_field(S: CyclixS, centers: np.ndarray, amps: np.ndarray, width: float, cutoff: float) -> np.ndarray:
    """sum_J amp_J exp(-|x - R_J|^2 / (2 width^2)) over all periodic images of R_J (within ``cutoff``)."""
    r = S.xin + np.arange(S.Nx) * S.dx
    t = np.arange(S.Ny) * S.dy
    z = np.arange(S.Nz) * S.dz
    Rg, Tg, Zg = np.meshgrid(r, t, z, indexing="ij")
    nodes = noncart2cart(S, np.stack([Rg.reshape(-1, order="F"), Tg.reshape(-1, order="F"),
                                      Zg.reshape(-1, order="F")], axis=1))
    zn = Zg.reshape(-1, order="F")
    out = np.zeros(S.N)
    # the distinct rotations of a cyclic group of order n_cyc = 2 pi / L2 (each counted once)
    n_cyc = int(round(2 * np.pi / S.L2)) if S.BCy == 0 else 1
    m_range = range(-(n_cyc // 2), n_cyc - n_cyc // 2)
    nz = int(math.ceil(cutoff / S.L3)) + 1 if S.BCz == 0 else 0
    # angular extent of the cell (with the helical twist over its length) for a quick image cull
    phi_lo = min(0.0, S.twist * S.L3)
    phi_hi = S.L2 + max(0.0, S.twist * S.L3)
    phi_c = 0.5 * (phi_lo + phi_hi)
    for J in range(centers.shape[0]):
        for m in m_range:
            for n in range(-nz, nz + 1):
                y, zz = centers[J, 1] + m * S.L2, centers[J, 2] + n * S.L3
                if zz < -cutoff or zz > S.L3 + cutoff:
                    continue
                phi = y + S.twist * zz
                phi = phi_c + math.remainder(phi - phi_c, 2 * math.pi)     # nearest copy of the angle
                dphi = max(phi_lo - phi, phi - phi_hi, 0.0)
                # every node has radius >= xin and angle >= dphi away from the image, hence distance
                # >= 2 sqrt(r0 xin) sin(dphi / 2): cull images that cannot reach the cutoff
                if 2 * math.sqrt(centers[J, 0] * S.xin) * math.sin(min(dphi, math.pi) / 2) > cutoff:
                    continue
                c = noncart2cart(S, np.array([[centers[J, 0], y, zz]]))[0]
                msk = np.abs(zn - c[2]) < cutoff
                d2 = ((nodes[msk] - c) ** 2).sum(axis=1)
                inc = d2 < cutoff * cutoff
                idx = np.nonzero(msk)[0][inc]
                out[idx] += amps[J] * np.exp(-0.5 * d2[inc] / (width * width))
    return out


def make_system(wl: Workload) -> CyclixS:
    """Build the struct-``S`` fields for a workload (deterministic in ``wl.seed``)."""
    rng = np.random.default_rng(wl.seed + 1234)
    cell_typ, BCx, BCy, BCz, L1, L2, L3, Nx, Ny, Nz, dx, dy, dz = _grid_fields(wl)
    FDn = 6
    w1, w2 = fd_weights(FDn)
    W = intg_weights(Nx, Ny, Nz, BCy, BCz, wl.xin, dx, dy, dz)
    kpt = np.array(wl.kpts, dtype=float).reshape(-1, 3)
    tnkpt = kpt.shape[0]
    S = CyclixS(Nx=Nx, Ny=Ny, Nz=Nz, FDn=FDn, cell_typ=cell_typ, BCx=BCx, BCy=BCy, BCz=BCz,
                dx=dx, dy=dy, dz=dz, xin=wl.xin, twist=wl.twist, L1=L1, L2=L2, L3=L3, w1=w1, w2=w2, W=W,
                Atoms=np.zeros((0, 3)), Atom=[], kptgrid=kpt, wkpt=np.ones(tnkpt) / tnkpt,
                nspin=wl.nspin, Nev=int(max(wl.Ns)), npl=wl.npl)
    S.Atoms = make_atoms(wl, rng)
    S.n_atm = wl.n_atm
    gammas = rng.choice([-1.0, 1.0], size=(wl.n_atm, 2))
    S.Atom = nloc_projectors(S, wl.rc, gammas)
    if not wl.scf:
        depth = rng.uniform(-3.0, -1.0, wl.n_atm)
        v = _gaussian_field(S, S.Atoms, depth, 0.8, 6.0)
        V = np.empty((S.N, wl.nspin))
        V[:, 0] = v
        if wl.nspin == 2:
            # the second spin channel sees a slightly different, seeded potential
            V[:, 1] = v + _gaussian_field(S, S.Atoms, rng.uniform(-0.2, 0.2, wl.n_atm), 0.8, 6.0)
        S.Veff = V
    else:
        Z = wl.zval
        sig_b = 0.6
        amp_b = -Z / (2 * np.pi * sig_b ** 2) ** 1.5
        S.b = _gaussian_field(S, S.Atoms, np.full(wl.n_atm, amp_b), sig_b, 6.0 * sig_b)
        PosCharge = abs(float(S.W @ S.b))
        S.NegCharge = -PosCharge
        sig_a = 1.0
        rho_at = _gaussian_field(S, S.Atoms, np.ones(wl.n_atm), sig_a, 6.0 * sig_a)
        S.rho_at = rho_at * abs(S.NegCharge / float(S.W @ rho_at))
        # self energy of the Gaussian pseudocharges, 0.5 * Z^2 / (sqrt(pi) sig_b) per atom
        S.Eself = wl.n_atm * 0.5 * Z * Z / (math.sqrt(math.pi) * sig_b)
        S.E_corr = 0.0
        S.bet = 27.21138602 / 0.2           # Gaussian smearing 0.2 eV, as the reference's default
        S.elec_T_type = 1
        S.occfac = 2.0 / wl.nspin
    S.extra["Ns"] = tuple(wl.Ns)
    S.extra["workload"] = wl.name
    return S


def block_layout(wl: Workload, S: CyclixS):
    """Blocks in the reference's ks order: all k-points of spin 1, then spin 2.

    Returns a list of ``(kvec (3,), spin (0-based), Ns)``.
    """
    out = []
    ks = 0
    for spin in range(wl.nspin):
        for k in range(S.tnkpt):
            out.append((S.kptgrid[k].copy(), spin, int(wl.Ns[ks])))
            ks += 1
    return out


def initial_psi(N: int, Ns: int, seed: int, dtype=np.complex128) -> np.ndarray:
    """Complex-normal block (seeded) with orthonormal columns (Euclidean QR)."""
    rng = np.random.default_rng(seed)
    X = (rng.standard_normal((N, Ns)) + 1j * rng.standard_normal((N, Ns))) / np.sqrt(2.0)
    Q, _ = np.linalg.qr(X)
    return np.asfortranarray(Q.astype(dtype))
