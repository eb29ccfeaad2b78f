"""Atomic forces of a converged Cyclix SCF (src/atomicForce.m:1-364) with the grid work on the GPU.

Paths relative to the reference project root ``Cyclix_MS_200220/``.

The force of atom J is the sum of three terms (src/atomicForce.m:111-127, 254-300):

* local, per image box:  fl = -sum_box W bJ (D phi - D V_J)
* correction, per image box:  fc = 1/2 sum_box W [(b + b_ref)(D V_J,ref - D V_J) - (bJ + bJ,ref) D V_c]
  both rotated back to the atom's frame by ROT = RotM1^fac1 RotM2^fac2, a rotation about z by
  A = fac1 L2 + fac2 twist L3;
* nonlocal: ``cx_nonlocal_force`` over the device-resident psi of every block.

The box terms depend on the SCF solution only through D phi, and on the set-up through D V_c.  The
set-up (:func:`local_force_setup`, host code over the pseudocharge boxes like the deck set-up of
``deck.py``) therefore reduces every atom to six grid vectors,
  a_c = sum_img cos(A) W bJ,  a_s = sum_img sin(A) W bJ,  a_z = sum_img W bJ, and the same of
  1/2 W (bJ + bJ,ref) as e_c, e_s, e_z,
and a constant vector (the rotated box sums of W bJ D V_J and of 1/2 W (b + b_ref)(D V_J,ref - D V_J)).
At force time (:func:`atomic_forces`) the GPU takes the Cartesian gradient of phi and of V_c and
projects it on those vectors (``cx_field_projections``):
  F_x = c_x - (a_c . D_x phi - a_s . D_y phi) - (e_c . D_x V_c - e_s . D_y V_c),
  F_y = c_y - (a_s . D_x phi + a_c . D_y phi) - (e_s . D_x V_c + e_c . D_y V_c),
  F_z = c_z - a_z . D_z phi - e_z . D_z V_c,
the same sums regrouped.  The drift along z, the one translation a Cyclix cell has, is removed
(src/electronicGroundState.m:108-115).
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

from . import deck as D


@dataclass
class LocalForceSetup:
    """Per-atom projection vectors (n_atm x 6 x N: a_c, a_s, a_z, e_c, e_s, e_z), the constant
    part of the local and correction forces (n_atm x 3), and V_c (N)."""
    vectors: np.ndarray
    const: np.ndarray
    V_c: np.ndarray


def box_gradient(S, V: np.ndarray, xx: np.ndarray, yy: np.ndarray, zz: np.ndarray) -> tuple:
    """Cartesian gradient of V on the interior of a box with FDn margins (Cychel/dpseudopot_cychel.m):
    D_x = cos(phi)/dx d_r - sin(phi)/(r dy) d_theta, D_y = sin(phi)/dx d_r + cos(phi)/(r dy) d_theta,
    D_z = d_z/dz - twist/dy d_theta, phi = theta + twist z, first-derivative weights S.w1."""
    n = S.FDn
    nx, ny, nz = V.shape
    I, J, K = slice(n, nx - n), slice(n, ny - n), slice(n, nz - n)
    R, T, Z = np.meshgrid(xx[I], yy[J], zz[K], indexing="ij")
    ang = T + S.twist * Z
    cs, sn = np.cos(ang), np.sin(ang)
    dr = np.zeros(R.shape)
    dt = np.zeros(R.shape)
    dz = np.zeros(R.shape)
    for p in range(1, n + 1):
        w = S.w1[p]
        dr += w * (V[n + p:nx - n + p, J, K] - V[n - p:nx - n - p, J, K])
        dt += w * (V[I, n + p:ny - n + p, K] - V[I, n - p:ny - n - p, K])
        dz += w * (V[I, J, n + p:nz - n + p] - V[I, J, n - p:nz - n - p])
    dr /= S.dx
    dt /= S.dy
    dz /= S.dz
    return cs * dr - sn / R * dt, sn * dr + cs / R * dt, dz - S.twist * dt


def local_force_setup(d) -> LocalForceSetup:
    """The set-up of the local and correction forces of a loaded deck ``d`` (``deck.load_deck``):
    the boxes, pseudocharges and local potentials of src/atomicForce.m:40-127, reduced per atom."""
    S, pc = d.S, d.pseudo
    n = S.FDn
    atom_type = S.extra["atom_type"]
    nat = S.Atoms.shape[0]
    vec = np.zeros((nat, 6, S.N))
    const = np.zeros((nat, 3))
    s4pi = -1.0 / (4 * math.pi)
    bsum = pc["b"] + pc["b_ref"]
    for J in range(nat):
        psp, rb = d.psps[atom_type[J]], d.rb[atom_type[J]]
        x0, y0, z0 = S.Atoms[J]
        for (x0i, y0i, z0i) in D._images(S, x0, y0, z0, rb[1], rb[2]):
            (is_, ie), (js, je), (ks, ke) = D._box(S, x0i, y0i, z0i, rb)
            if ie < is_ or je < js or ke < ks:
                continue
            xx = S.xin + np.arange(is_ - n - 1, ie + n) * S.dx
            yy = np.arange(js - n - 1, je + n) * S.dy
            zz = np.arange(ks - n - 1, ke + n) * S.dz
            dd = D._distance_box(S, xx, yy, zz, x0i, y0i, z0i)
            V = D._v_local(psp, dd)
            Vr = D._v_ref(psp.Z, dd)
            bJ = s4pi * D._pseudocharge_lap(S, V, float(xx[0]))
            bJr = s4pi * D._pseudocharge_lap(S, Vr, float(xx[0]))
            dV = box_gradient(S, V, xx, yy, zz)
            dVr = box_gradient(S, Vr, xx, yy, zz)
            I, Jj, K = np.meshgrid(np.arange(is_, ie + 1), np.arange(js, je + 1), np.arange(ks, ke + 1), indexing="ij")
            row = ((K - 1) * S.Nx * S.Ny + (Jj - 1) * S.Nx + I - 1)
            Wb = S.W[row]
            fl = np.array([np.sum(Wb * bJ * dV[q]) for q in range(3)])
            fc = np.array([0.5 * np.sum(Wb * bsum[row] * (dVr[q] - dV[q])) for q in range(3)])
            A = round((y0 - y0i) / S.L2) * S.L2 + round((z0 - z0i) / S.L3) * S.twist * S.L3
            c, s = math.cos(A), math.sin(A)
            ROT = np.array([[c, -s, 0.0], [s, c, 0.0], [0.0, 0.0, 1.0]])
            const[J] += ROT @ (fl + fc)
            wb = (Wb * bJ).reshape(-1)
            we = (0.5 * Wb * (bJ + bJr)).reshape(-1)
            r = row.reshape(-1)
            for o, w in ((0, wb), (3, we)):
                np.add.at(vec[J, o + 0], r, c * w)
                np.add.at(vec[J, o + 1], r, s * w)
                np.add.at(vec[J, o + 2], r, w)
    return LocalForceSetup(vectors=vec, const=const, V_c=np.asarray(pc["V_c"], dtype=np.float64).copy())


def occupations(EigVal: np.ndarray, lambda_f: float, bet: float, elec_T_type: int) -> np.ndarray:
    """Occupations of src/occupations.m at the Fermi level: Fermi-Dirac (elec_T_type 0) or Gaussian
    smearing (1)."""
    x = bet * (np.asarray(EigVal, dtype=np.float64) - lambda_f)
    if elec_T_type == 0:
        return 0.5 * (1.0 - np.tanh(0.5 * x))            # 1 / (1 + e^x) without overflow
    return 0.5 * np.vectorize(math.erfc)(x)


def atomic_forces(gpu, setup: LocalForceSetup, phi: np.ndarray, occ: np.ndarray, wkpt, occfac: float) -> np.ndarray:
    """Drift-free atomic forces (n_atm x 3, Ha/bohr) of a converged SCF on the handle ``gpu``
    (``msparc.CyclixGPU`` holding the converged psi): ``phi`` the SCF's electrostatic potential
    (S.phi; after a converged ``cx_scf``, Veff - Vxc[rho]), ``occ`` the occupations packed like
    EigVal, ``wkpt`` one weight per block."""
    nat = setup.const.shape[0]
    P = gpu.field_projections(phi, setup.vectors[:, :3].reshape(3 * nat, -1)).reshape(nat, 3, 3)
    Q = gpu.field_projections(setup.V_c, setup.vectors[:, 3:].reshape(3 * nat, -1)).reshape(nat, 3, 3)
    F = setup.const.copy()
    for M in (P, Q):                      # M[J, v, d] = vector v of atom J . D_d field
        F[:, 0] -= M[:, 0, 0] - M[:, 1, 1]
        F[:, 1] -= M[:, 1, 0] + M[:, 0, 1]
        F[:, 2] -= M[:, 2, 2]
    F += gpu.nonlocal_force(occ, wkpt, occfac)
    F[:, 2] -= F[:, 2].mean()
    return F
