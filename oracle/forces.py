"""Oracle restatement of the atomic forces of a converged Cyclix SCF (src/atomicForce.m:1-364).

Test infrastructure only (see ``oracle/__init__.py``).  Paths relative to the reference project
root ``Cyclix_MS_200220/``.  The box quantities of each atom image (V_J, the reference potential,
their pseudocharges) are those of the deck setup (``cyclix_msparc_gb300.deck``); the force terms:

* local:  f_l = -sum_box W b_J (D phi - D V_J)                         (:111-113)
* correction:  f_c = 1/2 sum_box W [(b + b_ref)(D V_J,ref - D V_J) - (b_J + b_J,ref) D V_c]  (:114-119)
  both rotated back to the atom's own frame by RotM1^fac1 RotM2^fac2   (:120-127);
* nonlocal:  f_nl = -occfac 2 w_k sum_n occ_n gamma^T Re[<chi|psi_n> * (-<psi_n| D chi>)]
  with the Bloch-summed projector of each atom and its Cartesian gradient (:141-183).
D is the Cartesian gradient on the (r, theta, z) grid (Cychel/gradIndicesValues_cychel.m), with
Bloch phases at the theta and z wraps (Cychel/blochGradient_cychel.m); the x / y derivatives of
the projector use the vector-field operators of Cychel/div_gradvec_cychel.m, which rotate the
field by the wedge angle across the theta wrap.
"""
from __future__ import annotations

import math

import numpy as np
import scipy.sparse as sp

from cyclix_msparc_gb300 import deck as D
from cyclix_msparc_gb300.cychel import rot_z


def _grad_entries(S):
    """(row, col, value, theta-wrap flag, z-wrap flag) of the three gradient stencils, with the
    wrapped neighbour's side: -1 left, +1 right, 0 inside (Cychel/gradIndicesValues_cychel.m)."""
    Nx, Ny, Nz, n = S.Nx, S.Ny, S.Nz, S.FDn
    N = Nx * Ny * Nz
    i, j, k = np.meshgrid(np.arange(Nx), np.arange(Ny), np.arange(Nz), indexing="ij")
    i, j, k = (a.reshape(-1, order="F") for a in (i, j, k))
    row = i + Nx * (j + Ny * k)
    r = S.xin + i * S.dx
    ph = j * S.dy + S.twist * (k * S.dz)
    c, sn = np.cos(ph), np.sin(ph)
    ent = {d: [] for d in range(3)}
    for p in range(1, n + 1):
        w = S.w1[p]
        for sgn in (1, -1):
            ii = i + sgn * p
            ok = (ii >= 0) & (ii < Nx)
            col = ii + Nx * (j + Ny * k)
            z0 = np.zeros(N, int)
            for d, wt in ((0, c / S.dx), (1, sn / S.dx)):
                ent[d].append((row[ok], col[ok], (sgn * w * wt)[ok], z0[ok], z0[ok]))
            jr = j + sgn * p
            tw = np.where(jr < 0, -1, np.where(jr >= Ny, 1, 0))
            col = i + Nx * (np.mod(jr, Ny) + Ny * k)
            for d, wt in ((0, -sn / (r * S.dy)), (1, c / (r * S.dy)), (2, np.full(N, -S.twist / S.dy))):
                ent[d].append((row, col, sgn * w * wt, tw, z0))
            kr = k + sgn * p
            zw = np.where(kr < 0, -1, np.where(kr >= Nz, 1, 0))
            col = i + Nx * (j + Ny * np.mod(kr, Nz))
            ent[2].append((row, col, np.full(N, sgn * w / S.dz), z0, zw))
    out = []
    for d in range(3):
        out.append(tuple(np.concatenate([e[q] for e in ent[d]]) for q in range(5)))
    return out


def bloch_gradients(S, kvec, entries=None):
    """D_x, D_y, D_z with the Bloch phases exp(+-i k_theta L2) / exp(+-i k_z L3) on wrapped entries
    (Cychel/blochGradient_cychel.m)."""
    entries = entries or _grad_entries(S)
    N = S.N
    mats = []
    for (R, C, V, tw, zw) in entries:
        ph = np.exp(1j * kvec[1] * S.L2 * tw) * np.exp(1j * kvec[2] * S.L3 * zw)
        mats.append(sp.csr_matrix((V * ph, (R, C)), shape=(N, N)))
    return mats


def vector_gradient_ops(S, kvec, entries=None):
    """(M1, M2) of Cychel/div_gradvec_cychel.m: the x and y derivative stencils whose theta-wrapped
    entries rotate the (F1, F2) field by the wedge angle L2 and carry the Bloch phase."""
    entries = entries or _grad_entries(S)
    (R, C, V1, tw, _), (_, _, V2, _, _) = entries[0], entries[1]
    cL, sL = math.cos(S.L2), math.sin(S.L2)
    ph = np.exp(1j * kvec[1] * S.L2 * tw)
    m1 = np.where(tw < 0, (V1 * cL - V2 * sL) * ph, np.where(tw > 0, (V1 * cL + V2 * sL) * ph, V1 + 0j))
    m2 = np.where(tw < 0, (V2 * cL + V1 * sL) * ph, np.where(tw > 0, (V2 * cL - V1 * sL) * ph, V2 + 0j))
    N = S.N
    return sp.csr_matrix((m1, (R, C)), shape=(N, N)), sp.csr_matrix((m2, (R, C)), shape=(N, N))


def _box_gradient(S, V, xx, yy, zz):
    """Cartesian gradient of V on the interior of a box with FDn margins (Cychel/dpseudopot_cychel.m)."""
    n = S.FDn
    nx, ny, nz = V.shape
    I, J, K = slice(n, nx - n), slice(n, ny - n), slice(n, nz - n)
    Rg, Tg, Zg = np.meshgrid(xx[I], yy[J], zz[K], indexing="ij")
    ph = Tg + S.twist * Zg
    c11, c12 = np.cos(ph) / S.dx, -np.sin(ph) / (Rg * S.dy)
    c21, c22 = np.sin(ph) / S.dx, np.cos(ph) / (Rg * S.dy)
    c31, c32 = -S.twist / S.dy, 1.0 / S.dz
    gx = np.zeros_like(Rg)
    gy = np.zeros_like(Rg)
    gz = np.zeros_like(Rg)
    for p in range(1, n + 1):
        w = S.w1[p]
        dr = V[n + p:nx - n + p, J, K] - V[n - p:nx - n - p, J, K]
        dt = V[I, n + p:ny - n + p, K] - V[I, n - p:ny - n - p, K]
        dz = V[I, J, n + p:nz - n + p] - V[I, J, n - p:nz - n - p]
        gx += w * (c11 * dr + c12 * dt)
        gy += w * (c21 * dr + c22 * dt)
        gz += w * (c31 * dt + c32 * dz)
    return gx, gy, gz


def _rot_pow(R, p):
    return np.linalg.matrix_power(R, p) if p >= 0 else np.linalg.matrix_power(R.T, -p)


def projector_fields(S, J, k):
    """(Ck, R1, R2) of atom J at Bloch vector k, N x angnum each: the Bloch sum of the image
    projectors, and the same weighted by ROT(1,1) and ROT(1,2) of each image's rotation
    (src/atomicForce.m:265-277)."""
    RotM1, RotM2 = rot_z(S.L2), rot_z(S.twist * S.L3)
    A = S.Atom[J]
    R1 = np.zeros((S.N, A.angnum), complex)
    R2 = np.zeros((S.N, A.angnum), complex)
    Ck = np.zeros((S.N, A.angnum), complex)
    for img in A.rcImage:
        disp = S.Atoms[J] - img.coordinates
        ph = np.exp(-1j * float(np.dot(k, disp)))
        ROT = _rot_pow(RotM1, int(round(disp[1] / S.L2))) @ _rot_pow(RotM2, int(round(disp[2] / S.L3)))
        pos = img.rc_pos - 1
        R1[pos] += ROT[0, 0] * img.Chi_mat * ph
        R2[pos] += ROT[0, 1] * img.Chi_mat * ph
        Ck[pos] += img.Chi_mat * ph
    return Ck, R1, R2


def projector_gradients(S, J, k, entries=None, ops=None):
    """(Ck, D_x, D_y, D_z) of atom J at Bloch vector k (src/atomicForce.m:278-280); ``ops`` the
    (M1, M2, G_z) of k when already built."""
    if ops is None:
        entries = entries or _grad_entries(S)
        ops = vector_gradient_ops(S, k, entries) + (bloch_gradients(S, k, entries)[2],)
    M1, M2, Gz = ops
    Ck, R1, R2 = projector_fields(S, J, k)
    return Ck, M1 @ R1 + M2 @ R2, -(M1 @ R2) + M2 @ R1, Gz @ Ck


def nonlocal_forces(S, kvecs, wkpt, psis, occ, occfac, entries=None):
    """Nonlocal atomic forces (n_atm, 3) of src/atomicForce.m:254-300: per Bloch block b (vector
    kvecs[b], weight wkpt[b], psi N x Ns, occupations occ[b]),
    F_J -= occfac 2 w_b gamma^T Re[conj(<psi|W Ck>) * (-<psi|W D Ck>)] occ."""
    entries = entries or _grad_entries(S)
    F_nl = np.zeros((S.n_atm, 3))
    for b, k in enumerate(kvecs):
        psi = psis[b]
        PsiW = (np.conj(psi) * S.W[:, None]).T                   # Ns x N
        fk = np.zeros((S.n_atm, 3))
        ops = vector_gradient_ops(S, k, entries) + (bloch_gradients(S, k, entries)[2],)
        for J, A in enumerate(S.Atom):
            Ck, DCx, DCy, DCz = projector_gradients(S, J, k, ops=ops)
            i1 = (np.conj(PsiW) @ np.conj(Ck)).T                  # angnum x Ns
            for q, DC in enumerate((DCx, DCy, DCz)):
                i2 = -(PsiW @ DC).T
                fk[J, q] = float(A.gamma_Jl @ np.real(i1 * i2) @ occ[b])
        F_nl -= occfac * 2 * wkpt[b] * fk
    return F_nl


def atomic_forces(d, psis, occ, phi):
    """Drift-free forces (n_atm, 3) in Ha/bohr of the converged SCF of a loaded deck ``d``: ``psis``
    and ``occ`` per Bloch block (W-normalised psi, N x Ns), ``phi`` the electrostatic potential.
    Also returns the three terms before the drift correction."""
    S, pc = d.S, d.pseudo
    n = S.FDn
    ent = _grad_entries(S)
    G0 = bloch_gradients(S, (0.0, 0.0, 0.0), ent)
    Dphi = [G @ phi for G in G0]
    DVc = [(G @ pc["V_c"]).real for G in G0]
    Dphi = [v.real for v in Dphi]
    RotM1, RotM2 = rot_z(S.L2), rot_z(S.twist * S.L3)
    atom_type = S.extra["atom_type"]
    F_loc = np.zeros((S.n_atm, 3))
    F_cor = np.zeros((S.n_atm, 3))
    for J in range(S.n_atm):
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
            bJ = -D._pseudocharge_lap(S, V, float(xx[0])) / (4 * math.pi)
            bJr = -D._pseudocharge_lap(S, Vr, float(xx[0])) / (4 * math.pi)
            dV = _box_gradient(S, V, xx, yy, zz)
            dVr = _box_gradient(S, Vr, xx, yy, zz)
            I, Jj, K = np.meshgrid(np.arange(is_, ie + 1), np.arange(js, je + 1), np.arange(ks, ke + 1), indexing="ij")
            row = ((K - 1) * S.Nx * S.Ny + (Jj - 1) * S.Nx + I - 1)
            Wb, bb, bref = S.W[row], S.b[row], pc["b_ref"][row]
            fl = np.array([-np.sum(Wb * bJ * (Dphi[q][row] - dV[q])) for q in range(3)])
            fc = np.array([0.5 * np.sum(Wb * ((bb + bref) * (dVr[q] - dV[q]) - (bJ + bJr) * DVc[q][row])) for q in range(3)])
            fac1 = int(round((y0 - y0i) / S.L2))
            fac2 = int(round((z0 - z0i) / S.L3))
            ROT = _rot_pow(RotM1, fac1) @ _rot_pow(RotM2, fac2)
            F_loc[J] += ROT @ fl
            F_cor[J] += ROT @ fc
    F_nl = nonlocal_forces(S, S.kptgrid, S.wkpt, psis, occ, S.occfac, ent)
    F = F_loc + F_cor + F_nl
    # drift-free forces: the mean force is removed along z, the translation a Cyclix cell has
    # (src/electronicGroundState.m:108-115)
    F[:, 2] -= F[:, 2].mean()
    return F, {"local": F_loc, "correction": F_cor, "nonlocal": F_nl}
