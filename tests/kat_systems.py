"""Bare Cyclix cells (no atoms, zero potential) for the known-answer tests of the oracle.

Grid conventions follow the reference: Dirichlet r with both end nodes
(``Nx = L1/dx + 1``, src/initialization.m:344), cyclic theta on ``L2 = 2 pi / n_cyc``,
periodic or helical z on ``L3 = Nz dz``.
"""
from __future__ import annotations

import numpy as np

from cyclix_msparc_gb300.cychel import CyclixS, cell_type, fd_weights, intg_weights


def bare_cell(Nx, Ny, Nz, *, xin=3.0, L1=4.0, n_cyc=12, L3=2.0, twist=0.0, kpts=((0.0, 0.0, 0.0),), FDn=6) -> CyclixS:
    cell_typ, BCx, BCy, BCz = cell_type(twist != 0.0)
    L2 = 2 * np.pi / n_cyc
    dx, dy, dz = L1 / (Nx - 1), L2 / Ny, L3 / Nz
    w1, w2 = fd_weights(FDn)
    W = intg_weights(Nx, Ny, Nz, BCy, BCz, xin, dx, dy, dz)
    kpt = np.array(kpts, dtype=float).reshape(-1, 3)
    S = CyclixS(Nx=Nx, Ny=Ny, Nz=Nz, FDn=FDn, cell_typ=cell_typ, BCx=BCx, BCy=BCy, BCz=BCz, dx=dx, dy=dy, dz=dz,
                xin=xin, twist=twist, L1=L1, L2=L2, L3=L3, w1=w1, w2=w2, W=W, Atoms=np.zeros((0, 3)), Atom=[],
                kptgrid=kpt, wkpt=np.ones(kpt.shape[0]) / kpt.shape[0], nspin=1)
    S.Veff = np.zeros((S.N, 1))
    return S


def grid_coords(S):
    """(r, theta, z) of every grid point in MATLAB column-major order (r fastest)."""
    r = S.xin + np.arange(S.Nx) * S.dx
    t = np.arange(S.Ny) * S.dy
    z = np.arange(S.Nz) * S.dz
    R, T, Z = np.meshgrid(r, t, z, indexing="ij")
    return R.reshape(-1, order="F"), T.reshape(-1, order="F"), Z.reshape(-1, order="F")


def tiny_cyclic_workload():
    """A tiny cyclic cell (16 x 8 x 10, 2 atoms, one Bloch block nu = 1, eta = 0.9)."""
    from cyclix_msparc_gb300.workloads import Workload
    return Workload("cyclic-tiny-16x8x10", 16, 8, 10, (6,), ((0.0, 1.0, 0.9),), 1, 6, 2, 12, L1=4.0, xin=4.0)


def tiny_helical_workload():
    """A tiny helical cell whose dense Hamiltonian is cheap (1280 points, 2 atoms, 2 blocks)."""
    from cyclix_msparc_gb300.workloads import Workload
    return Workload("helical-tiny-16x8x10", 16, 8, 10, (6, 6), ((0.0, 1.0, 0.0), (0.0, 0.0, 0.9)), 1, 6, 2, 4,
                    twist=0.05, L1=4.0, xin=4.0)


def xc_density(S, seed: int) -> np.ndarray:
    """A positive density with structure on every axis: the atomic superposition times a seeded
    smooth modulation, plus a seeded 2 % noise; 1 % of the points set to zero or below the 1e-14
    clip (the clipped branch of src/exchangeCorrelationPotential.m)."""
    rng = np.random.default_rng(seed)
    r = np.asarray(S.rho_at, dtype=np.float64).reshape(-1)
    i = np.arange(S.N)
    th = (i // S.Nx) % S.Ny * (2 * np.pi / S.Ny)
    z = i // (S.Nx * S.Ny) * (2 * np.pi / S.Nz)
    rho = np.abs(r) * (1.0 + 0.3 * np.sin(th + rng.uniform(0, 2 * np.pi)) * np.cos(z + rng.uniform(0, 2 * np.pi)))
    rho *= 1.0 + 0.02 * rng.standard_normal(S.N)
    low = rng.choice(S.N, S.N // 100, replace=False)
    rho[low] = rng.choice([0.0, 1e-16, -1e-12], low.size)
    return rho
