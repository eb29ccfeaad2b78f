"""Host-side Cyclix discretisation: the parts of the reference's ``S`` struct that
the GPU path consumes.

This module builds, with vectorised NumPy, the same quantities that the
reference computes during initialisation and hands to the Hamiltonian:

* central finite-difference weights ``w1`` / ``w2``
  (reference: src/initialization.m:403-419);
* the (r, theta, z) grid with the Dirichlet +1 radial node
  (src/initialization.m:330-345) and the cyclic / helical cell types
  (src/initialization.m:286-295);
* the quadrature weights ``W`` (Cychel/intgWts_cychel.m:1-14);
* the Bloch wavenumbers of a cyclic / helical cell (integer ``nu`` along
  theta, Monkhorst-Pack ``eta`` along z, optional time-reversal reduction;
  src/initialization.m:1591-1682).

The field names follow the reference's struct ``S`` so that a MEX shim, the
ctypes host mirror and the tests read alike.  Nothing here touches a GPU.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np


def fd_weights(FDn: int) -> tuple[np.ndarray, np.ndarray]:
    """Central FD weights of order 2*FDn for the first and second derivative.

    Returns ``(w1, w2)``, each of length FDn+1, indexed by the offset ``q``
    (``w[0]`` is the centre).  Closed form of src/initialization.m:403-419:
    ``w2[k] = 2(-1)^(k+1) (FDn!)^2 / (k^2 (FDn-k)! (FDn+k)!)``,
    ``w2[0] = -2 sum_k 1/k^2``, ``w1[k] = (-1)^(k+1) (FDn!)^2 / (k (FDn-k)! (FDn+k)!)``.
    """
    if FDn < 1:
        raise ValueError("FDn must be >= 1")
    f = math.factorial
    w1 = np.zeros(FDn + 1)
    w2 = np.zeros(FDn + 1)
    for k in range(1, FDn + 1):
        ratio = f(FDn) ** 2 / (f(FDn - k) * f(FDn + k))
        sgn = 1.0 if (k + 1) % 2 == 0 else -1.0
        w2[k] = 2.0 * sgn * ratio / (k * k)
        w2[0] -= 2.0 / (k * k)
        w1[k] = sgn * ratio / k
    return w1, w2


@dataclass
class RcImage:
    """One periodic image of an atom whose projector ball reaches the cell.

    Mirrors ``S.Atom(J).rcImage(img)`` (src/calculate_nloc_projector.m:185-198).
    ``rc_pos`` holds 1-based linear grid indices, as MATLAB does.
    """
    coordinates: np.ndarray          # (3,) image position in (r, theta, z)
    rc_pos: np.ndarray               # (rc_n_nodes,) int64, 1-based
    Chi_mat: np.ndarray              # (rc_n_nodes, angnum) float64

    @property
    def rc_n_nodes(self) -> int:
        return int(self.rc_pos.shape[0])


@dataclass
class AtomNL:
    """Nonlocal data of one atom: ``S.Atom(J)`` (src/calculate_nloc_projector.m:252-277)."""
    angnum: int
    gamma_Jl: np.ndarray             # (angnum,)
    rcImage: list = field(default_factory=list)

    @property
    def n_image_rc(self) -> int:
        return len(self.rcImage)


@dataclass
class CyclixS:
    """The subset of the reference struct ``S`` used by the CheFSI path."""
    Nx: int
    Ny: int
    Nz: int
    FDn: int
    cell_typ: int
    BCx: int
    BCy: int
    BCz: int
    dx: float
    dy: float
    dz: float
    xin: float
    twist: float
    L1: float
    L2: float
    L3: float
    w1: np.ndarray
    w2: np.ndarray
    W: np.ndarray
    Atoms: np.ndarray                # (n_atm, 3) positions in (r, theta, z)
    Atom: list                       # list[AtomNL]
    kptgrid: np.ndarray              # (tnkpt, 3)
    wkpt: np.ndarray                 # (tnkpt,)
    nspin: int = 1
    Nev: int = 0
    npl: int = 0
    Veff: np.ndarray | None = None   # (N, nspin)
    # SCF extras (only the full-SCF workload fills these)
    b: np.ndarray | None = None
    rho_at: np.ndarray | None = None
    NegCharge: float = 0.0
    Eself: float = 0.0
    E_corr: float = 0.0
    bet: float = 0.0
    elec_T_type: int = 1
    occfac: float = 2.0
    n_atm: int = 0
    extra: dict = field(default_factory=dict)

    @property
    def N(self) -> int:
        return self.Nx * self.Ny * self.Nz

    @property
    def tnkpt(self) -> int:
        return int(self.kptgrid.shape[0])

    @property
    def xout(self) -> float:
        return self.xin + self.L1


def periodic_images(S, x0: float, y0: float, z0: float, rby: float, rbz: float) -> list:
    """Periodic images of an atom whose box of half-widths (., rby, rbz) may reach the cell, in the
    reference's ndgrid order (theta before z; src/calculate_b_guessRho_Eself.m:38-69,
    src/calculate_nloc_projector.m:50-81).  Theta images only for a periodic theta, z images only
    for a periodic z."""
    nyl = math.floor((y0 + rby) / S.L2) if S.BCy == 0 else 0
    nyr = math.floor((S.L2 - y0 + rby - S.dy) / S.L2) if S.BCy == 0 else 0
    nzl = math.floor((z0 + rbz) / S.L3) if S.BCz == 0 else 0
    nzr = math.floor((S.L3 - z0 + rbz - S.dz) / S.L3) if S.BCz == 0 else 0
    return [(x0, y0 + j * S.L2, z0 + k * S.L3) for k in range(-nzl, nzr + 1) for j in range(-nyl, nyr + 1)]


def image_reaches_cell(S, x0i: float, y0i: float, z0i: float, rb) -> bool:
    """Whether the box of half-widths rb around an image overlaps the cell
    (src/calculate_nloc_projector.m:99-102; yin = zin = 0)."""
    rbx, rby, rbz = rb
    in_x = ((x0i - S.xin) - S.L1 + S.dx <= rbx) or (abs(x0i - S.xin) <= rbx)
    in_y = (y0i - S.L2 + S.dy <= rby) or (abs(y0i) <= rby)
    in_z = (z0i - S.L3 + S.dz <= rbz) or (abs(z0i) <= rbz)
    return in_x and in_y and in_z


def clipped_box(S, x0i: float, y0i: float, z0i: float, rb) -> tuple:
    """1-based (start, end) grid index ranges of the box of half-widths rb around an image,
    clipped to the cell (src/calculate_b_guessRho_Eself.m:81-103); empty when end < start."""
    rbx, rby, rbz = rb
    ii = (max(math.ceil(((x0i - S.xin) - rbx) / S.dx) + 1, 1), min(math.floor(((x0i - S.xin) + rbx) / S.dx) + 1, S.Nx))
    jj = (max(math.ceil((y0i - rby) / S.dy) + 1, 1), min(math.floor((y0i + rby) / S.dy) + 1, S.Ny))
    kk = (max(math.ceil((z0i - rbz) / S.dz) + 1, 1), min(math.floor((z0i + rbz) / S.dz) + 1, S.Nz))
    return ii, jj, kk


def split_projector_columns(atoms: list, width: int = 4) -> tuple[list, list]:
    """Atoms whose projector columns fit ``width``.

    The Kleinman-Bylander term sum_J sum_c gamma_Jc |chi_Jc><chi_Jc| (src/h_nonlocal_vector_mult.m:
    24-43) is a sum over the columns c of each atom with a diagonal gamma, so an atom with more
    columns (a psp8 atom with two projectors per l has 8, one with l <= 2 has 18) equals several
    atoms at the same position and images holding consecutive slices of its columns.  Returns the
    list of such atoms and, for each, the index of the atom it came from.
    """
    out, origin = [], []
    for J, A in enumerate(atoms):
        if A.angnum <= width:
            out.append(A)
            origin.append(J)
            continue
        for c0 in range(0, A.angnum, width):
            c1 = min(c0 + width, A.angnum)
            imgs = [RcImage(img.coordinates, img.rc_pos, np.ascontiguousarray(img.Chi_mat[:, c0:c1])) for img in A.rcImage]
            out.append(AtomNL(c1 - c0, np.asarray(A.gamma_Jl[c0:c1]), imgs))
            origin.append(J)
    return out, origin


def cell_type(helical: bool) -> tuple[int, int, int, int]:
    """(cell_typ, BCx, BCy, BCz) for ``BC: D C P`` (cyclic) or ``D C H`` (cyclic+helical).

    src/initialization.m:286-295: BC 5 -> (3; 1,0,0), BC 7 -> (5; 1,0,0).
    """
    return (5, 1, 0, 0) if helical else (3, 1, 0, 0)


def radial_nodes(S_or_xin, dx=None, Nx=None) -> np.ndarray:
    if dx is None:
        S = S_or_xin
        return S.xin + np.arange(S.Nx) * S.dx
    return S_or_xin + np.arange(Nx) * dx


def intg_weights(Nx, Ny, Nz, BCy, BCz, xin, dx, dy, dz) -> np.ndarray:
    """Quadrature weights ``W = kron(Wz, kron(Wy, Wx))`` (Cychel/intgWts_cychel.m:1-14).

    ``Wx = r dx`` with the trapezoid end corrections ``0.5 r dx +- dx^2/8``;
    ``Wy``, ``Wz`` are ``dy``, ``dz`` halved at Dirichlet ends.
    """
    r = xin + np.arange(Nx) * dx
    Wx = r * dx
    Wx[0] = 0.5 * xin * dx + 0.125 * dx * dx
    Wx[Nx - 1] = 0.5 * (xin + (Nx - 1) * dx) * dx - 0.125 * dx * dx
    Wy = np.full(Ny, dy)
    Wy[0] *= (1 - BCy * 0.5)
    Wy[Ny - 1] *= (1 - BCy * 0.5)
    Wz = np.full(Nz, dz)
    Wz[0] *= (1 - BCz * 0.5)
    Wz[Nz - 1] *= (1 - BCz * 0.5)
    return np.kron(Wz, np.kron(Wy, Wx))


def cyclix_kpoints(nkpt, L1, L2, L3, kptshift=(0.0, 0.0, 0.0), time_reversal=True):
    """Bloch wavenumbers of a cyclic / helical cell (src/initialization.m:1591-1682).

    x: Monkhorst-Pack (ABINIT convention) scaled by 2pi/L1; y (theta): integers
    ``round((2pi/L2) * (0..n-1)/n)``; z: MP grid shifted by ``kptshift[2]/n`` and
    mapped into (-1/2, 1/2], scaled by 2pi/L3.  With ``time_reversal`` the
    reference's pairing rule (sums of x, z equal to 0 and y equal to 0 or
    2pi/L2) halves the set and doubles the kept weights.
    Returns ``(kptgrid (tnkpt,3), wkpt (tnkpt,))`` in the reference's ndgrid
    order (x fastest).
    """
    n1, n2, n3 = (int(v) for v in nkpt)
    eps = np.finfo(float).eps

    def mp1(n):
        s = -((n - 1) // 2)
        return np.arange(s, s + n, dtype=float)

    kx = (1.0 / n1) * mp1(n1)
    ky = (1.0 / n2) * np.arange(n2, dtype=float)
    kz = (1.0 / n3) * mp1(n3)
    kz = kz + kptshift[2] * (1.0 / n3)
    kz = np.mod(kz + 0.5 - eps, 1.0) - 0.5 + eps
    sumx, sumy, sumz = 0.0, 2 * np.pi / L2, 0.0
    kx = (2 * np.pi / L1) * kx
    # MATLAB's round (half away from zero; ky >= 0 here), not NumPy's round-half-to-even:
    # an odd wedge order puts nu exactly on .5 (n_cyc = 5, 2 points: 2.5 -> 3)
    ky = np.floor((2 * np.pi / L2) * ky + 0.5)
    kz = (2 * np.pi / L3) * kz
    KX, KY, KZ = np.meshgrid(kx, ky, kz, indexing="ij")
    kpt = np.stack([KX.reshape(-1, order="F"), KY.reshape(-1, order="F"), KZ.reshape(-1, order="F")], axis=1)
    tn = n1 * n2 * n3
    w = np.ones(tn) / tn
    if time_reversal:
        tol = 1e-8
        drop = np.zeros(tn, bool)
        dbl = np.zeros(tn, bool)
        for i in range(tn):
            for j in range(i + 1, tn):
                if (abs(kpt[i, 0] + kpt[j, 0] - sumx) < tol
                        and (abs(kpt[i, 1] + kpt[j, 1] - sumy) < tol or abs(kpt[i, 1] + kpt[j, 1]) < tol)
                        and abs(kpt[i, 2] + kpt[j, 2] - sumz) < tol):
                    drop[i] = True
                    dbl[j] = True
        w[dbl] *= 2
        kpt = kpt[~drop]
        w = w[~drop]
    return kpt, w


def noncart2cart(S, X: np.ndarray) -> np.ndarray:
    """(r, theta, z) -> Cartesian with the helical twist (Cychel/coordinateTransformation_cychel.m:3-7)."""
    X = np.atleast_2d(X)
    ang = X[:, 1] + S.twist * X[:, 2]
    return np.stack([X[:, 0] * np.cos(ang), X[:, 0] * np.sin(ang), X[:, 2]], axis=1)


def rot_z(theta: float) -> np.ndarray:
    c, s = math.cos(theta), math.sin(theta)
    return np.array([[c, -s, 0.0], [s, c, 0.0], [0.0, 0.0, 1.0]])


def real_ylm(l: int, m: int, X, Y, Z) -> np.ndarray:
    """Real spherical harmonics for l <= 2 (src/sphericalHarmonics.m:58-100): the standard real
    combinations, normalised to 1 on the unit sphere, of the direction (X, Y, Z) / r."""
    r = np.sqrt(X * X + Y * Y + Z * Z)
    if l == 0:
        return 0.5 * math.sqrt(1.0 / math.pi) * np.ones_like(X)
    if l == 1:
        c = math.sqrt(3.0 / (4.0 * math.pi))
        return c * {-1: Y, 0: Z, 1: X}[m] / r
    if l == 2:
        r2 = r * r
        c = 0.5 * math.sqrt(15.0 / math.pi)
        if m == -2:
            return c * X * Y / r2
        if m == -1:
            return c * Y * Z / r2
        if m == 0:
            return 0.25 * math.sqrt(5.0 / math.pi) * (2 * Z * Z - X * X - Y * Y) / r2
        if m == 1:
            return c * Z * X / r2
        return 0.25 * math.sqrt(15.0 / math.pi) * (X * X - Y * Y) / r2
    raise ValueError("projectors with l > 2 are not supported")
