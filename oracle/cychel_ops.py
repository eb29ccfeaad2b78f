"""Oracle restatement of the Cyclix Hamiltonian and the CheFSI eigensolver.

Test infrastructure only (see ``oracle/__init__.py``).  Paths are relative to
the reference project root ``Cyclix_MS_200220/``.  The reference's per-slice
and per-state loops (``for i = 1:l_zs``) are written here as the same sparse
products applied along one grid axis at a time, which is the same arithmetic.
"""
from __future__ import annotations

import math

import numpy as np
import scipy.linalg as sla
import scipy.sparse as sp
import scipy.sparse.linalg as spla


# ---------------------------------------------------------------------------
# src/initialization.m:403-419 -- FD weights, written as the reference's loop
# ---------------------------------------------------------------------------
def fd_weights(FDn: int):
    w2 = np.zeros(FDn + 1)
    for k in range(1, FDn + 1):
        w2[k] = (2 * (-1) ** (k + 1)) * (math.factorial(FDn) ** 2) / (
            k * k * math.factorial(FDn - k) * math.factorial(FDn + k))
        w2[0] = w2[0] - 2 * (1 / (k * k))
    w1 = np.zeros(FDn + 1)
    for k in range(1, FDn + 1):
        w1[k] = ((-1) ** (k + 1)) * (math.factorial(FDn) ** 2) / (
            k * math.factorial(FDn - k) * math.factorial(FDn + k))
    return w1, w2


# ---------------------------------------------------------------------------
# Cychel/intgWts_cychel.m:1-14
# ---------------------------------------------------------------------------
def intg_wts_cychel(S):
    Nx, Ny, Nz = S.Nx, S.Ny, S.Nz
    W_x = np.array([(S.xin + i * S.dx) * S.dx for i in range(Nx)])
    W_x[0] = 0.5 * S.xin * S.dx + 0.125 * S.dx * S.dx
    W_x[Nx - 1] = 0.5 * (S.xin + (Nx - 1) * S.dx) * S.dx - 0.125 * S.dx * S.dx
    W_y = np.ones(Ny) * S.dy
    W_y[0] = W_y[0] * (1 - S.BCy * 0.5)
    W_y[Ny - 1] = W_y[Ny - 1] * (1 - S.BCy * 0.5)
    W_z = np.ones(Nz) * S.dz
    W_z[0] = W_z[0] * (1 - S.BCz * 0.5)
    W_z[Nz - 1] = W_z[Nz - 1] * (1 - S.BCz * 0.5)
    return np.kron(W_z, np.kron(W_y, W_x))


# ---------------------------------------------------------------------------
# Cychel/lapIndicesValues_1d_cychel.m:1-262 (indices here are 1-based, as in MATLAB)
# ---------------------------------------------------------------------------
def _second_derivative_entries(n, n0, w2, coef):
    I, II, V = [], [], []
    for ii in range(1, n + 1):
        I.append(ii); II.append(ii); V.append(w2[0] * coef)
        for q in range(1, n0 + 1):
            I.append(ii); II.append(ii + q); V.append(w2[q] * coef)
            I.append(ii); II.append(ii - q); V.append(w2[q] * coef)
    return np.array(I), np.array(II), np.array(V)


def _first_derivative_entries(n, n0, w1, coef_of_row):
    G, R, A = [], [], []
    for ii in range(1, n + 1):
        c = coef_of_row(ii)
        for q in range(1, n0 + 1):
            G.append(ii); R.append(ii + q); A.append(w1[q] * c)
            G.append(ii); R.append(ii - q); A.append(-w1[q] * c)
    return np.array(G), np.array(R), np.array(A)


def lap_indices_values_1d_cychel(S):
    T = {}
    n0, w1, w2 = S.FDn, S.w1, S.w2
    Nx, Ny, Nz = S.Nx, S.Ny, S.Nz
    # D_xx (Dirichlet r: out-of-range entries dropped, :53-54)
    I, II, V = _second_derivative_entries(Nx, n0, w2, 1 / S.dx ** 2)
    keep = (II >= 1) & (II <= Nx)
    T["I_11"], T["II_11"], T["V_11"] = I[keep], II[keep], V[keep]
    # D_yy (:56-99)
    I, II, V = _second_derivative_entries(Ny, n0, w2, 1 / S.dy ** 2)
    if S.BCy == 1:
        keep = (II >= 1) & (II <= Ny)
        T["I_22"], T["II_22"], T["V_22"] = I[keep], II[keep], V[keep]
    else:
        T["isOutl_22"], T["isOutr_22"] = II < 1, II > Ny
        T["I_22"], T["II_22"], T["V_22"] = I, np.mod(II + (Ny - 1), Ny) + 1, V
    if S.cell_typ in (4, 5):                                  # :101-103
        T["V_22"] = T["V_22"] * (S.twist * S.twist)
    # D_zz (:105-148)
    I, II, V = _second_derivative_entries(Nz, n0, w2, 1 / S.dz ** 2)
    if S.BCz == 1:
        keep = (II >= 1) & (II <= Nz)
        T["I_33"], T["II_33"], T["V_33"] = I[keep], II[keep], V[keep]
    else:
        T["isOutl_33"], T["isOutr_33"] = II < 1, II > Nz
        T["I_33"], T["II_33"], T["V_33"] = I, np.mod(II + (Nz - 1), Nz) + 1, V
    # x gradient (1/r) d/dx (:154-180)
    G, R, A = _first_derivative_entries(Nx, n0, w1, lambda ii: 1 / ((S.xin + (ii - 1) * S.dx) * S.dx))
    keep = (R >= 1) & (R <= Nx)
    T["I_1"], T["II_1"], T["V_1"] = G[keep], R[keep], A[keep]
    # y gradient, coefficient -2*twist/dy (:182-214)
    G, R, A = _first_derivative_entries(Ny, n0, w1, lambda jj: -2 * S.twist / S.dy)
    if S.BCy == 1:
        keep = (R >= 1) & (R <= Ny)
        T["I_2"], T["II_2"], T["V_2"] = G[keep], R[keep], A[keep]
    else:
        T["isOutl_2"], T["isOutr_2"] = R < 1, R > Ny
        T["I_2"], T["II_2"], T["V_2"] = G, np.mod(R + (Ny - 1), Ny) + 1, A
    # z gradient (:217-252)
    G, R, A = _first_derivative_entries(Nz, n0, w1, lambda kk: 1 / S.dz)
    if S.BCz == 1:
        keep = (R >= 1) & (R <= Nz)
        T["I_3"], T["II_3"], T["V_3"] = G[keep], R[keep], A[keep]
    else:
        T["isOutl_3"], T["isOutr_3"] = R < 1, R > Nz
        T["I_3"], T["II_3"], T["V_3"] = G, np.mod(R + (Nz - 1), Nz) + 1, A
    # 1/r^2 (:254-261)
    Rr = S.xin + np.arange(Nx) * S.dx
    if S.cell_typ == 3:
        r2inv = 1.0 / (Rr * Rr)
    else:
        r2inv = (1 / (S.twist * S.twist)) * (1.0 / (Rr * Rr))
    T["R2inv"] = sp.diags(r2inv, 0, shape=(Nx, Nx), format="csr")
    return T


# ---------------------------------------------------------------------------
# src/blochLaplacian_1d.m:1-124
# ---------------------------------------------------------------------------
def bloch_laplacian_1d(S, T, kptvec):
    Nx, Ny, Nz = S.Nx, S.Ny, S.Nz

    def phases(k, L):
        if k == 0:
            return 1.0, 1.0
        return np.exp(-1j * k * L), np.exp(1j * k * L)

    xl, xr = phases(kptvec[0], S.L1)
    yl, yr = phases(kptvec[1], S.L2)
    zl, zr = phases(kptvec[2], S.L3)

    def build(I, II, V, n, BC, outl, outr, pl, pr):
        V = V.astype(complex) if (BC == 0 and (pl != 1.0 or pr != 1.0)) else V.astype(float)
        if BC == 0:
            V = V.copy()
            V[T[outl]] = V[T[outl]] * pl
            V[T[outr]] = V[T[outr]] * pr
        return sp.csr_matrix((V, (I - 1, II - 1)), shape=(n, n))

    DL11 = sp.csr_matrix((T["V_11"], (T["I_11"] - 1, T["II_11"] - 1)), shape=(Nx, Nx))   # BCx = 1
    DL22 = build(T["I_22"], T["II_22"], T["V_22"], Ny, S.BCy, "isOutl_22", "isOutr_22", yl, yr)
    DL33 = build(T["I_33"], T["II_33"], T["V_33"], Nz, S.BCz, "isOutl_33", "isOutr_33", zl, zr)
    DG1 = sp.csr_matrix((T["V_1"], (T["I_1"] - 1, T["II_1"] - 1)), shape=(Nx, Nx))
    DG2 = build(T["I_2"], T["II_2"], T["V_2"], Ny, S.BCy, "isOutl_2", "isOutr_2", yl, yr)
    DG3 = build(T["I_3"], T["II_3"], T["V_3"], Nz, S.BCz, "isOutl_3", "isOutr_3", zl, zr)
    return DL11, DL22, DL33, DG1, DG2, DG3


# ---------------------------------------------------------------------------
# Cychel/lapVec_cychel.m:1-52 (dispatched from src/lapVec.m:59-60)
# ---------------------------------------------------------------------------
def _along(D, X4, axis):
    """out[..., j, ...] = sum_k D[j, k] X[..., k, ...] along ``axis`` of a 4-D block."""
    Xm = np.moveaxis(X4, axis, 0)
    sh = Xm.shape
    out = D @ Xm.reshape(sh[0], -1)
    return np.moveaxis(np.asarray(out).reshape(sh), 0, axis)


def lapvec_cychel(DL11, DL22, DL33, DG1, DG2, DG3, X, S, T):
    Nx, Ny, Nz = S.Nx, S.Ny, S.Nz
    Ns = X.shape[1]
    X4 = X.reshape((Nx, Ny, Nz, Ns), order="F")
    r2 = T["R2inv"].diagonal()
    if S.cell_typ == 3:
        # Hlx1 = (DL11+DG1)*X1 + R2inv*X1*DL22.' ; then + X2*DL33.'   (:19-33)
        H = _along(DL11 + DG1, X4, 0)
        H = H + r2[:, None, None, None] * _along(DL22, X4, 1)
        H = H + _along(DL33, X4, 2)
    else:
        # (:34-52) adds X1*DL22.' and the cross term (X1*DG2.')*DG3.'
        t = _along(DL22, X4, 1)
        H = _along(DL11 + DG1, X4, 0) + t + r2[:, None, None, None] * t
        H2 = _along(DG2, X4, 1)
        H = H + _along(DL33, X4, 2) + _along(DG3, H2, 2)
    return H.reshape((Nx * Ny * Nz, Ns), order="F")


# ---------------------------------------------------------------------------
# src/h_nonlocal_vector_mult.m:1-43
# ---------------------------------------------------------------------------
def h_nonlocal_vector_mult(DL11, DL22, DL33, DG1, DG2, DG3, Veff, X, S, T, kptvec):
    X = np.asarray(X)
    Hnlx = -0.5 * lapvec_cychel(DL11, DL22, DL33, DG1, DG2, DG3, X, S, T) + Veff[:, None] * X
    fac = 1.0 if (kptvec[0] == 0 and kptvec[1] == 0 and kptvec[2] == 0) else 1.0j
    if not np.iscomplexobj(Hnlx) and fac != 1.0:
        Hnlx = Hnlx.astype(complex)
    for J in range(len(S.Atom)):
        A = S.Atom[J]
        CX = np.zeros((A.angnum, X.shape[1]), dtype=complex if (fac != 1.0 or np.iscomplexobj(X)) else float)
        for img in A.rcImage:
            pos = img.rc_pos - 1
            ph = np.exp(np.dot(kptvec, (S.Atoms[J, :] - img.coordinates) * fac))
            CX = CX + (img.Chi_mat * S.W[pos][:, None]).T @ X[pos, :] * ph
        CX = CX * A.gamma_Jl[:, None]
        for img in A.rcImage:
            pos = img.rc_pos - 1
            Chi = img.Chi_mat * np.exp(-np.dot(kptvec, (S.Atoms[J, :] - img.coordinates) * fac))
            Hnlx[pos, :] = Hnlx[pos, :] + Chi @ CX
    return Hnlx


class Hamiltonian:
    """The operator of one (k-point, spin) block: ``Hfun`` in src/eigSolver.m:41-42."""

    def __init__(self, S, kptvec, Veff):
        self.S = S
        self.T = lap_indices_values_1d_cychel(S)
        self.k = np.asarray(kptvec, dtype=float)
        self.D = bloch_laplacian_1d(S, self.T, self.k)
        self.Veff = np.asarray(Veff, dtype=float)

    def __call__(self, X):
        X = np.asarray(X)
        one = X.ndim == 1
        if one:
            X = X[:, None]
        Y = h_nonlocal_vector_mult(*self.D, self.Veff, X, self.S, self.T, self.k)
        return Y[:, 0] if one else Y

    def dense(self):
        N = self.S.N
        return self(np.eye(N, dtype=complex))


# ---------------------------------------------------------------------------
# src/chebyshev_filter.m:1-44 (argument order: a = cutoff, b = upper bound, a0 = lower bound)
# ---------------------------------------------------------------------------
def chebyshev_filter(X, m, a, b, a0, H):
    e = (b - a) / 2
    c = (b + a) / 2
    sigma = e / (a0 - c)
    sigma1 = sigma
    gamma = 2 / sigma1
    HX = H(X)
    Y = (sigma1 / e) * (HX - c * X)
    ii = 2
    while ii <= m:
        sigma2 = 1 / (gamma - sigma)
        HX = H(Y)
        Ynew = (2 * sigma2 / e) * (HX - c * Y) - ((sigma * sigma2) * X)
        X = Y
        Y = Ynew
        sigma = sigma2
        ii += 1
    return Y


def matlab_rand(seed: int, n: int) -> np.ndarray:
    """MATLAB ``rng(seed); rand(n,1)`` (Mersenne twister, 53-bit doubles)."""
    return np.random.RandomState(seed).random_sample(n)


def spectral_bounds(H, N, ks, tol=1e-2, maxit=300, complex_op=True):
    """eigs(Hfun,N,1,'lr'/'sr',opts) bounds of src/eigSolver.m:47-67 (first SCF step).

    ``bup = 1.01 * real(lambda_lr)``, ``a0 = real(lambda_sr) - 0.1``; v0 = rand(N,1)
    after ``rng(ks+1)`` (ks 1-based).  ARPACK is SciPy's; MATLAB's ARPACK build
    is closed and unversioned, so these bounds agree only to the tolerance.
    """
    v0 = matlab_rand(ks + 1, N)
    dt = complex if complex_op else float
    op = spla.LinearOperator((N, N), matvec=lambda x: H(np.asarray(x, dtype=dt)), dtype=dt)
    lr, vec = spla.eigs(op, k=1, which="LR", tol=tol, maxiter=maxit, v0=v0.astype(dt))
    sr = spla.eigs(op, k=1, which="SR", tol=tol, maxiter=maxit, v0=v0.astype(dt), return_eigenvectors=False)
    return float(np.real(lr[0])) * 1.01, float(np.real(sr[0])) - 0.1, vec[:, 0]


def eig_solver_bounds(H, N, ks, count, ubgv, EigVal_prev, bounds, rhoTrigger=4, elecgs_Count=1, chefsibound_flag=0,
                      tol_lanczos=1e-2, complex_op=True):
    """Bounds and cutoff of one block, src/eigSolver.m:21-94, line by line.

    ``ubgv`` is the block's column of S.upper_bound_guess_vecs, ``EigVal_prev`` its S.EigVal
    column and ``bounds`` the previous ``(a0, bup, lambda_cutoff)``.  Returns
    ``(a0, bup, lambda_cutoff, ubgv)``: ``ubgv`` is the eigs vector of every new upper-bound
    estimate, else the input column.
      * :21-23   rhoTrigger = 1 when elecgs_Count > 1;
      * :47-64   count == 1: eigs 'lr' from rand (elecgs_Count == 1) or from ubgv (later
                 relaxation steps), bup = 1.01 real(lambda);
      * :65-72   count == 1: a0 = real(eigs 'sr') - 0.1, or min(EigVal) on later relaxation steps;
      * :74-83   count > rhoTrigger: with chefsibound_flag, bup again from eigs started at ubgv;
                 a0 = min(EigVal);
      * :88-94   cutoff (bup + a0)/2 on the first SCF step of the first relaxation step, else
                 max(EigVal) + 0.1.
    """
    a0, bup, lc = bounds
    if elecgs_Count > 1:
        rhoTrigger = 1
    dt = complex if complex_op else float
    op = spla.LinearOperator((N, N), matvec=lambda x: H(np.asarray(x, dtype=dt)), dtype=dt)

    def upper(v0, tol, maxit):
        lam, vec = spla.eigs(op, k=1, which="LR", tol=tol, maxiter=maxit, v0=np.asarray(v0, dtype=dt))
        return float(np.real(lam[0])) * 1.01, vec[:, 0]

    if count == 1:
        if elecgs_Count == 1:
            bup, a0, ubgv = spectral_bounds(H, N, ks, tol=tol_lanczos, maxit=300, complex_op=complex_op)
        else:
            bup, ubgv = upper(ubgv, tol_lanczos, 300)
            a0 = float(np.min(EigVal_prev))
    elif count > rhoTrigger:
        if chefsibound_flag == 1:
            bup, ubgv = upper(ubgv, tol_lanczos, 100)
        a0 = float(np.min(EigVal_prev))
    if count == 1 and elecgs_Count == 1:
        lc = 0.5 * (bup + a0)
    else:
        lc = float(np.max(EigVal_prev)) + 0.10
    return a0, bup, lc, ubgv


def rayleigh_ritz(psi, H, S, W):
    """src/eigSolver.m:99-124: orth, Hs = psi'*H*psi, eig, real, sort, rotate, W-normalise."""
    psi = sla.orth(psi)
    if psi.shape[1] != S.Nev_block:
        raise AssertionError("Number of states have changed within SCF")
    Hs = psi.conj().T @ H(psi)
    if S.cell_typ < 3:
        Hs = 0.5 * (Hs + Hs.conj().T)
    D, Q = sla.eig(Hs)
    EigVal = np.real(D)
    if S.cell_typ >= 3:
        ind = np.argsort(EigVal, kind="stable")
        EigVal = EigVal[ind]
        Q = Q[:, ind]
    psi = psi @ Q
    scfac = 1.0 / np.sqrt(np.sum(W[:, None] * (psi * np.conj(psi)).real, axis=0))
    psi = psi * scfac[None, :]
    return psi, EigVal


class _Nev:
    def __init__(self, S, nev):
        self._S = S
        self.Nev_block = nev

    def __getattr__(self, k):
        return getattr(self._S, k)


def eig_solver_block(S, H, psi, count, bounds, EigVal_prev, rhoTrigger=4, elecgs_Count=1):
    """One block of the serial branch of src/eigSolver.m:26-125.

    ``bounds`` is ``(a0, bup, lambda_cutoff)`` from the previous call (or the
    first-step estimates).  The cutoff is ``(bup+a0)/2`` on the first step of
    the first relaxation step, else ``max(EigVal)+0.1`` (:88-94); after
    ``rhoTrigger`` the lower bound becomes ``min(EigVal)`` (:72-82).
    """
    a0, bup, lc = bounds
    if count > 1 and count > rhoTrigger:
        a0 = float(np.min(EigVal_prev))
    if count == 1 and elecgs_Count == 1:
        lc = 0.5 * (bup + a0)
    else:
        lc = float(np.max(EigVal_prev)) + 0.10
    psi = chebyshev_filter(psi, S.npl, lc, bup, a0, H)
    psi, ev = rayleigh_ritz(psi, H, _Nev(S, psi.shape[1]), S.W)
    return psi, ev, (a0, bup, lc)


# ---------------------------------------------------------------------------
# src/initialization.m:734-740 -- assembled Laplacian for the Poisson solve
# ---------------------------------------------------------------------------
def lap_std(S, T=None):
    T = T if T is not None else lap_indices_values_1d_cychel(S)
    DL11, DL22, DL33, DG1, DG2, DG3 = bloch_laplacian_1d(S, T, [0.0, 0.0, 0.0])
    Ix, Iy, Iz = sp.identity(S.Nx), sp.identity(S.Ny), sp.identity(S.Nz)
    L = sp.kron(Iz, sp.kron(Iy, DL11 + DG1)) + sp.kron(DL33, sp.kron(Iy, Ix)) + \
        sp.kron(Iz, sp.kron(DL22, T["R2inv"]))
    if S.cell_typ in (4, 5):
        L = L + sp.kron(Iz, sp.kron(DL22, Ix)) + sp.kron(DG3, sp.kron(DG2, Ix))
    return sp.csr_matrix(L)


def lap_full_k(S, kptvec, T=None):
    """The same assembled operator with Bloch phases (the kron form of lapVec_cychel)."""
    T = T if T is not None else lap_indices_values_1d_cychel(S)
    DL11, DL22, DL33, DG1, DG2, DG3 = bloch_laplacian_1d(S, T, kptvec)
    Ix, Iy, Iz = sp.identity(S.Nx), sp.identity(S.Ny), sp.identity(S.Nz)
    L = sp.kron(Iz, sp.kron(Iy, DL11 + DG1)) + sp.kron(DL33, sp.kron(Iy, Ix)) + \
        sp.kron(Iz, sp.kron(DL22, T["R2inv"]))
    if S.cell_typ in (4, 5):
        L = L + sp.kron(Iz, sp.kron(DL22, Ix)) + sp.kron(DG3, sp.kron(DG2, Ix))
    return sp.csr_matrix(L)
