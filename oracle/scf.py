"""Oracle restatement of the SCF bookkeeping around the CheFSI path.

Test infrastructure only (see ``oracle/__init__.py``).  Paths relative to the reference project
root ``Cyclix_MS_200220/``.  Covers the non-spin LDA (PW or PZ) and GGA_PBE potential-mixing SCF of src/scf.m with the
reference defaults (MixingVariable = 1, MixingPrecond = 0, PulayFrequency = 1, MixingHistory = 7,
MixingParameter = 0.3, rhoTrigger = 4, MINIT_SCF = 3; src/initialization.m:1004-1040).
"""
from __future__ import annotations

import math

import numpy as np
import scipy.linalg as sla
import scipy.optimize as so
import scipy.sparse as sp
import scipy.sparse.linalg as spla
from scipy.special import erf, expit

from . import cychel_ops as O

XC_RHOTOL = 1e-14   # src/initialization.m:143


# ---------------------------------------------------------------------------------------------
# src/aar.m:1-74 with the ILU(1e-5) preconditioner of src/initialization.m:752
# ---------------------------------------------------------------------------------------------
def aar(A, b, x_guess, tol, max_iter, omega, beta, m, p, M_solve):
    N = b.shape[0]
    DX = np.zeros((N, m))
    DF = np.zeros((N, m))
    nb = 1 / np.linalg.norm(b)
    x_prev = np.ones(N) if x_guess is None else x_guess.copy()
    relres = 1 + tol
    count = 1
    x = x_prev
    Xold = Fold = None
    while count <= max_iter and relres > tol:
        res1 = b - A @ x_prev
        relres = np.linalg.norm(res1) * nb
        res = M_solve(res1)
        if count > 1:
            DX[:, (count - 2) % m] = x_prev - Xold
            DF[:, (count - 2) % m] = res - Fold
        Xold = x_prev
        Fold = res
        if count % p != 0:
            x_new = x_prev + omega * res
        else:
            x_new = x_prev + beta * res - (DX + beta * DF) @ (np.linalg.pinv(DF.T @ DF) @ (DF.T @ res))
        x = x_prev
        x_prev = x_new
        count += 1
    return x, relres, count - 1


class PoissonOperator:
    """Lap_std and its ILU factors (src/initialization.m:734-752)."""

    def __init__(self, S):
        self.L = O.lap_std(S).tocsc()
        self.ilu = spla.spilu(self.L, drop_tol=1e-5)

    def solve(self, f, guess, tol, maxit=1000):
        # src/poissonSolve.m:36: aar(Lap_std, f, guess, tol, MAXIT_POISSON, 0.6, 0.6, 7, 6, L, U)
        return aar(self.L, f, guess, tol, maxit, 0.6, 0.6, 7, 6, self.ilu.solve)


# ---------------------------------------------------------------------------------------------
# src/exchangeCorrelationPotential.m:82-106 (LDA_PW potential) and
# src/evaluateTotalEnergy.m:28-43 (LDA_PW energy)
# ---------------------------------------------------------------------------------------------
def lda_pw_potential(rho):
    rho = np.where(rho < XC_RHOTOL, XC_RHOTOL, rho)
    p, A, alpha1 = 1, 0.031091, 0.21370
    beta1, beta2, beta3, beta4 = 7.5957, 3.5876, 1.6382, 0.49294
    C3 = 0.9847450218427
    rs = (0.75 / (np.pi * rho)) ** (1 / 3)
    Q = 2 * A * (beta1 * rs ** 0.5 + beta2 * rs + beta3 * rs ** 1.5 + beta4 * rs ** (p + 1))
    V = -C3 * rho ** (1 / 3) + (-2 * A * (1 + alpha1 * rs)) * np.log(1 + 1 / Q) \
        - (rs / 3) * (-2 * A * alpha1 * np.log(1 + 1 / Q)
                      - ((-2 * A * (1 + alpha1 * rs)) * (A * (beta1 * rs ** -0.5 + 2 * beta2 + 3 * beta3 * rs ** 0.5
                                                               + 2 * (p + 1) * beta4 * rs ** p)))
                      / (Q * Q + Q))
    return V


def lda_pw_energy(rho, W):
    rho = np.where(rho < XC_RHOTOL, XC_RHOTOL, rho)
    C2 = 0.73855876638202
    p, A, alpha1 = 1, 0.031091, 0.21370
    beta1, beta2, beta3, beta4 = 7.5957, 3.5876, 1.6382, 0.49294
    rs = (0.75 / (np.pi * rho)) ** (1 / 3)
    ec = -2 * A * (1 + alpha1 * rs) * np.log(1 + 1 / (2 * A * (beta1 * rs ** 0.5 + beta2 * rs + beta3 * rs ** 1.5
                                                               + beta4 * rs ** (p + 1.0))))
    return float(np.sum(ec * rho * W) - C2 * np.sum(rho ** (4 / 3) * W))


# ---------------------------------------------------------------------------------------------
# LDA_PZ: Slater exchange and the Perdew-Zunger (1981) parametrisation of the Ceperley-Alder
# correlation, unpolarised.  The reference's potential comes from compiled libxc (functional ids
# 1 and 9, src/exchangeCorrelationPotential.m:109-130), restated here from the published
# formulas; its energy is src/evaluateTotalEnergy.m:44-60.
# ---------------------------------------------------------------------------------------------
PZ = dict(A=0.0311, B=-0.048, C=0.002, D=-0.0116, gamma=-0.1423, beta1=1.0529, beta2=0.3334)


def _pz_corr(rho):
    """(eps_c, v_c) of Perdew-Zunger: rs >= 1 Pade form, rs < 1 logarithmic form."""
    rs = (0.75 / (np.pi * rho)) ** (1 / 3)
    A, B, C, D = PZ["A"], PZ["B"], PZ["C"], PZ["D"]
    g, b1, b2 = PZ["gamma"], PZ["beta1"], PZ["beta2"]
    eps = np.empty_like(rs)
    v = np.empty_like(rs)
    hi = rs >= 1.0
    sq = np.sqrt(rs[hi])
    den = 1.0 + b1 * sq + b2 * rs[hi]
    eps[hi] = g / den
    v[hi] = eps[hi] * (1.0 + (7.0 / 6.0) * b1 * sq + (4.0 / 3.0) * b2 * rs[hi]) / den
    lo = ~hi
    r = rs[lo]
    lr = np.log(r)
    eps[lo] = A * lr + B + C * r * lr + D * r
    v[lo] = A * lr + (B - A / 3.0) + (2.0 / 3.0) * C * r * lr + (2.0 * D - C) / 3.0 * r
    return eps, v


def lda_pz_potential(rho):
    rho = np.where(rho < XC_RHOTOL, XC_RHOTOL, rho)
    vx = -((3.0 / np.pi) * rho) ** (1 / 3)          # d(rho eps_x)/d rho, eps_x = -(3/4)(3 rho/pi)^(1/3)
    return vx + _pz_corr(rho)[1]


def lda_pz_energy(rho, W):
    rho = np.where(rho < XC_RHOTOL, XC_RHOTOL, rho)
    C2 = 0.73855876638202                         # (3/4)(3/pi)^(1/3)
    return float(np.sum(_pz_corr(rho)[0] * rho * W) - C2 * np.sum(rho ** (4 / 3) * W))


# ---------------------------------------------------------------------------------------------
# GGA_PBE (src/exchangeCorrelationPotential.m:156-326, nspin = 1) on the Cyclix gradients of
# Cychel/gradIndicesValues_cychel.m and Cychel/blochGradient_cychel.m (k = 0)
# ---------------------------------------------------------------------------------------------
def cyclix_gradients(S):
    """Cartesian derivative operators on the (r, theta, z) grid, FD order 2 FDn:
    D_x = cos(phi) d_r - sin(phi)/r d_theta, D_y = sin(phi) d_r + cos(phi)/r d_theta,
    D_z = d_z - tau d_theta, phi = theta + tau z; zero outside the radial Dirichlet ends,
    periodic in theta and z (Cychel/gradIndicesValues_cychel.m:1-141)."""
    Nx, Ny, Nz, n = S.Nx, S.Ny, S.Nz, S.FDn
    N = Nx * Ny * Nz
    i, j, k = np.meshgrid(np.arange(Nx), np.arange(Ny), np.arange(Nz), indexing="ij")
    i, j, k = (a.reshape(-1, order="F") for a in (i, j, k))
    row = i + Nx * (j + Ny * k)
    r = S.xin + i * S.dx
    ph = j * S.dy + S.twist * (k * S.dz)
    c, sn = np.cos(ph), np.sin(ph)
    ops = [[], [], []]
    for p in range(1, n + 1):
        w = S.w1[p]
        for sgn in (1, -1):
            ii = i + sgn * p
            ok = (ii >= 0) & (ii < Nx)                               # radial: Dirichlet zero ghosts
            col = ii + Nx * (j + Ny * k)
            for d, wt in ((0, c / S.dx), (1, sn / S.dx)):
                ops[d].append((row[ok], col[ok], (sgn * w * wt)[ok]))
            jj = np.mod(j + sgn * p, Ny)                             # theta: periodic (k = 0)
            col = i + Nx * (jj + Ny * k)
            for d, wt in ((0, -sn / (r * S.dy)), (1, c / (r * S.dy)), (2, np.full(N, -S.twist / S.dy))):
                ops[d].append((row, col, sgn * w * wt))
            kk = np.mod(k + sgn * p, Nz)                             # z: periodic
            col = i + Nx * (j + Ny * kk)
            ops[2].append((row, col, np.full(N, sgn * w / S.dz)))
    mats = []
    for d in range(3):
        R = np.concatenate([a for a, _, _ in ops[d]])
        Cc = np.concatenate([b for _, b, _ in ops[d]])
        V = np.concatenate([v for _, _, v in ops[d]])
        mats.append(sp.csr_matrix((V, (R, Cc)), shape=(N, N)))
    return mats


PBE = dict(kappa=0.804, mu=0.2195149727645171, beta=0.066725)


def _pbe_f(rho, sigma):
    """rho * e_xc of unpolarised PBE (Perdew, Burke, Ernzerhof, PRL 77, 3865 (1996)) with the
    PW92 correlation of LDA_PW; written for complex arguments (complex-step derivatives)."""
    kappa, mu, beta = PBE["kappa"], PBE["mu"], PBE["beta"]
    gam = (1.0 - math.log(2.0)) / math.pi ** 2
    kf = (3.0 * math.pi ** 2 * rho) ** (1.0 / 3.0)
    ex_lda = -0.75 * (3.0 / math.pi) ** (1.0 / 3.0) * rho ** (1.0 / 3.0)
    s2 = sigma / (4.0 * kf * kf * rho * rho)
    Fx = 1.0 + kappa - kappa / (1.0 + mu * s2 / kappa)
    rs = (0.75 / (math.pi * rho)) ** (1.0 / 3.0)
    A0, a1, b1, b2, b3, b4 = 0.031091, 0.21370, 7.5957, 3.5876, 1.6382, 0.49294
    ec = -2.0 * A0 * (1.0 + a1 * rs) * np.log(1.0 + 1.0 / (2.0 * A0 * (b1 * rs ** 0.5 + b2 * rs + b3 * rs ** 1.5 + b4 * rs * rs)))
    ks2 = 4.0 * kf / math.pi
    t2 = sigma / (4.0 * ks2 * rho * rho)
    Ac = (beta / gam) / (np.exp(-ec / gam) - 1.0)
    At2 = Ac * t2
    H = gam * np.log(1.0 + (beta / gam) * t2 * (1.0 + At2) / (1.0 + At2 + At2 * At2))
    return rho * (ex_lda * Fx + ec + H)


def _pbe_parts(rho, sigma):
    """(f, df/drho, df/dsigma) by complex-step differentiation (exact to rounding)."""
    h = 1e-30
    f = _pbe_f(rho, sigma).real
    fr = _pbe_f(rho + 1j * h * rho, sigma + 0j).imag / (h * rho)
    hs = h * (sigma + rho ** (8.0 / 3.0))            # sigma's natural scale; nonzero where sigma = 0
    fs = _pbe_f(rho + 0j, sigma + 1j * hs).imag / hs
    return f, fr, fs


def gga_pbe(rho, grads):
    """(Vxc, e_xc) of src/exchangeCorrelationPotential.m:156-326: gradients of the clipped density,
    v = d(rho e)/d rho, and Vxc = v - sum_i D_i (2 d(rho e)/d sigma D_i rho)."""
    rho = np.where(rho < XC_RHOTOL, XC_RHOTOL, rho)
    d = [G @ rho for G in grads]
    sigma = d[0] * d[0] + d[1] * d[1] + d[2] * d[2]
    f, fr, fs = _pbe_parts(rho, sigma)
    V = fr - sum(G @ (2.0 * fs * di) for G, di in zip(grads, d))
    return V, f / rho


def xc_functions(name, S=None):
    """(potential(rho), energy(rho, W)) of an XC functional by the reference's EXCHANGE_CORRELATION name."""
    if name == "LDA_PW":
        return lda_pw_potential, lda_pw_energy
    if name == "LDA_PZ":
        return lda_pz_potential, lda_pz_energy
    if name == "GGA_PBE":
        grads = cyclix_gradients(S)

        def energy(rho, W):
            e = gga_pbe(rho, grads)[1]
            rho_c = np.where(rho < XC_RHOTOL, XC_RHOTOL, rho)
            return float(np.sum(e * rho_c * W))          # src/evaluateTotalEnergy.m:61-62
        return (lambda rho: gga_pbe(rho, grads)[0]), energy
    raise ValueError(f"exchange-correlation {name}: the oracle implements LDA_PW, LDA_PZ and GGA_PBE")


# ---------------------------------------------------------------------------------------------
# src/occupations.m:1-35 (Fermi-Dirac, elec_T_type = 0; Gaussian smearing, elec_T_type = 1)
# and src/electronDensity.m:9-12
# ---------------------------------------------------------------------------------------------
def _occ(ev, lf, bet, elec_T_type):
    if elec_T_type == 0:
        return expit(-bet * (ev - lf))            # 1 / (1 + exp(bet (lambda - lambda_f)))
    return 0.5 * (1.0 - erf(bet * (ev - lf)))


def occupations(EigVals, wkpt, bet, occfac, NegCharge, elec_T_type=1):
    def f(lf):
        s = 0.0
        for k, ev in enumerate(EigVals):
            s += occfac * np.sum(wkpt[k] * _occ(ev, lf, bet, elec_T_type))
        return s + NegCharge
    lo, hi = min(ev.min() for ev in EigVals) - 10.0, max(ev.max() for ev in EigVals) + 10.0
    lam_f = so.brentq(f, lo, hi, xtol=1e-15, rtol=4 * np.finfo(float).eps, maxiter=500)
    occ = [_occ(ev, lam_f, bet, elec_T_type) for ev in EigVals]
    return lam_f, occ


def electron_density(psis, occ, wkpt, N):
    rho = np.zeros(N)
    for k, psi in enumerate(psis):
        rho += 2 * wkpt[k] * np.sum((psi * np.conj(psi)).real * occ[k][None, :], axis=1)
    return rho


# ---------------------------------------------------------------------------------------------
# src/evaluateTotalEnergy.m:12-93 (nspin = 1, LDA_PW; Fermi-Dirac or Gaussian smearing)
# ---------------------------------------------------------------------------------------------
def total_energy(EigVals, occ, wkpt, occfac, bet, lam_f, rho, b, phi, Vxc, W, Eself, E_corr, elec_T_type=1,
                 exc_energy=None):
    Eband = sum(occfac * wkpt[k] * np.sum(EigVals[k] * occ[k]) for k in range(len(EigVals)))
    Exc = (exc_energy or lda_pw_energy)(rho, W)
    rho_c = np.where(rho < XC_RHOTOL, XC_RHOTOL, rho)
    Exc_dc = float(np.sum(Vxc * rho_c * W))
    Eelec_dc = 0.5 * float(np.sum((b - rho) * phi * W))
    Eent = 0.0
    for k in range(len(EigVals)):
        if elec_T_type == 0:
            o = occ[k]
            with np.errstate(divide="ignore", invalid="ignore"):
                Eent_v = occfac * (1 / bet) * (o * np.log(o) + (1 - o) * np.log(1 - o))
            Eent_v[np.isnan(Eent_v)] = 0.0          # 0 log 0 (src/evaluateTotalEnergy.m:83)
        else:
            Eent_v = -occfac * (1 / bet) * 1 / (2 * np.sqrt(np.pi)) * np.exp(-(bet * (EigVals[k] - lam_f)) ** 2)
        Eent += wkpt[k] * np.sum(Eent_v)
    Etot = Eband + Exc - Exc_dc + Eelec_dc - Eself + E_corr + Eent
    return Etot, dict(Eband=Eband, Exc=Exc, Exc_dc=Exc_dc, Eelec_dc=Eelec_dc, Eent=Eent)


# ---------------------------------------------------------------------------------------------
# src/mixing.m:20-116 (Periodic Pulay, no preconditioner) and src/andersonWtdAvg.m:1-23
# ---------------------------------------------------------------------------------------------
class PeriodicPulay:
    def __init__(self, N, m=7, beta=0.3, omega=0.3, p=1):
        self.X = np.zeros((N, m))
        self.F = np.zeros((N, m))
        self.m, self.beta, self.omega, self.p = m, beta, omega, p
        self.fkm1 = np.zeros(N)
        self.xkm1 = None

    def __call__(self, g_k, x_k, it):
        f_k = g_k - x_k
        if it > 1:
            i_hist = (it - 2) % self.m
            self.X[:, i_hist] = x_k - self.xkm1
            self.F[:, i_hist] = f_k - self.fkm1
        if it % self.p == 0 and it > 1:
            Gamma = np.linalg.pinv(self.F.T @ self.F) @ (self.F.T @ f_k)
            x_wavg = x_k - self.X @ Gamma
            f_wavg = f_k - self.F @ Gamma
        else:
            x_wavg, f_wavg = x_k, f_k
        x_kp1 = x_wavg + (self.beta if it % self.p == 0 else self.omega) * f_wavg
        self.fkm1 = f_k
        self.xkm1 = x_k
        return x_kp1


# ---------------------------------------------------------------------------------------------
# src/scf.m:1-327 (first relaxation step, nspin = 1, potential mixing)
# ---------------------------------------------------------------------------------------------
def scf(S, psis, blocks, scf_tol=1e-6, poisson_tol=None, rhoTrigger=4, max_scf=100, min_scf=3, bounds=None, log=None):
    """Run the reference SCF on the CPU.  ``psis``: initial psi per block; ``blocks``: (kvec, spin, Ns).

    ``bounds``: optional per-block (a0, bup) for the first eigSolver call instead of eigs.
    Returns a dict with Etotal, EigVal (list), lambda_f, rho, Veff, n_scf, history.
    """
    N = S.N
    T_type = getattr(S, "elec_T_type", 1)
    vxc_fn, exc_fn = xc_functions(S.extra.get("xc", "LDA_PW"), S)
    poisson_tol = poisson_tol if poisson_tol is not None else 0.01 * scf_tol
    P = PoissonOperator(S)
    wk = np.asarray(S.wkpt)
    rho = S.rho_at.copy()
    phi, _, _ = P.solve(-4 * np.pi * (rho + S.b), None, poisson_tol)
    Vxc = vxc_fn(rho)
    Veff = phi + Vxc
    mixer = PeriodicPulay(N)
    Veff_temp = Veff.copy()
    psis = [p.copy() for p in psis]
    nblk = len(blocks)
    EigVal = [np.zeros(n) for (_, _, n) in blocks]
    a0 = np.zeros(nblk)
    bup = np.zeros(nblk)
    count, count_scf, err = 1, 1, 100.0
    hist = []
    Etot = None
    while (err > scf_tol and count_scf <= max_scf) or count_scf <= min_scf:
        for b_, (k, spin, n) in enumerate(blocks):
            H = O.Hamiltonian(S, k, Veff)
            if count == 1:
                if bounds is not None:
                    bup[b_], a0[b_] = bounds[b_][1], bounds[b_][0]
                else:
                    bup[b_], a0[b_], _ = O.spectral_bounds(H, N, b_ + 1)
            psis[b_], EigVal[b_], (a0[b_], bup[b_], _) = O.eig_solver_block(S, H, psis[b_], count, (a0[b_], bup[b_], 0.0),
                                                                              EigVal[b_], rhoTrigger=rhoTrigger)
        lam_f, occ = occupations(EigVal, wk, S.bet, S.occfac, S.NegCharge, T_type)
        if count >= rhoTrigger:
            rho = electron_density(psis, occ, wk, N)
            phi, _, _ = P.solve(-4 * np.pi * (rho + S.b), phi, poisson_tol)
            Vxc = vxc_fn(rho)
            Veff = phi + Vxc
            Etot, parts = total_energy(EigVal, occ, wk, S.occfac, S.bet, lam_f, rho, S.b, phi, Vxc, S.W, S.Eself, S.E_corr,
                                       T_type, exc_fn)
            Escc = float(np.sum((Veff - Veff_temp) * rho * S.W))
            Etot += Escc
            err = np.linalg.norm(Veff - Veff_temp) / np.linalg.norm(Veff)
            hist.append((count_scf, Etot / S.n_atm, err))
            if log:
                log(count_scf, Etot / S.n_atm, err)
            if err > scf_tol or count_scf < min_scf:
                Veff = mixer(Veff, Veff_temp, count_scf)
                Veff_temp = Veff.copy()
            count_scf += 1
        count += 1
    return dict(Etotal=Etot, EigVal=EigVal, lambda_f=lam_f, occ=occ, rho=rho, phi=phi, Veff=Veff, n_scf=count_scf - 1,
                history=hist, psis=psis)
