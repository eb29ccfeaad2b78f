"""Known-answer tests of the oracle's SCF pieces (no GPU): the AAR solver (src/aar.m), the Poisson
operator (src/poissonSolve.m, src/initialization.m:734-752), LDA_PW (src/exchangeCorrelationPotential.m,
src/evaluateTotalEnergy.m), Gaussian-smearing occupations (src/occupations.m) and Periodic Pulay
mixing (src/mixing.m, src/andersonWtdAvg.m)."""
import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from kat_systems import bare_cell
from oracle import scf as OS


def test_aar_solves_a_nonsymmetric_system():
    rng = np.random.default_rng(0)
    n = 200
    A = sp.diags([np.full(n - 1, -1.0), np.full(n, 4.0), np.full(n - 1, -1.3)], [-1, 0, 1]).tocsr()
    b = rng.standard_normal(n)
    x, relres, it = OS.aar(A, b, None, 1e-10, 500, 0.6, 0.6, 7, 6, lambda r: r / 4.0)
    assert relres <= 1e-10
    assert np.max(np.abs(x - spla.spsolve(A.tocsc(), b))) < 1e-8


def test_poisson_operator_recovers_a_potential():
    S = bare_cell(17, 8, 12)
    P = OS.PoissonOperator(S)
    rng = np.random.default_rng(1)
    phi0 = rng.standard_normal(S.N)
    f = P.L @ phi0
    phi, relres, it = P.solve(f, None, 1e-11)
    assert relres <= 1e-11
    assert np.max(np.abs(phi - phi0)) < 1e-7 * np.max(np.abs(phi0))


@pytest.mark.parametrize("rho", [1e-4, 3e-3, 0.05, 0.7, 4.0])
def test_lda_pw_potential_is_the_energy_derivative(rho):
    # V_xc = d(rho eps_xc)/d rho: central difference of the energy density
    W = np.ones(1)
    h = 1e-6 * rho
    e = lambda r: OS.lda_pw_energy(np.array([r]), W)
    dnum = (e(rho + h) - e(rho - h)) / (2 * h)
    v = OS.lda_pw_potential(np.array([rho]))[0]
    assert abs(v - dnum) < 1e-6 * max(1.0, abs(v))


def test_lda_pw_exchange_limit():
    # high density: exchange dominates, eps_x = -(3/4)(3/pi)^(1/3) rho^(1/3)
    rho = 1e4
    ex = -0.75 * (3 / np.pi) ** (1 / 3) * rho ** (1 / 3)
    exc = OS.lda_pw_energy(np.array([rho]), np.ones(1)) / rho
    assert abs(exc - ex) / abs(ex) < 0.05


def test_occupations_count_electrons():
    rng = np.random.default_rng(2)
    evs = [np.sort(rng.uniform(-1, 1, 20)), np.sort(rng.uniform(-1, 1, 18))]
    wk = np.array([0.5, 0.5])
    bet = 27.21138602 / 0.2
    ne = 21.3
    lam_f, occ = OS.occupations(evs, wk, bet, 2.0, -ne)
    total = sum(2.0 * wk[k] * np.sum(occ[k]) for k in range(2))
    assert abs(total - ne) < 1e-10
    for o in occ:
        assert np.all((o >= 0) & (o <= 1))
    assert min(e.min() for e in evs) < lam_f < max(e.max() for e in evs)


def test_periodic_pulay_finds_the_fixed_point():
    # g(x) = M x + c with a contractive M: the fixed point solves (I - M) x = c
    rng = np.random.default_rng(3)
    n = 40
    Q, _ = np.linalg.qr(rng.standard_normal((n, n)))
    M = Q @ np.diag(np.linspace(-0.8, 0.9, n)) @ Q.T
    c = rng.standard_normal(n)
    xs = np.linalg.solve(np.eye(n) - M, c)
    mixer = OS.PeriodicPulay(n)
    x = np.zeros(n)
    for it in range(1, 60):
        x = mixer(M @ x + c, x, it)
    assert np.max(np.abs(x - xs)) < 1e-8 * np.max(np.abs(xs))
    # simple mixing with the same parameter is far slower
    y = np.zeros(n)
    for it in range(1, 60):
        y = y + 0.3 * (M @ y + c - y)
    assert np.max(np.abs(y - xs)) > 1e-3 * np.max(np.abs(xs))


def test_fermi_dirac_occupations_and_entropy():
    # src/occupations.m (elec_T_type = 0) and the entropy term of src/evaluateTotalEnergy.m:82-83:
    # occupations sum to the electron count; the free-energy entropy term equals
    # T * sum f ln f + (1 - f) ln (1 - f) and vanishes as T -> 0
    rng = np.random.default_rng(4)
    evs = [np.sort(rng.uniform(-1, 1, 12)), np.sort(rng.uniform(-1, 1, 10))]
    wk = np.array([0.25, 0.75])
    for bet in (50.0, 1000.0, 1e5):
        lam_f, occ = OS.occupations(evs, wk, bet, 2.0, -9.0, elec_T_type=0)
        assert abs(sum(2.0 * wk[k] * np.sum(occ[k]) for k in range(2)) - 9.0) < 1e-10
        with np.errstate(over="ignore"):
            fd = [1.0 / (1.0 + np.exp(bet * (e - lam_f))) for e in evs]
        assert all(np.allclose(o, f, atol=1e-15) for o, f in zip(occ, fd))
        N = 4
        z = np.zeros(N)
        _, parts = OS.total_energy(evs, occ, wk, 2.0, bet, lam_f, z, z, z, z, np.ones(N), 0.0, 0.0, elec_T_type=0)
        with np.errstate(divide="ignore", invalid="ignore"):
            ent = sum(wk[k] * np.nansum(2.0 / bet * (o * np.log(o) + (1 - o) * np.log(1 - o))) for k, o in enumerate(occ))
        assert abs(parts["Eent"] - ent) < 1e-14 and parts["Eent"] <= 0.0
    assert abs(parts["Eent"]) < 1e-4


@pytest.mark.parametrize("rho", [1e-4, 3e-3, 0.05, 0.7, 4.0])
def test_lda_pz_potential_is_the_energy_derivative(rho):
    # both branches of the Perdew-Zunger fit (rs >= 1 and rs < 1 at rho > 0.24) and their
    # potentials: V_xc = d(rho eps_xc)/d rho
    W = np.ones(1)
    h = 1e-6 * rho
    e = lambda r: OS.lda_pz_energy(np.array([r]), W)
    dnum = (e(rho + h) - e(rho - h)) / (2 * h)
    v = OS.lda_pz_potential(np.array([rho]))[0]
    assert abs(v - dnum) < 1e-6 * max(1.0, abs(v))


def test_lda_pz_close_to_pw():
    # two fits of the same Ceperley-Alder data: within a few mHa per electron over metallic densities
    rho = np.geomspace(1e-3, 1.0, 20)
    W = np.ones(1)
    for r in rho:
        a = OS.lda_pz_energy(np.array([r]), W) / r
        b = OS.lda_pw_energy(np.array([r]), W) / r
        assert abs(a - b) < 3e-3


def test_pbe_reduces_to_lda_pw_for_a_uniform_density():
    # sigma = 0: F_x = 1 and H = 0, so PBE is the PW92 LDA (same correlation parameters)
    rho = np.geomspace(1e-4, 5.0, 30)
    f, fr, fs = OS._pbe_parts(rho, np.zeros_like(rho))
    e_lda = np.array([OS.lda_pw_energy(np.array([r]), np.ones(1)) for r in rho])
    assert np.allclose(f, e_lda, rtol=1e-12)
    assert np.allclose(fr, OS.lda_pw_potential(rho), rtol=1e-10)
    # second-order gradient terms at sigma = 0: exchange -3 mu / (16 pi k_F rho), correlation
    # beta pi / (16 k_F rho); PBE's mu = beta pi^2 / 3 makes them cancel
    kf = (3 * np.pi ** 2 * rho) ** (1 / 3)
    beta, mu = OS.PBE["beta"], OS.PBE["mu"]
    assert np.allclose(fs * 16 * kf * rho, np.pi * beta - 3 * mu / np.pi, rtol=0, atol=1e-9)
    assert abs(np.pi * beta - 3 * mu / np.pi) < 2e-5


@pytest.mark.parametrize("rho,sigma", [(0.01, 1e-5), (0.2, 0.03), (1.5, 2.0)])
def test_pbe_complex_step_derivatives(rho, sigma):
    f0 = lambda r, s: OS._pbe_f(np.array([r]), np.array([s]))[0]
    f, fr, fs = (v[0] for v in OS._pbe_parts(np.array([rho]), np.array([sigma])))
    hr, hs = 1e-5 * rho, 1e-5 * sigma
    assert abs(fr - (f0(rho + hr, sigma) - f0(rho - hr, sigma)) / (2 * hr)) < 1e-7 * max(1, abs(fr))
    assert abs(fs - (f0(rho, sigma + hs) - f0(rho, sigma - hs)) / (2 * hs)) < 1e-6 * max(1, abs(fs))


def test_cyclix_gradients_on_a_smooth_field():
    # f = x^2 + y^2 + sin(2 pi z / L3) is periodic in theta and z: D_x f = 2x, D_y f = 2y,
    # D_z f = (2 pi / L3) cos(2 pi z / L3), away from the radial Dirichlet ends, on a cyclic and on
    # a helical cell (Cychel/gradIndicesValues_cychel.m)
    for twist in (0.0, 0.05):
        S = bare_cell(30, 12, 16, twist=twist)
        G = OS.cyclix_gradients(S)
        r = S.xin + np.arange(S.Nx) * S.dx
        R, T, Z = np.meshgrid(r, np.arange(S.Ny) * S.dy, np.arange(S.Nz) * S.dz, indexing="ij")
        R, T, Z = (a.reshape(-1, order="F") for a in (R, T, Z))
        X, Y = R * np.cos(T + twist * Z), R * np.sin(T + twist * Z)
        k = 2 * np.pi / S.L3
        f = X * X + Y * Y + np.sin(k * Z)
        inner = (R > r[S.FDn]) & (R < r[-S.FDn - 1])
        assert np.allclose((G[0] @ f)[inner], 2 * X[inner], atol=1e-8)
        assert np.allclose((G[1] @ f)[inner], 2 * Y[inner], atol=1e-8)
        assert np.allclose((G[2] @ f)[inner], k * np.cos(k * Z[inner]), atol=1e-7)
