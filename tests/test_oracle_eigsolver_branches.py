"""The oracle's restatement of eigSolver's bound and cutoff control flow (src/eigSolver.m:21-94)
on the tiny cyclic cell, checked against the dense spectrum.

Known answers: on later relaxation steps (elecgs_Count > 1) rhoTrigger is 1, a0 is min(EigVal),
the cutoff max(EigVal) + 0.1 and the upper bound comes from eigs started at the previous
upper-bound vector; chefsibound_flag re-estimates it once count > rhoTrigger; with neither, the
bounds of count <= rhoTrigger are kept.  The eigs estimates are checked against the largest real
part of the dense spectrum (ARPACK tolerance 1e-2: within 2 %).
"""
import numpy as np
import pytest

from oracle import cychel_ops as O


@pytest.fixture(scope="module")
def tiny(tiny_cyclic):
    S = tiny_cyclic
    H = O.Hamiltonian(S, S.kptgrid[0], S.Veff[:, 0])
    lam = np.linalg.eigvals(H.dense())
    return S, H, float(lam.real.max()), float(lam.real.min())


def test_first_relaxation_step_bounds(tiny):
    S, H, lmax, lmin = tiny
    ev_prev = np.linspace(-1.0, 0.4, 6)
    a0, bup, lc, u = O.eig_solver_bounds(H, S.N, 1, 1, None, ev_prev, (0.0, 0.0, 0.0))
    assert lmax <= bup <= 1.02 * lmax
    assert a0 == pytest.approx(lmin - 0.1, abs=0.02 * (lmax - lmin))
    assert lc == pytest.approx(0.5 * (bup + a0))
    assert u.shape == (S.N,)


def test_later_relaxation_step_restarts_from_ubgv(tiny):
    S, H, lmax, lmin = tiny
    _, _, _, u = O.eig_solver_bounds(H, S.N, 1, 1, None, np.zeros(6), (0.0, 0.0, 0.0))
    ev_prev = np.array([-0.7, -0.2, 0.1, 0.3, 0.5, 0.9])
    a0, bup, lc, u2 = O.eig_solver_bounds(H, S.N, 1, 1, u, ev_prev, (0.0, 0.0, 0.0), elecgs_Count=2)
    assert a0 == ev_prev.min()                      # min(S.EigVal(:,ks)), not eigs 'sr'
    assert lc == ev_prev.max() + 0.10               # max(S.EigVal) + 0.1 already on count == 1
    assert lmax <= bup <= 1.02 * lmax
    # count 2 > rhoTrigger = 1 on later relaxation steps: a0 follows EigVal, bup is kept
    a0b, bupb, lcb, u3 = O.eig_solver_bounds(H, S.N, 1, 2, u2, ev_prev - 0.05, (a0, bup, lc), rhoTrigger=4, elecgs_Count=2)
    assert a0b == (ev_prev - 0.05).min() and bupb == bup and u3 is u2


def test_chefsibound_flag_reestimates_bup_after_rhotrigger(tiny):
    S, H, lmax, lmin = tiny
    _, _, _, u = O.eig_solver_bounds(H, S.N, 1, 1, None, np.zeros(6), (0.0, 0.0, 0.0))
    ev_prev = np.array([-0.7, -0.2, 0.1, 0.3, 0.5, 0.9])
    old = (-2.0, 123.0, 1.0)
    # count <= rhoTrigger: nothing is re-estimated, only the cutoff follows EigVal
    a0, bup, lc, _ = O.eig_solver_bounds(H, S.N, 1, 3, u, ev_prev, old, rhoTrigger=4, chefsibound_flag=1)
    assert (a0, bup) == old[:2] and lc == ev_prev.max() + 0.10
    # count > rhoTrigger: a0 = min(EigVal); bup again from eigs only with the flag
    a0, bup, lc, _ = O.eig_solver_bounds(H, S.N, 1, 5, u, ev_prev, old, rhoTrigger=4, chefsibound_flag=0)
    assert a0 == ev_prev.min() and bup == old[1]
    a0, bup, lc, u2 = O.eig_solver_bounds(H, S.N, 1, 5, u, ev_prev, old, rhoTrigger=4, chefsibound_flag=1)
    assert a0 == ev_prev.min() and lmax <= bup <= 1.02 * lmax
    # the returned vector is an approximate top eigenvector: its Rayleigh quotient is near lmax
    rq = np.real(np.vdot(u2, H(u2[:, None])[:, 0]) / np.vdot(u2, u2))
    assert rq == pytest.approx(bup / 1.01, rel=1e-6)
