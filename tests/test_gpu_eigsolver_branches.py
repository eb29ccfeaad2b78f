"""GPU eigSolver control flow (cx_eigsolver_full through the C-ABI) against the oracle's
restatement of src/eigSolver.m:21-94, complex128, on the 40 x 12 x 20 cyclic cell.

Tolerances:
  * a0 and the cutoff are set from EigVal and the bounds given (min(EigVal), max(EigVal) + 0.1,
    (bup + a0) / 2): equal to 1e-12;
  * the upper bound is 1.01 x a Krylov estimate of the largest eigenvalue; the GPU's 64-step
    Lanczos and the oracle's ARPACK (tolerance 1e-2) agree within 2 %;
  * the returned upper-bound vector is the Ritz vector of that estimate: its 2-norm is 1 and its
    Rayleigh quotient in the W inner product is within 2 % of bup / 1.01 (a 64-step Lanczos run
    without reorthogonalisation, like eigs at tolerance 1e-2, gives an approximate eigenvector);
  * eigenvalues of the step equal the oracle's eigSolver step run with the GPU's bounds to 1e-9 Ha.
"""
import numpy as np
import pytest

from oracle import cychel_ops as O

pytestmark = pytest.mark.gpu


def _w_rq(S, H, u):
    Hu = H(u[:, None])[:, 0]
    return float(np.real(np.sum(S.W * np.conj(u) * Hu)) / np.real(np.sum(S.W * np.conj(u) * u)))


@pytest.fixture(scope="module")
def case(small_cyclic):
    from cyclix_msparc_gb300.msparc import CyclixGPU
    from cyclix_msparc_gb300.workloads import WORKLOADS, block_layout, initial_psi
    S = small_cyclic
    bl = block_layout(WORKLOADS["cyclic-40x12x20-ns48-m20"], S)
    g = CyclixGPU(S, bl, "fp64")
    psi0 = initial_psi(S.N, bl[0][2], 21)
    H = O.Hamiltonian(S, S.kptgrid[0], S.Veff[:, 0])
    yield S, g, psi0, H
    g.close()


def _step(g, psi0, count, EV, bounds, **kw):
    g.set_psi(0, psi0)
    a0, bup, lc = (np.array([v], dtype=float) for v in bounds)
    EV = np.ascontiguousarray(EV, dtype=float).copy()
    g.eigsolve(count, kw.pop("npl"), EV, a0, bup, lc, **kw)
    return EV, a0[0], bup[0], lc[0]


def test_first_step_returns_upper_bound_vector(case):
    S, g, psi0, H = case
    u = np.zeros((S.N, 1), dtype=np.complex128, order="F")
    EV, a0, bup, lc = _step(g, psi0, 1, np.zeros(48), (0, 0, 0), npl=S.npl, ubgv=u)
    bup_ref, a0_ref, _ = O.spectral_bounds(H, S.N, 1)
    assert bup == pytest.approx(bup_ref, rel=0.02)
    assert lc == pytest.approx(0.5 * (bup + a0), rel=1e-12)
    assert np.linalg.norm(u[:, 0]) == pytest.approx(1.0, rel=1e-12)
    assert _w_rq(S, H, u[:, 0]) == pytest.approx(bup / 1.01, rel=0.02)


def test_later_relaxation_step(case):
    S, g, psi0, H = case
    u = np.zeros((S.N, 1), dtype=np.complex128, order="F")
    _step(g, psi0, 1, np.zeros(48), (0, 0, 0), npl=S.npl, ubgv=u)
    u_prev = u.copy()
    ev_prev = np.linspace(-2.0, 0.5, 48)
    EV, a0, bup, lc = _step(g, psi0, 1, ev_prev, (0, 0, 0), npl=S.npl, ubgv=u, elecgs_Count=2)
    a0_ref, bup_ref, lc_ref, _ = O.eig_solver_bounds(H, S.N, 1, 1, u_prev[:, 0], ev_prev, (0, 0, 0), elecgs_Count=2)
    assert a0 == a0_ref and lc == pytest.approx(lc_ref, abs=1e-12)
    assert bup == pytest.approx(bup_ref, rel=0.02)
    assert _w_rq(S, H, u[:, 0]) == pytest.approx(bup / 1.01, rel=0.02)
    # the step itself: eigenvalues of the oracle's eigSolver step with these bounds
    _, ev_ref, _ = O.eig_solver_block(S, H, psi0, 1, (a0, bup, lc), ev_prev, elecgs_Count=2)
    assert np.max(np.abs(EV - ev_ref)) < 1e-9


def test_chefsibound_flag(case):
    S, g, psi0, H = case
    u = np.zeros((S.N, 1), dtype=np.complex128, order="F")
    _step(g, psi0, 1, np.zeros(48), (0, 0, 0), npl=S.npl, ubgv=u)
    ev_prev = np.linspace(-2.0, 0.5, 48)
    old = (-3.0, 900.0, 0.0)
    # count > rhoTrigger without the flag: bup kept, a0 = min(EigVal)
    EV, a0, bup, lc = _step(g, psi0, 5, ev_prev, old, npl=S.npl, ubgv=u, rhoTrigger=4)
    assert bup == 900.0 and a0 == ev_prev.min() and lc == pytest.approx(ev_prev.max() + 0.1, abs=1e-12)
    # with the flag: bup re-estimated from ubgv, the vector updated
    u_prev = u.copy()
    EV, a0, bup, lc = _step(g, psi0, 5, ev_prev, old, npl=S.npl, ubgv=u, rhoTrigger=4, chefsibound_flag=1)
    _, bup_ref, _, _ = O.eig_solver_bounds(H, S.N, 1, 5, u_prev[:, 0], ev_prev, old, rhoTrigger=4, chefsibound_flag=1)
    assert bup == pytest.approx(bup_ref, rel=0.02) and a0 == ev_prev.min()
    assert _w_rq(S, H, u[:, 0]) == pytest.approx(bup / 1.01, rel=0.02)
    _, ev_ref, _ = O.eig_solver_block(S, H, psi0, 5, (a0, bup, lc), ev_prev)
    assert np.max(np.abs(EV - ev_ref)) < 1e-9


def test_eigSolver_mirror_returns_ubgv(case):
    """The MATLAB-signature mirror passes S.upper_bound_guess_vecs through the library and returns the update."""
    from cyclix_msparc_gb300 import msparc
    S, g, psi0, H = case
    S.gpu = g
    S.elecgs_Count, S.chefsibound_flag = 1, 0
    try:
        ubgv = np.zeros((S.N, 1), dtype=np.complex128)
        out = msparc.eigSolver(S, 1, ubgv, psi0[:, :, None], np.zeros((48, 1)), np.zeros(1), np.zeros(1), np.zeros(1))
    finally:
        del S.gpu, S.elecgs_Count, S.chefsibound_flag
    u, psi, ev, a0, bup, lc = out
    assert u.shape == (S.N, 1) and np.linalg.norm(u) == pytest.approx(1.0, rel=1e-12)
    assert _w_rq(S, H, u[:, 0]) == pytest.approx(bup[0] / 1.01, rel=0.02)
    assert psi.shape == (S.N, 48, 1) and ev.shape == (48, 1)
