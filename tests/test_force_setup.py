"""The host set-up of the local and correction forces (cyclix_msparc_gb300/forces.py) against the
oracle (oracle/forces.py, src/atomicForce.m:40-127) on the CNT_chiral deck's saved set-up
(helical, twist 0.1636 rad/bohr, psp8 local potentials): the per-atom projection vectors and
constants, projected on the gradients of a seeded potential phi and of V_c (here with the oracle's
sparse gradient in place of cx_field_projections), give the oracle's drift-free local + correction
forces.  Tolerance 1e-12 relative to the largest component (the sums are regrouped)."""
import numpy as np

from golden.make_deck_fixtures import load_force_deck


def test_local_force_setup_matches_oracle():
    from cyclix_msparc_gb300 import forces as PF
    from oracle import forces as OF
    d, _, _, _ = load_force_deck("CNT_chiral")
    S = d.S
    st = PF.local_force_setup(d)
    G = OF.bloch_gradients(S, (0.0, 0.0, 0.0))

    class Projector:
        def field_projections(self, f, A):
            return A @ np.stack([(g @ f).real for g in G], axis=1)

        def nonlocal_force(self, occ, wkpt, occfac):
            return np.zeros((S.Atoms.shape[0], 3))

    phi = 0.1 * np.random.default_rng(2).standard_normal(S.N) + d.pseudo["V_c"]
    F = PF.atomic_forces(Projector(), st, phi, np.zeros(1), [1.0], S.occfac)
    zero = [np.zeros((S.N, 1), complex) for _ in range(S.tnkpt)]
    _, parts = OF.atomic_forces(d, zero, [np.zeros(1)] * S.tnkpt, phi)
    ref = parts["local"] + parts["correction"]
    ref[:, 2] -= ref[:, 2].mean()
    assert np.max(np.abs(F - ref)) <= 1e-12 * np.max(np.abs(ref))


def test_occupations_match_oracle():
    from cyclix_msparc_gb300.forces import occupations
    from oracle.scf import _occ
    ev = np.linspace(-0.5, 0.5, 101)
    for T in (0, 1):
        assert np.max(np.abs(occupations(ev, 0.03, 50.0, T) - _occ(ev, 0.03, 50.0, T))) < 1e-15


def test_force_deck_rebuilds_the_saved_setup():
    """The local-potential tables of the fixture reproduce its saved pseudocharge set-up exactly."""
    from golden.make_deck_fixtures import load
    d, _, _, _ = load_force_deck("CNT_chiral")
    S0 = load("CNT_chiral")[0]
    assert np.array_equal(d.pseudo["b"], S0.b)
    assert np.array_equal(d.pseudo["rho_at"], S0.rho_at)
    assert d.pseudo["Eself"] == S0.Eself and d.pseudo["E_corr"] == S0.E_corr
