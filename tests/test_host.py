"""Host-side logic (no GPU): Bloch points, synthetic systems, block layout, projector tables."""
import numpy as np
import pytest

from cyclix_msparc_gb300.cychel import cyclix_kpoints, intg_weights, fd_weights
from cyclix_msparc_gb300.workloads import WORKLOADS, block_layout, initial_psi, make_system


def test_cyclix_kpoints_nu_and_time_reversal():
    # n_cyc = 12 (L2 = 2 pi / 12), 4 theta points: nu = round(12 j / 4) = 0, 3, 6, 9; the pair
    # (3, 9) sums to 2 pi / L2 = 12 and is merged into nu = 9 with double weight
    # (src/initialization.m:1624-1636, 1657-1674)
    L2 = 2 * np.pi / 12
    k, w = cyclix_kpoints((1, 4, 1), 8.0, L2, 4.0, time_reversal=False)
    assert np.array_equal(k[:, 1], [0.0, 3.0, 6.0, 9.0])
    assert np.allclose(w, 0.25)
    k, w = cyclix_kpoints((1, 4, 1), 8.0, L2, 4.0, time_reversal=True)
    assert np.array_equal(k[:, 1], [0.0, 6.0, 9.0])
    assert np.allclose(w, [0.25, 0.25, 0.5])
    assert abs(np.sum(w) - 1) < 1e-15


def test_cyclix_kpoints_eta_grid():
    # Monkhorst-Pack along z, mapped into (-1/2, 1/2] and scaled by 2 pi / L3
    L3 = 4.0
    k, w = cyclix_kpoints((1, 1, 4), 8.0, 2 * np.pi / 12, L3, time_reversal=False)
    eta = k[:, 2] * L3 / (2 * np.pi)
    assert np.allclose(np.sort(eta), [-0.25, 0.0, 0.25, 0.5])
    k2, w2 = cyclix_kpoints((1, 1, 4), 8.0, 2 * np.pi / 12, L3, time_reversal=True)
    assert abs(np.sum(w2) - 1) < 1e-15 and len(k2) == 3


def test_intg_weights_volume():
    xin, dx, Nx = 3.0, 0.25, 33
    W = intg_weights(Nx, 10, 8, 0, 0, xin, dx, 0.05, 0.2)
    vol = 0.5 * ((xin + (Nx - 1) * dx) ** 2 - xin ** 2) * 10 * 0.05 * 8 * 0.2
    assert abs(W.sum() - vol) < 1e-12 * vol


def test_fd_weights_shapes():
    w1, w2 = fd_weights(6)
    assert w1.shape == (7,) and w2.shape == (7,) and w1[0] == 0.0


def test_batched_block_sizes():
    wl = WORKLOADS["cyclic-batched-16nu-64x16x48-ns96to320-m24"]
    assert len(wl.Ns) == 16 and sum(wl.Ns) == 3345
    assert all(96 <= n <= 320 for n in wl.Ns)
    assert [k[1] for k in wl.kpts] == list(range(16))


def test_helical_block_count():
    wl = WORKLOADS["helical-80x32x40-96k2s-ns192-m24"]
    assert wl.nblocks == 192 and wl.nspin == 2 and len(wl.kpts) == 96


def test_make_system_deterministic_and_layout():
    wl = WORKLOADS["scf-small-24x12x20-12at-2k-ns40"]
    S1, S2 = make_system(wl), make_system(wl)
    assert np.array_equal(S1.b, S2.b) and np.array_equal(S1.rho_at, S2.rho_at)
    assert np.array_equal(S1.Atoms, S2.Atoms)
    # the pseudocharges integrate to -Z per atom, the initial density to the electron count
    assert abs(float(S1.W @ S1.b) + 4.0 * wl.n_atm) < 1e-3 * 4.0 * wl.n_atm
    assert abs(float(S1.W @ S1.rho_at) + S1.NegCharge) < 1e-12 * abs(S1.NegCharge)
    bl = block_layout(wl, S1)
    assert [n for (_, _, n) in bl] == list(wl.Ns)
    assert all(spin == 0 for (_, spin, _) in bl)


def test_block_layout_spin_major():
    from cyclix_msparc_gb300.workloads import Workload
    wl = Workload("t", 16, 8, 10, (4, 5, 6, 7), ((0.0, 0.0, 0.0), (0.0, 1.0, 0.0)), 2, 4, 2, 12, L1=4.0, xin=4.0)
    S = make_system(wl)
    bl = block_layout(wl, S)
    assert [(int(k[1]), s, n) for (k, s, n) in bl] == [(0, 0, 4), (1, 0, 5), (0, 1, 6), (1, 1, 7)]
    assert S.Veff.shape == (S.N, 2)


def test_projector_tables_in_range():
    wl = WORKLOADS["cyclic-40x12x20-ns48-m20"]
    S = make_system(wl)
    assert len(S.Atom) == wl.n_atm
    for A in S.Atom:
        assert A.angnum == 4 and A.gamma_Jl.shape == (4,)
        for img in A.rcImage:
            assert img.rc_pos.min() >= 1 and img.rc_pos.max() <= S.N       # 1-based, as in MATLAB
            assert img.Chi_mat.shape == (img.rc_n_nodes, 4)
            assert len(np.unique(img.rc_pos)) == img.rc_n_nodes


def test_initial_psi_orthonormal():
    X = initial_psi(500, 7, 3)
    assert np.allclose(X.conj().T @ X, np.eye(7), atol=1e-12)
    assert X.flags.f_contiguous


def test_host_buffer_checks_reject_what_the_library_would_overrun():
    # arrays handed to the C library by pointer are checked before the call (not by assert)
    from cyclix_msparc_gb300.msparc import _host_buffer
    _host_buffer(np.zeros(5), np.float64, 5, "EigVal")
    _host_buffer(np.zeros((4, 3), dtype=np.complex128, order="F"), np.complex128, 12, "psi")
    bad = [
        (np.zeros(4), np.float64, 5, "elements"),                        # too short
        (np.zeros(5, dtype=np.float32), np.float64, 5, "float64"),       # wrong dtype
        ([0.0] * 5, np.float64, 5, "numpy array"),                       # not an array
        (np.zeros(10)[::2], np.float64, 5, "contiguous"),                # strided view
    ]
    for a, dt, n, msg in bad:
        with pytest.raises(ValueError, match=msg):
            _host_buffer(a, dt, n, "x")
    ro = np.zeros(5)
    ro.setflags(write=False)
    with pytest.raises(ValueError, match="writable"):
        _host_buffer(ro, np.float64, 5, "x")


def test_operator_inputs_need_n_rows():
    # hpsi / filter read N x ncol values: other row counts are refused on the host
    from cyclix_msparc_gb300.msparc import CyclixGPU
    g = CyclixGPU.__new__(CyclixGPU)         # no handle: only the host-side check runs
    g.N = 12
    assert g._columns(np.ones(12), "hpsi").shape == (12, 1)
    assert g._columns(np.ones((12, 3)), "hpsi").flags.f_contiguous
    with pytest.raises(ValueError, match="N = 12 rows"):
        g._columns(np.ones((11, 3)), "hpsi")
    with pytest.raises(ValueError, match="N = 12 rows"):
        g._columns(np.ones((12, 3, 2)), "filter")


@pytest.mark.parametrize("n_cyc,expect", [(5, [0.0, 3.0]), (9, [0.0, 5.0]), (13, [0.0, 7.0])])
def test_cyclix_kpoints_round_half_away_from_zero(n_cyc, expect):
    # nu = round((2 pi / L2) * j / n) with MATLAB's round (src/initialization.m:1640): an odd
    # wedge order with two theta points puts nu exactly on a half, which rounds up
    k, w = cyclix_kpoints((1, 2, 1), 8.0, 2 * np.pi / n_cyc, 4.0, time_reversal=False)
    assert k[:, 1].tolist() == expect
