"""CPU oracle for the Cyclix CheFSI path — TEST INFRASTRUCTURE ONLY.

This package restates, in NumPy/SciPy, the reference MATLAB functions on the
Chebyshev-filtered subspace iteration path (eigSolver -> chebyshev_filter ->
h_nonlocal_vector_mult -> lapVec_cychel), the AAR Poisson solve, the SCF
bookkeeping (LDA_PW, LDA_PZ, GGA_PBE; Gaussian and Fermi-Dirac smearing) and
the atomic forces.  Each function cites the reference file:line it follows
(paths relative to the reference project root ``Cyclix_MS_200220/``).

It is the checker, never the product: only ``tests/``, ``__graft_entry__.smoke()``
and the CPU-baseline leg of ``bench.py`` may import it.

Parity status: pinned to the reference's own outputs.  The reference is MATLAB;
neither MATLAB nor Octave exists on the build or GPU machines, and it ships no
golden vectors for this path.  Its ``.out`` / ``.static`` files of full psp8
runs are used instead: loaded from the same decks, the oracle reproduces the
printed self and correction energies, free energies and forces of cyclic and
helical decks (``tests/golden/pin_decks.py``, ``tests/golden/deck_pins.json``,
``tests/test_decks.py``).  Below that it is pinned to mathematical known
answers the reference's algorithm must satisfy (``tests/test_oracle_kat.py``,
``tests/test_oracle_scf_kat.py``): exactness of the FD weights on polynomials,
12th-order convergence of the Cyclix Laplacian on analytic fields with Bloch
factors, agreement of the matrix-free operator with the assembled ``Lap_std``,
the Chebyshev filter against a dense eigendecomposition, and subspace
eigenvalues against dense ``eig`` on tiny grids.  The golden fixtures under
``tests/golden/`` were produced by this oracle by ``tests/golden/make_golden.py``.
"""
