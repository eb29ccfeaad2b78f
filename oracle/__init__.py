"""CPU oracle for the Cyclix CheFSI path — TEST INFRASTRUCTURE ONLY.

This package restates, in NumPy/SciPy, the reference MATLAB functions on the
Chebyshev-filtered subspace iteration path (eigSolver -> chebyshev_filter ->
h_nonlocal_vector_mult -> lapVec_cychel), the AAR Poisson solve and the SCF
bookkeeping.  Each function cites the reference file:line it follows (paths
relative to the reference project root ``Cyclix_MS_200220/``).

It is the checker, never the product: only ``tests/``, ``__graft_entry__.smoke()``
and the CPU-baseline leg of ``bench.py`` may import it.

Parity status: UNPINNED against reference-run vectors.  The reference is
MATLAB; neither MATLAB nor Octave exists on the build or GPU machines, and the
reference ships no golden vectors or known-answer tests for this path (its
``tests/`` hold only end-to-end ``.out`` files of full psp8 runs).  The oracle
is instead pinned to mathematical known answers that the reference's
algorithm must satisfy (see ``tests/test_oracle_kat.py``): exactness of the
FD weights on polynomials, 12th-order convergence of the Cyclix Laplacian on
analytic fields with Bloch factors, agreement of the matrix-free operator with
the assembled ``Lap_std``, the Chebyshev filter against a dense
eigendecomposition, and subspace eigenvalues against dense ``eig`` on tiny
grids.  The golden fixtures under ``tests/golden/`` were produced by this
oracle by ``tests/golden/make_golden.py``.
"""
