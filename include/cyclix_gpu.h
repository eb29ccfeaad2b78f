/*
 * cyclix_gpu.h -- C-ABI of libcyclix_gpu.so, the GB300 (sm_103a) implementation of
 * Cyclix's Chebyshev-filtered subspace iteration.
 *
 * The entry points replace the reference's MATLAB functions on the CheFSI path
 * (paths relative to the reference project root Cyclix_MS_200220/):
 *
 *   cx_hpsi             h_nonlocal_vector_mult(DL11,DL22,DL33,DG1,DG2,DG3,Veff,X,S,kptvec)
 *                         src/h_nonlocal_vector_mult.m:1 (with lapVec src/lapVec.m:1 ->
 *                         Cychel/lapVec_cychel.m:1)
 *   cx_chebyshev_filter chebyshev_filter(X,m,a,b,a0,DL11,...,Veff,S,kpt_vec)
 *                         src/chebyshev_filter.m:1
 *   cx_eigsolver        [ubgv,psi,EigVal,a0,bup,lambda_cutoff] = eigSolver(S,count,ubgv,psi,EigVal,a0,bup,lambda_cutoff)
 *                         src/eigSolver.m:1, called from src/scf.m:123-124
 *   cx_poisson          S = poissonSolve(S,poisson_tol,Isguess) -> aar(Lap_std,f,...)
 *                         src/poissonSolve.m:1, src/aar.m:1
 *   cx_scf              S = scf(S): the SCF loop around eigSolver (first relaxation step,
 *                         nspin = 1, potential mixing) src/scf.m:1-327
 *   cx_xc               S = exchangeCorrelationPotential(S) (nspin = 1: LDA_PW, LDA_PZ, GGA_PBE)
 *                         src/exchangeCorrelationPotential.m:1-80
 *   cx_nonlocal_force   the nonlocal term of S = atomicForce(S) src/atomicForce.m:254-300
 *   cx_gradient         S.grad_1..3 * f (blochGradient(S,[0 0 0],d), src/initialization.m:743-745)
 *   cx_field_projections  the grid sums of the local and correction forces src/atomicForce.m:111-127
 *
 * The operator data that MATLAB keeps in the struct S (grid, FD weights,
 * quadrature weights, KB projector images) is handed over once in cx_create;
 * the Bloch blocks (k-point, spin, number of states) in cx_set_blocks.
 *
 * Conventions
 *  - Host arrays are MATLAB column-major.  Complex arrays are interleaved
 *    (re, im) doubles, i.e. the R2018a mxGetComplexDoubles layout.
 *  - psi of one block is N x Ns, N = Nx*Ny*Nz with x (r) fastest, then y (theta), then z.
 *  - Every call returns a cx_status; CX_OK is 0.  No call aborts or exits the
 *    process.  cx_last_error() gives the message of the last failure.
 *  - One CUDA stream per handle; calls on one handle are not thread-safe.
 */
#ifndef CYCLIX_GPU_H
#define CYCLIX_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int32_t cx_status;
enum {
  CX_OK = 0,
  CX_ERR_ARG = 1,        /* invalid argument (sizes, null pointers, unsupported FD order) */
  CX_ERR_CUDA = 2,       /* CUDA runtime error */
  CX_ERR_NOMEM = 3,      /* device allocation failed */
  CX_ERR_LIB = 4,        /* cuBLAS / cuSOLVER error */
  CX_ERR_NOTPD = 5,      /* Gram matrix not positive definite (filtered block lost rank) */
  CX_ERR_STATE = 6,      /* call out of order (e.g. eigensolver before cx_set_blocks) */
  CX_ERR_NOCONV = 7      /* iterative solver hit its iteration limit */
};

/* Arithmetic of the filter / subspace path. */
enum {
  CX_PREC_FP64 = 0,      /* complex128 everywhere: the plain FP64 path */
  CX_PREC_MIXED = 1      /* complex64 filter and H*psi, tcgen05 3xTF32 Rayleigh-Ritz products (FP32
                            accumulation over short ranges, FP64 across them), FP64 Cholesky /
                            eigensolver / refinement */
};

typedef struct cx_handle_s* cx_handle;

/* Grid and discretisation: the S fields that lapIndicesValues_1d_cychel
 * (Cychel/lapIndicesValues_1d_cychel.m:9-15) and intgWts_cychel read. */
typedef struct {
  int32_t Nx, Ny, Nz;        /* nodes (S.Nx etc. after the +BC node) */
  int32_t FDn;               /* half FD order; 1..8 supported (FD order 12 -> 6) */
  int32_t cell_typ;          /* 3 cyclic, 4/5 helical */
  int32_t BCx, BCy, BCz;     /* 1 Dirichlet, 0 periodic; BCx must be 1 (radial walls) */
  double dx, dy, dz;
  double xin;                /* inner radius */
  double twist;              /* S.twist (rad/bohr); 0 for cell_typ 3 */
  double L1, L2, L3;
  const double* w1;          /* S.w1, FDn+1 entries (src/initialization.m:413-418) */
  const double* w2;          /* S.w2, FDn+1 entries (src/initialization.m:404-410) */
  const double* W;           /* S.W, N quadrature weights (Cychel/intgWts_cychel.m) */
} cx_grid;

/* S.Atom(J).rcImage(img) (src/calculate_nloc_projector.m:185-198) */
typedef struct {
  int32_t rc_n_nodes;
  const int64_t* rc_pos;     /* 1-based linear grid indices */
  const double* Chi_mat;     /* rc_n_nodes x angnum, column-major */
  double coordinates[3];     /* image position (r, theta, z) */
} cx_rc_image;

/* S.Atom(J) and S.Atoms(J,:) (src/calculate_nloc_projector.m:252-277) */
typedef struct {
  int32_t angnum;
  int32_t n_image_rc;
  const double* gamma_Jl;    /* angnum */
  double position[3];        /* S.Atoms(J,:) */
  const cx_rc_image* rcImage;
} cx_atom;

/* One (k-point, spin) block: eigSolver's ks (src/eigSolver.m:26-33). */
typedef struct {
  double kpt_vec[3];         /* S.kptgrid(kpt,:) */
  int32_t spin;              /* 0-based spin channel (column of S.Veff) */
  int32_t Ns;                /* states in this block (S.Nev; may differ per block) */
} cx_block;

/* ---- lifecycle ---------------------------------------------------------- */
cx_status cx_create(const cx_grid* grid, int32_t n_atm, const cx_atom* atoms, int32_t nspin, cx_handle* out);
cx_status cx_destroy(cx_handle h);
/* Message of the last failed call on h (or of the last failed cx_create when h is NULL). */
const char* cx_last_error(cx_handle h);
/* Library version string. */
const char* cx_version(void);
/* Device of the handles the calling thread creates next (default: device 0).  One process per
 * GPU selects its local device once before cx_create; no reference counterpart (MATLAB runs one
 * process on one device). */
cx_status cx_set_device(int32_t device);

/* Blocks and working precision; allocates two device buffers per block
 * (psi and one work array).  Replaces any previous block set. */
cx_status cx_set_blocks(cx_handle h, int32_t nblk, const cx_block* blocks, int32_t prec);
/* S.Veff: N x nspin, column-major (src/scf.m:39). */
cx_status cx_set_veff(cx_handle h, const double* Veff);
/* Device-resident psi of one block: host N x Ns complex (interleaved). */
cx_status cx_set_psi(cx_handle h, int32_t blk, const double* psi);
cx_status cx_get_psi(cx_handle h, int32_t blk, double* psi);

/* ---- the MATLAB functions ---------------------------------------------- */
/* Hnlx = h_nonlocal_vector_mult(..., Veff, X, S, kptvec) for block blk:
 * X, Y host N x ncol complex.  prec selects complex128 or complex64 arithmetic. */
cx_status cx_hpsi(cx_handle h, int32_t blk, int32_t ncol, const double* X, double* Y, int32_t prec);

/* Y = chebyshev_filter(X, m, a, b, a0, ...) for block blk (a = cutoff, b = upper
 * bound, a0 = lower bound, as the reference names them at src/chebyshev_filter.m:1). */
cx_status cx_chebyshev_filter(cx_handle h, int32_t blk, int32_t ncol, const double* X, double* Y,
                              int32_t m, double a, double b, double a0, int32_t prec);

/* The eigSolver step over all blocks on the device-resident psi (src/eigSolver.m:26-125) for the
 * first relaxation step without upper-bound vectors (cx_eigsolver_full with elecgs_Count = 1,
 * chefsibound_flag = 0, ubgv = NULL): spectral bounds when count == 1 (Lanczos), filter cutoff, Chebyshev filter of degree npl,
 * orthonormalisation, projected Hamiltonian, general FP64 subspace eigensolver, sort,
 * rotation and W-normalisation.  EigVal is packed: block b's Ns_b values follow block b-1's.
 * a0, bup, lambda_cutoff have nblk entries each (in/out).  rhoTrigger as src/scf.m:93. */
cx_status cx_eigsolver(cx_handle h, int32_t count, int32_t npl, int32_t rhoTrigger,
                       double* EigVal, double* a0, double* bup, double* lambda_cutoff);

/* The same step with host psi in and out (N x Ns_b per block, blocks back to back),
 * the drop-in for a MEX call that passes S.psi: the copies are part of the call. */
cx_status cx_eigsolver_host(cx_handle h, int32_t count, int32_t npl, int32_t rhoTrigger, double* psi,
                            double* EigVal, double* a0, double* bup, double* lambda_cutoff);

/* The S fields that steer eigSolver's bounds and cutoff (src/eigSolver.m:21-94). */
typedef struct {
  int32_t npl;               /* S.npl: Chebyshev degree */
  int32_t rhoTrigger;        /* S.rhoTrigger (taken as 1 when elecgs_Count > 1, src/eigSolver.m:21-23) */
  int32_t elecgs_Count;      /* S.elecgs_Count: 1 on the first relaxation / MD step, > 1 after it */
  int32_t chefsibound_flag;  /* S.chefsibound_flag: 1 re-estimates bup from ubgv once count > rhoTrigger */
} cx_eig_params;

/* [ubgv,psi,EigVal,a0,bup,lambda_cutoff] = eigSolver(S,count,ubgv,psi,EigVal,a0,bup,lambda_cutoff)
 * with the whole control flow of src/eigSolver.m:21-94:
 *  - count == 1, elecgs_Count == 1: bup = 1.01 x the largest and a0 = the smallest Ritz value - 0.1
 *    of a Lanczos run from a random vector; cutoff (bup + a0) / 2;
 *  - count == 1, elecgs_Count > 1: bup from a Lanczos run started at ubgv, a0 = min(EigVal)
 *    (the previous relaxation step's eigenvalues), cutoff max(EigVal) + 0.1;
 *  - count > rhoTrigger: a0 = min(EigVal); with chefsibound_flag == 1 also bup from a Lanczos
 *    run started at ubgv;
 *  - otherwise the bounds are kept; cutoff max(EigVal) + 0.1.
 * ubgv is S.upper_bound_guess_vecs: N x nblk complex (interleaved), in and out.  Every upper-bound
 * estimate writes the Ritz vector of its largest Ritz value (2-norm 1) into the block's column;
 * a zero column, or ubgv == NULL, starts that block from the seeded random vector (ubgv == NULL
 * also returns no vector).  psi is device-resident (cx_set_psi / cx_get_psi). */
cx_status cx_eigsolver_full(cx_handle h, const cx_eig_params* p, int32_t count, double* ubgv, double* EigVal, double* a0,
                            double* bup, double* lambda_cutoff);
/* The same with host psi in and out (blocks back to back), copied in and out by the call. */
cx_status cx_eigsolver_full_host(cx_handle h, const cx_eig_params* p, int32_t count, double* ubgv, double* psi, double* EigVal,
                                 double* a0, double* bup, double* lambda_cutoff);

/* Number of subspace eigen-decompositions (since cx_create) that could not use the fast
 * Hermitian-plus-refinement path and ran the general FP64 solver instead. */
cx_status cx_eig_fallback_count(cx_handle h, int64_t* count);
/* Number of subspace eigen-decompositions (since cx_create) answered by the eigenpairs of the
 * Hermitian part of the W-similar projected matrix: blocks of more than 512 states whose
 * refinement did not converge, and any block whose other results would have left the rotated
 * block ill-conditioned (eigenvalues equal to the real parts of the exact ones up to second order
 * in the non-Hermitian part, W-orthonormal rotation). */
cx_status cx_eig_hermitian_count(cx_handle h, int64_t* count);

/* phi = aar(Lap_std, f, guess, tol, maxit, 0.6, 0.6, 7, 6, ...) (src/poissonSolve.m:36,
 * src/aar.m:1-74) with f = -4*pi*(rho+b) given; a Jacobi preconditioner replaces ILU.
 * phi is the initial guess when use_guess != 0 (else ones, as aar.m:51-53) and the result. */
cx_status cx_poisson(cx_handle h, const double* f, double* phi, double tol, int32_t maxit,
                     int32_t use_guess, int32_t* iters, double* relres);

/* H*psi of block blk on caller-owned DEVICE buffers that allocates no device memory.
 * No counterpart in the reference: it exists for callers that cannot let a library call
 * cudaMalloc because another allocator owns their device memory (a framework's caching
 * allocator, a MEX session that must leave nothing allocated when interrupted).
 * X_dev, Y_dev: N x ncol column-major, complex128 (prec CX_PREC_FP64) or complex64
 * (CX_PREC_MIXED), distinct.  The projector scratch lives in a fixed 16 MiB device array of
 * the library (held by every GPU that loads it until exit); a call that needs more returns
 * CX_ERR_ARG naming the largest ncol that fits.  Calls share the array: calls whose work
 * overlaps on the GPU race.  Each call waits for its own work before returning (a stream
 * synchronisation), so a call cannot be recorded into a CUDA graph.  The call
 * runs on the handle's own stream, which is not ordered after the caller's streams: X_dev must be
 * completely written (the caller synchronises the stream that wrote it) before the call. */
cx_status cx_hpsi_noalloc(cx_handle h, int32_t blk, int32_t ncol, const void* X_dev, void* Y_dev, int32_t prec);

/* Exchange-correlation functional: the reference's S.xc codes (src/initialization.m:145-154). */
enum {
  CX_XC_LDA_PW = 0,      /* Perdew-Wang 1992 LDA (src/exchangeCorrelationPotential.m:82-106) */
  CX_XC_LDA_PZ = 1,      /* Perdew-Zunger 1981 LDA (src/evaluateTotalEnergy.m:44-60) */
  CX_XC_GGA_PBE = 2      /* PBE GGA on the Cyclix gradients (src/exchangeCorrelationPotential.m:156-362) */
};

/* S = exchangeCorrelationPotential(S) for nspin = 1 on the density rho (N, host): Vxc (N) and
 * e_xc (N), the energy per particle at the density clipped below at 1e-14 (S.xc_rhotol), so that
 * Exc = sum(e_xc .* max(rho, 1e-14) .* W) (src/evaluateTotalEnergy.m:25-62).  xc is a CX_XC_*
 * code.  GGA_PBE differentiates the clipped density with the order-2 FDn first-derivative
 * stencils of the Cyclix grid (Cartesian components through the local angle theta + twist z,
 * Cychel/gradIndicesValues_cychel.m) and forms Vxc = d(rho e_xc)/d rho - div(2 d(rho e_xc)/d sigma
 * grad rho) with the same operators (src/exchangeCorrelationPotential.m:354-362); it needs theta
 * and z periodic.  Allocates and frees its device work arrays. */
cx_status cx_xc(cx_handle h, int32_t xc, const double* rho, double* Vxc, double* e_xc);

/* Nonlocal part of the atomic forces (src/atomicForce.m:254-300) from the device-resident psi of
 * every block: for each block (Bloch vector k, weight wkpt[b], occupations occ packed like EigVal)
 * the Bloch-summed projectors of every atom and their Cartesian gradients on the grid (the x / y
 * pair with the wedge rotation across the theta wrap, Cychel/div_gradvec_cychel.m), and
 *   F_J -= occfac 2 wkpt[b] sum_n occ_n sum_c gamma_c Re[conj(<psi_n|W chi_c>) (-<psi_n|W D chi_c>)].
 * F is n_atm x 3, column-major, for the atoms of cx_create (an atom passed as several 4-column
 * atoms gets one row per part; their sum is its force).  complex64 blocks are widened to
 * complex128 for the products.  Allocates and frees its device work arrays (7 N x 4 n_atm complex
 * values and one block of psi). */
cx_status cx_nonlocal_force(cx_handle h, const double* occ, const double* wkpt, double occfac, double* F);

/* Cartesian gradient of a real grid field at k = 0 (the S.grad_1, S.grad_2, S.grad_3 products
 * src/atomicForce.m applies to phi and V_c): D_x = cos(phi) d_r - sin(phi)/r d_theta,
 * D_y = sin(phi) d_r + cos(phi)/r d_theta, D_z = d_z - twist d_theta with phi = theta + twist z,
 * order-2 FDn first-derivative stencils, zero beyond the radial walls, theta and z periodic.
 * f: N values; Df: N x 3, column-major. */
cx_status cx_gradient(cx_handle h, const double* f, double* Df);

/* Projections of the gradient of a real grid field on nvec grid vectors: out (nvec x 3,
 * column-major) = A^T [D_x f, D_y f, D_z f], A N x nvec column-major, D as cx_gradient.  The local
 * and correction terms of src/atomicForce.m:111-127 are such projections of D phi and D V_c on
 * per-atom sums of W bJ over the atom's image boxes (the host set-up reduces them so). */
cx_status cx_field_projections(cx_handle h, const double* f, int32_t nvec, const double* A, double* out);

/* SCF parameters: the S fields read by src/scf.m (nspin = 1, potential mixing). */
typedef struct {
  double scf_tol;            /* S.SCF_tol: stop when ||Veff - Veff_in|| / ||Veff|| <= scf_tol */
  double poisson_tol;        /* S.poisson_tol (<= 0: 0.01 * scf_tol, src/initialization.m:548-552) */
  int32_t max_scf, min_scf;  /* S.MAXIT_SCF, S.MINIT_SCF */
  int32_t rhoTrigger;        /* S.rhoTrigger (Chebyshev cycles of the first SCF step) */
  int32_t npl;               /* S.npl */
  int32_t maxit_poisson;     /* S.MAXIT_POISSON */
  int32_t elec_T_type;       /* 0 Fermi-Dirac, 1 Gaussian smearing */
  double bet;                /* S.bet (1 / smearing) */
  double occfac;             /* S.occfac */
  double NegCharge;          /* S.NegCharge */
  double Eself, E_corr;      /* S.Eself, S.E_corr */
  int32_t n_atm;             /* S.n_atm (energy per atom in hist) */
  double mixing_param;       /* S.MixingParameter */
  const double* wkpt;        /* k-point weight of each block (nblk) */
  const double* b;           /* S.b, pseudocharge density (N) */
  const double* rho0;        /* initial density (N) */
  int32_t refine;            /* != 0: after the loop, replace the eigenvalues by FP64 Rayleigh quotients of
                                H[Veff_in] (cx_refine_eigenvalues) and re-evaluate occupations and energy */
  double fp64_tol;           /* > 0 with complex64 blocks (cx_scf only): after the mixed-precision loop,
                                switch the blocks to complex128 (psi converted) and continue with FP64
                                passes until the error is <= fp64_tol (at most max_scf more): the fixed
                                point of the reference's arithmetic.  The blocks stay complex128. */
  int32_t xc;                /* S.xc: CX_XC_LDA_PW (0, the value of a zeroed struct), CX_XC_LDA_PZ or
                                CX_XC_GGA_PBE; the potential and energy of every SCF step use it */
} cx_scf_params;

typedef struct {
  double Etotal;             /* free energy (Ha) of the last SCF step, with Escc */
  double lambda_f;           /* Fermi level */
  double err;                /* last SCF error */
  int32_t n_scf;             /* SCF steps taken */
  int32_t converged;
} cx_scf_result;

/* S = scf(S) (src/scf.m:1-327) on the device-resident psi of the handle's blocks: initial
 * potential from rho0, then eigSolver / occupations / density / Poisson / Vxc (p->xc) / energy /
 * Periodic-Pulay potential mixing until converged.  EigVal (packed, sum Ns), rho (N), Veff (N)
 * and hist (max_scf x 2, or 2 max_scf x 2 with p->fp64_tol > 0: energy per atom, error per SCF
 * step) are outputs (rho, Veff, hist may be NULL). */
cx_status cx_scf(cx_handle h, const cx_scf_params* p, double* EigVal, double* rho, double* Veff, double* hist,
                 cx_scf_result* res);

/* One SCF step at a time: the same loop as cx_scf, driven by the caller (src/scf.m:111-306).
 * cx_scf_init sets the initial potential from p->rho0 (src/scf.m:32-39); each cx_scf_step is
 * one pass of the loop body: the eigSolver step, occupations and, once count >= rhoTrigger, the
 * density, Poisson solve, exchange-correlation potential, energy, error and Pulay mixing; cx_scf_finish
 * applies the optional FP64 refinement and returns the results (EigVal, rho, Veff may be NULL).
 * The caller stops when info.converged is set or its step limit is reached, as src/scf.m:111. */
typedef struct {
  double Etotal;             /* free energy (Ha) after this step (of the last density update) */
  double lambda_f;           /* Fermi level of this step's occupations */
  double err;                /* SCF error ||Veff - Veff_in|| / ||Veff|| of the last density update */
  int32_t count;             /* eigSolver passes so far (the reference's count) */
  int32_t n_scf;             /* density updates so far (the reference's count_SCF - 1) */
  int32_t density_updated;   /* 1 when this pass updated the density (count >= rhoTrigger) */
  int32_t converged;         /* err <= scf_tol after at least min_scf density updates */
  int32_t poisson_iters;     /* AAR iterations of this pass's Poisson solve (0 without one) */
  int32_t pad;
  double step_ms;            /* device time of the pass (CUDA events on the handle's stream; the
                                copies of psi_host are outside it) */
  double poisson_ms;         /* device time of the Poisson solve within it */
  double filter_ms;          /* device time of the spectral bounds, the filter and H X within it */
  double rr_ms;              /* device time of the Rayleigh-Ritz steps of all blocks within it */
} cx_scf_step_info;

cx_status cx_scf_init(cx_handle h, const cx_scf_params* p);
/* psi_host (may be NULL): S.psi on the host, blocks back to back (N x Ns_b complex each); copied
 * to the device before the pass and back after it, as a MEX eigSolver call passes S.psi.
 * EigVal (may be NULL): this pass's eigenvalues, packed over blocks. */
cx_status cx_scf_step(cx_handle h, double* psi_host, double* EigVal, cx_scf_step_info* info);
cx_status cx_scf_finish(cx_handle h, double* EigVal, double* rho, double* Veff, cx_scf_result* res);

/* FP64 refinement of the Ritz values of the device-resident psi: lambda_j = Re(psi_j^H W H psi_j) /
 * (psi_j^H W psi_j) with H applied in complex128 (the Hamiltonian is self-adjoint in the W inner
 * product, so the error is second order in the error of psi).  EigVal packed (sum Ns), output. */
cx_status cx_refine_eigenvalues(cx_handle h, double* EigVal);

/* ---- measurement -------------------------------------------------------- */
/* Wait for all work of h. */
cx_status cx_sync(cx_handle h);
/* CUDA-event timer on the handle's stream. */
cx_status cx_timer_start(cx_handle h);
cx_status cx_timer_stop(cx_handle h, double* ms);
/* Per-kernel device timing of the Chebyshev stencil launches (enable, then read
 * launches and total ms since enabling). */
cx_status cx_profile_stencil(cx_handle h, int32_t enable);
cx_status cx_profile_read(cx_handle h, int64_t* launches, double* total_ms, double* bytes);
/* Device time (ms) of the separate projector-apply launches that follow the complex64 stencil
 * launches, over the same profiling window (0 for the complex128 path, which fuses it). */
cx_status cx_profile_read_apply(cx_handle h, double* apply_ms);
/* Kernels of the complex64 projector term: 0 (default) the CUDA-core contraction and apply,
 * 1 the tcgen05 tensor-core contraction and apply (3xTF32; the apply on grids eligible for the
 * TMA stencil).  Both compute the same term; the CUDA-core pair is the faster one on the
 * benchmarked cells. */
cx_status cx_set_nl_kernels(cx_handle h, int32_t tensor_cores);
/* Summed time (ms) of the projector contraction launches since cx_profile_stencil enabled profiling. */
cx_status cx_profile_read_contract(cx_handle h, double* contract_ms);
/* Page-lock a caller-owned host buffer for faster copies (cudaHostRegister) and release it. */
cx_status cx_host_register(void* ptr, size_t bytes);
cx_status cx_host_unregister(void* ptr);
/* Configuration of the complex64 stencil kernel on h: rows per thread and TMA prefetch depth
 * (0: the default rule), whether the autotuner chose them (it times every configuration on the
 * first full-size filter step of the handle), and its log ("rows/depth:ms ...", may be NULL). */
cx_status cx_stencil_config(cx_handle h, int32_t* rows_per_thread, int32_t* ring_depth, int32_t* tuned, char* log, int32_t log_bytes);
/* Number of this library's kernel launches issued on h since the last reset. */
cx_status cx_launch_count(cx_handle h, int64_t* count, int32_t reset);

#ifdef __cplusplus
}
#endif
#endif /* CYCLIX_GPU_H */
