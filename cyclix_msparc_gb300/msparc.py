"""Host mirror of the reference's MATLAB functions on the CheFSI path, backed by libcyclix_gpu.so.

The function names, argument order and meaning follow the reference (paths relative to the
reference project root ``Cyclix_MS_200220/``):

* ``h_nonlocal_vector_mult(DL11,DL22,DL33,DG1,DG2,DG3,Veff,X,S,kptvec)``  src/h_nonlocal_vector_mult.m:1
* ``chebyshev_filter(X,m,a,b,a0,DL11,DL22,DL33,DG1,DG2,DG3,Veff,S,kpt_vec)``  src/chebyshev_filter.m:1
* ``eigSolver(S,count,upper_bound_guess_vecs,psi,EigVal,a0,bup,lambda_cutoff)``  src/eigSolver.m:1
* ``poissonSolve(S,poisson_tol,Isguess)``  src/poissonSolve.m:1
* ``exchangeCorrelationPotential(S)`` (nspin = 1)  src/exchangeCorrelationPotential.m:1
* ``scf(S)``  src/scf.m:1

MATLAB hands the six 1-D operators to the first two; on the GPU the operator is rebuilt from
the grid in ``S`` and the Bloch vector, so those arguments are accepted and not read.  The GPU
state (a ``cx_handle``) lives in ``S.gpu`` (see :func:`attach`).  Every failure of the library
raises :class:`CxError`; nothing falls back to a CPU implementation.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import CxError, check, cptr, dptr
from .cychel import split_projector_columns

__all__ = ["CyclixGPU", "attach", "h_nonlocal_vector_mult", "chebyshev_filter", "eigSolver", "poissonSolve",
           "exchangeCorrelationPotential", "scf", "CxError"]


def _host_buffer(a, dtype, size: int, name: str) -> None:
    """Check an array that the library reads or writes through a raw pointer: its dtype, one
    contiguous block, at least ``size`` elements and, since the library writes into it, writable.
    Anything else would make the library touch memory outside the array, so it raises
    ``ValueError`` before the call (independently of ``python -O``)."""
    if not isinstance(a, np.ndarray) or a.dtype != np.dtype(dtype):
        got = a.dtype if isinstance(a, np.ndarray) else type(a).__name__
        raise ValueError(f"{name}: need a numpy array of {np.dtype(dtype).name}, got {got}")
    if not (a.flags.c_contiguous or a.flags.f_contiguous):
        raise ValueError(f"{name}: the array must be one contiguous block")
    if not a.flags.writeable:
        raise ValueError(f"{name}: the array must be writable (the library updates it in place)")
    if a.size < size:
        raise ValueError(f"{name}: {a.size} elements, the library needs {size}")


class CyclixGPU:
    """Owns one ``cx_handle``: the discretised operator of ``S`` and its Bloch blocks."""

    def __init__(self, S, blocks, prec: str = "mixed"):
        self.lib = _lib.load()
        self.S = S
        self.prec = prec
        self.N = int(S.Nx * S.Ny * S.Nz)
        keep = []

        def darr(a):
            a = np.ascontiguousarray(a, dtype=np.float64)
            keep.append(a)
            return dptr(a)

        g = _lib.cx_grid(Nx=S.Nx, Ny=S.Ny, Nz=S.Nz, FDn=S.FDn, cell_typ=S.cell_typ, BCx=S.BCx, BCy=S.BCy, BCz=S.BCz,
                         dx=S.dx, dy=S.dy, dz=S.dz, xin=S.xin, twist=S.twist, L1=S.L1, L2=S.L2, L3=S.L3,
                         w1=darr(S.w1), w2=darr(S.w2), W=darr(S.W))
        # the library's projector kernels hold 4 columns per atom: psp8 atoms with more are passed
        # as several atoms at the same position (the same operator, see split_projector_columns)
        nl_atoms, origin = split_projector_columns(S.Atom, 4)
        self.nl_origin = np.asarray(origin, dtype=np.int64)
        atoms = (_lib.cx_atom * max(1, len(nl_atoms)))()
        for J, A in enumerate(nl_atoms):
            imgs = (_lib.cx_rc_image * max(1, A.n_image_rc))()
            keep.append(imgs)
            for k, img in enumerate(A.rcImage):
                pos = np.ascontiguousarray(img.rc_pos, dtype=np.int64)
                chi = np.asfortranarray(img.Chi_mat, dtype=np.float64)
                keep.extend([pos, chi])
                imgs[k].rc_n_nodes = int(pos.shape[0])
                imgs[k].rc_pos = pos.ctypes.data_as(C.POINTER(C.c_int64))
                imgs[k].Chi_mat = chi.ctypes.data_as(C.POINTER(C.c_double))
                for d in range(3):
                    imgs[k].coordinates[d] = float(img.coordinates[d])
            atoms[J].angnum = int(A.angnum)
            atoms[J].n_image_rc = int(A.n_image_rc)
            atoms[J].gamma_Jl = darr(A.gamma_Jl)
            for d in range(3):
                atoms[J].position[d] = float(S.Atoms[origin[J], d])
            atoms[J].rcImage = C.cast(imgs, C.POINTER(_lib.cx_rc_image))
        h = C.c_void_p()
        st = self.lib.cx_create(C.byref(g), len(nl_atoms), atoms, int(S.nspin), C.byref(h))
        if st != _lib.CX_OK:
            raise CxError(st, self.lib.cx_last_error(None).decode())
        self.h = h
        self.set_blocks(blocks, prec)
        if S.Veff is not None:
            self.set_veff(S.Veff)

    # -- state -----------------------------------------------------------------------------
    def set_blocks(self, blocks, prec):
        self.blocks = [(np.asarray(k, float), int(s), int(n)) for (k, s, n) in blocks]
        arr = (_lib.cx_block * len(self.blocks))()
        for i, (k, s, n) in enumerate(self.blocks):
            for d in range(3):
                arr[i].kpt_vec[d] = float(k[d])
            arr[i].spin = s
            arr[i].Ns = n
        self.prec = prec
        check(self.lib, self.h, self.lib.cx_set_blocks(self.h, len(self.blocks), arr, _lib.PREC[prec]))
        self.Ns = [n for (_, _, n) in self.blocks]
        self.offsets = np.concatenate([[0], np.cumsum(self.Ns)]).astype(int)

    def set_veff(self, Veff):
        V = np.asfortranarray(np.asarray(Veff, dtype=np.float64).reshape(self.N, -1, order="F"))
        if V.shape[1] != int(self.S.nspin):
            raise ValueError(f"set_veff: need N x nspin = {self.N} x {int(self.S.nspin)} values, got {V.shape}")
        check(self.lib, self.h, self.lib.cx_set_veff(self.h, dptr(V)))

    def set_psi(self, blk, psi):
        a = np.asfortranarray(psi, dtype=np.complex128)
        if a.shape != (self.N, self.Ns[blk]):
            raise ValueError(f"set_psi: block {blk} is {self.N} x {self.Ns[blk]}, got {a.shape}")
        check(self.lib, self.h, self.lib.cx_set_psi(self.h, blk, cptr(a)))

    def get_psi(self, blk):
        a = np.empty((self.N, self.Ns[blk]), dtype=np.complex128, order="F")
        check(self.lib, self.h, self.lib.cx_get_psi(self.h, blk, cptr(a)))
        return a

    # -- operators ---------------------------------------------------------------------------
    def _columns(self, X, name):
        X = np.asfortranarray(X, dtype=np.complex128)
        if X.ndim == 1:
            X = X[:, None]
        if X.ndim != 2 or X.shape[0] != self.N:
            raise ValueError(f"{name}: need N = {self.N} rows, got shape {X.shape}")
        return X

    def hpsi(self, blk, X, prec=None):
        X = self._columns(X, "hpsi")
        Y = np.empty_like(X, order="F")
        check(self.lib, self.h, self.lib.cx_hpsi(self.h, blk, X.shape[1], cptr(X),
                                                 cptr(Y), _lib.PREC[prec or self.prec]))
        return Y

    def filter(self, blk, X, m, a, b, a0, prec=None):
        X = self._columns(X, "filter")
        Y = np.empty_like(X, order="F")
        check(self.lib, self.h, self.lib.cx_chebyshev_filter(self.h, blk, X.shape[1], cptr(X),
                                                             cptr(Y), int(m), float(a), float(b), float(a0),
                                                             _lib.PREC[prec or self.prec]))
        return Y

    def _check_step_arrays(self, EigVal, a0, bup, lambda_cutoff):
        _host_buffer(EigVal, np.float64, int(sum(self.Ns)), "EigVal")
        for name, v in (("a0", a0), ("bup", bup), ("lambda_cutoff", lambda_cutoff)):
            _host_buffer(v, np.float64, len(self.blocks), name)

    def _ubgv(self, ubgv):
        """S.upper_bound_guess_vecs as the library reads it: N x nblk complex128, column-major (or None)."""
        if ubgv is None:
            return None
        u = np.asarray(ubgv)
        if u.dtype != np.complex128 or u.shape != (self.N, len(self.blocks)) or not u.flags.f_contiguous or not u.flags.writeable:
            raise ValueError(f"ubgv: need a writable Fortran-ordered complex128 array of shape ({self.N}, {len(self.blocks)})")
        return u

    @staticmethod
    def _eig_params(npl, rhoTrigger, elecgs_Count, chefsibound_flag):
        return _lib.cx_eig_params(npl=int(npl), rhoTrigger=int(rhoTrigger), elecgs_Count=int(elecgs_Count),
                                  chefsibound_flag=int(chefsibound_flag))

    def eigsolve(self, count, npl, EigVal, a0, bup, lambda_cutoff, rhoTrigger=4, elecgs_Count=1, chefsibound_flag=0,
                 ubgv=None):
        """Device-resident eigSolver step (src/eigSolver.m:21-125): arrays are updated in place.

        ``ubgv`` (S.upper_bound_guess_vecs, N x nblk complex128, Fortran order) is read where the
        reference restarts the upper-bound estimate from it and receives every new estimate."""
        self._check_step_arrays(EigVal, a0, bup, lambda_cutoff)
        u = self._ubgv(ubgv)
        p = self._eig_params(npl, rhoTrigger, elecgs_Count, chefsibound_flag)
        check(self.lib, self.h, self.lib.cx_eigsolver_full(self.h, C.byref(p), int(count), cptr(u) if u is not None else None,
                                                           dptr(EigVal), dptr(a0), dptr(bup), dptr(lambda_cutoff)))

    def eigsolve_host(self, count, npl, psi_packed, EigVal, a0, bup, lambda_cutoff, rhoTrigger=4, elecgs_Count=1,
                      chefsibound_flag=0, ubgv=None):
        _host_buffer(psi_packed, np.complex128, self.N * int(sum(self.Ns)), "psi")
        self._check_step_arrays(EigVal, a0, bup, lambda_cutoff)
        u = self._ubgv(ubgv)
        p = self._eig_params(npl, rhoTrigger, elecgs_Count, chefsibound_flag)
        check(self.lib, self.h, self.lib.cx_eigsolver_full_host(self.h, C.byref(p), int(count),
                                                                cptr(u) if u is not None else None, cptr(psi_packed),
                                                                dptr(EigVal), dptr(a0), dptr(bup), dptr(lambda_cutoff)))

    def _scf_params(self, S, scf_tol, poisson_tol, max_scf, min_scf, rhoTrigger, maxit_poisson, mixing_param, refine, fp64_tol=0.0):
        xc = self._xc_code(S)
        wk = np.ascontiguousarray([S.wkpt[i % S.tnkpt] for i in range(len(self.blocks))], dtype=np.float64)
        b = np.ascontiguousarray(S.b, dtype=np.float64)
        rho0 = np.ascontiguousarray(S.rho_at, dtype=np.float64)
        p = _lib.cx_scf_params(scf_tol=scf_tol, poisson_tol=poisson_tol, max_scf=max_scf, min_scf=min_scf, rhoTrigger=rhoTrigger,
                               npl=int(S.npl), maxit_poisson=maxit_poisson, elec_T_type=int(S.elec_T_type), bet=float(S.bet),
                               occfac=float(S.occfac), NegCharge=float(S.NegCharge), Eself=float(S.Eself), E_corr=float(S.E_corr),
                               n_atm=int(S.n_atm), mixing_param=mixing_param, wkpt=dptr(wk), b=dptr(b), rho0=dptr(rho0),
                               refine=int(self.prec == "mixed" if refine is None else refine), fp64_tol=float(fp64_tol),
                               xc=xc)
        return p, (wk, b, rho0)

    @staticmethod
    def _xc_code(S):
        """The CX_XC_* code of the system's functional (S.XC, held in ``S.extra['xc']``; LDA_PW by default)."""
        name = S.extra.get("xc", "LDA_PW") if hasattr(S, "extra") else "LDA_PW"
        if name not in _lib.XC:
            raise CxError(_lib.CX_ERR_ARG, f"exchange-correlation {name}: the library implements {', '.join(_lib.XC)}")
        return _lib.XC[name]

    def xc(self, rho, xc="LDA_PW"):
        """(Vxc, e_xc) of ``exchangeCorrelationPotential`` for nspin = 1 on the density ``rho`` (cx_xc):
        e_xc is the energy per particle at the density clipped at 1e-14."""
        rho = np.ascontiguousarray(rho, dtype=np.float64).reshape(-1)
        if rho.size != self.N:
            raise ValueError(f"xc: rho needs N = {self.N} values, got {rho.size}")
        if xc not in _lib.XC:
            raise CxError(_lib.CX_ERR_ARG, f"exchange-correlation {xc}: the library implements {', '.join(_lib.XC)}")
        V = np.zeros(self.N)
        e = np.zeros(self.N)
        check(self.lib, self.h, self.lib.cx_xc(self.h, _lib.XC[xc], dptr(rho), dptr(V), dptr(e)))
        return V, e

    def nonlocal_force(self, occ, wkpt, occfac):
        """Nonlocal part of the atomic forces (cx_nonlocal_force, src/atomicForce.m:254-300) from the
        device-resident psi: ``occ`` packed like EigVal, ``wkpt`` one weight per block.  Returns
        (n_atm, 3) for the atoms of ``S.Atom`` (the parts of an atom passed as several 4-column atoms
        summed)."""
        occ = np.ascontiguousarray(occ, dtype=np.float64).reshape(-1)
        wkpt = np.ascontiguousarray(wkpt, dtype=np.float64).reshape(-1)
        if occ.size != int(sum(self.Ns)) or wkpt.size != len(self.blocks):
            raise ValueError(f"nonlocal_force: occ needs {int(sum(self.Ns))} values and wkpt {len(self.blocks)}")
        nat = self.nl_origin.size
        F = np.zeros(3 * max(nat, 1))
        check(self.lib, self.h, self.lib.cx_nonlocal_force(self.h, dptr(occ), dptr(wkpt), float(occfac), dptr(F)))
        parts = F[:3 * nat].reshape(3, nat).T
        out = np.zeros((int(self.S.Atoms.shape[0]), 3))
        np.add.at(out, self.nl_origin, parts)
        return out

    def gradient(self, f):
        """Cartesian gradient (N, 3) of a real grid field at k = 0 (cx_gradient: S.grad_1..3 * f)."""
        f = np.ascontiguousarray(f, dtype=np.float64).reshape(-1)
        if f.size != self.N:
            raise ValueError(f"gradient: f needs N = {self.N} values, got {f.size}")
        D = np.zeros(3 * self.N)
        check(self.lib, self.h, self.lib.cx_gradient(self.h, dptr(f), dptr(D)))
        return D.reshape(3, self.N).T

    def field_projections(self, f, A):
        """(nvec, 3): the projections A[v] . D_d f of the Cartesian gradient of a real grid field on
        the rows of ``A`` (nvec x N) (cx_field_projections)."""
        f = np.ascontiguousarray(f, dtype=np.float64).reshape(-1)
        A = np.ascontiguousarray(A, dtype=np.float64)
        if f.size != self.N or A.ndim != 2 or A.shape[1] != self.N:
            raise ValueError(f"field_projections: f needs N = {self.N} values and A shape (nvec, {self.N})")
        out = np.zeros(3 * max(A.shape[0], 1))
        check(self.lib, self.h, self.lib.cx_field_projections(self.h, dptr(f), int(A.shape[0]), dptr(A), dptr(out)))
        return out[:3 * A.shape[0]].reshape(3, A.shape[0]).T

    def scf(self, S, scf_tol=1e-6, poisson_tol=-1.0, max_scf=100, min_scf=3, rhoTrigger=4, maxit_poisson=1000,
            mixing_param=0.3, refine=None, fp64_tol=0.0):
        """Full SCF on the device-resident psi (cx_scf); returns (result, EigVal packed, rho, Veff, history).
        ``fp64_tol`` > 0 with mixed blocks: finish with FP64 passes down to that error (the blocks
        are complex128 afterwards)."""
        p, keep = self._scf_params(S, scf_tol, poisson_tol, max_scf, min_scf, rhoTrigger, maxit_poisson, mixing_param, refine,
                                   fp64_tol)
        EV = np.zeros(int(sum(self.Ns)))
        rho = np.zeros(self.N)
        V = np.zeros(self.N)
        hist = np.zeros((2 * max_scf if fp64_tol > 0 else max_scf, 2))
        res = _lib.cx_scf_result()
        check(self.lib, self.h, self.lib.cx_scf(self.h, C.byref(p), dptr(EV), dptr(rho), dptr(V), dptr(hist), C.byref(res)))
        if fp64_tol > 0:
            self.prec = "fp64"
        return res, EV, rho, V, hist[: res.n_scf]

    def scf_init(self, S, scf_tol=1e-6, poisson_tol=-1.0, max_scf=100, min_scf=3, rhoTrigger=4, maxit_poisson=1000,
                 mixing_param=0.3, refine=None):
        """Start a caller-driven SCF (cx_scf_init): the initial potential from ``S.rho_at``."""
        p, keep = self._scf_params(S, scf_tol, poisson_tol, max_scf, min_scf, rhoTrigger, maxit_poisson, mixing_param, refine)
        check(self.lib, self.h, self.lib.cx_scf_init(self.h, C.byref(p)))

    def scf_step(self, psi_host=None, EigVal=None):
        """One pass of the SCF loop (cx_scf_step); ``psi_host`` (packed complex128 blocks) is copied
        in and out around it when given.  Returns the step record (cx_scf_step_info)."""
        info = _lib.cx_scf_step_info()
        if psi_host is not None:
            _host_buffer(psi_host, np.complex128, self.N * int(sum(self.Ns)), "psi")
        if EigVal is not None:
            _host_buffer(EigVal, np.float64, int(sum(self.Ns)), "EigVal")
        check(self.lib, self.h, self.lib.cx_scf_step(self.h, cptr(psi_host) if psi_host is not None else None,
                                                     dptr(EigVal) if EigVal is not None else None, C.byref(info)))
        return info

    def scf_finish(self):
        """End the caller-driven SCF (cx_scf_finish): (result, EigVal packed, rho, Veff)."""
        EV = np.zeros(int(sum(self.Ns)))
        rho = np.zeros(self.N)
        V = np.zeros(self.N)
        res = _lib.cx_scf_result()
        check(self.lib, self.h, self.lib.cx_scf_finish(self.h, dptr(EV), dptr(rho), dptr(V), C.byref(res)))
        return res, EV, rho, V

    def poisson(self, f, phi0=None, tol=1e-8, maxit=1000):
        f = np.ascontiguousarray(f, dtype=np.float64).reshape(-1)
        phi = np.ascontiguousarray(phi0 if phi0 is not None else np.zeros(self.N), dtype=np.float64).reshape(-1).copy()
        if f.size != self.N or phi.size != self.N:
            raise ValueError(f"poisson: f and phi need N = {self.N} values, got {f.size} and {phi.size}")
        it = C.c_int32(0)
        rr = C.c_double(0)
        st = self.lib.cx_poisson(self.h, dptr(f), dptr(phi), float(tol), int(maxit), 1 if phi0 is not None else 0,
                                 C.byref(it), C.byref(rr))
        if st not in (_lib.CX_OK, _lib.CX_ERR_NOCONV):
            check(self.lib, self.h, st)
        return phi, int(it.value), float(rr.value), st == _lib.CX_OK

    # -- measurement --------------------------------------------------------------------------
    def sync(self):
        check(self.lib, self.h, self.lib.cx_sync(self.h))

    def timer_start(self):
        check(self.lib, self.h, self.lib.cx_timer_start(self.h))

    def timer_stop(self) -> float:
        ms = C.c_double(0)
        check(self.lib, self.h, self.lib.cx_timer_stop(self.h, C.byref(ms)))
        return ms.value

    def profile(self, enable: bool):
        check(self.lib, self.h, self.lib.cx_profile_stencil(self.h, 1 if enable else 0))

    def profile_read(self):
        n = C.c_int64(0)
        ms = C.c_double(0)
        by = C.c_double(0)
        check(self.lib, self.h, self.lib.cx_profile_read(self.h, C.byref(n), C.byref(ms), C.byref(by)))
        return n.value, ms.value, by.value

    def profile_read_apply(self) -> float:
        ms = C.c_double(0)
        check(self.lib, self.h, self.lib.cx_profile_read_apply(self.h, C.byref(ms)))
        return ms.value

    def set_nl_kernels(self, tensor_cores: bool):
        """Select the projector kernels of the complex64 path (cx_set_nl_kernels)."""
        check(self.lib, self.h, self.lib.cx_set_nl_kernels(self.h, 1 if tensor_cores else 0))

    def profile_read_contract(self) -> float:
        """Summed device time (ms) of the projector contraction launches in the profiling window."""
        ms = C.c_double(0)
        check(self.lib, self.h, self.lib.cx_profile_read_contract(self.h, C.byref(ms)))
        return ms.value

    def eig_fallbacks(self) -> int:
        n = C.c_int64(0)
        check(self.lib, self.h, self.lib.cx_eig_fallback_count(self.h, C.byref(n)))
        return n.value

    def eig_hermitian(self) -> int:
        n = C.c_int64(0)
        check(self.lib, self.h, self.lib.cx_eig_hermitian_count(self.h, C.byref(n)))
        return n.value

    def stencil_config(self) -> dict:
        """The complex64 stencil kernel's configuration and the autotuner's log (cx_stencil_config)."""
        r, d, t = C.c_int32(0), C.c_int32(0), C.c_int32(0)
        buf = C.create_string_buffer(1024)
        check(self.lib, self.h, self.lib.cx_stencil_config(self.h, C.byref(r), C.byref(d), C.byref(t), buf, 1024))
        return {"rows_per_thread": r.value, "ring_depth": d.value, "tuned": bool(t.value), "candidates_ms": buf.value.decode()}

    def launch_count(self, reset=False) -> int:
        n = C.c_int64(0)
        check(self.lib, self.h, self.lib.cx_launch_count(self.h, C.byref(n), 1 if reset else 0))
        return n.value

    def close(self):
        if getattr(self, "h", None):
            self.lib.cx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def select_device(device: int) -> None:
    """Device of the handles this process creates next (one process per GPU)."""
    lib = _lib.load()
    check(lib, None, lib.cx_set_device(int(device)))


def attach(S, blocks, prec="mixed") -> CyclixGPU:
    """Create the GPU operator for ``S`` and keep it in ``S.gpu``."""
    S.gpu = CyclixGPU(S, blocks, prec)
    return S.gpu


def _block_of(S, kptvec, Veff=None):
    gpu = S.gpu
    k = np.asarray(kptvec, float)
    cands = [i for i, (kk, s, n) in enumerate(gpu.blocks) if np.allclose(kk, k, atol=0, rtol=0)]
    if not cands:
        raise CxError(_lib.CX_ERR_ARG, "no block with this kptvec; pass it in the block list of attach()")
    if Veff is not None and len(cands) > 1 and S.Veff is not None:
        for i in cands:
            if np.array_equal(np.asarray(S.Veff)[:, gpu.blocks[i][1]], np.asarray(Veff).reshape(-1)):
                return i
    return cands[0]


def h_nonlocal_vector_mult(DL11, DL22, DL33, DG1, DG2, DG3, Veff, X, S, kptvec):
    """``Hnlx = (-0.5*Lap + Veff) X + Vnl X`` for the block of ``kptvec`` (src/h_nonlocal_vector_mult.m:1-43)."""
    blk = _block_of(S, kptvec, Veff)
    return S.gpu.hpsi(blk, X)


def chebyshev_filter(X, m, a, b, a0, DL11, DL22, DL33, DG1, DG2, DG3, Veff, S, kpt_vec):
    """Scaled Chebyshev filter of degree m (src/chebyshev_filter.m:1-44); a = cutoff, b = upper, a0 = lower."""
    blk = _block_of(S, kpt_vec, Veff)
    return S.gpu.filter(blk, X, m, a, b, a0)


def eigSolver(S, count, upper_bound_guess_vecs, psi, EigVal, a0, bup, lambda_cutoff):
    """``[ubgv,psi,EigVal,a0,bup,lambda_cutoff] = eigSolver(S,count,...)`` (src/eigSolver.m:1-125).

    ``psi`` is N x Nev x (tnkpt*nspin) as in MATLAB (or a list of per-block N x Ns arrays for
    uneven blocks); it is copied to the GPU, updated there and copied back, like a MEX call.
    ``S.elecgs_Count``, ``S.chefsibound_flag`` and ``S.rhoTrigger`` steer the bounds as in
    src/eigSolver.m:21-94 (defaults 1, 0, 4).  ``upper_bound_guess_vecs`` (N x tnkpt*nspin) is
    the start of the upper-bound estimate where the reference restarts it (later relaxation steps,
    ``chefsibound_flag``); the returned copy holds every new estimate's vector.
    """
    gpu = S.gpu
    uniform = not isinstance(psi, (list, tuple))
    blocks = [psi[:, :, k] for k in range(psi.shape[2])] if uniform else list(psi)
    packed = np.concatenate([np.asarray(b, np.complex128).reshape(-1, order="F") for b in blocks])
    EV = np.ascontiguousarray(np.concatenate([np.asarray(EigVal)[:gpu.Ns[k], k] for k in range(len(gpu.Ns))])
                              if uniform and np.ndim(EigVal) == 2 else np.asarray(EigVal, float).reshape(-1), dtype=np.float64)
    a0 = np.ascontiguousarray(a0, dtype=np.float64).reshape(-1).copy()
    bup = np.ascontiguousarray(bup, dtype=np.float64).reshape(-1).copy()
    lc = np.ascontiguousarray(lambda_cutoff, dtype=np.float64).reshape(-1).copy()
    nblk = len(gpu.Ns)
    if upper_bound_guess_vecs is None:
        ubgv = np.zeros((gpu.N, nblk), dtype=np.complex128, order="F")
    else:
        ubgv = np.array(np.asarray(upper_bound_guess_vecs, dtype=np.complex128).reshape(gpu.N, nblk, order="F"), order="F")
    gpu.eigsolve_host(count, S.npl, packed, EV, a0, bup, lc, rhoTrigger=getattr(S, "rhoTrigger", 4),
                      elecgs_Count=getattr(S, "elecgs_Count", 1), chefsibound_flag=getattr(S, "chefsibound_flag", 0), ubgv=ubgv)
    out = []
    for k, n in enumerate(gpu.Ns):
        o = gpu.offsets[k] * gpu.N
        out.append(packed[o:o + gpu.N * n].reshape(gpu.N, n, order="F"))
    if uniform:
        psi_out = np.stack(out, axis=2)
        EigVal_out = np.stack([EV[gpu.offsets[k]:gpu.offsets[k + 1]] for k in range(len(gpu.Ns))], axis=1)
    else:
        psi_out = out
        EigVal_out = EV
    return ubgv, psi_out, EigVal_out, a0, bup, lc


def scf(S, scf_tol=1e-6):
    """``S = scf(S)`` (src/scf.m:1-327): the whole SCF on the GPU from ``S.rho_at`` and the psi held in ``S.gpu``.

    Sets ``S.Etotal``, ``S.EigVal`` (packed per block), ``S.lambda_f``, ``S.rho``, ``S.Veff`` and ``S.extra['scf']``.
    """
    res, EV, rho, V, hist = S.gpu.scf(S, scf_tol=scf_tol, rhoTrigger=getattr(S, "rhoTrigger", 4))
    S.Etotal, S.EigVal, S.lambda_f, S.rho = res.Etotal, EV, res.lambda_f, rho
    S.Veff = V.reshape(-1, 1)
    S.extra["scf"] = dict(n_scf=res.n_scf, converged=bool(res.converged), err=res.err, history=hist)
    return S


def exchangeCorrelationPotential(S):
    """``S = exchangeCorrelationPotential(S)`` for nspin = 1 (src/exchangeCorrelationPotential.m:1-80):
    ``S.Vxc`` and ``S.e_xc`` of ``S.rho`` for the functional ``S.extra['xc']`` (LDA_PW, LDA_PZ or GGA_PBE)."""
    rho = np.asarray(S.rho).reshape(S.N, -1, order="F")[:, 0]
    S.Vxc, S.e_xc = S.gpu.xc(rho, S.extra.get("xc", "LDA_PW"))
    return S


def poissonSolve(S, poisson_tol, Isguess):
    """``S = poissonSolve(S, poisson_tol, Isguess)`` for Cyclix cells (src/poissonSolve.m:1-51).

    ``f = -4 pi (rho + b)`` (:19-23), AAR with omega = beta = 0.6, m = 7, p = 6 (:36) and
    ``S.MAXIT_POISSON`` iterations; the converged potential is stored in ``S.phi``.
    """
    f = -4 * np.pi * (np.asarray(S.rho).reshape(S.N, -1, order="F")[:, 0] + S.b)
    guess = S.phi if (Isguess and getattr(S, "phi", None) is not None) else None
    phi, it, rr, ok = S.gpu.poisson(f, guess, poisson_tol, getattr(S, "MAXIT_POISSON", 1000))
    S.phi = phi
    S.extra["poisson_iters"] = it
    S.extra["poisson_relres"] = rr
    return S
