"""ctypes binding of ``libcyclix_gpu.so`` (declarations in ``include/cyclix_gpu.h``).

Loading fails loudly: there is no CPU implementation behind these names.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "libcyclix_gpu.so"

CX_OK, CX_ERR_ARG, CX_ERR_CUDA, CX_ERR_NOMEM, CX_ERR_LIB, CX_ERR_NOTPD, CX_ERR_STATE, CX_ERR_NOCONV = range(8)
CX_PREC_FP64, CX_PREC_MIXED = 0, 1
PREC = {"fp64": CX_PREC_FP64, "mixed": CX_PREC_MIXED}
CX_XC_LDA_PW, CX_XC_LDA_PZ, CX_XC_GGA_PBE = 0, 1, 2
XC = {"LDA_PW": CX_XC_LDA_PW, "LDA_PZ": CX_XC_LDA_PZ, "GGA_PBE": CX_XC_GGA_PBE}

EXPORTS = ["cx_create", "cx_destroy", "cx_last_error", "cx_version", "cx_set_blocks", "cx_set_veff", "cx_set_psi",
           "cx_get_psi", "cx_hpsi", "cx_chebyshev_filter", "cx_eigsolver", "cx_eigsolver_host", "cx_poisson", "cx_sync",
           "cx_timer_start", "cx_timer_stop", "cx_profile_stencil", "cx_profile_read", "cx_launch_count",
           "cx_host_register", "cx_host_unregister", "cx_hpsi_noalloc", "cx_profile_read_apply", "cx_profile_read_contract", "cx_set_nl_kernels", "cx_eig_fallback_count", "cx_scf", "cx_refine_eigenvalues", "cx_set_device",
           "cx_eigsolver_full", "cx_eigsolver_full_host", "cx_scf_init", "cx_scf_step", "cx_scf_finish",
           "cx_eig_hermitian_count", "cx_stencil_config", "cx_xc", "cx_nonlocal_force", "cx_gradient",
           "cx_field_projections"]


class cx_grid(C.Structure):
    _fields_ = [("Nx", C.c_int32), ("Ny", C.c_int32), ("Nz", C.c_int32), ("FDn", C.c_int32), ("cell_typ", C.c_int32),
                ("BCx", C.c_int32), ("BCy", C.c_int32), ("BCz", C.c_int32),
                ("dx", C.c_double), ("dy", C.c_double), ("dz", C.c_double), ("xin", C.c_double), ("twist", C.c_double),
                ("L1", C.c_double), ("L2", C.c_double), ("L3", C.c_double),
                ("w1", C.POINTER(C.c_double)), ("w2", C.POINTER(C.c_double)), ("W", C.POINTER(C.c_double))]


class cx_rc_image(C.Structure):
    _fields_ = [("rc_n_nodes", C.c_int32), ("rc_pos", C.POINTER(C.c_int64)), ("Chi_mat", C.POINTER(C.c_double)),
                ("coordinates", C.c_double * 3)]


class cx_atom(C.Structure):
    _fields_ = [("angnum", C.c_int32), ("n_image_rc", C.c_int32), ("gamma_Jl", C.POINTER(C.c_double)),
                ("position", C.c_double * 3), ("rcImage", C.POINTER(cx_rc_image))]


class cx_scf_params(C.Structure):
    _fields_ = [("scf_tol", C.c_double), ("poisson_tol", C.c_double), ("max_scf", C.c_int32), ("min_scf", C.c_int32),
                ("rhoTrigger", C.c_int32), ("npl", C.c_int32), ("maxit_poisson", C.c_int32), ("elec_T_type", C.c_int32),
                ("bet", C.c_double), ("occfac", C.c_double), ("NegCharge", C.c_double), ("Eself", C.c_double),
                ("E_corr", C.c_double), ("n_atm", C.c_int32), ("mixing_param", C.c_double),
                ("wkpt", C.POINTER(C.c_double)), ("b", C.POINTER(C.c_double)), ("rho0", C.POINTER(C.c_double)),
                ("refine", C.c_int32), ("fp64_tol", C.c_double), ("xc", C.c_int32)]


class cx_scf_result(C.Structure):
    _fields_ = [("Etotal", C.c_double), ("lambda_f", C.c_double), ("err", C.c_double), ("n_scf", C.c_int32),
                ("converged", C.c_int32)]


class cx_eig_params(C.Structure):
    _fields_ = [("npl", C.c_int32), ("rhoTrigger", C.c_int32), ("elecgs_Count", C.c_int32), ("chefsibound_flag", C.c_int32)]


class cx_scf_step_info(C.Structure):
    _fields_ = [("Etotal", C.c_double), ("lambda_f", C.c_double), ("err", C.c_double), ("count", C.c_int32),
                ("n_scf", C.c_int32), ("density_updated", C.c_int32), ("converged", C.c_int32),
                ("poisson_iters", C.c_int32), ("pad", C.c_int32), ("step_ms", C.c_double), ("poisson_ms", C.c_double),
                ("filter_ms", C.c_double), ("rr_ms", C.c_double)]


class cx_block(C.Structure):
    _fields_ = [("kpt_vec", C.c_double * 3), ("spin", C.c_int32), ("Ns", C.c_int32)]


_lib = None


def load(build_if_missing: bool = True):
    """Load the library (building it in-tree first when it is missing or stale)."""
    global _lib
    if _lib is not None:
        return _lib
    if build_if_missing:
        from .build import build
        build()
    if not LIB_PATH.exists():
        raise ImportError(f"libcyclix_gpu.so not found at {LIB_PATH}; run cyclix_msparc_gb300.build")
    lib = C.CDLL(str(LIB_PATH))
    P = C.POINTER
    dp = P(C.c_double)
    h = C.c_void_p
    sig = {
        "cx_create": ([P(cx_grid), C.c_int32, P(cx_atom), C.c_int32, P(C.c_void_p)], C.c_int32),
        "cx_destroy": ([h], C.c_int32),
        "cx_last_error": ([h], C.c_char_p),
        "cx_version": ([], C.c_char_p),
        "cx_set_blocks": ([h, C.c_int32, P(cx_block), C.c_int32], C.c_int32),
        "cx_set_veff": ([h, dp], C.c_int32),
        "cx_set_psi": ([h, C.c_int32, dp], C.c_int32),
        "cx_get_psi": ([h, C.c_int32, dp], C.c_int32),
        "cx_hpsi": ([h, C.c_int32, C.c_int32, dp, dp, C.c_int32], C.c_int32),
        "cx_chebyshev_filter": ([h, C.c_int32, C.c_int32, dp, dp, C.c_int32, C.c_double, C.c_double, C.c_double, C.c_int32],
                                C.c_int32),
        "cx_eigsolver": ([h, C.c_int32, C.c_int32, C.c_int32, dp, dp, dp, dp], C.c_int32),
        "cx_eigsolver_host": ([h, C.c_int32, C.c_int32, C.c_int32, dp, dp, dp, dp, dp], C.c_int32),
        "cx_eigsolver_full": ([h, P(cx_eig_params), C.c_int32, dp, dp, dp, dp, dp], C.c_int32),
        "cx_eigsolver_full_host": ([h, P(cx_eig_params), C.c_int32, dp, dp, dp, dp, dp, dp], C.c_int32),
        "cx_poisson": ([h, dp, dp, C.c_double, C.c_int32, C.c_int32, P(C.c_int32), dp], C.c_int32),
        "cx_sync": ([h], C.c_int32),
        "cx_timer_start": ([h], C.c_int32),
        "cx_timer_stop": ([h, dp], C.c_int32),
        "cx_profile_stencil": ([h, C.c_int32], C.c_int32),
        "cx_profile_read": ([h, P(C.c_int64), dp, dp], C.c_int32),
        "cx_launch_count": ([h, P(C.c_int64), C.c_int32], C.c_int32),
        "cx_host_register": ([C.c_void_p, C.c_size_t], C.c_int32),
        "cx_host_unregister": ([C.c_void_p], C.c_int32),
        "cx_hpsi_noalloc": ([h, C.c_int32, C.c_int32, C.c_void_p, C.c_void_p, C.c_int32], C.c_int32),
        "cx_profile_read_apply": ([h, dp], C.c_int32),
        "cx_profile_read_contract": ([h, dp], C.c_int32),
        "cx_set_nl_kernels": ([h, C.c_int32], C.c_int32),
        "cx_eig_fallback_count": ([h, P(C.c_int64)], C.c_int32),
        "cx_eig_hermitian_count": ([h, P(C.c_int64)], C.c_int32),
        "cx_stencil_config": ([h, P(C.c_int32), P(C.c_int32), P(C.c_int32), C.c_char_p, C.c_int32], C.c_int32),
        "cx_scf": ([h, P(cx_scf_params), dp, dp, dp, dp, P(cx_scf_result)], C.c_int32),
        "cx_refine_eigenvalues": ([h, dp], C.c_int32),
        "cx_scf_init": ([h, P(cx_scf_params)], C.c_int32),
        "cx_scf_step": ([h, dp, dp, P(cx_scf_step_info)], C.c_int32),
        "cx_scf_finish": ([h, dp, dp, dp, P(cx_scf_result)], C.c_int32),
        "cx_set_device": ([C.c_int32], C.c_int32),
        "cx_xc": ([h, C.c_int32, dp, dp, dp], C.c_int32),
        "cx_nonlocal_force": ([h, dp, dp, C.c_double, dp], C.c_int32),
        "cx_gradient": ([h, dp, dp], C.c_int32),
        "cx_field_projections": ([h, dp, C.c_int32, dp, dp], C.c_int32),
    }
    for name, (args, res) in sig.items():
        f = getattr(lib, name)
        f.argtypes = args
        f.restype = res
    _lib = lib
    return lib


class CxError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"cyclix_gpu status {status}: {msg}")
        self.status = status


def dptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def cptr(a: np.ndarray):
    """Pointer to a contiguous complex128 array as interleaved doubles."""
    if a.dtype != np.complex128 or not (a.flags.c_contiguous or a.flags.f_contiguous):
        raise ValueError("expected a contiguous complex128 array")
    return a.ctypes.data_as(C.POINTER(C.c_double))


def check(lib, h, status):
    if status != CX_OK:
        msg = lib.cx_last_error(h)
        raise CxError(status, msg.decode() if msg else "")
    return status
