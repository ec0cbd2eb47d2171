"""ctypes binding of libefgpu.so (the C ABI declared in include/efgpu.h).

The library is built in-tree by ``edelweissfe_gb300.build``.  There is no CPU
fallback: if the library is missing or cannot be loaded, every entry point
raises.
"""

import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libefgpu.so")

c_int = ctypes.c_int
c_i64 = ctypes.c_int64
c_dbl = ctypes.c_double
c_vp = ctypes.c_void_p
c_char_p = ctypes.c_char_p

EF_OK = 0
EF_CUTBACK = 1
EF_NAN = 2
EF_NOT_CONVERGED = 3
EF_ERR_ARG = 10
EF_ERR_CUDA = 11
EF_ERR_STATE = 12
EF_ERR_DEVICE = 13

EF_OPT_KE_FP64 = 1
EF_OPT_NO_SCALAR_CSR = 2

EF_SOLVE_PCG = 0
EF_SOLVE_FGMRES = 1

EF_FGMRES_PC_MULTIGRID = 0
EF_FGMRES_PC_JACOBI = 1


class EfInfo(ctypes.Structure):
    _fields_ = [
        ("nDof", c_i64),
        ("nNodes", c_i64),
        ("nElements", c_i64),
        ("nVIJ", c_i64),
        ("nnz", c_i64),
        ("nBlocks", c_i64),
        ("nPe", c_i64),
        ("keFp64", c_int),
    ]


class EfSolveOpts(ctypes.Structure):
    _fields_ = [
        ("method", c_int),
        ("mixed", c_int),
        ("rtol", c_dbl),
        ("innerRtol", c_dbl),
        ("maxIter", c_int),
        ("restart", c_int),
        ("maxRefine", c_int),
        ("profile", c_int),
    ]


class EfSolveInfo(ctypes.Structure):
    _fields_ = [
        ("iterations", c_int),
        ("refinements", c_int),
        ("relResidual", c_dbl),
        ("status", c_int),
        ("kernelMs", c_dbl),
        ("kernelLaunches", c_int),
        ("spmvMs", c_dbl),
        ("spmvLaunches", c_int),
        ("precondMs", c_dbl),
        ("orthoMs", c_dbl),
        ("reorths", c_int),
        ("setupMs", c_dbl),
    ]


class EfNewtonOpts(ctypes.Structure):
    _fields_ = [("fluxTol", c_dbl), ("fluxTolAlt", c_dbl), ("corrTol", c_dbl), ("fluxFloor", c_dbl),
                ("nAccFluxes", c_dbl)]  # fmt: skip


class EfNewtonCheck(ctypes.Structure):
    _fields_ = [("converged", c_int), ("nGrew", c_int), ("fluxResidual", c_dbl), ("fieldCorrection", c_dbl),
                ("spatialAveragedFlux", c_dbl)]  # fmt: skip


# name -> (restype, argtypes); the exported surface of include/efgpu.h
SIGNATURES = {
    "ef_abi_version": (c_int, []),
    "ef_last_error": (c_char_p, []),
    "ef_create": (c_int, [c_i64, c_vp, ctypes.POINTER(c_vp)]),
    "ef_destroy": (None, [c_vp]),
    "ef_add_group": (c_int, [c_vp, c_char_p, c_char_p, c_vp, c_int, c_int, c_vp, ctypes.POINTER(c_int)]),
    "ef_finalize": (c_int, [c_vp, c_int]),
    "ef_get_info": (c_int, [c_vp, ctypes.POINTER(EfInfo)]),
    "ef_compute_elements": (c_int, [c_vp, c_vp, c_vp, c_vp, c_dbl, c_vp, c_vp, c_vp]),
    "ef_element_status": (c_int, [c_vp, c_vp, ctypes.POINTER(c_dbl)]),
    "ef_get_state_size": (c_int, [c_vp, c_int, ctypes.POINTER(c_int), ctypes.POINTER(c_int)]),
    "ef_set_state": (c_int, [c_vp, c_int, c_vp]),
    "ef_get_state": (c_int, [c_vp, c_int, c_int, c_vp]),
    "ef_results_create": (c_int, [c_vp, c_int, c_vp, c_int, c_vp, c_int, c_int, c_int, ctypes.POINTER(c_int)]),
    "ef_results_update": (c_int, [c_vp, c_int, c_int, c_vp, c_vp]),
    "ef_results_device": (c_int, [c_vp, c_int, ctypes.POINTER(c_vp), ctypes.POINTER(c_i64)]),
    "ef_results_destroy": (c_int, [c_vp, c_int]),
    "ef_accept_state": (c_int, [c_vp]),
    "ef_reset_state": (c_int, [c_vp]),
    "ef_add_body_force": (c_int, [c_vp, c_int, c_vp, c_vp, c_vp]),
    "ef_export_vij": (c_int, [c_vp, c_vp, c_vp]),
    "ef_csr_pattern": (c_int, [c_vp, c_vp, c_vp]),
    "ef_update_csr": (c_int, [c_vp, c_vp, c_vp, c_vp]),
    "ef_csr_dirichlet_rows": (c_int, [c_vp, c_vp, c_vp, c_i64, c_vp]),
    "ef_set_dirichlet": (c_int, [c_vp, c_vp, c_i64]),
    "ef_assemble_bsr": (c_int, [c_vp, c_vp]),
    "ef_solve": (c_int, [c_vp, ctypes.POINTER(EfSolveOpts), c_vp, c_vp, ctypes.POINTER(EfSolveInfo), c_vp]),
    "ef_bsr_matvec": (c_int, [c_vp, c_vp, c_vp, c_vp]),
    "ef_norms": (c_int, [c_vp, c_vp, c_vp, c_vp, c_vp, c_vp]),
    "ef_newton_residual": (
        c_int,
        [c_vp, c_int, c_vp, c_vp, c_vp, c_vp, c_vp, c_int, c_dbl, c_int, ctypes.POINTER(EfNewtonOpts), c_vp,
         ctypes.POINTER(EfNewtonCheck), c_vp],
    ),
    "ef_pcg_noalloc_max_nodes": (c_i64, []),
    "ef_kernel_launches": (c_i64, []),
    "ef_fgmres_set_preconditioner": (c_int, [c_vp, c_int]),
    "ef_fgmres_set_reuse": (c_int, [c_vp, c_int]),
    "ef_fine_kernel_profile": (c_int, [c_vp, c_int, c_vp, c_vp, c_vp]),
    "ef_set_group_props": (c_int, [c_vp, c_int, c_vp, c_int, c_int, c_vp]),
    "ef_set_group_cutback": (c_int, [c_vp, c_int, c_dbl]),
    "ef_set_ties": (c_int, [c_vp, c_vp, c_vp, c_vp, c_i64]),
    "ef_mpnn_dense_eval": (c_int, [c_int, c_int, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp]),
    "ef_batch_setup": (c_int, [c_vp, c_int, c_vp]),
    "ef_batch_tile_count": (c_int, []),
    "ef_batch_tile_info": (c_int, [c_int, ctypes.POINTER(c_int), ctypes.POINTER(c_int)]),
    "ef_batch_set_tile": (c_int, [c_vp, c_int]),
    "ef_batch_solve": (c_int, [c_vp, c_dbl, c_int, c_vp, c_vp, c_vp, c_vp, c_vp]),
    "ef_batch_autotune": (c_int, [c_vp, c_dbl, c_int, c_vp, c_vp, c_vp, c_vp, c_vp, ctypes.POINTER(c_int), c_vp]),
    "ef_batch_norms": (c_int, [c_vp, c_vp, c_vp, c_vp, c_vp, c_vp]),
    "ef_mpnn_param_count": (c_int, []),
    "ef_mpnn_init": (c_int, [c_vp, ctypes.c_uint64, c_int]),
    "ef_mpnn_set_params": (c_int, [c_vp, c_vp, c_vp]),
    "ef_mpnn_get_params": (c_int, [c_vp, c_vp, c_vp]),
    "ef_mpnn_enable": (c_int, [c_vp, c_int]),
    "ef_mpnn_collect": (c_int, [c_vp, c_int, c_int, c_int]),
    "ef_mpnn_add_sample": (c_int, [c_vp, c_vp, c_vp, c_vp]),
    "ef_mpnn_num_samples": (c_int, [c_vp, ctypes.POINTER(c_int)]),
    "ef_mpnn_clear_samples": (c_int, [c_vp]),
    "ef_mpnn_train": (c_int, [c_vp, c_int, ctypes.c_float, c_int, ctypes.POINTER(c_dbl), ctypes.POINTER(c_dbl), c_vp]),
    "ef_mpnn_eval": (
        c_int,
        [c_int, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, ctypes.c_float, ctypes.c_float, c_vp, c_vp,
         ctypes.POINTER(c_dbl), c_vp],
    ),
    "ef_pcg_solve_noalloc": (
        c_int,
        [c_i64, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_int, c_dbl, ctypes.POINTER(EfSolveInfo), c_vp],
    ),
}

_lib = None


class EfError(RuntimeError):
    def __init__(self, status, where, msg):
        super().__init__(f"{where} failed with status {status}: {msg}")
        self.status = status


def load(path: str = LIB_PATH):
    """Load the library (without building it) and attach the signatures."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise ImportError(f"libefgpu.so not built ({path} missing); run edelweissfe_gb300.build.build()")
    lib = ctypes.CDLL(path, mode=os.RTLD_NOW)  # every symbol resolved at load: a missing one fails here
    for name, (res, args) in SIGNATURES.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


def lib():
    return load()


def check(status, where):
    if status != EF_OK:
        msg = lib().ef_last_error()
        raise EfError(status, where, msg.decode() if msg else "")
    return status


def ptr(t):
    """Raw device/host address of a torch tensor or numpy array (None -> NULL)."""
    if t is None:
        return None
    if hasattr(t, "data_ptr"):
        return t.data_ptr()
    return t.ctypes.data
