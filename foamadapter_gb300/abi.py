"""ctypes binding of the libfvgb C ABI (include/fvgb.h).

This is the binding a Python caller of the drop-in uses (the C++ façade in
``foamadapter_gb300/adapter`` is the one a C++ caller uses).  It loads the
in-tree ``_lib/libfvgb.so`` and fails loudly when the library is missing:
there is no fallback implementation.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "_lib" / "libfvgb.so"

# status codes (fvgb_status)
OK, ERR_INVALID_ARG, ERR_OOM, ERR_NOT_CONVERGED, ERR_BREAKDOWN, ERR_CUDA, ERR_UNSUPPORTED, \
    ERR_BUDGET, ERR_CANCELLED = range(9)
BC_CALCULATED, BC_FIXED_VALUE, BC_FIXED_GRADIENT = 0, 1, 2
SCHEME_LINEAR, SCHEME_UPWIND, SCHEME_CORRECTED = 0, 1, 2
TERM_DDT, TERM_LAPLACIAN, TERM_DIV, TERM_SOURCE, TERM_EXPLICIT, TERM_DIV_FLUX, TERM_DIV_EXPLICIT = range(7)
PREC_FP64, PREC_MIXED_IR = 0, 1
TOK_WORD, TOK_STRING, TOK_LABEL, TOK_SCALAR, TOK_PUNCT = 1, 2, 3, 4, 5

vp = C.c_void_p
i32 = C.c_int32
i64 = C.c_int64
dbl = C.c_double
P_i32 = C.POINTER(C.c_int32)
P_i64 = C.POINTER(C.c_int64)
P_dbl = C.POINTER(C.c_double)


class MeshDesc(C.Structure):
    _fields_ = [("n_cells", i32), ("n_ifaces", i32), ("n_bfaces", i32), ("n_patches", i32),
                ("cell_volumes", vp), ("cell_centres", vp), ("owner", vp), ("neighbour", vp),
                ("face_areas", vp), ("mag_face_areas", vp), ("weights", vp), ("delta_coeffs", vp),
                ("bface_cells", vp), ("bface_areas", vp), ("bmag_face_areas", vp), ("bweights", vp),
                ("bdelta_coeffs", vp), ("patch_offsets", vp)]


class BC(C.Structure):
    _fields_ = [("patch_type", vp), ("ref", vp)]


class Term(C.Structure):
    _fields_ = [("kind", i32), ("scheme", i32), ("coeff", dbl), ("cell", vp), ("face", vp)]


class SolverCfg(C.Structure):
    _fields_ = [("rel_tol", dbl), ("abs_tol", dbl), ("max_iter", i32), ("precision", i32),
                ("inner_rel_tol", dbl), ("inner_max_iter", i32), ("max_outer", i32), ("kernel_mode", i32),
                ("flags", i32), ("method", i32), ("preconditioner", i32)]


SOLVER_CG, SOLVER_BICGSTAB, SOLVER_BICG, SOLVER_MULTIGRID = 0, 1, 2, 3
PRECOND_JACOBI, PRECOND_MULTIGRID, PRECOND_ILU = 0, 1, 2


SOLVE_NO_TUNE = 1
SOLVE_RHS_BASELINE = 2  # rel_tol relative to ||b|| (Ginkgo ResidualNorm, baseline rhs_norm)


class SolverStats(C.Structure):
    _fields_ = [("init_res_norm", dbl), ("final_res_norm", dbl), ("num_iter", i32),
                ("num_outer", i32), ("status", i32), ("reserved", i32)]


class BoxSpec(C.Structure):
    _fields_ = [("nx", i32), ("ny", i32), ("nz", i32), ("lx", dbl), ("ly", dbl), ("lz", dbl),
                ("jitter", dbl), ("seed", C.c_uint64), ("two_d", i32)]


class ServerCfg(C.Structure):
    _fields_ = [("budget_bytes", i64), ("n_streams", i32), ("max_active", i32)]


class ServeRequest(C.Structure):
    _fields_ = [("nx", i32), ("ny", i32), ("nz", i32), ("steps", i32), ("U", dbl * 3), ("D", dbl), ("dt", dbl),
                ("precision", i32), ("kernel_mode", i32), ("flags", i32), ("reserved", i32), ("T_out", vp),
                ("T_init", vp)]


SERVE_REASSEMBLE = 1
IO_BINARY, IO_SURFACE = 1, 2


class ServeResult(C.Structure):
    _fields_ = [("id", i64), ("status", i32), ("steps_done", i32), ("total_iters", i32), ("reserved", i32),
                ("submit_s", dbl), ("start_s", dbl), ("finish_s", dbl), ("device_bytes", i64)]


class MeshArrays(C.Structure):
    _fields_ = [(name, vp) for name in (
        "points", "cell_volumes", "cell_centres", "owner", "neighbour", "face_areas", "face_centres",
        "mag_face_areas", "weights", "delta_coeffs", "bface_cells", "bface_areas", "bface_centres",
        "bmag_face_areas", "bweights", "bdelta_coeffs", "patch_offsets")]


_SIGS = {
    "fvgb_status_string": (C.c_char_p, [C.c_int]),
    "fvgb_last_error": (C.c_char_p, []),
    "fvgb_abi_version": (i32, []),
    "fvgb_mesh_create": (C.c_int, [C.POINTER(MeshDesc), C.POINTER(vp)]),
    "fvgb_mesh_destroy": (C.c_int, [vp]),
    "fvgb_mesh_sizes": (C.c_int, [vp, P_i64]),
    "fvgb_mesh_device_bytes": (i64, [vp]),
    "fvgb_mesh_sparsity": (C.c_int, [vp, vp, vp, vp, vp, vp]),
    "fvgb_mesh_create_boxes": (C.c_int, [vp, i32, C.POINTER(vp), vp, vp]),
    "fvgb_bc_correct": (C.c_int, [vp, i32, C.POINTER(BC), vp, vp, vp]),
    "fvgb_interp_linear": (C.c_int, [vp, i32, vp, vp, vp, vp]),
    "fvgb_interp_upwind": (C.c_int, [vp, i32, vp, vp, vp, vp, vp]),
    "fvgb_div_explicit": (C.c_int, [vp, i32, i32, vp, vp, vp, dbl, vp, vp]),
    "fvgb_grad": (C.c_int, [vp, vp, vp, dbl, vp, vp]),
    "fvgb_laplacian_explicit": (C.c_int, [vp, i32, vp, vp, vp, dbl, vp, vp]),
    "fvgb_sngrad": (C.c_int, [vp, vp, vp, vp, vp]),
    "fvgb_laplacian_explicit_corrected": (C.c_int, [vp, i32, vp, vp, vp, dbl, vp, vp]),
    "fvgb_sngrad_corrected": (C.c_int, [vp, vp, vp, vp, vp]),
    "fvgb_nonorth_flux": (C.c_int, [vp, i32, vp, vp, vp, dbl, vp, vp]),
    "fvgb_advect_euler_step": (C.c_int, [vp, vp, vp, vp, dbl, C.POINTER(BC), vp, vp, vp]),
    "fvgb_advect_euler_steps": (C.c_int, [vp, vp, vp, vp, dbl, C.POINTER(BC), C.c_int32, vp, vp, vp]),
    "fvgb_mesh_face_tile": (C.c_int, [vp, C.c_int32]),
    "fvgb_explicit_tune": (C.c_int, [vp, vp, C.POINTER(C.c_int32), C.POINTER(C.c_float)]),
    "fvgb_ls_create": (C.c_int, [vp, i32, C.POINTER(vp)]),
    "fvgb_ls_destroy": (C.c_int, [vp]),
    "fvgb_assemble": (C.c_int, [vp, C.POINTER(Term), i32, dbl, C.POINTER(BC), vp, vp]),
    "fvgb_assemble_rhs": (C.c_int, [vp, C.POINTER(Term), i32, dbl, C.POINTER(BC), vp, vp]),
    "fvgb_set_reference": (C.c_int, [vp, i32, dbl, vp]),
    "fvgb_apply_operator": (C.c_int, [vp, vp, vp, vp]),
    "fvgb_ls_diag": (C.c_int, [vp, vp, vp]),
    "fvgb_ls_export": (C.c_int, [vp, vp, vp, vp, vp, vp]),
    "fvgb_solve": (C.c_int, [vp, vp, C.POINTER(SolverCfg), C.POINTER(SolverStats), vp]),
    "fvgb_solve_async": (C.c_int, [vp, vp, C.POINTER(SolverCfg), vp, vp]),
    "fvgb_solve_kernel_times": (C.c_int, [vp, vp, i32, vp, vp]),
    "fvgb_solve_tuning": (C.c_int, [vp, vp, vp, vp]),
    "fvgb_batch_tuning": (C.c_int, [vp, vp, vp, vp]),
    "fvgb_tuning_cache_load": (C.c_int, [C.c_char_p]),
    "fvgb_tuning_cache_save": (C.c_int, [C.c_char_p]),
    "fvgb_tuning_cache_clear": (C.c_int, []),
    "fvgb_tuning_cache_size": (C.c_int32, []),
    "fvgb_step_create": (C.c_int, [vp, vp, C.POINTER(Term), i32, dbl, C.POINTER(BC), vp, vp, vp,
                                   C.POINTER(SolverCfg), vp, C.POINTER(vp)]),
    "fvgb_step_launch": (C.c_int, [vp, vp]),
    "fvgb_polymesh_read": (C.c_int, [C.c_char_p, C.POINTER(vp), vp]),
    "fvgb_polymesh_patch": (C.c_int, [vp, i32, C.POINTER(C.c_char_p), C.POINTER(C.c_char_p)]),
    "fvgb_polymesh_geometry": (C.c_int, [vp, C.POINTER(i32), C.POINTER(vp), C.POINTER(vp), C.POINTER(vp)]),
    "fvgb_polymesh_free": (C.c_int, [vp]),
    "fvgb_field_read": (C.c_int, [C.c_char_p, i32, i32, vp]),
    "fvgb_field_read_bc": (C.c_int, [C.c_char_p, vp, i32, vp, vp, vp]),
    "fvgb_field_write": (C.c_int, [C.c_char_p, C.c_char_p, vp, i32, vp, vp, i32]),
    "fvgb_step_destroy": (C.c_int, [vp]),
    "fvgb_batch_create": (C.c_int, [vp, i32, vp, C.POINTER(vp)]),
    "fvgb_batch_destroy": (C.c_int, [vp]),
    "fvgb_batch_solve": (C.c_int, [vp, vp, C.POINTER(SolverCfg), vp, vp]),
    "fvgb_batch_solve_async": (C.c_int, [vp, vp, C.POINTER(SolverCfg), vp, vp]),
    "fvgb_pcg_csr_noalloc": (C.c_int, [i32, vp, vp, vp, vp, vp, vp, C.POINTER(SolverCfg),
                                       C.POINTER(SolverStats), vp]),
    "fvgb_piso_rau_hbya": (C.c_int, [vp, vp, vp, vp, vp]),
    "fvgb_piso_constrain_hbya": (C.c_int, [vp, vp, vp, vp, vp]),
    "fvgb_flux_vec": (C.c_int, [vp, vp, vp, vp, vp]),
    "fvgb_piso_face_update": (C.c_int, [vp, vp, vp, vp, vp]),
    "fvgb_piso_velocity_update": (C.c_int, [vp, vp, vp, vp, vp, vp, vp]),
    "fvgb_piso_ddt_corr": (C.c_int, [vp, vp, vp, vp, vp, vp, dbl, vp, vp]),
    "fvgb_piso_constrain_pressure": (C.c_int, [vp, vp, vp, vp, vp, vp, vp]),
    "fvgb_server_create": (C.c_int, [C.POINTER(ServerCfg), C.POINTER(vp)]),
    "fvgb_server_submit": (C.c_int, [vp, C.POINTER(ServeRequest), P_i64]),
    "fvgb_server_cancel": (C.c_int, [vp, i64]),
    "fvgb_server_poll": (C.c_int, [vp, vp, i32, C.POINTER(i32)]),
    "fvgb_server_info": (C.c_int, [vp, P_i64]),
    "fvgb_server_destroy": (C.c_int, [vp]),
    "fvgb_box_sizes": (C.c_int, [C.POINTER(BoxSpec), P_i64]),
    "fvgb_box_build": (C.c_int, [C.POINTER(BoxSpec), C.POINTER(MeshArrays)]),
    "fvgb_geometry_compute": (C.c_int, [i32, vp, i32, i32, vp, vp, vp, i32, vp, i32,
                                        C.POINTER(MeshArrays)]),
    "fvgb_dict_read": (C.c_int, [C.c_char_p, C.POINTER(vp)]),
    "fvgb_dict_parse": (C.c_int, [C.c_char_p, C.c_char_p, C.POINTER(vp)]),
    "fvgb_dict_create": (C.c_int, [C.POINTER(vp)]),
    "fvgb_dict_copy": (C.c_int, [vp, C.POINTER(vp)]),
    "fvgb_dict_free": (C.c_int, [vp]),
    "fvgb_dict_size": (i32, [vp]),
    "fvgb_dict_key": (C.c_char_p, [vp, i32]),
    "fvgb_dict_is_pattern": (i32, [vp, i32]),
    "fvgb_dict_find": (i32, [vp, C.c_char_p]),
    "fvgb_dict_sub": (vp, [vp, i32]),
    "fvgb_dict_ntokens": (i32, [vp, i32]),
    "fvgb_dict_token": (C.c_int, [vp, i32, i32, P_i32, C.POINTER(C.c_char_p), P_i64, C.POINTER(dbl)]),
    "fvgb_dict_set": (C.c_int, [vp, C.c_char_p, C.c_char_p]),
    "fvgb_dict_set_dict": (C.c_int, [vp, C.c_char_p, vp, C.POINTER(vp)]),
    "fvgb_dict_remove": (C.c_int, [vp, C.c_char_p]),
    "fvgb_dict_write": (C.c_int, [vp, C.c_char_p, i64, P_i64]),
    "fvgb_fvsolution_update_solver": (C.c_int, [vp]),
    "fvgb_fvsolution_update_preconditioner": (C.c_int, [vp]),
    "fvgb_fvsolution_update_criteria": (C.c_int, [vp]),
    "fvgb_fvsolution_map": (C.c_int, [vp, C.POINTER(vp)]),
    "fvgb_solver_cfg_from_dict": (C.c_int, [vp, C.POINTER(SolverCfg)]),
    "fvgb_solver_cfg_from_json": (C.c_int, [C.c_char_p, C.POINTER(SolverCfg)]),
    "fvgb_scheme_from_dict": (C.c_int, [vp, C.c_char_p, C.c_char_p, P_i32]),
    "fvgb_amg_apply": (C.c_int, [vp, vp, vp, vp]),
    "fvgb_amg_info": (C.c_int, [vp, P_i32, vp, vp, i32]),
    "fvgb_pgm_aggregate": (C.c_int, [i32, vp, vp, vp, vp, P_i32]),
}

_lib = None


class FvgbError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{status_string(status)}: {msg}")
        self.status = status


def lib() -> C.CDLL:
    """The loaded libfvgb; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(f"{LIB_PATH} is missing: run __graft_entry__.build() (no CPU fallback exists)")
        L = C.CDLL(str(LIB_PATH))
        for name, (res, args) in _SIGS.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def status_string(st: int) -> str:
    return lib().fvgb_status_string(st).decode()


def check(st: int, allow=()) -> int:
    if st != OK and st not in allow:
        raise FvgbError(st, lib().fvgb_last_error().decode())
    return st


def ptr(a) -> int | None:
    """Address of a numpy array or torch tensor (None for None)."""
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        assert a.flags["C_CONTIGUOUS"]
        return a.ctypes.data
    if hasattr(a, "data_ptr"):
        assert a.is_contiguous()
        return a.data_ptr()
    return int(a)
