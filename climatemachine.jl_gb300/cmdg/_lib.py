"""ctypes binding of libcmdg.so (the C ABI declared in include/cmdg.h).

The library is built in-tree by ``climatemachine.jl_gb300/build.py``.  There
is no CPU fallback: if the shared library is missing or cannot be loaded,
every entry point raises ``CmdgError``.
"""
from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
PKG_ROOT = os.path.dirname(HERE)
LIB_PATH = os.path.join(PKG_ROOT, "_build", "libcmdg.so")

CMDG_OK = 0
ERRORS = {1: "CMDG_ERR_ARG", 2: "CMDG_ERR_CUDA", 3: "CMDG_ERR_UNSUPPORTED", 4: "CMDG_ERR_NONFINITE",
          5: "CMDG_ERR_TIMEOUT", 6: "CMDG_ERR_ALLOC", 7: "CMDG_ERR_STATE"}
CMDG_FP64, CMDG_MIXED = 0, 1
CMDG_DIR_EVERY, CMDG_DIR_HORIZONTAL, CMDG_DIR_VERTICAL = 0, 1, 2
CMDG_TOPOLOGY_LIBRARY, CMDG_TOPOLOGY_BRICK, CMDG_TOPOLOGY_STACKED_BRICK = 0, 1, 2

# Every exported symbol of include/cmdg.h (checked by the CPU test suite).
EXPORTS = (
    "cmdg_last_error", "cmdg_version", "cmdg_mesh_create_brick", "cmdg_mesh_create_shell", "cmdg_mesh_destroy", "cmdg_mesh_info",
    "cmdg_mesh_coordinates", "cmdg_mesh_mass", "cmdg_model_create", "cmdg_model_destroy",
    "cmdg_model_reference_state", "cmdg_tendency", "cmdg_lsrk54_step", "cmdg_to_perturbation",
    "cmdg_from_perturbation", "cmdg_tendency_mixed", "cmdg_lsrk54_step_mixed", "cmdg_weighted_sums",
    "cmdg_weighted_sums_mixed", "cmdg_courant_dt", "cmdg_status_word", "cmdg_lsrk54_step_noalloc",
    "cmdg_model_set_kernel", "cmdg_model_get_kernel", "cmdg_model_autotune", "cmdg_gradient_flux",
    "cmdg_hyperdiffusive_state", "cmdg_lsrk54_step_mixed_host", "cmdg_mesh_create_arrays", "cmdg_model_set_reference",
    "cmdg_batch_create", "cmdg_batch_destroy", "cmdg_batch_set_tiling", "cmdg_batch_get_tiling",
    "cmdg_batch_lsrk54_step", "cmdg_batch_autotune",
    "cmdg_filter_matrix", "cmdg_apply_filter", "cmdg_apply_tmar",
    "cmdg_linear_tendency", "cmdg_hevi_create", "cmdg_hevi_destroy", "cmdg_hevi_info", "cmdg_hevi_solve",
    "cmdg_hevi_step", "cmdg_apply_mp_filter", "cmdg_model_set_mms", "cmdg_model_set_staging_test",
    "cmdg_brick_element_order", "cmdg_mesh_create_brick_ordered", "cmdg_batch_set_kernel", "cmdg_batch_get_kernel",
)


class CmdgError(RuntimeError):
    """A libcmdg entry point returned an error code."""

    def __init__(self, fn: str, code: int, msg: str):
        super().__init__(f"{fn} -> {ERRORS.get(code, code)}: {msg}")
        self.code = code


class BrickDesc(ctypes.Structure):
    _fields_ = [("N", ctypes.c_int), ("ne", ctypes.c_int * 3), ("lo", ctypes.c_double * 3),
                ("hi", ctypes.c_double * 3), ("periodic", ctypes.c_int * 3), ("bc_lo", ctypes.c_int * 3),
                ("bc_hi", ctypes.c_int * 3)]


class AtmosParams(ctypes.Structure):
    _fields_ = [("R_d", ctypes.c_double), ("cp_d", ctypes.c_double), ("cv_d", ctypes.c_double),
                ("T_0", ctypes.c_double), ("grav", ctypes.c_double), ("MSLP", ctypes.c_double),
                ("inv_Pr_turb", ctypes.c_double), ("numflux", ctypes.c_int), ("orientation", ctypes.c_int),
                ("gravity", ctypes.c_int), ("ref_state", ctypes.c_int), ("subtract_off", ctypes.c_int),
                ("profile", ctypes.c_int), ("T_surface", ctypes.c_double), ("T_min", ctypes.c_double),
                ("turbulence", ctypes.c_int), ("rho_nu", ctypes.c_double), ("with_divergence", ctypes.c_int),
                ("C_smag", ctypes.c_double), ("planet_radius", ctypes.c_double),
                ("hyperdiffusion", ctypes.c_int), ("tau_hyper", ctypes.c_double), ("hyper_direction", ctypes.c_int)]


class ShellDesc(ctypes.Structure):
    _fields_ = [("N", ctypes.c_int), ("nhorz", ctypes.c_int), ("nvert", ctypes.c_int), ("r_inner", ctypes.c_double),
                ("r_outer", ctypes.c_double), ("bc_inner", ctypes.c_int), ("bc_outer", ctypes.c_int)]


class GridArrays(ctypes.Structure):
    _fields_ = [("N", ctypes.c_int), ("nelem", ctypes.c_int64), ("vgeo", ctypes.c_void_p),
                ("vmap_plus", ctypes.c_void_p), ("elemtobndy", ctypes.c_void_p)]


_lib = None


def load(path: str | None = None):
    """Loads libcmdg.so and declares the prototypes; raises if it is absent."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise CmdgError("load", 3, f"{path} is missing: build it with climatemachine.jl_gb300/build.py")
    L = ctypes.CDLL(path)
    P = ctypes.c_void_p
    PP = ctypes.POINTER(ctypes.c_void_p)
    D = ctypes.c_double
    I = ctypes.c_int
    L.cmdg_last_error.restype = ctypes.c_char_p
    L.cmdg_version.restype = ctypes.c_char_p
    proto = {
        "cmdg_mesh_create_brick": [ctypes.POINTER(BrickDesc), PP],
        "cmdg_mesh_create_shell": [ctypes.POINTER(ShellDesc), PP],
        "cmdg_mesh_destroy": [P],
        "cmdg_mesh_info": [P, ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int)],
        "cmdg_mesh_coordinates": [P, P],
        "cmdg_mesh_mass": [P, P],
        "cmdg_model_create": [P, ctypes.POINTER(AtmosParams), I, PP],
        "cmdg_model_destroy": [P],
        "cmdg_model_reference_state": [P, P],
        "cmdg_tendency": [P, P, P, D, D, D, P],
        "cmdg_lsrk54_step": [P, P, P, D, D, I, P],
        "cmdg_to_perturbation": [P, P, P, P],
        "cmdg_from_perturbation": [P, P, P, P],
        "cmdg_tendency_mixed": [P, P, P, D, D, D, P],
        "cmdg_lsrk54_step_mixed": [P, P, P, D, D, I, P],
        "cmdg_weighted_sums": [P, P, I, P, P, P],
        "cmdg_weighted_sums_mixed": [P, P, I, P, P, P],
        "cmdg_courant_dt": [P, P, D, P, P],
        "cmdg_status_word": [P, P, P],
        "cmdg_lsrk54_step_noalloc": [P, P, P, D, D, I, P],
        "cmdg_model_set_kernel": [P, I, I],
        "cmdg_model_get_kernel": [P, ctypes.POINTER(I), ctypes.POINTER(I)],
        "cmdg_model_autotune": [P, I, P, I, ctypes.POINTER(I), P],
        "cmdg_gradient_flux": [P, P, P, P],
        "cmdg_hyperdiffusive_state": [P, P, P, P],
        "cmdg_lsrk54_step_mixed_host": [P, P, P, P, D, D, I, P],
        "cmdg_mesh_create_arrays": [ctypes.POINTER(GridArrays), PP],
        "cmdg_model_set_reference": [P, P],
        "cmdg_batch_create": [P, I, PP],
        "cmdg_batch_destroy": [P],
        "cmdg_batch_set_tiling": [P, I, I, I],
        "cmdg_batch_get_tiling": [P, I, ctypes.POINTER(I), ctypes.POINTER(I)],
        "cmdg_batch_lsrk54_step": [P, P, P, P, I, P],
        "cmdg_batch_autotune": [P, P, P, I, P, I, ctypes.POINTER(I), P],
        "cmdg_filter_matrix": [I, I, I, I, D, P],
        "cmdg_apply_filter": [P, P, P, P, I, P, I, P],
        "cmdg_apply_tmar": [P, P, P, I, P],
        "cmdg_linear_tendency": [P, P, P, D, D, D, P],
        "cmdg_hevi_create": [P, D, I, I, I, PP],
        "cmdg_hevi_destroy": [P],
        "cmdg_hevi_info": [P, ctypes.POINTER(D), ctypes.POINTER(I), ctypes.POINTER(ctypes.c_int64)],
        "cmdg_hevi_solve": [P, P, P, P],
        "cmdg_hevi_step": [P, P, D, I, P],
        "cmdg_apply_mp_filter": [P, P, P, P, I, P, I, P],
        "cmdg_model_set_mms": [P, P, P, I],
        "cmdg_model_set_staging_test": [P, I, I],
        "cmdg_brick_element_order": [ctypes.POINTER(BrickDesc), I, P],
        "cmdg_mesh_create_brick_ordered": [ctypes.POINTER(BrickDesc), I, PP],
        "cmdg_batch_set_kernel": [P, I, I, I, I],
        "cmdg_batch_get_kernel": [P, ctypes.POINTER(I), ctypes.POINTER(I), ctypes.POINTER(I), ctypes.POINTER(I)],
    }
    for name, args in proto.items():
        fn = getattr(L, name)
        fn.restype = ctypes.c_int
        fn.argtypes = args
    _lib = L
    return L


def check(fn_name: str, rc: int):
    if rc != CMDG_OK:
        msg = load().cmdg_last_error().decode(errors="replace")
        raise CmdgError(fn_name, rc, msg)


def call(fn_name: str, *args):
    rc = getattr(load(), fn_name)(*args)
    check(fn_name, rc)
