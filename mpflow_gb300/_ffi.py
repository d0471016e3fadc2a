"""ctypes binding of libmpflow_gb300.so (the C ABI in include/mpflow_gb300.h).

The library is loaded from the package's in-tree ``_lib`` directory.  There is
no fallback: if the shared library is missing or a call fails, an exception is
raised with the library's own message.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libmpflow_gb300.so")

MPF_OK = 0
STATUS_NAMES = {0: "MPF_OK", 1: "MPF_EINVAL", 2: "MPF_ENOMEM", 3: "MPF_ECUDA", 4: "MPF_ENOCONV",
                5: "MPF_EBREAKDOWN", 6: "MPF_ETIMEOUT", 7: "MPF_EFULL", 8: "MPF_ENOTSUP"}


class MpfError(RuntimeError):
    """A C-ABI call returned a non-zero status."""

    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


class EitDesc(ctypes.Structure):
    _fields_ = [
        ("n_nodes", ctypes.c_int32), ("n_elements", ctypes.c_int32),
        ("nodes", ctypes.c_void_p), ("elements", ctypes.c_void_p),
        ("edges", ctypes.c_void_p), ("n_edges", ctypes.c_int32),
        ("ports", ctypes.c_int32), ("port_edges", ctypes.c_void_p), ("port_edges_cap", ctypes.c_int32),
        ("drive_count", ctypes.c_int32), ("meas_count", ctypes.c_int32),
        ("drive_pattern", ctypes.c_void_p), ("meas_pattern", ctypes.c_void_p),
        ("source_values", ctypes.c_void_p), ("source_type", ctypes.c_int32),
        ("reference_value", ctypes.c_double), ("logarithmic", ctypes.c_int32),
        ("components", ctypes.c_int32), ("height", ctypes.c_double), ("port_height", ctypes.c_double),
        ("device", ctypes.c_int32), ("jacobian_mode", ctypes.c_int32),
        ("contact_impedance", ctypes.c_double),
    ]


class EitInfo(ctypes.Structure):
    _fields_ = [(name, ctypes.c_int32) for name in (
        "n_nodes", "n_elements", "data_rows", "ports", "drive_count", "meas_count",
        "drive_cols_pad", "meas_cols_pad", "jacobian_rows", "elements_pad", "density", "levels",
        "unique_columns", "components", "active_components")]


class SolveOpts(ctypes.Structure):
    _fields_ = [("tol", ctypes.c_double), ("max_iter", ctypes.c_int32), ("refine_tol", ctypes.c_double),
                ("max_refine", ctypes.c_int32), ("warm_start", ctypes.c_int32),
                ("check_every", ctypes.c_int32), ("preconditioner", ctypes.c_int32), ("solver", ctypes.c_int32),
                ("gn_factor", ctypes.c_int32), ("accept_tol", ctypes.c_double), ("accept_margin", ctypes.c_double)]


class SolveStats(ctypes.Structure):
    _fields_ = [("iterations", ctypes.c_int32), ("refinements", ctypes.c_int32),
                ("not_converged", ctypes.c_int32), ("max_rel_residual", ctypes.c_double),
                ("seconds", ctypes.c_double)]


class GnStats(ctypes.Structure):
    _fields_ = [("gn_iterations", ctypes.c_int32), ("cg_iterations", ctypes.c_int32),
                ("frames_converged", ctypes.c_int32), ("seconds", ctypes.c_double),
                ("solves_fp32", ctypes.c_int32), ("solves_fp64", ctypes.c_int32),
                ("accepted_loose", ctypes.c_int32)]


_P = ctypes.c_void_p
_I = ctypes.c_int32
_D = ctypes.c_double

# name -> (restype, argtypes); every symbol declared in include/mpflow_gb300.h
SIGNATURES = {
    "mpf_last_error": (ctypes.c_char_p, []),
    "mpf_version": (ctypes.c_char_p, []),
    "mpf_kernel_launches": (ctypes.c_longlong, []),
    "mpf_selftest_bounded_wait": (_I, [_I, _P]),
    "mpf_data_rows": (ctypes.c_uint32, [ctypes.c_uint32]),
    "mpf_ring_mesh_counts": (_I, [_I, _P, _P]),
    "mpf_ring_mesh": (_I, [_I, _D, _P, _P]),
    "mpf_mesh_edges": (_I, [_I, _I, _P, _P, _P, _P, _P, _P, _P]),
    "mpf_ports_circular": (_I, [_I, _P, _I, _P, _P, _I, _P, _I, _D, _D, _I, _P, _I, _P]),
    "mpf_p1_elemental": (_I, [_I, _P, _P, _P, _P]),
    "mpf_ell_layout": (_I, [_I, _I, _P, _P, _P]),
    "mpf_excitation_matrix": (_I, [_I, _P, _P, _I, _P, _I, _P, _I]),
    "mpf_eit_create": (_I, [ctypes.POINTER(EitDesc), _P]),
    "mpf_eit_destroy": (_I, [_P]),
    "mpf_eit_get_info": (_I, [_P, ctypes.POINTER(EitInfo)]),
    "mpf_eit_assemble": (_I, [_P, _I, _P, _P, _P, _P]),
    "mpf_eit_forward": (_I, [_P, _I, _P, _P, _P, ctypes.POINTER(SolveOpts), ctypes.POINTER(SolveStats), _P]),
    "mpf_eit_fields": (_I, [_P, _I, _P, _P]),
    "mpf_eit_fields_complex": (_I, [_P, _I, _P, _P]),
    "mpf_eit_forward_complex": (_I, [_P, _I, _P, _P, _P, ctypes.POINTER(SolveOpts), ctypes.POINTER(SolveStats), _P]),
    "mpf_gn_step": (_I, [_P, _I, _P, _P, _D, ctypes.POINTER(SolveOpts), _P, ctypes.POINTER(SolveStats), _P]),
    "mpf_gn_solve": (_I, [_P, _I, _P, _P, _D, _D, _I, ctypes.POINTER(SolveOpts), _P, _P,
                          ctypes.POINTER(GnStats), _P]),
    "mpf_eit_profile_cg": (_I, [_P, _I, _P, _I, _P, _P, _P]),
    "mpf_eit_profile_cg_loop": (_I, [_P, _I, _P, _I, _P, _P]),
    "mpf_eit_phase_times": (_I, [_P, _I, _P, _I, _P]),
    "mpf_eit_group_iterations": (_I, [_P, _P, _I, _P]),
    "mpf_eit_cg_variants": (_I, [_P, _P, _I, _P]),
    "mpf_inverse_solve": (_I, [_P, _I, _D, _I, _P, _P, _P, _P, _P]),
    "mpf_matrix_elementwise": (_I, [_I, _I, _I, _P, _P, _P, _I, ctypes.c_float, _P]),
    "mpf_matrix_column_reduce": (_I, [_I, _I, _I, _P, _P, _I, _P, _I, _P]),
    "mpf_convert_values": (_I, [_I, ctypes.c_int64, _P, _P, _P]),
    "mpf_matrix_multiply": (_I, [_I, _I, _I, _I, _I, _P, _I, _P, _I, _P, _I, _P]),
    "mpf_sparse_create": (_I, [_I, _P, _P, ctypes.c_uint32, _P]),
    "mpf_sparse_destroy": (_I, [_P]),
    "mpf_sparse_multiply": (_I, [_P, _P, _I, _I, _P, _I, _P]),
    "mpf_sparse_solve": (_I, [_P, _I, _P, _I, _P, _I, _I, _I, _D, _I, _P, _P]),
    "mpf_batch_create": (_I, [_P, _I, _P]),
    "mpf_batch_destroy": (_I, [_P]),
    "mpf_batch_forward": (_I, [_P, _I, _P, _P, ctypes.POINTER(SolveOpts), ctypes.POINTER(SolveStats), _P]),
    "mpf_batch_iterations": (_I, [_P, _P, _I, _P]),
    "mpf_batch_cg_stats": (_I, [_P, _P, _P]),
    "mpf_batch_cg_variants": (_I, [_P, _P, _I, _P, _I, _P]),
    "mpf_gram_split_bf16": (_I, [_I, _I, _I, _P, _I, _P, _P]),
    "mpf_cholesky_solve_f64": (_I, [_I, _I, _P, _D, _P, _I, _P, _P]),
    "mpf_gram_split_bf16_noalloc": (_I, [_I, _I, _I, _P, _I, _P, _P]),
    "mpf_mlp_create": (_I, [_I, _I, _I, _I, ctypes.c_uint64, _I, _P]),
    "mpf_mlp_destroy": (_I, [_P]),
    "mpf_mlp_layout": (_I, [_P, _P]),
    "mpf_mlp_forward": (_I, [_P, _I, _P, _P, _I, _P]),
    "mpf_mlp_backward": (_I, [_P, _I, _P, _P, _I, _I, _P, _P]),
    "mpf_mlp_adam": (_I, [_P, ctypes.c_float, ctypes.c_float, ctypes.c_float, ctypes.c_float, ctypes.c_float, _P]),
    "mpf_mlp_train_step": (_I, [_P, _I, _P, _I, _P, _P, _I, _I, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                                ctypes.c_float, ctypes.c_float, _P, _P]),
    "mpf_mlp_params": (_I, [_P, _P, _I, _P]),
    "mpf_eit_learned_input": (_I, [_P, _I, _P, _P, _P]),
    "mpf_eit_learned_prior": (_I, [_P, _D, _P]),
    "mpf_profile_gram": (_I, [_I, _I, _I, _I, _P, _P]),
    "mpf_eit_profile_fem": (_I, [_P, _I, _P, _I, _P, _P, _P]),
    "mpf_inverse_solve_complex": (_I, [_P, _I, _D, _I, _P, _P, _P, _P, _P]),
    "mpf_eit_learned_prior_apply": (_I, [_P, _I, _P, _P, _I, _I, _P]),
    "mpf_gn_solve_learned": (_I, [_P, _P, _I, _P, _P, _D, _D, _I, ctypes.POINTER(SolveOpts), _P, _P, _P,
                                  ctypes.POINTER(GnStats), _P]),
}

_lib = None


def lib() -> ctypes.CDLL:
    """Load the in-tree CUDA library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(
                f"{LIB_PATH} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`")
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def check(status: int) -> None:
    if status != MPF_OK:
        msg = lib().mpf_last_error()
        raise MpfError(status, msg.decode() if msg else "")


def ptr(a) -> ctypes.c_void_p:
    """Address of a numpy array or a torch tensor (host or device)."""
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        return a.ctypes.data_as(ctypes.c_void_p)
    return ctypes.c_void_p(a.data_ptr())
