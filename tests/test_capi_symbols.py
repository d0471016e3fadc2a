"""The C-ABI library loads without a GPU and exports every entry point that
include/*.h declares (no compute calls)."""
import ctypes
import glob
import os
import re

import mpflow_gb300
from mpflow_gb300 import _ffi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for header in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(header).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"\b(mpf_[a-z0-9_]+)\s*\(", text):
            names.add(m.group(1))
    return names


def test_header_declares_entry_points():
    names = declared_functions()
    assert {"mpf_eit_create", "mpf_eit_forward", "mpf_gn_step", "mpf_gram_split_bf16",
            "mpf_cholesky_solve_f64"} <= names


def test_library_exports_all_declared_symbols():
    L = ctypes.CDLL(_ffi.LIB_PATH)
    missing = [n for n in sorted(declared_functions()) if not hasattr(L, n)]
    assert not missing, missing


def test_binding_covers_header():
    assert declared_functions() <= set(_ffi.SIGNATURES)


def test_host_only_calls_work_without_gpu():
    L = mpflow_gb300.lib()
    assert L.mpf_version().startswith(b"mpflow_gb300")
    assert L.mpf_data_rows(19441) == 19456
    n, e = ctypes.c_int32(), ctypes.c_int32()
    assert L.mpf_ring_mesh_counts(80, ctypes.byref(n), ctypes.byref(e)) == 0
    assert (n.value, e.value) == (19441, 38400)
    assert L.mpf_ring_mesh_counts(0, ctypes.byref(n), ctypes.byref(e)) == 1
    assert b"rings" in L.mpf_last_error()


def test_invalid_model_arguments_are_rejected():
    L = mpflow_gb300.lib()
    h = ctypes.c_void_p()
    assert L.mpf_eit_create(None, ctypes.byref(h)) == 1
    assert L.mpf_eit_forward(None, 1, None, None, None, None, None, None) == 1
    assert b"model == nullptr" in L.mpf_last_error()


def test_selftest_rejects_bad_timeout_without_gpu():
    L = mpflow_gb300.lib()
    assert L.mpf_selftest_bounded_wait(0, None) == 1
    assert L.mpf_selftest_bounded_wait(3000000, None) == 1


def test_new_entry_points_reject_bad_arguments_without_gpu():
    """Argument checks of the complex inverse, the learned prior and the
    Gram measurement hook run before any device work."""
    L = mpflow_gb300.lib()
    assert L.mpf_inverse_solve_complex(None, 0, 1.0, 1, None, None, None, None, None) == 1
    assert b"model == nullptr" in L.mpf_last_error()
    assert L.mpf_eit_learned_prior(None, 1.0, None) == 1
    assert L.mpf_eit_learned_prior_apply(None, 1, None, None, 0, 0, None) == 1
    ms = ctypes.c_double(0.0)
    assert L.mpf_profile_gram(1, 100, 64, 1, ctypes.byref(ms), None) == 1
    assert b"rows" in L.mpf_last_error()
    assert L.mpf_profile_gram(0, 128, 64, 1, ctypes.byref(ms), None) == 1


def test_entry_points_of_this_build_reject_bad_arguments_without_gpu():
    """Argument checks of the device conversion, the training step, the
    complex field export and the CG loop hook run before any device work;
    the solve options carry the acceptance-solve fields in header order."""
    L = mpflow_gb300.lib()
    assert L.mpf_convert_values(2, 4, None, None, None) == 1
    assert b"direction" in L.mpf_last_error()
    assert L.mpf_convert_values(0, -1, None, None, None) == 1
    assert L.mpf_convert_values(0, 0, None, None, None) == 0  # nothing to convert
    assert L.mpf_mlp_train_step(None, 1, None, 0, None, None, 0, 1, 1e-3, 0.9, 0.999, 1e-8, 0.0, None, None) == 1
    assert L.mpf_eit_fields_complex(None, 1, None, None) == 1
    assert b"model == nullptr" in L.mpf_last_error()
    assert L.mpf_eit_profile_cg_loop(None, 1, None, 1, None, None) == 1
    from mpflow_gb300 import _ffi
    from mpflow_gb300.eit import SolveOptions
    o = SolveOptions(tol=1e-5, gn_factor="fp32-refined", accept_tol=1e-4, accept_margin=0.2).c()
    assert (o.gn_factor, o.accept_tol, o.accept_margin) == (1, 1e-4, 0.2)
    names = [f[0] for f in _ffi.SolveOpts._fields_]
    assert names[-3:] == ["gn_factor", "accept_tol", "accept_margin"]
    assert [f[0] for f in _ffi.GnStats._fields_][-1] == "accepted_loose"
