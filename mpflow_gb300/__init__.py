"""mpflow_gb300 -- GB300-native (sm_103a) EIT hot path with mpFlow's interface.

The numerics live in the CUDA library ``_lib/libmpflow_gb300.so`` (C ABI in
``include/mpflow_gb300.h``); this package only binds it.  Importing the
package does not touch the GPU; the first call that needs the library loads
it and raises if it is missing (there is no CPU fallback).
"""
from .eit import (EIT, FIXED, EITBatch, OPEN, IrregularMesh, Ports, SolveOptions, Sources, SparseMatrix,
                  adjacent_pattern, cholesky_solve_f64, data_rows, gram_split_bf16, profile_gram)
from ._ffi import MpfError, lib
from .learned import MLP, generate_pairs, gn_labels, inclusion_frames, train_warm_start, zero_network

__all__ = ["EIT", "EITBatch", "SparseMatrix", "IrregularMesh", "Ports", "Sources", "SolveOptions",
           "adjacent_pattern", "data_rows", "gram_split_bf16", "profile_gram", "cholesky_solve_f64", "MpfError", "lib",
           "OPEN", "FIXED", "MLP", "generate_pairs", "gn_labels", "inclusion_frames", "train_warm_start",
           "zero_network"]
__version__ = "0.1.0"
