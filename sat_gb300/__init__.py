"""sat_gb300 -- summed-area tables (integral images) on one GB300 (sm_103a).

A drop-in for pengdada/SAT's three algorithm entry points (ScanRow-BRLT,
BRLT-ScanRow, ScanRowColumn) and their input -> output type pairs, computed by
a single-pass tiled CUDA kernel with decoupled look-back (libsatgb.so, C ABI in
include/satgb.h).  Adds a compensated f32 mode, batched persistent launches in
a CUDA graph, a reverse (suffix) SAT and a torch.autograd box filter.
"""
from ._lib import (F32, F64, I8, I32, KOGGE_STONE_SCAN, LF_SCAN, U8, U32, SatError,
                   launch_count)
from .api import (ALGORITHMS, PAIRS, BatchPlan, autotune, box_means_adjoint, box_means_from_sat, box_means_grad_x,
                  brlt_scanrow, config_names, release, sat, scan_cols, scan_rows, scan_rows_transposed,
                  scanrow_brlt, scanrowcolumn, set_config, set_wait_limit_us, stream_check)
from .autograd import BoxFilter, SATFunction, box_filter_means

__all__ = [
    "ALGORITHMS", "PAIRS", "BatchPlan", "BoxFilter", "SATFunction", "SatError", "autotune",
    "box_filter_means", "box_means_adjoint", "box_means_from_sat", "box_means_grad_x", "brlt_scanrow", "config_names",
    "launch_count", "release", "sat", "scan_cols", "scan_rows", "scan_rows_transposed", "scanrow_brlt",
    "scanrowcolumn", "set_config", "set_wait_limit_us", "stream_check", "U8", "I8", "U32", "I32", "F32", "F64",
    "KOGGE_STONE_SCAN", "LF_SCAN",
]
