"""bsam1.2_gb300 -- GB300 (sm_103a) FAS multigrid V-cycle for BSAM 1.2.

The compute path is libbsamg.so (CUDA C++ behind the C ABI in
include/bsamg.h); this package is its Python host mirror.
"""
from .api import (BsamgError, Context, Hierarchy, exported_symbols, format_f25, format_stats_line,  # noqa: F401
                  lib, pin, regrid_params, unpin)
from . import initial  # noqa: F401
from . import serve  # noqa: F401
