"""stzpp_gb300: GB300-native multigrid for stzpp's quasi-static projection solve.

The compute path is the CUDA library ``libstz_mg.so`` (sources in csrc/, C-ABI
in include/stz_mg.h) built for sm_103a; :mod:`stzpp_gb300.mg` is the Python
mirror of the reference's multigrid interface over that ABI.
"""
from .mg import (BOTTOM_DIRECT, BOTTOM_GS, DEVICE, FP64, HOST, MIXED, Multigrid, StzMgError,
                 elastic_stencil, load_library)

__all__ = ["Multigrid", "StzMgError", "elastic_stencil", "load_library", "FP64", "MIXED",
           "BOTTOM_DIRECT", "BOTTOM_GS", "HOST", "DEVICE"]
