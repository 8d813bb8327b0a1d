"""ish_gb300 -- GB300-native batch alignment scoring for ish.

Exact-integer striped semi-global and striped local (Smith-Waterman/Gotoh)
scoring of queries against record sets, on hand-written sm_103a CUDA kernels
behind the C ABI of ``libish_gpu.so`` (include/ish_gpu.h).  This package is
the host-side mirror of ish's matcher plugin API.
"""
from .matcher import (BatchResult, SemiGlobalEndsFreeness, StripedLocalMatcher,  # noqa: F401
                      StripedSemiGlobalMatcher)
from .native import Context, IshGpuError, pack_records  # noqa: F401
from .scoring import ScoringMatrix  # noqa: F401

__all__ = ["BatchResult", "Context", "IshGpuError", "ScoringMatrix", "SemiGlobalEndsFreeness",
           "StripedLocalMatcher", "StripedSemiGlobalMatcher", "pack_records"]
