"""scft_gb300 -- the SCFT inner loop of giantsda/SCFT on one GB300 GPU.

The compute path is libscft.so (hand-written sm_103a CUDA behind the C ABI of
include/scft.h); this package is the host-side mirror of the reference's
interface over that ABI.  Importing the package does not load the library;
``scft_gb300.api`` functions load it on first use and raise ImportError when it
has not been built.
"""
from ._lib import (F32, F64, MIX_LINEAR, MIX_LOG, RULE_ROMBERG, RULE_TRAPEZOID, SCHEME_IE, SCHEME_IRK2,
                   ST_CONVERGED, ST_FORKED, ST_FP64, ST_MAXIT, ST_NONFINITE, ST_NOT_DOMINANT, ST_RESTARTED,
                   ST_WATCHDOG, W_CONSISTENT, W_ROWSCALED, ScftError, load)

__all__ = ["F32", "F64", "MIX_LINEAR", "MIX_LOG", "RULE_ROMBERG", "RULE_TRAPEZOID", "SCHEME_IE", "SCHEME_IRK2",
           "ST_CONVERGED", "ST_FORKED", "ST_FP64", "ST_MAXIT", "ST_NONFINITE", "ST_NOT_DOMINANT", "ST_RESTARTED",
           "ST_WATCHDOG", "W_CONSISTENT", "W_ROWSCALED", "ScftError", "load"]
