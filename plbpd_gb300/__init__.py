"""GB300 lattice-Boltzmann engine with plbpd's BGK/SRT operator API.

The compute path is libplb_gb300.so (CUDA, sm_103a), reached through the C ABI
declared in include/plb.h.  ``plbpd_gb300.capi`` binds it for Python callers;
the C++ classes of plbpd (LBModel, Domain, Boundary, SimData, PLBPD, ...) are in
include/plbpd/ over the same ABI.
"""
from . import capi  # noqa: F401
from .capi import Solve, make_params  # noqa: F401

__all__ = ["capi", "Solve", "make_params"]
