"""doci_gb300 -- GB300-native (sm_103a) DOCI eigensolver.

The engine is libdoci_gb300.so (CUDA kernels + a C ABI, include/doci_gb300.h):
a drop-in for the reference's matvec plug-in (doci_matvec / fill_doci_data)
and solver dispatch (sparse_eigensolve), plus a status-returning device API.
This package loads that library through ctypes and adds the synthetic
FCIDUMP generator used by the benchmark workloads.
"""
from ._lib import (FP32, FP64, MODE_FP64, MODE_MIXED, SOLVER_CG, SOLVER_CGP,  # noqa: F401
                   SOLVER_D, DociError, Hamiltonian, LIB_PATH, Server, SolveOpts, SolveResult, batch_opts,
                   batch_solve, default_opts, fcidump_integrals, footprint, lib, solve_roots)
from .fcidump import raw_integrals, synthetic_integrals, write_fcidump, write_synthetic_fcidump  # noqa: F401

__all__ = ["FP32", "FP64", "MODE_FP64", "MODE_MIXED", "SOLVER_D", "SOLVER_CG", "SOLVER_CGP", "DociError",
           "Hamiltonian", "LIB_PATH", "Server", "SolveOpts", "SolveResult", "batch_opts", "batch_solve",
           "default_opts", "fcidump_integrals", "footprint", "lib", "solve_roots",
           "raw_integrals", "synthetic_integrals", "write_fcidump", "write_synthetic_fcidump"]
