"""GB300-native drop-in for ParaFROST's GPU simplify phase.

The product is the CUDA library `libpfgpu.so` behind the C ABI of
include/pfgpu.h; this package loads it (ctypes) and mirrors the reference's
`Solver::simplify` entry point and option names.
"""
from ._abi import (PFG_SAT, PFG_UNKNOWN, PFG_UNSAT, PfgOptions, PfgStats, default_options, options_dict,
                   options_from)
from .cnf import (Cnf, generate, lit_to_int, int_to_lit, parse_dimacs, random_ksat, read_dimacs, scale_free, tseitin,
                  write_dimacs)
from .simplifier import SimplifyError, SimplifyResult, Simplifier, proof_text, run_many, simplify, simplify_batch
from .server import JobInfo, Server
from .incremental import Incremental
from .writeback import Mapped, map_result, reconstruct_model

__all__ = [
    "Cnf", "Simplifier", "SimplifyResult", "SimplifyError", "simplify", "generate", "random_ksat", "tseitin",
    "scale_free", "read_dimacs", "write_dimacs", "lit_to_int", "int_to_lit", "default_options", "options_from",
    "simplify_batch", "run_many", "proof_text", "Server", "JobInfo", "parse_dimacs", "Mapped", "map_result", "reconstruct_model",
    "options_dict", "Incremental", "PfgOptions", "PfgStats", "PFG_SAT", "PFG_UNSAT", "PFG_UNKNOWN",
]
