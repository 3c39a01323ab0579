"""Write-back of a simplification result into a host solver.

`map_result` compacts the variables that are still active (Solver::map,
src/gpu/vmap.cpp:61) and renumbers the simplified CNF and the pending units
accordingly; `reconstruct_model` takes a model of the mapped formula back to
the original numbering, adds the units fixed by device propagation and walks
the model stack (MODEL::extend, src/gpu/model.cpp:101). Both run the library's
host functions (pfg_map_vars, pfg_map_lits, pfg_extend_model).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib
from .cnf import Cnf


def _p(a, t):
    return a.ctypes.data_as(C.POINTER(t))


@dataclass
class Mapped:
    cnf: Cnf                 # simplified clauses over variables 1..cnf.max_var
    units: np.ndarray        # pending units, mapped
    old_of_new: np.ndarray   # uint32[cnf.max_var + 1]
    new_of_old: np.ndarray   # uint32[original max_var + 1], 0 for dropped variables


def map_result(res) -> Mapped:
    L = _lib.lib()
    V = int(res.cnf.max_var)
    elim = np.ascontiguousarray(res.eliminated, dtype=np.uint8)
    new_of_old = np.zeros(V + 1, dtype=np.uint32)
    old_of_new = np.zeros(V + 1, dtype=np.uint32)
    nv = C.c_uint32()
    if L.pfg_map_vars(V, _p(elim, C.c_uint8), _p(new_of_old, C.c_uint32), _p(old_of_new, C.c_uint32), C.byref(nv)):
        raise ValueError("pfg_map_vars failed")
    n = int(nv.value)
    lits = np.empty_like(res.cnf.lits)
    src = np.ascontiguousarray(res.cnf.lits, dtype=np.uint32)
    if len(src) and L.pfg_map_lits(_p(new_of_old, C.c_uint32), V, len(src), _p(src, C.c_uint32), _p(lits, C.c_uint32)):
        raise ValueError("a clause holds an eliminated or fixed variable")
    pend = np.ascontiguousarray(res.pending_units, dtype=np.uint32)
    units = np.empty_like(pend)
    if len(pend) and L.pfg_map_lits(_p(new_of_old, C.c_uint32), V, len(pend), _p(pend, C.c_uint32), _p(units, C.c_uint32)):
        raise ValueError("a pending unit belongs to a dropped variable")
    cnf = Cnf(n, lits, np.array(res.cnf.off, dtype=np.uint64), res.cnf.learnt, res.cnf.lbd, res.cnf.usage)
    return Mapped(cnf, units, old_of_new[: n + 1].copy(), new_of_old)


def reconstruct_model(res, mapped: Mapped, values_new) -> np.ndarray:
    """values_new[1..n]: a model of the mapped formula (0/1). Returns a model of
    the original formula, uint8[max_var + 1]."""
    L = _lib.lib()
    V = int(res.cnf.max_var)
    value = np.zeros(V + 1, dtype=np.uint8)
    vn = np.asarray(values_new, dtype=np.uint8)
    value[mapped.old_of_new[1:]] = vn[1: len(mapped.old_of_new)]
    units = np.asarray(res.units, dtype=np.uint32)
    value[units >> 1] = (1 - (units & 1)).astype(np.uint8)
    stack = np.ascontiguousarray(res.stack, dtype=np.uint32)
    if L.pfg_extend_model(len(stack), _p(stack, C.c_uint32), V, _p(value, C.c_uint8)):
        raise ValueError("malformed model stack")
    return value
