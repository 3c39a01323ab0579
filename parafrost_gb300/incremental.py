"""The simplify side of the reference's incremental interface.

ParaFROST's IPASIR front end adds clauses and freezes variables between calls,
and every `Solver::isolve` (src/gpu/solverinc.cpp:73-150) marks the frozen
and assumed variables in `assumed` (`ifreeze` / `iassume`,
src/gpu/assume.cpp:193-245) before it simplifies, so that simplification never
eliminates a variable the caller still talks about. `Incremental` keeps that
flow on the host around the engine: the live formula is held in external
(DIMACS) numbering; every call uploads it over the variables still active,
renumbered 1..n with `vorg` mapping back (as `Solver::map` does), with the
frozen and assumed variables kept out of elections and BVE counting only
original clauses from the second call on (`in_ve_k_1`); the result is folded
back: the simplified clauses replace the formula, eliminated variables are
recorded, device units fix their variables, and the model stack (already in
external numbering) grows. `extend` turns a model of the current formula into
a model of everything added so far.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import Dict, Iterable, List, Optional

import numpy as np

from . import _lib
from .cnf import Cnf
from .simplifier import Simplifier

MELTING, FORCED = 0x1, 0x4


@dataclass
class Prepared:
    """The inputs of one call: the live formula over the active variables."""
    cnf: Cnf                  # clauses over 1..n (every clause has >= 2 literals)
    assumed: np.ndarray       # uint8[n+1]: frozen or assumed variables
    vorg: np.ndarray          # uint32[n+1]: external variable of each internal one
    ve_inprocess: int         # 1 from the second call on


class Incremental:
    def __init__(self, **options):
        self.options = options
        self.max_var = 0
        self.clauses: List[tuple] = []        # live formula, DIMACS literals
        self.fixed: Dict[int, bool] = {}      # top-level values (units)
        self.eliminated: set = set()
        self.frozen: set = set()
        self.assumptions: List[int] = []
        self.stack: List[int] = []            # model stack words, 2v|s in external numbering
        self.calls = 0
        self.unsat = False

    # ---- ipasir_add / ifreeze / iassume ----
    def add(self, clause: Iterable[int]) -> None:
        c = tuple(int(l) for l in clause)
        for l in c:
            if l == 0:
                raise ValueError("literal 0 in a clause")
            if abs(l) in self.eliminated:
                raise ValueError(f"variable {abs(l)} was eliminated; freeze variables that are used later")
            self.max_var = max(self.max_var, abs(l))
        self.clauses.append(c)

    def freeze(self, v: int) -> None:
        if v in self.eliminated:
            raise ValueError(f"variable {v} was eliminated")
        self.frozen.add(int(v))
        self.max_var = max(self.max_var, int(v))

    def melt(self, v: int) -> None:
        self.frozen.discard(int(v))

    def assume(self, lit: int) -> None:
        if abs(lit) in self.eliminated:
            raise ValueError(f"variable {abs(lit)} was eliminated")     # assert(!ieliminated(v)), assume.cpp:233
        self.assumptions.append(int(lit))
        self.max_var = max(self.max_var, abs(int(lit)))

    # ---- one Solver::simplify call ----
    def _propagate_fixed(self) -> None:
        """Apply the top-level values: drop satisfied clauses, remove false
        literals, turn one-literal clauses into values (to a fixpoint)."""
        changed = True
        while changed and not self.unsat:
            changed = False
            out = []
            for c in self.clauses:
                keep, sat = [], False
                for l in c:
                    v = self.fixed.get(abs(l))
                    if v is None:
                        if l not in keep:
                            keep.append(l)
                    elif v == (l > 0):
                        sat = True
                        break
                if sat:
                    continue
                if any(-l in keep for l in keep):
                    continue
                if not keep:
                    self.unsat = True
                    return
                if len(keep) == 1:
                    self.fixed[abs(keep[0])] = keep[0] > 0
                    changed = True
                    continue
                out.append(tuple(keep))
            self.clauses = out

    def prepare(self) -> Optional[Prepared]:
        """Inputs of the next call, or None when the formula is decided on the
        host (UNSAT, or no clause left)."""
        self._propagate_fixed()
        if self.unsat or not self.clauses:
            return None
        active = sorted({abs(l) for c in self.clauses for l in c})
        new_of = {v: i + 1 for i, v in enumerate(active)}
        n = len(active)
        vorg = np.zeros(n + 1, dtype=np.uint32)
        vorg[1:] = np.array(active, dtype=np.uint32)
        assumed = np.zeros(n + 1, dtype=np.uint8)
        for v in self.frozen | {abs(a) for a in self.assumptions}:
            if v in new_of:
                assumed[new_of[v]] = 1
        mapped = [[new_of[abs(l)] if l > 0 else -new_of[abs(l)] for l in c] for c in self.clauses]
        return Prepared(Cnf.from_ints(n, mapped), assumed, vorg, 1 if self.calls else 0)

    def absorb(self, prep: Prepared, res) -> None:
        """Fold a result of `prep` back into the session."""
        self.calls += 1
        self.assumptions = []
        if int(res.status) == 20:
            self.unsat = True
            return
        vorg = prep.vorg
        elim = np.asarray(res.eliminated)
        for v in np.nonzero((elim & MELTING) & ~(elim & FORCED))[0]:
            if v:
                self.eliminated.add(int(vorg[v]))
        for u in list(np.asarray(res.units)) + list(np.asarray(res.pending_units)):
            u = int(u)
            self.fixed[int(vorg[u >> 1])] = not (u & 1)
        self.stack.extend(int(w) for w in np.asarray(res.stack))
        cnf = res.cnf
        out = []
        for i in range(cnf.num_clauses):
            lits = cnf.clause(i)
            out.append(tuple(int(vorg[l >> 1]) * (-1 if l & 1 else 1) for l in lits))
        self.clauses = out

    def simplify(self):
        """One call on the GPU engine; returns the engine's result (None when
        the host decided the formula)."""
        prep = self.prepare()
        if prep is None:
            self.calls += 1
            self.assumptions = []
            return None
        opts = dict(self.options, ve_inprocess=prep.ve_inprocess)
        with Simplifier(**opts) as s:
            res = s.simplify(prep.cnf, assumed=prep.assumed, vorg=prep.vorg)
        self.absorb(prep, res)
        return res

    # ---- model ----
    def extend(self, values) -> np.ndarray:
        """values[v] (0/1) for the variables of the current formula (indexed by
        external variable); returns a model of every clause added so far:
        fixed values set, then the model stack walked backwards
        (MODEL::extend, src/gpu/model.cpp:101-160)."""
        V = self.max_var
        value = np.zeros(V + 1, dtype=np.uint8)
        vals = np.asarray(values, dtype=np.uint8)
        value[: min(len(vals), V + 1)] = vals[: V + 1]
        for v, b in self.fixed.items():
            value[v] = 1 if b else 0
        st = np.ascontiguousarray(np.array(self.stack, dtype=np.uint32))
        L = _lib.lib()
        if len(st) and L.pfg_extend_model(len(st), st.ctypes.data_as(C.POINTER(C.c_uint32)), V,
                                          value.ctypes.data_as(C.POINTER(C.c_uint8))):
            raise ValueError("malformed model stack")
        return value

    def formula(self) -> Cnf:
        """The live formula (external numbering) plus the top-level values as units."""
        cls = [list(c) for c in self.clauses] + [[v if b else -v] for v, b in self.fixed.items()]
        return Cnf.from_ints(self.max_var, cls)
