"""CNF containers, DIMACS I/O and the seeded instance generators.

Literals use the reference's internal encoding lit = 2*v | sign
(src/gpu/constants.hpp:72-80); clauses are stored flat with uint64 offsets.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field
from typing import Iterable, List, Optional

import os

import numpy as np

from . import _lib

FAMILY_KSAT = 0
FAMILY_TSEITIN = 1
FAMILY_SCALEFREE = 2


@dataclass
class Cnf:
    max_var: int
    lits: np.ndarray                      # uint32, internal literals
    off: np.ndarray                       # uint64, num_clauses + 1
    learnt: Optional[np.ndarray] = None   # uint8 per clause (1 = learnt)
    lbd: Optional[np.ndarray] = None      # uint32 per clause
    usage: Optional[np.ndarray] = None    # uint8 per clause

    def __post_init__(self):
        self.lits = np.ascontiguousarray(self.lits, dtype=np.uint32)
        self.off = np.ascontiguousarray(self.off, dtype=np.uint64)
        if self.learnt is not None:
            self.learnt = np.ascontiguousarray(self.learnt, dtype=np.uint8)
        if self.lbd is not None:
            self.lbd = np.ascontiguousarray(self.lbd, dtype=np.uint32)
        if self.usage is not None:
            self.usage = np.ascontiguousarray(self.usage, dtype=np.uint8)

    @property
    def num_clauses(self) -> int:
        return len(self.off) - 1

    @property
    def num_literals(self) -> int:
        return int(self.off[-1]) if len(self.off) else 0

    def clause(self, i: int) -> np.ndarray:
        return self.lits[int(self.off[i]):int(self.off[i + 1])]

    def pinned(self) -> "Cnf":
        """A copy whose arrays live in page-locked host memory (uploads from it
        are direct DMA transfers)."""
        from . import pinned as pm
        cp = lambda a: None if a is None else pm.copy(a)
        return Cnf(self.max_var, pm.copy(self.lits), pm.copy(self.off), cp(self.learnt), cp(self.lbd), cp(self.usage))

    def clauses(self) -> List[List[int]]:
        """Clauses as lists of DIMACS integers."""
        out = []
        for i in range(self.num_clauses):
            out.append([lit_to_int(int(l)) for l in self.clause(i)])
        return out

    @staticmethod
    def from_ints(max_var: int, clauses: Iterable[Iterable[int]], learnt: Optional[Iterable[int]] = None) -> "Cnf":
        lits, off = [], [0]
        for c in clauses:
            for x in c:
                lits.append(int_to_lit(int(x)))
            off.append(len(lits))
        lr = None if learnt is None else np.asarray(list(learnt), dtype=np.uint8)
        return Cnf(max_var, np.asarray(lits, dtype=np.uint32), np.asarray(off, dtype=np.uint64), lr)


def int_to_lit(x: int) -> int:
    return (abs(x) << 1) | (1 if x < 0 else 0)


def lit_to_int(lit: int) -> int:
    v = lit >> 1
    return -v if lit & 1 else v


def generate(family: int, a: int, b: int, c: int, seed: int) -> Cnf:
    """Seeded instance from the C generators (pfg_generate of the host-only
    libpfgen.so, the same code libpfgpu.so exports)."""
    lib = _lib.gen_lib()
    mv = C.c_uint32()
    nc = C.c_uint64()
    nl = C.c_uint64()
    rc = lib.pfg_generate(family, a, b, c, seed, C.byref(mv), C.byref(nc), C.byref(nl), None, None)
    if rc != 0:
        raise ValueError(f"pfg_generate failed ({rc})")
    lits = np.empty(nl.value, dtype=np.uint32)
    off = np.empty(nc.value + 1, dtype=np.uint64)
    rc = lib.pfg_generate(family, a, b, c, seed, None, None, None,
                          lits.ctypes.data_as(C.POINTER(C.c_uint32)), off.ctypes.data_as(C.POINTER(C.c_uint64)))
    if rc != 0:
        raise ValueError(f"pfg_generate failed ({rc})")
    return Cnf(int(mv.value), lits, off)


def random_ksat(num_vars: int, num_clauses: int, k: int = 3, seed: int = 1) -> Cnf:
    return generate(FAMILY_KSAT, num_vars, num_clauses, k, seed)


def tseitin(gates: int, inputs: int, outputs: int, seed: int = 1) -> Cnf:
    return generate(FAMILY_TSEITIN, gates, inputs, outputs, seed)


def scale_free(num_vars: int, num_clauses: int, seed: int = 1, planted: bool = False) -> Cnf:
    """Scale-free CNF; `planted` keeps it satisfiable with a hidden model."""
    return generate(FAMILY_SCALEFREE, num_vars, num_clauses, 1 if planted else 0, seed)


def write_dimacs(cnf: Cnf, path: str, extra_units: Iterable[int] = ()) -> None:
    """DIMACS text of `cnf` (clause order kept), then `extra_units` as unit
    clauses. The literals and 0 terminators are laid out in one array first,
    so the text is formatted in one pass."""
    units = list(extra_units)
    lits = np.asarray(cnf.lits, dtype=np.int64)
    ints = np.where(lits & 1, -(lits >> 1), lits >> 1)
    n = cnf.num_clauses
    lens = np.diff(np.asarray(cnf.off, dtype=np.int64))
    words = np.zeros(len(ints) + n, dtype=np.int64)
    words[np.arange(len(ints)) + np.repeat(np.arange(n), lens)] = ints
    with open(path, "w") as f:
        f.write(f"p cnf {cnf.max_var} {n + len(units)}\n")
        if n:
            f.write(" ".join(map(str, words.tolist())).replace(" 0 ", " 0\n") + "\n")
        for u in units:
            f.write(f"{u} 0\n")


def parse_dimacs(path: str):
    """Native DIMACS ingest (pfg_dimacs_read): returns (cnf, units, status).

    Clauses are normalised as the reference's parser does (repeated literals
    and tautologies dropped, earlier unit clauses applied); one-literal clauses
    come back in `units` (literals 2v|s) and `status` is 20 when the formula
    has an empty clause."""
    import ctypes as C
    from . import _abi, _lib
    L = _lib.lib()
    h = C.c_void_p()
    rc = L.pfg_dimacs_read(os.fsencode(path), C.byref(h))
    try:
        if rc != 0:
            msg = L.pfg_dimacs_error(h)
            raise ValueError(f"{path}: {msg.decode() if msg else 'parse error'}")
        info = _abi.PfgDimacsInfo()
        L.pfg_dimacs_get_info(h, C.byref(info))
        lits = np.empty(info.num_literals, dtype=np.uint32)
        off = np.empty(info.num_clauses + 1, dtype=np.uint64)
        units = np.empty(info.num_units, dtype=np.uint32)
        L.pfg_dimacs_copy(h, lits.ctypes.data_as(C.POINTER(C.c_uint32)), off.ctypes.data_as(C.POINTER(C.c_uint64)),
                          units.ctypes.data_as(C.POINTER(C.c_uint32)))
        return Cnf(info.max_var, lits, off), units, int(info.status)
    finally:
        L.pfg_dimacs_free(h)


def read_dimacs(path: str) -> Cnf:
    max_var = 0
    clauses = []
    cur = []
    with open(path) as f:
        for line in f:
            line = line.strip()
            if not line or line[0] in "c%":
                continue
            if line[0] == "p":
                max_var = int(line.split()[2])
                continue
            for tok in line.split():
                x = int(tok)
                if x == 0:
                    clauses.append(cur)
                    cur = []
                else:
                    cur.append(x)
                    max_var = max(max_var, abs(x))
    return Cnf.from_ints(max_var, clauses)
