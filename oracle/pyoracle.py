"""Python bindings of the oracle (TEST INFRASTRUCTURE ONLY).

Loads oracle/libpfo.so (built by oracle/build.py) and exposes the CPU
restatement of the GPU simplify path, the canonicalizer, model extension and a
small DPLL solver. Only the tests, the smoke check and the benchmark's
CPU-baseline leg use it.
"""
import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

from parafrost_gb300._abi import PfgOptions  # noqa: E402
from parafrost_gb300.cnf import Cnf  # noqa: E402

from . import build as _build  # noqa: E402

u8p = C.POINTER(C.c_uint8)
u32p = C.POINTER(C.c_uint32)
u64p = C.POINTER(C.c_uint64)


class PfoRound(C.Structure):
    _fields_ = [
        ("elected", C.c_uint32), ("mis_rounds", C.c_uint32), ("eliminated", C.c_uint32),
        ("units", C.c_uint32), ("resolvents", C.c_uint32),
        ("clauses_before", C.c_uint64), ("literals_before", C.c_uint64),
        ("clauses_after", C.c_uint64), ("literals_after", C.c_uint64),
    ]


class PfoResult(C.Structure):
    _fields_ = [
        ("status", C.c_int32), ("simpstate", C.c_int32), ("rounds", C.c_int32), ("ere_ran", C.c_int32),
        ("max_var", C.c_uint32),
        ("ncls", C.c_uint64), ("nlits", C.c_uint64),
        ("lits", u32p), ("cls_off", u64p), ("cls_learnt", u8p), ("cls_lbd", u32p), ("cls_usage", u8p),
        ("eliminated", u8p),
        ("nunits", C.c_uint64), ("units", u32p),
        ("npending", C.c_uint64), ("pending", u32p),
        ("nstack", C.c_uint64), ("stack", u32p),
        ("nround_ends", C.c_uint64), ("round_ends", u64p),
        ("nround_stats", C.c_uint64), ("round_stats", C.POINTER(PfoRound)),
        ("nproof", C.c_uint64), ("proof", u8p),
    ]


_L = None


def lib():
    global _L
    if _L is None:
        path = _build.build()
        L = C.CDLL(path)
        L.pfo_simplify.argtypes = [C.POINTER(PfgOptions), C.c_uint32, C.c_uint64, u32p, u64p, u8p, u32p, u8p,
                                   u8p, u8p, u32p, C.POINTER(C.POINTER(PfoResult))]
        L.pfo_simplify.restype = C.c_int
        L.pfo_free.argtypes = [C.POINTER(PfoResult)]
        L.pfo_canon_cnf.argtypes = [C.c_uint64, u32p, u64p, u8p, u32p, u8p, u32p, u64p, u8p, u32p, u8p]
        L.pfo_canon_cnf.restype = C.c_int
        L.pfo_canon_stack.argtypes = [C.c_uint64, u32p, C.c_uint64, u64p, u32p]
        L.pfo_canon_stack.restype = C.c_int
        L.pfo_extend_model.argtypes = [C.c_uint64, u32p, u8p]
        L.pfo_extend_model.restype = None
        L.pfo_solve.argtypes = [C.c_uint32, C.c_uint64, u32p, u64p, u8p, C.c_uint64]
        L.pfo_solve.restype = C.c_int
        L.pfo_check_rup.argtypes = [C.c_uint32, C.c_uint64, u32p, u64p, u8p, C.c_uint64, u64p]
        L.pfo_check_rup.restype = C.c_int64
        _L = L
    return _L


def _p(a, t):
    return None if a is None else a.ctypes.data_as(C.POINTER(t))


def _arr(ptr, n, dtype):
    if n == 0:
        return np.empty(0, dtype=dtype)
    return np.ctypeslib.as_array(ptr, shape=(int(n),)).astype(dtype, copy=True)


class OracleResult:
    def __init__(self, r: PfoResult):
        self.status = r.status
        self.simpstate = r.simpstate
        self.rounds = r.rounds
        self.ere_ran = r.ere_ran
        V = r.max_var
        self.cnf = Cnf(V, _arr(r.lits, r.nlits, np.uint32), _arr(r.cls_off, r.ncls + 1, np.uint64),
                       _arr(r.cls_learnt, r.ncls, np.uint8), _arr(r.cls_lbd, r.ncls, np.uint32),
                       _arr(r.cls_usage, r.ncls, np.uint8))
        self.eliminated = _arr(r.eliminated, V + 1, np.uint8)
        self.units = _arr(r.units, r.nunits, np.uint32)
        self.pending_units = _arr(r.pending, r.npending, np.uint32)
        self.stack = _arr(r.stack, r.nstack, np.uint32)
        self.round_ends = _arr(r.round_ends, r.nround_ends, np.uint64)
        self.round_stats = [{f[0]: getattr(r.round_stats[i], f[0]) for f in PfoRound._fields_}
                            for i in range(r.nround_stats)]
        self.proof = bytes(_arr(r.proof, r.nproof, np.uint8))


def simplify(cnf: Cnf, opts: PfgOptions, var_state=None, assumed=None, vorg=None) -> OracleResult:
    L = lib()
    out = C.POINTER(PfoResult)()
    vs = None if var_state is None else np.ascontiguousarray(var_state, dtype=np.uint8)
    asd = None if assumed is None else np.ascontiguousarray(assumed, dtype=np.uint8)
    vo = None if vorg is None else np.ascontiguousarray(vorg, dtype=np.uint32)
    rc = L.pfo_simplify(C.byref(opts), cnf.max_var, cnf.num_clauses, _p(cnf.lits, C.c_uint32),
                        _p(cnf.off, C.c_uint64), _p(cnf.learnt, C.c_uint8), _p(cnf.lbd, C.c_uint32),
                        _p(cnf.usage, C.c_uint8), _p(vs, C.c_uint8), _p(asd, C.c_uint8), _p(vo, C.c_uint32),
                        C.byref(out))
    if rc != 0:
        raise ValueError(f"pfo_simplify failed ({rc})")
    try:
        return OracleResult(out.contents)
    finally:
        L.pfo_free(out)


def canon_cnf(cnf: Cnf):
    """Canonical (sorted) clause list: returns (lits, off, learnt, lbd, usage)."""
    L = lib()
    n = cnf.num_clauses
    ol = np.empty(max(cnf.num_literals, 1), dtype=np.uint32)
    oo = np.empty(n + 1, dtype=np.uint64)
    olr = np.empty(max(n, 1), dtype=np.uint8)
    olb = np.empty(max(n, 1), dtype=np.uint32)
    ous = np.empty(max(n, 1), dtype=np.uint8)
    L.pfo_canon_cnf(n, _p(cnf.lits, C.c_uint32), _p(cnf.off, C.c_uint64), _p(cnf.learnt, C.c_uint8),
                    _p(cnf.lbd, C.c_uint32), _p(cnf.usage, C.c_uint8), _p(ol, C.c_uint32), _p(oo, C.c_uint64),
                    _p(olr, C.c_uint8), _p(olb, C.c_uint32), _p(ous, C.c_uint8))
    nl = cnf.num_literals
    return ol[:nl], oo, olr[:n], olb[:n], ous[:n]


def canon_stack(stack: np.ndarray, round_ends: np.ndarray) -> np.ndarray:
    L = lib()
    st = np.ascontiguousarray(stack, dtype=np.uint32)
    re = np.ascontiguousarray(round_ends, dtype=np.uint64)
    out = np.empty(max(len(st), 1), dtype=np.uint32)
    rc = L.pfo_canon_stack(len(st), _p(st, C.c_uint32), len(re), _p(re, C.c_uint64), _p(out, C.c_uint32))
    if rc != 0:
        raise ValueError(f"malformed model stack ({rc})")
    return out[:len(st)]


def extend_model(stack: np.ndarray, value: np.ndarray) -> np.ndarray:
    L = lib()
    st = np.ascontiguousarray(stack, dtype=np.uint32)
    v = np.ascontiguousarray(value, dtype=np.uint8).copy()
    L.pfo_extend_model(len(st), _p(st, C.c_uint32), _p(v, C.c_uint8))
    return v


def solve(cnf: Cnf, max_decisions: int = 10_000_000):
    """Returns (status, model) with status 10/20/0 and model uint8[max_var+1]."""
    L = lib()
    model = np.zeros(cnf.max_var + 1, dtype=np.uint8)
    rc = L.pfo_solve(cnf.max_var, cnf.num_clauses, _p(cnf.lits, C.c_uint32), _p(cnf.off, C.c_uint64),
                     _p(model, C.c_uint8), max_decisions)
    return rc, model


def check_rup(cnf: Cnf, proof: bytes):
    """RUP-check a binary DRAT proof against `cnf`: returns (first failing
    line or 0, deletions of absent clauses)."""
    L = lib()
    pb = np.frombuffer(proof, dtype=np.uint8) if proof else np.zeros(1, dtype=np.uint8)
    pb = np.ascontiguousarray(pb)
    missing = C.c_uint64(0)
    bad = L.pfo_check_rup(cnf.max_var, cnf.num_clauses, _p(cnf.lits, C.c_uint32), _p(cnf.off, C.c_uint64),
                          _p(pb, C.c_uint8), len(proof), C.byref(missing))
    return int(bad), int(missing.value)


def satisfies(cnf: Cnf, value: np.ndarray) -> bool:
    """value[v] in {0,1} for every variable: does it satisfy every clause?"""
    lits = cnf.lits.astype(np.int64)
    v = value[lits >> 1].astype(bool)
    sat_lit = np.where(lits & 1, ~v, v)
    if cnf.num_clauses == 0:
        return True
    cls_idx = np.repeat(np.arange(cnf.num_clauses), np.diff(cnf.off).astype(np.int64))
    sat = np.zeros(cnf.num_clauses, dtype=bool)
    np.logical_or.at(sat, cls_idx, sat_lit)
    return bool(sat.all())
