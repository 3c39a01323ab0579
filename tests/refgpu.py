"""Canonical digests shared by the reference-GPU fixtures and their tests.

The golden fixtures under tests/golden/refgpu hold, for each seeded instance
and option set, what the reference's own GPU simplifier (src/gpu, built by
oracle/ref_gpu_build.py and driven by oracle/refgpu/dump_main.cpp) produced,
as per-field SHA-256 digests of the canonical form plus a few counts:

  status    0 unknown, 10 SAT (no clause left), 20 UNSAT (propagation conflict)
  cnf       clauses sorted lexicographically, literals sorted, with (learnt,
            lbd, usage) — the reference's clause order is an atomic-order
            artifact (src/gpu/cnf.cu:200-236)
  elim      eliminated bytes per variable (MELTING|ADDING|FORCED)
  units     set of literals device propagation assigned
  pending   set of units the last round produced and nothing propagated
  stack     model-reconstruction blocks grouped per witness variable and
            sorted by it; the reference appends blocks through atomics and
            records no round boundaries (model.cuh:29-49, vector.cu:85-90),
            so the fixtures compare the set of per-variable blocks
  rounds    SUB+BVE rounds run (the reference's `phase`)

On a conflict the reference ends the process (killSolver), so only the
status is compared then.
"""
from __future__ import annotations

import hashlib
import struct

import numpy as np

from oracle import pyoracle as po
from parafrost_gb300.cnf import Cnf

FIELDS = ("cnf", "elim", "units", "pending", "stack", "rounds")


def _h(*arrays) -> str:
    h = hashlib.sha256()
    for a in arrays:
        a = np.ascontiguousarray(a)
        h.update(struct.pack("<Q", a.nbytes))
        h.update(a.tobytes())
    return h.hexdigest()[:32]


def input_digest(cnf: Cnf) -> str:
    """Ordered clause list with each clause's literals sorted (clause ids
    follow this order on the device, so it is part of the input)."""
    lits = np.asarray(cnf.lits, dtype=np.uint32).copy()
    off = np.asarray(cnf.off, dtype=np.uint64)
    for i in range(cnf.num_clauses):
        a, b = int(off[i]), int(off[i + 1])
        lits[a:b].sort()
    learnt = np.zeros(cnf.num_clauses, np.uint8) if cnf.learnt is None else np.asarray(cnf.learnt, np.uint8)
    return _h(off, lits, learnt)


def canon(status: int, cnf: Cnf | None, elim, units, pending, stack, rounds: int) -> dict:
    """Per-field digests and counts of one result."""
    d = {"status": int(status)}
    if int(status) == 20:
        return d
    lits, off, learnt, lbd, usage = po.canon_cnf(cnf)
    st = np.asarray(stack, dtype=np.uint32)
    cs = po.canon_stack(st, np.array([len(st)], dtype=np.uint64)) if len(st) else st
    e = np.asarray(elim, dtype=np.uint8)
    d.update({
        "cnf": _h(off, lits, learnt, lbd, usage),
        "elim": _h(e),
        "units": _h(np.unique(np.asarray(units, dtype=np.uint32))),
        "pending": _h(np.unique(np.asarray(pending, dtype=np.uint32))),
        "stack": _h(cs),
        "rounds": int(rounds),
        "n_clauses": int(cnf.num_clauses),
        "n_literals": int(cnf.num_literals),
        "n_eliminated": int(((e & 1) & ~((e >> 2) & 1)).sum()),
        "n_units": int(len(np.unique(np.asarray(units, dtype=np.uint32)))),
        "n_stack": int(len(st)),
    })
    return d


def canon_result(res) -> dict:
    """Canonical digests of an engine SimplifyResult or an oracle result."""
    return canon(res.status, res.cnf, res.eliminated, res.units, res.pending_units, res.stack, len(res.round_ends))


def differences(got: dict, want: dict) -> list:
    if got["status"] != want["status"]:
        return [f"status {got['status']} vs {want['status']}"]
    if got["status"] == 20:
        return []
    out = []
    for k in FIELDS:
        if got[k] != want[k]:
            extra = ""
            if k == "cnf":
                extra = f" ({got['n_clauses']}/{got['n_literals']} vs {want['n_clauses']}/{want['n_literals']})"
            elif k == "elim":
                extra = f" ({got['n_eliminated']} vs {want['n_eliminated']} eliminated)"
            elif k == "stack":
                extra = f" ({got['n_stack']} vs {want['n_stack']} words)"
            elif k == "units":
                extra = f" ({got['n_units']} vs {want['n_units']})"
            out.append(f"{k}{extra}")
    return out


def matches_any(got: dict, outputs: list) -> tuple:
    """(True, i) when `got` equals the i-th reference output, else (False,
    differences from the most frequent one)."""
    for i, o in enumerate(outputs):
        if not differences(got, o["canon"]):
            return True, i
    best = max(outputs, key=lambda o: o["count"])
    return False, differences(got, best["canon"])


def read_dump(path: str, with_results: bool):
    """Parse a file written by oracle/refgpu/dump_main.cpp."""
    with open(path, "rb") as f:
        buf = f.read()
    if buf[:8] != b"PFREFDMP":
        raise ValueError(f"{path}: not a reference dump")
    version, max_var, status = struct.unpack_from("<III", buf, 8)
    p = 20
    out = {"max_var": max_var, "status": status}

    def arr(dtype, n):
        nonlocal p
        a = np.frombuffer(buf, dtype=dtype, count=n, offset=p).copy()
        p += a.nbytes
        return a

    def u64():
        nonlocal p
        v = struct.unpack_from("<Q", buf, p)[0]
        p += 8
        return v

    if p >= len(buf):
        return out
    n = u64()
    nl = u64()
    off = arr(np.uint64, n + 1)
    lits = arr(np.uint32, nl)
    learnt = arr(np.uint8, n)
    lbd = arr(np.uint32, n)
    usage = arr(np.uint8, n)
    out["cnf"] = Cnf(max_var, lits, off, learnt, lbd, usage)
    if with_results:
        out["elim"] = arr(np.uint8, max_var + 1)
        out["units"] = arr(np.uint32, u64())
        out["pending"] = arr(np.uint32, u64())
        out["stack"] = arr(np.uint32, u64())
        out["rounds"] = struct.unpack_from("<I", buf, p)[0]
    return out
