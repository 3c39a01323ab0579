"""Serving: simplification jobs submitted over time to a native request loop.

`Server` wraps the pfg_server_* entry points of include/pfgpu.h: jobs are
copied at submit, admitted in arrival order while their estimated device
footprint fits the arena budget, and run as batches on `slots` concurrent
workers (one engine context and stream each). Every job's result is the one
the instance gives alone.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import Optional

import numpy as np

from . import _abi, _lib
from .cnf import Cnf
from .simplifier import SimplifyError, SimplifyResult, _addr, _ptr


@dataclass
class JobInfo:
    ticket: int
    rc: int
    status: int
    batch_size: int
    slot: int
    est_bytes: int
    latency_s: float          # done - submit
    queue_s: float            # admit - submit
    clauses_processed: int
    t_submit_ns: int
    t_admit_ns: int
    t_done_ns: int


class Server:
    def __init__(self, arena_bytes: int = 0, slots: int = 2, max_batch: int = 256, **options):
        self.lib = _lib.lib()
        self.options = _abi.options_from(**options)
        self._srv = C.c_void_p()
        rc = self.lib.pfg_server_create(C.byref(self._srv), C.byref(self.options), arena_bytes, slots, max_batch)
        if rc != 0:
            raise SimplifyError(rc, "pfg_server_create failed")
        self._info = {}

    def submit(self, cnf: Cnf, var_state=None, assumed=None, vorg=None) -> int:
        keep = []

        def arr(a, dtype):
            if a is None:
                return None
            a = np.ascontiguousarray(a, dtype=dtype)
            keep.append(a)
            return a

        q = _abi.PfgInstance()
        q.max_var = cnf.max_var
        q.num_clauses = cnf.num_clauses
        q.lits = _addr(cnf.lits)
        q.cls_off = _addr(cnf.off)
        q.cls_learnt = _addr(cnf.learnt)
        q.cls_lbd = _addr(cnf.lbd)
        q.cls_usage = _addr(cnf.usage)
        q.var_state = _addr(arr(var_state, np.uint8))
        q.assumed = _addr(arr(assumed, np.uint8))
        q.vorg = _addr(arr(vorg, np.uint32))
        t = C.c_uint64()
        rc = self.lib.pfg_server_submit(self._srv, C.byref(q), C.byref(t))
        if rc != 0:
            msg = self.lib.pfg_server_last_error(self._srv)
            raise SimplifyError(rc, "pfg_server_submit: " + (msg.decode() if msg else ""))
        return int(t.value)

    def poll(self, ticket: int, wait_ms: int = 0) -> Optional[JobInfo]:
        info = _abi.PfgJobInfo()
        rc = self.lib.pfg_server_poll(self._srv, ticket, int(wait_ms), C.byref(info))
        if rc == _abi.PFG_PENDING:
            return None
        if rc != 0:
            raise SimplifyError(rc, f"pfg_server_poll({ticket})")
        self._info[ticket] = info
        return JobInfo(ticket, info.rc, info.status, info.batch_size, info.slot, info.est_bytes,
                       (info.t_done_ns - info.t_submit_ns) * 1e-9, (info.t_admit_ns - info.t_submit_ns) * 1e-9,
                       info.clauses_processed, info.t_submit_ns, info.t_admit_ns, info.t_done_ns)

    def wait(self, ticket: int, timeout_s: float = 600.0) -> JobInfo:
        waited = 0.0
        while True:
            j = self.poll(ticket, 200)
            if j is not None:
                return j
            waited += 0.2
            if waited > timeout_s:
                raise TimeoutError(f"job {ticket} not done after {timeout_s} s")

    def fetch(self, ticket: int) -> SimplifyResult:
        info = self._info.pop(ticket, None)
        if info is None:
            self.wait(ticket)
            info = self._info.pop(ticket)
        sz = info.sizes
        lits = np.empty(sz.literals, dtype=np.uint32)
        off = np.empty(sz.clauses + 1, dtype=np.uint64)
        learnt = np.empty(sz.clauses, dtype=np.uint8)
        lbd = np.empty(sz.clauses, dtype=np.uint32)
        usage = np.empty(sz.clauses, dtype=np.uint8)
        elim = np.empty(sz.max_var + 1, dtype=np.uint8)
        units = np.empty(sz.units, dtype=np.uint32)
        pend = np.empty(sz.pending_units, dtype=np.uint32)
        stack = np.empty(sz.stack_words, dtype=np.uint32)
        rends = np.empty(sz.rounds, dtype=np.uint64)
        proof = b""
        if sz.proof_bytes:       # before the fetch, which forgets the job
            pb = np.empty(sz.proof_bytes, dtype=np.uint8)
            rc = self.lib.pfg_server_fetch_proof(self._srv, ticket, _ptr(pb, C.c_uint8))
            if rc != 0:
                raise SimplifyError(rc, f"pfg_server_fetch_proof({ticket})")
            proof = pb.tobytes()
        rc = self.lib.pfg_server_fetch(self._srv, ticket, _ptr(lits, C.c_uint32), _ptr(off, C.c_uint64),
                                       _ptr(learnt, C.c_uint8), _ptr(lbd, C.c_uint32), _ptr(usage, C.c_uint8),
                                       _ptr(elim, C.c_uint8), _ptr(units, C.c_uint32), _ptr(pend, C.c_uint32),
                                       _ptr(stack, C.c_uint32), _ptr(rends, C.c_uint64))
        if rc != 0:
            raise SimplifyError(rc, f"pfg_server_fetch({ticket})")
        stats = {"clauses_processed": info.clauses_processed, "batch_size": info.batch_size, "slot": info.slot}
        return SimplifyResult(int(info.status), Cnf(sz.max_var, lits, off, learnt, lbd, usage), elim, units, pend,
                              stack, rends, stats, proof)

    def stats(self) -> dict:
        st = _abi.PfgServerStats()
        self.lib.pfg_server_stats_get(self._srv, C.byref(st))
        return {f[0]: int(getattr(st, f[0])) for f in _abi.PfgServerStats._fields_}

    def close(self) -> None:
        if self._srv:
            self.lib.pfg_server_destroy(self._srv)
            self._srv = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
