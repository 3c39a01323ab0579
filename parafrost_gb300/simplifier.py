"""Host-side mirror of ParaFROST's GPU simplify entry point.

`Simplifier.simplify(cnf)` does what `Solver::simplify` (src/gpu/simplify.cu:57)
does for one clause database: upload (awaken, simplify.cu:77-134), run the
simplification rounds until the reference's stop rule (simplify.cu:163-186),
and return the simplified CNF, the eliminated-variable bytes, the units fixed
by device propagation and the model-reconstruction stack (simplify.cu:190-240).
Options use the reference's CLI names (`phases`, `electionsmax`, `ere`, ...).

Every call goes through the C ABI of include/pfgpu.h into the CUDA engine.
"""
from __future__ import annotations

import ctypes as C
import threading
from concurrent.futures import ThreadPoolExecutor
from dataclasses import dataclass, field
from typing import Optional

import numpy as np

from . import _abi, _lib
from .cnf import Cnf


class SimplifyError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(f"{_abi.RETURN_NAMES.get(code, code)}: {message}")
        self.code = code


def _ptr(a, t):
    return None if a is None else a.ctypes.data_as(C.POINTER(t))


def _addr(a):
    """Address of a contiguous numpy array (or None), for PfgInstance fields."""
    return None if a is None else a.ctypes.data


@dataclass
class SimplifyResult:
    status: int                      # 0 unknown, 10 SAT (no clause left), 20 UNSAT
    cnf: Cnf                         # simplified clause database (clause order kept)
    eliminated: np.ndarray           # uint8[max_var+1]: MELTING 1 | ADDING 2 | FORCED 4
    units: np.ndarray                # literals fixed by device propagation (sorted)
    pending_units: np.ndarray        # units of the last round not yet propagated (sorted)
    stack: np.ndarray                # model-reconstruction words
    round_ends: np.ndarray           # stack length after each SUB+BVE round
    stats: dict = field(default_factory=dict)
    proof: bytes = b""               # binary DRAT lines of the passes (proof=True)

    def eliminated_vars(self) -> np.ndarray:
        e = self.eliminated
        return np.nonzero((e & 1) & ~((e >> 2) & 1))[0].astype(np.uint32)


def split_runs(sizes, k: int) -> list:
    """k runs [b, e) of consecutive indices covering `sizes`, cut where the
    running total passes j/k of the sum; every run holds at least one index."""
    n = len(sizes)
    k = max(1, min(int(k), n))
    total = float(sum(sizes)) or 1.0
    cuts, acc, j = [0], 0.0, 1
    for i, sz in enumerate(sizes):
        acc += sz
        while j < k and acc >= total * j / k and i + 1 - cuts[-1] >= 1 and n - (i + 1) >= k - j:
            cuts.append(i + 1)
            j += 1
    while len(cuts) < k:          # too few cuts: split the tail one index at a time
        cuts.append(n - (k - len(cuts)))
    cuts.append(n)
    return [(cuts[i], cuts[i + 1]) for i in range(k)]


class Simplifier:
    """One device context (a `pfg_ctx`): one instance, or a batch of instances
    simplified together with per-instance results."""

    def __init__(self, arena_bytes: int = 0, **options):
        self.lib = _lib.lib()
        self.options = _abi.options_from(**options)
        self._ctx = C.c_void_p()
        self._arena_bytes = arena_bytes
        self._pool = None          # host threads of simplify_batch(streams > 1)
        self._peer_ctx = []        # its other contexts
        rc = self.lib.pfg_create(C.byref(self._ctx), C.byref(self.options), arena_bytes)
        if rc != 0:
            raise SimplifyError(rc, "pfg_create failed (is a CUDA device visible?)")
        self.last_stats: Optional[_abi.PfgStats] = None

    def _check(self, rc: int, what: str):
        if rc != 0:
            msg = self.lib.pfg_last_error(self._ctx)
            raise SimplifyError(rc, f"{what}: {msg.decode() if msg else ''}")

    def upload(self, cnf: Cnf, var_state: Optional[np.ndarray] = None, assumed: Optional[np.ndarray] = None,
               vorg: Optional[np.ndarray] = None) -> None:
        vs = None if var_state is None else np.ascontiguousarray(var_state, dtype=np.uint8)
        asd = None if assumed is None else np.ascontiguousarray(assumed, dtype=np.uint8)
        vo = None if vorg is None else np.ascontiguousarray(vorg, dtype=np.uint32)
        rc = self.lib.pfg_upload(self._ctx, cnf.max_var, cnf.num_clauses, _ptr(cnf.lits, C.c_uint32),
                                 _ptr(cnf.off, C.c_uint64), _ptr(cnf.learnt, C.c_uint8), _ptr(cnf.lbd, C.c_uint32),
                                 _ptr(cnf.usage, C.c_uint8), _ptr(vs, C.c_uint8), _ptr(asd, C.c_uint8),
                                 _ptr(vo, C.c_uint32))
        self._check(rc, "pfg_upload")

    def run(self) -> _abi.PfgStats:
        st = _abi.PfgStats()
        rc = self.lib.pfg_simplify(self._ctx, C.byref(st))
        self.last_stats = st
        self._check(rc, "pfg_simplify")
        return st

    def download(self, into=None) -> SimplifyResult:
        """Results of a one-instance context. `into`: a pinned.ResultBuffers to
        download into (page-locked, reused across calls; the result's arrays
        are views into it, valid until the next download into it)."""
        sz = _abi.PfgResultSizes()
        self._check(self.lib.pfg_result_sizes_get(self._ctx, C.byref(sz)), "pfg_result_sizes_get")
        alloc = (lambda name, k, dt: np.empty(k, dtype=dt)) if into is None else \
            (lambda name, k, dt: into.get(name, k))
        lits = alloc("lits", sz.literals, np.uint32)
        off = alloc("off", sz.clauses + 1, np.uint64)
        learnt = alloc("learnt", sz.clauses, np.uint8)
        lbd = alloc("lbd", sz.clauses, np.uint32)
        usage = alloc("usage", sz.clauses, np.uint8)
        elim = alloc("elim", sz.max_var + 1, np.uint8)
        units = alloc("units", sz.units, np.uint32)
        pend = alloc("pend", sz.pending_units, np.uint32)
        stack = alloc("stack", sz.stack_words, np.uint32)
        rends = alloc("rends", sz.rounds, np.uint64)
        rc = self.lib.pfg_download(self._ctx, _ptr(lits, C.c_uint32), _ptr(off, C.c_uint64), _ptr(learnt, C.c_uint8),
                                   _ptr(lbd, C.c_uint32), _ptr(usage, C.c_uint8), _ptr(elim, C.c_uint8),
                                   _ptr(units, C.c_uint32), _ptr(pend, C.c_uint32), _ptr(stack, C.c_uint32),
                                   _ptr(rends, C.c_uint64))
        self._check(rc, "pfg_download")
        proof = np.empty(max(sz.proof_bytes, 1), dtype=np.uint8)
        self._check(self.lib.pfg_download_proof(self._ctx, _ptr(proof, C.c_uint8)), "pfg_download_proof")
        st = self.last_stats
        stats = {}
        if st is not None:
            stats = {f[0]: getattr(st, f[0]) for f in _abi.PfgStats._fields_ if f[0] != "pass_ms"}
            stats["pass_ms"] = dict(zip(_abi.PASS_NAMES, list(st.pass_ms)))
        return SimplifyResult(int(st.status) if st is not None else 0,
                              Cnf(sz.max_var, lits, off, learnt, lbd, usage), elim, units, pend, stack, rends, stats,
                              proof[:sz.proof_bytes].tobytes())

    def simplify(self, cnf: Cnf, var_state=None, assumed=None, vorg=None, into=None) -> SimplifyResult:
        self.upload(cnf, var_state, assumed, vorg)
        self.run()
        return self.download(into)

    # ---- batches: n instances simplified together, results per instance ----

    def upload_batch(self, cnfs, var_states=None, assumeds=None, vorgs=None) -> None:
        arr, keep = self._instances(cnfs, var_states, assumeds, vorgs)
        self._check(self.lib.pfg_batch_upload(self._ctx, len(cnfs), arr), "pfg_batch_upload")

    @staticmethod
    def _instances(cnfs, var_states=None, assumeds=None, vorgs=None):
        """The pfg_instance array of `cnfs` and the arrays it points into (keep
        both alive across the call)."""
        n = len(cnfs)
        arr = (_abi.PfgInstance * max(n, 1))()
        keep = []   # the arrays must outlive the call

        def opt(seq, i, dtype):
            if seq is None or seq[i] is None:
                return None
            a = np.ascontiguousarray(seq[i], dtype=dtype)
            keep.append(a)
            return a

        for i, cnf in enumerate(cnfs):
            q = arr[i]
            q.max_var = cnf.max_var
            q.num_clauses = cnf.num_clauses
            q.lits = _addr(cnf.lits)
            q.cls_off = _addr(cnf.off)
            q.cls_learnt = _addr(cnf.learnt)
            q.cls_lbd = _addr(cnf.lbd)
            q.cls_usage = _addr(cnf.usage)
            q.var_state = _addr(opt(var_states, i, np.uint8))
            q.assumed = _addr(opt(assumeds, i, np.uint8))
            q.vorg = _addr(opt(vorgs, i, np.uint32))
        return arr, keep

    # ---- launch shapes (pfg_tuning) ----

    @property
    def tuning(self) -> dict:
        """Launch shapes per pass (pfg_tuning); 0 is the built-in choice.
        Assigning a dict sets every field: the ones it leaves out go back to 0."""
        t = _abi.PfgTuning()
        self._check(self.lib.pfg_tuning_get(self._ctx, C.byref(t)), "pfg_tuning_get")
        return {f[0]: getattr(t, f[0]) for f in _abi.PfgTuning._fields_ if not f[0].startswith("_")}

    @tuning.setter
    def tuning(self, values: dict) -> None:
        t = _abi.PfgTuning()
        for k, v in values.items():
            if k.startswith("_") or not any(f[0] == k for f in _abi.PfgTuning._fields_):
                raise KeyError(f"unknown tuning field {k!r}")
            setattr(t, k, int(v))
        self._check(self.lib.pfg_tuning_set(self._ctx, C.byref(t)), "pfg_tuning_set")

    def autotune(self, cnfs, repeats: int = 1) -> dict:
        """Measure the launch shapes on `cnfs` (pfg_autotune) and keep the best;
        returns them. Upload again before the next simplify."""
        arr, keep = self._instances(cnfs)
        t = _abi.PfgTuning()
        self._check(self.lib.pfg_autotune(self._ctx, len(cnfs), arr, int(repeats), C.byref(t)), "pfg_autotune")
        return {f[0]: getattr(t, f[0]) for f in _abi.PfgTuning._fields_ if not f[0].startswith("_")}

    def batch_size(self) -> int:
        return int(self.lib.pfg_batch_size(self._ctx))

    def download_instance(self, i: int) -> SimplifyResult:
        sz = _abi.PfgResultSizes()
        self._check(self.lib.pfg_batch_result_sizes(self._ctx, i, C.byref(sz)), "pfg_batch_result_sizes")
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
        rc = self.lib.pfg_batch_download(self._ctx, i, _ptr(lits, C.c_uint32), _ptr(off, C.c_uint64),
                                         _ptr(learnt, C.c_uint8), _ptr(lbd, C.c_uint32), _ptr(usage, C.c_uint8),
                                         _ptr(elim, C.c_uint8), _ptr(units, C.c_uint32), _ptr(pend, C.c_uint32),
                                         _ptr(stack, C.c_uint32), _ptr(rends, C.c_uint64))
        self._check(rc, "pfg_batch_download")
        proof = self._proof_of(i, sz.proof_bytes)
        st = _abi.PfgStats()
        self._check(self.lib.pfg_batch_stats(self._ctx, i, C.byref(st)), "pfg_batch_stats")
        stats = {f[0]: getattr(st, f[0]) for f in _abi.PfgStats._fields_ if f[0] != "pass_ms"}
        return SimplifyResult(int(st.status), Cnf(sz.max_var, lits, off, learnt, lbd, usage), elim, units, pend,
                              stack, rends, stats, proof)

    def _proof_of(self, i: int, nbytes: int) -> bytes:
        if not nbytes:
            return b""
        buf = np.empty(nbytes, dtype=np.uint8)
        self._check(self.lib.pfg_batch_download_proof(self._ctx, i, _ptr(buf, C.c_uint8)), "pfg_batch_download_proof")
        return buf.tobytes()

    def download_all(self, into=None) -> list:
        """Results of every instance of the batch, one copy per output array
        (each instance's arrays are views into them). `into`: a
        pinned.ResultBuffers to download into (page-locked, reused across calls)."""
        n = self.batch_size()
        sizes = (_abi.PfgResultSizes * max(n, 1))()
        self._check(self.lib.pfg_batch_result_sizes_all(self._ctx, sizes), "pfg_batch_result_sizes_all")
        f = lambda name: np.array([getattr(sizes[i], name) for i in range(n)], dtype=np.int64)
        ncls, nlit, nvar = f("clauses"), f("literals"), f("max_var")
        nun, npend, nstk, nrnd = f("units"), f("pending_units"), f("stack_words"), f("rounds")
        alloc = (lambda name, k, dt: np.empty(k, dtype=dt)) if into is None else \
            (lambda name, k, dt: into.get(name, k))
        lits = alloc("lits", int(nlit.sum()), np.uint32)
        off = alloc("off", int((ncls + 1).sum()), np.uint64)
        learnt = alloc("learnt", int(ncls.sum()), np.uint8)
        lbd = alloc("lbd", int(ncls.sum()), np.uint32)
        usage = alloc("usage", int(ncls.sum()), np.uint8)
        elim = alloc("elim", int((nvar + 1).sum()), np.uint8)
        units = alloc("units", int(nun.sum()), np.uint32)
        pend = alloc("pend", int(npend.sum()), np.uint32)
        stack = alloc("stack", int(nstk.sum()), np.uint32)
        rends = alloc("rends", int(nrnd.sum()), np.uint64)
        rc = self.lib.pfg_batch_download_all(self._ctx, _ptr(lits, C.c_uint32), _ptr(off, C.c_uint64),
                                             _ptr(learnt, C.c_uint8), _ptr(lbd, C.c_uint32), _ptr(usage, C.c_uint8),
                                             _ptr(elim, C.c_uint8), _ptr(units, C.c_uint32), _ptr(pend, C.c_uint32),
                                             _ptr(stack, C.c_uint32), _ptr(rends, C.c_uint64))
        self._check(rc, "pfg_batch_download_all")

        def starts(counts):
            return np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)

        sl, so, sc, se = starts(nlit), starts(ncls + 1), starts(ncls), starts(nvar + 1)
        su, sp, ss, sr = starts(nun), starts(npend), starts(nstk), starts(nrnd)
        out = []
        for i in range(n):
            st = _abi.PfgStats()
            self._check(self.lib.pfg_batch_stats(self._ctx, i, C.byref(st)), "pfg_batch_stats")
            stats = {k[0]: getattr(st, k[0]) for k in _abi.PfgStats._fields_ if k[0] != "pass_ms"}
            cnf = Cnf(int(nvar[i]), lits[sl[i]:sl[i + 1]], off[so[i]:so[i + 1]], learnt[sc[i]:sc[i + 1]],
                      lbd[sc[i]:sc[i + 1]], usage[sc[i]:sc[i + 1]])
            out.append(SimplifyResult(int(st.status), cnf, elim[se[i]:se[i + 1]], units[su[i]:su[i + 1]],
                                      pend[sp[i]:sp[i + 1]], stack[ss[i]:ss[i + 1]], rends[sr[i]:sr[i + 1]], stats,
                                      self._proof_of(i, int(sizes[i].proof_bytes))))
        return out

    def simplify_batch(self, cnfs, var_states=None, assumeds=None, vorgs=None, into=None, streams: int = 1) -> list:
        """Simplify every CNF of `cnfs` in one device store; one result per
        instance (views into `into`, a pinned.ResultBuffers, when given).

        streams > 1 splits the batch into that many runs of consecutive
        instances with about equal clause counts, each simplified by its own
        context (same options and launch shapes) on its own stream from its
        own host thread, so one run's host copies overlap another's kernels
        (the runs are uploaded one after another: the first computes while the
        next ones are copied up).
        Instances are independent, so the results are the ones of one batch.
        `into` is then a list of pinned.ResultBuffers, one per run."""
        streams = max(1, min(int(streams), len(cnfs) // 2))
        if streams == 1:
            if isinstance(into, (list, tuple)):
                into = into[0]
            self.upload_batch(cnfs, var_states, assumeds, vorgs)
            self.run()
            return self.download_all(into)
        runs = split_runs([c.num_clauses for c in cnfs], streams)
        sims = [self] + self.peers(streams - 1)
        bufs = list(into) if isinstance(into, (list, tuple)) else [into] + [None] * (streams - 1)
        if len(bufs) < streams:
            raise ValueError(f"`into` holds {len(bufs)} result buffers for {streams} runs")
        pick = lambda seq, b, e: None if seq is None else seq[b:e]
        # the uploads go one after another, so the first run's rounds start while
        # the later runs are still being copied up (together they would all wait
        # for the whole batch to cross the host link)
        uploaded = [threading.Event() for _ in range(streams)]

        def work(j):
            b, e = runs[j]
            sim = sims[j]
            try:
                if j:
                    uploaded[j - 1].wait()
                sim.upload_batch(cnfs[b:e], pick(var_states, b, e), pick(assumeds, b, e), pick(vorgs, b, e))
            finally:
                uploaded[j].set()
            sim.run()
            return sim.download_all(bufs[j])

        if self._pool is None or self._pool._max_workers < streams:
            if self._pool is not None:
                self._pool.shutdown()
            self._pool = ThreadPoolExecutor(streams)
        out = []
        for part in self._pool.map(work, range(streams)):
            out.extend(part)
        return out

    def peers(self, k: int) -> list:
        """k more contexts with this one's options and launch shapes, owned by
        this Simplifier (kept for later calls, closed with it): the other runs
        of simplify_batch(streams=k + 1), or contexts for run_many."""
        while len(self._peer_ctx) < k:
            peer = Simplifier.__new__(Simplifier)
            peer.lib = self.lib
            peer.options = self.options
            peer._ctx = C.c_void_p()
            peer._pool = None
            peer._peer_ctx = []
            peer.last_stats = None
            rc = self.lib.pfg_create(C.byref(peer._ctx), C.byref(peer.options), self._arena_bytes)
            if rc != 0:
                raise SimplifyError(rc, "pfg_create failed")
            self._peer_ctx.append(peer)
        tuning = self.tuning
        for peer in self._peer_ctx[:k]:
            peer.tuning = tuning
        return self._peer_ctx[:k]

    def profile(self, on: bool = True) -> None:
        """Per-kernel CUDA-event timing of the following simplify calls."""
        self.lib.pfg_profile_enable(self._ctx, 1 if on else 0)

    def profile_reset(self) -> None:
        self.lib.pfg_profile_reset(self._ctx)

    def profile_report(self) -> dict:
        """{kernel group: {launches, ms, alg_bytes}} accumulated since the last reset."""
        out = {}
        for i in range(self.lib.pfg_profile_count()):
            n = C.c_uint64()
            ms = C.c_double()
            b = C.c_uint64()
            self.lib.pfg_profile_get(self._ctx, i, C.byref(n), C.byref(ms), C.byref(b))
            out[self.lib.pfg_profile_name(i).decode()] = {"launches": n.value, "ms": ms.value, "alg_bytes": b.value}
        return out

    def set_loop_limits(self, max_bcp_levels: int = 0, max_mis_rounds: int = 0) -> None:
        """Bounds of the device propagation levels and MIS rounds of a simplify
        call (pfg_set_loop_limits); beyond one the call raises SimplifyError
        with code PFG_TIMEOUT. 0 keeps the built-in bound."""
        self._check(self.lib.pfg_set_loop_limits(self._ctx, int(max_bcp_levels), int(max_mis_rounds)),
                    "pfg_set_loop_limits")

    def kernel_launches(self) -> int:
        return int(self.lib.pfg_kernel_launches(self._ctx))

    def close(self) -> None:
        if getattr(self, "_pool", None) is not None:
            self._pool.shutdown()
            self._pool = None
        for peer in getattr(self, "_peer_ctx", []):
            peer.close()
        self._peer_ctx = []
        if self._ctx:
            self.lib.pfg_destroy(self._ctx)
            self._ctx = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def run_many(sims) -> tuple:
    """pfg_simplify_many over uploaded Simplifiers (distinct contexts): each
    one's rounds on its own stream and host thread at once. Returns their
    stats and the device time of the whole job in ms."""
    sims = list(sims)
    if not sims:
        raise ValueError("no contexts")
    lib = sims[0].lib
    ctxs = (C.c_void_p * len(sims))(*[s._ctx.value for s in sims])
    stats = (_abi.PfgStats * len(sims))()
    ms = C.c_float(0)
    rc = lib.pfg_simplify_many(ctxs, len(sims), stats, C.byref(ms))
    for s, st in zip(sims, stats):
        s.last_stats = st
    if rc != 0:
        msgs = [lib.pfg_last_error(s._ctx) for s in sims]
        raise SimplifyError(rc, "pfg_simplify_many: " + "; ".join(m.decode() for m in msgs if m))
    return list(stats), float(ms.value)


def simplify(cnf: Cnf, **options) -> SimplifyResult:
    with Simplifier(**options) as s:
        return s.simplify(cnf)


def simplify_batch(cnfs, **options) -> list:
    with Simplifier(**options) as s:
        return s.simplify_batch(cnfs)


def proof_text(proof: bytes) -> str:
    """Text form of a binary DRAT proof ("d " before deletions, signed decimal
    literals, "0" at the end of each line), as pfg_proof_text writes it."""
    L = _lib.lib()
    pb = np.frombuffer(proof, dtype=np.uint8) if proof else np.zeros(1, dtype=np.uint8)
    pb = np.ascontiguousarray(pb)
    n = C.c_uint64(0)
    rc = L.pfg_proof_text(_ptr(pb, C.c_uint8), len(proof), None, 0, C.byref(n))
    if rc != 0:
        raise SimplifyError(rc, "malformed proof")
    out = C.create_string_buffer(max(n.value, 1))
    L.pfg_proof_text(_ptr(pb, C.c_uint8), len(proof), out, n.value, C.byref(n))
    return out.raw[:n.value].decode("ascii")
