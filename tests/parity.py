"""Shared helpers of the parity tests: run the CUDA engine and the oracle on
the same input and compare canonical outputs."""
import numpy as np

import parafrost_gb300 as pg
from oracle import pyoracle as po


def canon(res):
    """Canonical outputs. Units are sets. When device propagation finds a
    conflict (UNSAT) the reference stops the solver on the spot
    (src/gpu/elimbcp.cu:180, simplify.cu:168): the CNF is left untouched, and
    which units were assigned before the conflict was seen depends on the
    propagation schedule, so forced units are not compared then."""
    lits, off, learnt, lbd, usage = po.canon_cnf(res.cnf)
    unsat = int(res.status) == pg.PFG_UNSAT
    elim = np.asarray(res.eliminated)
    out = {
        "lits": lits, "off": off, "learnt": learnt, "lbd": lbd, "usage": usage,
        "eliminated": (elim & 0x3) if unsat else elim,
        "stack": po.canon_stack(res.stack, res.round_ends),
        "rounds": len(res.round_ends),
        "status": int(res.status),
    }
    if not unsat:
        out["units"] = np.unique(np.asarray(res.units))
        out["pending"] = np.unique(np.asarray(res.pending_units))
    return out


def diff(a, b):
    out = []
    for k in a:
        x, y = a[k], b[k]
        if isinstance(x, np.ndarray):
            if x.shape != y.shape or not np.array_equal(x, y):
                out.append(f"{k}: engine {x.shape} vs oracle {y.shape}")
        elif x != y:
            out.append(f"{k}: engine {x} vs oracle {y}")
    return out


def run_both(cnf, var_state=None, assumed=None, vorg=None, **opts):
    with pg.Simplifier(**opts) as s:
        res = s.simplify(cnf, var_state=var_state, assumed=assumed, vorg=vorg)
    ref = po.simplify(cnf, pg.options_from(**opts), var_state=var_state, assumed=assumed, vorg=vorg)
    return res, ref


def assert_parity(cnf, var_state=None, assumed=None, vorg=None, **opts):
    res, ref = run_both(cnf, var_state, assumed, vorg, **opts)
    d = diff(canon(res), canon(ref))
    assert not d, "engine differs from the oracle: " + "; ".join(d) + f" (oracle rounds {ref.round_stats})"
    return res, ref


def decode_proof(proof: bytes):
    """Binary DRAT lines as (kind, literals) with kind 'a' or 'd' and literals
    in the 2v+s encoding."""
    out, p, n = [], 0, len(proof)
    while p < n:
        kind = chr(proof[p]); p += 1
        lits = []
        while proof[p] != 0:
            v, sh = 0, 0
            while True:
                b = proof[p]; p += 1
                v |= (b & 0x7F) << sh
                sh += 7
                if not b & 0x80:
                    break
            lits.append(v)
        p += 1
        out.append((kind, tuple(lits)))
    return out


def proof_diff(engine: bytes, oracle: bytes) -> str:
    """'' when equal, else the first differing line."""
    if engine == oracle:
        return ""
    a, b = decode_proof(engine), decode_proof(oracle)
    for i, (x, y) in enumerate(zip(a, b)):
        if x != y:
            return f"line {i}: engine {x} vs oracle {y} ({len(a)} vs {len(b)} lines)"
    return f"{len(a)} vs {len(b)} lines"
