"""Shared helpers of the parity tests: run the CUDA engine and the oracle on
the same input and compare canonical outputs."""
import numpy as np

import parafrost_gb300 as pg
from oracle import pyoracle as po


def canon(res):
    lits, off, learnt, lbd, usage = po.canon_cnf(res.cnf)
    return {
        "lits": lits, "off": off, "learnt": learnt, "lbd": lbd, "usage": usage,
        "eliminated": np.asarray(res.eliminated),
        "units": np.asarray(res.units),
        "pending": np.asarray(res.pending_units),
        "stack": po.canon_stack(res.stack, res.round_ends),
        "rounds": len(res.round_ends),
        "status": int(res.status),
    }


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
