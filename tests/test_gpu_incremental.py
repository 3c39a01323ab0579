"""The incremental path on the GPU engine: every call of an IPASIR-style
session (clauses added over frozen and fresh variables, per-call assumptions)
runs the engine on the prepared inputs, is compared with the oracle on the same
inputs, and the session's models are checked as in the CPU test."""
import pytest

import parafrost_gb300 as pg
from oracle import pyoracle as po
from tests.parity import canon, diff
from tests.test_incremental import run_session

pytestmark = pytest.mark.gpu


def engine_call(opts):
    def call(s, prep):
        o = dict(opts, ve_inprocess=prep.ve_inprocess)
        with pg.Simplifier(**o) as sim:
            res = sim.simplify(prep.cnf, assumed=prep.assumed, vorg=prep.vorg)
        ref = po.simplify(prep.cnf, pg.options_from(**o), assumed=prep.assumed, vorg=prep.vorg)
        d = diff(canon(res), canon(ref))
        assert not d, "; ".join(d)
        return res
    return call


@pytest.mark.parametrize("seed", range(1, 9))
def test_incremental_session_on_the_engine(seed):
    opts = dict(mupos=10, muneg=10, electionsmin=1, bce=bool(seed % 2))
    s, outcomes = run_session(seed, engine_call(opts), **opts)
    assert outcomes


def test_session_simplify_runs_the_engine():
    from parafrost_gb300.incremental import Incremental
    s = Incremental(mupos=10, muneg=10, electionsmin=1)
    for c in pg.random_ksat(120, 400, 3, 5).clauses():
        s.add(c)
    s.freeze(1)
    s.assume(-1)
    res = s.simplify()
    assert res is not None and s.calls == 1 and s.eliminated
    assert 1 not in s.eliminated
