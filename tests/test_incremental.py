"""The incremental path (IPASIR add / freeze / assume, Solver::isolve): a
session of simplify calls with clauses added between calls over frozen
variables and fresh ones, and per-call assumptions. After every call the
current formula plus the assumptions is solved (the oracle's DPLL), the model
is extended through the session's model stack and checked against every clause
ever added and the assumptions, and SAT/UNSAT is checked against solving all
added clauses with the assumptions directly. CPU side: the calls run the
oracle on the inputs the session prepares."""
import numpy as np
import pytest

import parafrost_gb300 as pg
from oracle import pyoracle as po
from parafrost_gb300.incremental import Incremental


def with_assumptions(cnf, assumptions):
    cls = [cnf.clause(i).tolist() for i in range(cnf.num_clauses)]
    ints = [[pg.lit_to_int(l) for l in c] for c in cls] + [[a] for a in assumptions]
    return pg.Cnf.from_ints(cnf.max_var, ints)


def random_clauses(rng, pool, n, k=3):
    out = []
    for _ in range(n):
        vs = rng.choice(pool, k, replace=False)
        out.append([int(v) if rng.random() < 0.5 else -int(v) for v in vs])
    return out


def run_session(seed, call, calls=4, **opts):
    """`call(session, prep)` performs one call and returns the result."""
    rng = np.random.default_rng(seed)
    V0 = int(rng.integers(60, 140))
    s = Incremental(**opts)
    added = random_clauses(rng, np.arange(1, V0 + 1), int(V0 * rng.uniform(2.5, 3.8)))
    for c in added:
        s.add(c)
    frozen = [int(v) for v in rng.choice(np.arange(1, V0 + 1), max(4, V0 // 6), replace=False)]
    for v in frozen:
        s.freeze(v)
    nxt = V0 + 1
    outcomes = []
    for k in range(calls):
        assumptions = [int(v) if rng.random() < 0.5 else -int(v) for v in rng.choice(frozen, 3, replace=False)]
        for a in assumptions:
            s.assume(a)
        prep = s.prepare()
        if prep is not None:
            res = call(s, prep)
            s.absorb(prep, res)
        else:                      # decided on the host: no device call
            s.calls += 1
            s.assumptions = []
        # the session's formula under the assumptions against everything added
        full = pg.Cnf.from_ints(s.max_var, added)
        want, _ = po.solve(with_assumptions(full, assumptions), 50_000_000)
        if s.unsat:
            assert want == 20
            outcomes.append(20)
            break
        cur = s.formula()
        got, model = po.solve(with_assumptions(cur, assumptions), 50_000_000)
        assert got == want, f"call {k}: session formula {got} vs all clauses {want}"
        if got == 10:
            value = s.extend(model)
            assert po.satisfies(full, value), f"call {k}: extended model violates an added clause"
            for a in assumptions:
                assert value[abs(a)] == (1 if a > 0 else 0)
        outcomes.append(got)
        # clauses over frozen and fresh variables
        fresh = list(range(nxt, nxt + 10))
        nxt += 10
        new = random_clauses(rng, np.array(frozen + fresh), 25)
        for c in new:
            s.add(c)
        added.extend(new)
        frozen.extend(fresh[:3])
        for v in fresh[:3]:
            s.freeze(v)
    return s, outcomes


def oracle_call(opts):
    def call(s, prep):
        o = pg.options_from(**dict(opts, ve_inprocess=prep.ve_inprocess))
        return po.simplify(prep.cnf, o, assumed=prep.assumed, vorg=prep.vorg)
    return call


@pytest.mark.parametrize("seed", range(1, 13))
def test_incremental_session(seed):
    opts = dict(mupos=10, muneg=10, electionsmin=1, bce=bool(seed % 2))
    s, outcomes = run_session(seed, oracle_call(opts), **opts)
    assert s.calls >= 1 and outcomes


def test_frozen_and_assumed_variables_are_never_eliminated():
    for seed in range(1, 9):
        opts = dict(mupos=10, muneg=10, electionsmin=1)
        s, _ = run_session(seed, oracle_call(opts), **opts)
        assert not (s.eliminated & s.frozen)


def test_eliminated_variables_cannot_come_back():
    s = Incremental(mupos=10, muneg=10, electionsmin=1)
    for c in ([1, 2], [-1, 3], [2, 3, 4], [-2, -4, 5], [4, -5, 6]):
        s.add(c)
    s.freeze(3)
    prep = s.prepare()
    s.absorb(prep, po.simplify(prep.cnf, pg.options_from(mupos=10, muneg=10, electionsmin=1), assumed=prep.assumed,
                               vorg=prep.vorg))
    assert s.eliminated and 3 not in s.eliminated
    v = next(iter(s.eliminated))
    with pytest.raises(ValueError):
        s.add([v, 3])
    with pytest.raises(ValueError):
        s.assume(-v)
