"""The host-side give-up paths of the two device loops a simplify call drives:
unit propagation levels (bcp.cu) and Luby MIS rounds (lcve.cu). The bounds
are lowered through pfg_set_loop_limits, so no device wait is involved: the
host stops launching, pfg_simplify returns PFG_TIMEOUT naming the loop, and
the context (and a fresh one) still simplify correctly afterwards."""
import pytest

import parafrost_gb300 as pg
from tests.parity import assert_parity, canon, diff
from tests.test_gpu_variants import inst
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu

PFG_TIMEOUT = 4


def _timeout(sim, cnf):
    with pytest.raises(pg.SimplifyError) as e:
        sim.simplify(cnf)
    assert e.value.code == PFG_TIMEOUT
    return str(e.value)


def chain_instance(n=120):
    """Round 1 eliminates b from (a | b), (a | -b), which forces the unit a;
    round 2 starts by propagating it down the implications a -> x1 -> ... -> xn,
    one level per link. Every x_i also sits in 32 clauses of each polarity
    whose other literals are pure, so round 1 cannot elect an x_i (both
    polarities reach the mu bound) while it removes those clauses."""
    a, b = 1, 2
    xs = list(range(3, 3 + n))
    nxt = 3 + n
    clauses = [[a, b], [a, -b], [-a, xs[0]]]
    clauses += [[-xs[i], xs[i + 1]] for i in range(n - 1)]
    for x in xs:
        for sign in (1, -1):
            for _ in range(32):
                clauses.append([sign * x, nxt, nxt + 1])
                nxt += 2
    return pg.Cnf.from_ints(nxt - 1, clauses)


def test_chain_instance_propagates_the_whole_chain():
    cnf = chain_instance()
    res = po.simplify(cnf, pg.options_from())
    assert len(res.units) >= 120      # the oracle's propagation reaches every link


@pytest.mark.parametrize("bound", [1, 8])
def test_propagation_gives_up_beyond_the_level_bound(bound):
    cnf = chain_instance()
    with pg.Simplifier() as sim:
        sim.set_loop_limits(max_bcp_levels=bound)
        msg = _timeout(sim, cnf)
        assert "unit propagation" in msg
        # the same context simplifies correctly once the bound is back
        sim.set_loop_limits(0, 0)
        res = sim.simplify(cnf)
    ref = po.simplify(cnf, pg.options_from())
    assert not diff(canon(res), canon(ref))
    assert_parity(cnf)          # and a fresh context


@pytest.mark.parametrize("seed", [3, 17])
def test_mis_gives_up_beyond_the_round_bound(seed):
    cnf = inst(seed, scale=2)
    with pg.Simplifier() as sim:
        sim.set_loop_limits(max_mis_rounds=1)
        msg = _timeout(sim, cnf)
        assert "MIS" in msg
    assert_parity(cnf)


def test_bounds_that_are_never_reached_change_nothing():
    cnf = chain_instance()
    with pg.Simplifier() as sim:
        sim.set_loop_limits(max_bcp_levels=1 << 30, max_mis_rounds=1 << 30)
        res = sim.simplify(cnf)
    assert not diff(canon(res), canon(po.simplify(cnf, pg.options_from())))
