"""The host-side give-up paths of the two device loops a simplify call drives:
unit propagation levels (bcp.cu) and Luby MIS rounds (lcve.cu). The bounds
are lowered through pfg_set_loop_limits, so no device wait is involved: the
host stops launching, pfg_simplify returns PFG_TIMEOUT naming the loop, and
the context (and a fresh one) still simplify correctly afterwards."""
import pytest

import parafrost_gb300 as pg
from parafrost_gb300 import _abi
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


@pytest.mark.parametrize("seed", [17, 41])
def test_propagation_gives_up_beyond_the_level_bound(seed):
    # these instances force units in BVE that propagate through long chains
    cnf = inst(seed)
    with pg.Simplifier() as sim:
        sim.set_loop_limits(max_bcp_levels=1)
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
    cnf = inst(17)
    with pg.Simplifier() as sim:
        sim.set_loop_limits(max_bcp_levels=1 << 30, max_mis_rounds=1 << 30)
        res = sim.simplify(cnf)
    assert not diff(canon(res), canon(po.simplify(cnf, pg.options_from())))
