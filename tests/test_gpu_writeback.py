"""Write-back of the engine's results (single and batched): the mapped
formula keeps the original's satisfiability and its models extend to models
of the original formula through pfg_extend_model."""
import numpy as np
import pytest

import parafrost_gb300 as pg
from oracle import pyoracle as po
from tests.test_writeback import small, solve_dpll, with_units

pytestmark = pytest.mark.gpu


def check(cnf, res):
    orig, _ = solve_dpll(cnf)
    if int(res.status) == pg.PFG_UNSAT:
        assert orig == 20
        return
    m = pg.map_result(res)
    status, model = solve_dpll(with_units(m.cnf, m.units))
    assert status == orig
    if status == 10:
        assert po.satisfies(cnf, pg.reconstruct_model(res, m, model))


@pytest.mark.parametrize("seed", range(1, 13))
def test_engine_result_writes_back(seed):
    cnf = small(seed)
    with pg.Simplifier(mupos=10, muneg=10, electionsmin=1, bce=bool(seed % 2)) as s:
        res = s.simplify(cnf)
    check(cnf, res)


def test_batched_results_write_back():
    cnfs = [small(s) for s in range(20, 32)]
    with pg.Simplifier(mupos=10, muneg=10, electionsmin=1) as s:
        outs = s.simplify_batch(cnfs)
    for cnf, res in zip(cnfs, outs):
        check(cnf, res)
