"""Occurrence lists longer than the warp passes take (the hub literals of
scale-free instances): the table update between rounds and the filter after
unit propagation hand them to whole blocks (ot.cu, prune_move_long_k and
ot_filter_long_k). These instances have dozens of lists above that length
and propagate ~90k forced units, so both kernels run in several rounds; the
results must equal the oracle's, alone and inside a batch."""
import numpy as np
import pytest

import parafrost_gb300 as pg
from oracle import pyoracle as po
from tests.parity import assert_parity, canon, diff
from tests.test_gpu_variants import inst

pytestmark = pytest.mark.gpu

LONG = 1024


def hub_instance(seed):
    cnf = pg.scale_free(200_000, 800_000, seed, planted=True)
    hist = np.bincount(cnf.lits, minlength=2 * cnf.max_var + 2)
    assert (hist > LONG).sum() >= 10
    return cnf


@pytest.mark.parametrize("seed", [3, 4])
def test_long_lists_alone(seed):
    res, ref = assert_parity(hub_instance(seed))
    assert len(ref.units) > 10_000 and len(ref.round_ends) >= 3
    # a trail this long is sorted on the device by pfg_download; the ABI promises ascending units
    u = np.asarray(res.units)
    assert np.all(u[1:] > u[:-1])


def test_long_lists_in_a_batch():
    cnfs = [inst(5), hub_instance(3), inst(6), inst(7)]
    with pg.Simplifier() as sim:
        outs = sim.simplify_batch(cnfs)
    for cnf, out in zip(cnfs, outs):
        ref = po.simplify(cnf, pg.options_from())
        d = diff(canon(out), canon(ref))
        assert not d, "; ".join(d)
