"""Launch shapes (pfg_tuning) and the autotuner (pfg_autotune).

The shapes only move speed: every pass is schedule-independent, so the
simplified CNF, eliminated set and model stack (canonical form) must be the
same under any valid shapes, including extreme ones (one block per SM, a
work-stealing ticket of one variable, 32-thread blocks), and after the
autotuner has picked its own."""
import pytest

import parafrost_gb300 as pg
from tests.parity import canon, diff
from tests.test_gpu_variants import inst

pytestmark = pytest.mark.gpu

EXTREME = dict(sub_blocks_per_sm=1, ve1_blocks_per_sm=1, ve3_blocks_per_sm=1, ve3_ticket=1, mis_threads=32,
               list_threads=32, bcp_blocks_per_sm=1)
WIDE = dict(sub_blocks_per_sm=64, ve1_blocks_per_sm=64, ve3_blocks_per_sm=64, ve3_ticket=4096, mis_threads=1024,
            list_threads=1024, bcp_blocks_per_sm=64)


def batch():
    return [inst(900 + j, scale=1 + (j % 3)) for j in range(6)]


def run(cnfs, tuning=None):
    with pg.Simplifier() as s:
        if tuning is not None:
            s.tuning = tuning
        return s.simplify_batch(cnfs)


def same(a, b, what):
    for i, (x, y) in enumerate(zip(a, b)):
        d = diff(canon(x), canon(y))
        assert not d, f"instance {i}: {what} differs from the built-in shapes: " + "; ".join(d)


def test_get_set_roundtrip_and_defaults():
    with pg.Simplifier() as s:
        assert all(v == 0 for v in s.tuning.values())
        s.tuning = EXTREME
        assert s.tuning == EXTREME
        s.upload(inst(3))          # kept across uploads
        assert s.tuning == EXTREME


@pytest.mark.parametrize("bad", [dict(mis_threads=48), dict(list_threads=2048), dict(ve3_ticket=70000),
                                 dict(bcp_blocks_per_sm=65)])
def test_out_of_range_rejected(bad):
    with pg.Simplifier() as s:
        s.tuning = EXTREME
        with pytest.raises(pg.SimplifyError):
            s.tuning = bad
        assert s.tuning == EXTREME     # unchanged
        with pytest.raises(KeyError):
            s.tuning = dict(no_such_knob=1)


@pytest.mark.parametrize("shapes", [EXTREME, WIDE], ids=["extreme", "wide"])
def test_results_do_not_depend_on_shapes(shapes):
    cnfs = batch()
    same(run(cnfs, shapes), run(cnfs), "shapes " + str(shapes))


def test_autotune_picks_valid_shapes_and_keeps_results():
    cnfs = batch()
    ref = run(cnfs)
    with pg.Simplifier() as s:
        s.profile(False)
        best = s.autotune(cnfs)
        assert best == s.tuning
        assert best["mis_threads"] in (64, 128, 256, 512)
        assert best["list_threads"] in (64, 128, 256, 512)
        assert best["ve3_ticket"] in (1, 4, 16, 64)
        assert best["bcp_blocks_per_sm"] in (2, 4, 8, 16)
        for k in ("sub_blocks_per_sm", "ve1_blocks_per_sm", "ve3_blocks_per_sm"):
            assert best[k] in (0, 2, 4, 6)
        tuned = s.simplify_batch(cnfs)     # upload again after tuning
    same(tuned, ref, "autotuned shapes")
