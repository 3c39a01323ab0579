"""GPU parity of the DRAT proof (proof_en): the engine's proof stream equals
the oracle's byte for byte, alone and per instance of a batch, through the
warp-staged and the thread-per-variable kernels, and with the proof-byte
guard changing an elimination decision."""
import numpy as np
import pytest

import parafrost_gb300 as pg
from oracle import pyoracle as po
from tests.parity import canon, diff, proof_diff
from tests.test_gpu_variants import inst, with_learnts
from tests.test_proof import GUARD_OPTS, guard_instance
from tests.test_writeback import small

pytestmark = pytest.mark.gpu

VARIANTS = [dict(), dict(bce=True), dict(all=True), dict(mupos=10, muneg=10), dict(phases=1),
            dict(ere=False, bce=True, mupos=10, muneg=10), dict(collectfreq=1, eliminatedlitsmin=1)]


def check(cnf, var_state=None, assumed=None, vorg=None, **opts):
    o = dict(opts, proof=True)
    with pg.Simplifier(**o) as s:
        res = s.simplify(cnf, var_state=var_state, assumed=assumed, vorg=vorg)
    ref = po.simplify(cnf, pg.options_from(**o), var_state=var_state, assumed=assumed, vorg=vorg)
    d = diff(canon(res), canon(ref))
    assert not d, "; ".join(d)
    pd = proof_diff(res.proof, ref.proof)
    assert not pd, pd
    return res


@pytest.mark.parametrize("vi", range(len(VARIANTS)))
@pytest.mark.parametrize("seed", range(1, 9))
def test_proof_equals_oracle(seed, vi):
    check(inst(seed, scale=1 + seed % 2), **VARIANTS[vi])


@pytest.mark.parametrize("seed", range(1, 9))
def test_proof_of_small_instances_checks_by_unit_propagation(seed):
    cnf = small(seed)
    res = check(cnf, mupos=10, muneg=10, electionsmin=1, bce=bool(seed % 2))
    assert po.check_rup(cnf, res.proof) == (0, 0)


@pytest.mark.parametrize("seed", range(1, 7))
def test_proof_with_learnts_state_and_vorg(seed):
    cnf = with_learnts(inst(seed), seed)
    V = cnf.max_var
    rng = np.random.default_rng(seed)
    vorg = np.zeros(V + 1, dtype=np.uint32)
    vorg[1:] = rng.permutation(np.arange(1, V + 1)).astype(np.uint32) * 131 + 5
    vs = np.zeros(V + 1, dtype=np.uint8)
    vs[rng.random(V + 1) < 0.05] = 2
    check(cnf, var_state=vs, vorg=vorg, ve_inprocess=seed % 2, mupos=10, muneg=10)


def test_large_lists_take_the_thread_kernels():
    # scale-free lists longer than the warp stage holds
    check(pg.scale_free(3000, 12000, 11, planted=True), mupos=64, muneg=64)


@pytest.mark.parametrize("big", [False, True])
def test_proof_byte_guard(big):
    cnf, vs, bigv = guard_instance()
    res = check(cnf, var_state=vs, vorg=bigv if big else None, **GUARD_OPTS)
    assert bool(res.eliminated[1] & 1) == (not big)


def test_batch_proofs_are_the_ones_alone():
    cnfs = [inst(90 + j, scale=1 + j % 2) for j in range(6)] + [with_learnts(inst(99), 99)]
    with pg.Simplifier(proof=True, bce=True) as s:
        outs = s.simplify_batch(cnfs)
        assert s.batch_size() == len(cnfs)
    with pg.Simplifier(proof=True, bce=True) as s:
        s.upload_batch(cnfs)
        s.run()
        bulk = s.download_all()
    o = pg.options_from(proof=True, bce=True)
    for i, cnf in enumerate(cnfs):
        ref = po.simplify(cnf, o)
        assert not proof_diff(outs[i].proof, ref.proof), f"instance {i}: " + proof_diff(outs[i].proof, ref.proof)
        assert bulk[i].proof == outs[i].proof


def test_proof_off_writes_nothing():
    with pg.Simplifier() as s:
        res = s.simplify(inst(4))
    assert res.proof == b""
