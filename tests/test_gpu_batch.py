"""GPU parity of batched simplification (pfg_batch_upload / pfg_batch_download).

A batch simplifies n independent instances in one device clause store. Every
instance of a batch must give exactly what it gives alone: the canonical
output of each instance is compared with the oracle on that instance alone
and with the engine's own one-instance run, for mixed families, sizes,
solver-state inputs and option variants."""
import numpy as np
import pytest

import parafrost_gb300 as pg
from oracle import pyoracle as po
from tests.parity import canon, diff
from tests.test_gpu_variants import inst, with_learnts

pytestmark = pytest.mark.gpu


def check_batch(cnfs, var_states=None, assumeds=None, vorgs=None, alone=True, **opts):
    with pg.Simplifier(**opts) as s:
        outs = s.simplify_batch(cnfs, var_states, assumeds, vorgs)
        assert s.batch_size() == len(cnfs)
    assert len(outs) == len(cnfs)
    o = pg.options_from(**opts)
    for i, (cnf, res) in enumerate(zip(cnfs, outs)):
        vs = None if var_states is None else var_states[i]
        asd = None if assumeds is None else assumeds[i]
        vo = None if vorgs is None else vorgs[i]
        ref = po.simplify(cnf, o, var_state=vs, assumed=asd, vorg=vo)
        d = diff(canon(res), canon(ref))
        assert not d, f"instance {i}: batch differs from the oracle: " + "; ".join(d)
        assert res.stats["clauses_in"] == cnf.num_clauses
        assert res.stats["clauses_out"] == res.cnf.num_clauses
        if alone:
            with pg.Simplifier(**opts) as s1:
                one = s1.simplify(cnf, var_state=vs, assumed=asd, vorg=vo)
            d = diff(canon(res), canon(one))
            assert not d, f"instance {i}: batch differs from the same instance alone: " + "; ".join(d)
            assert res.stats["rounds"] == one.stats["rounds"]
    return outs


@pytest.mark.parametrize("seed", range(6))
def test_mixed_families(seed):
    cnfs = [inst(100 * seed + j, scale=1 + (j % 3)) for j in range(7)]
    check_batch(cnfs)


def test_single_instance_batch_matches_plain_download():
    cnf = inst(11, scale=2)
    with pg.Simplifier() as s:
        a = s.simplify_batch([cnf])[0]
    with pg.Simplifier() as s:
        b = s.simplify(cnf)
    assert not diff(canon(a), canon(b))
    # clause order is deterministic; the raw stack is in atomic append order
    # within a round, so only its canonical form (compared above) and the
    # round boundaries are fixed
    assert np.array_equal(a.cnf.lits, b.cnf.lits) and np.array_equal(a.cnf.off, b.cnf.off)
    assert len(a.stack) == len(b.stack) and np.array_equal(a.round_ends, b.round_ends)


VARIANTS = [
    dict(lcvefast=False), dict(vefunction=False), dict(ere=False), dict(phases=1), dict(phases=8),
    dict(collectfreq=1), dict(mupos=10, muneg=10), dict(electionsmax=6), dict(literalsmul=0.0),
    dict(velitsbound=True), dict(sub=False, veextend=False), dict(eliminatedlitsmin=1),
    dict(all=True), dict(bce=True, ve=False, veextend=False),
]


@pytest.mark.parametrize("vi", range(len(VARIANTS)))
def test_option_variants(vi):
    cnfs = [inst(7 * vi + j) for j in range(5)]
    check_batch(cnfs, alone=False, **VARIANTS[vi])


@pytest.mark.parametrize("inprocess", [0, 1])
def test_learnts_and_solver_state(inprocess):
    cnfs, vss, asds, vos = [], [], [], []
    for j in range(6):
        cnf = inst(40 + j)
        if j % 2:
            cnf = with_learnts(cnf, j)
        rng = np.random.default_rng(j)
        V = cnf.max_var
        asd = (rng.random(V + 1) < 0.05).astype(np.uint8) if j % 3 == 0 else None
        vs = np.zeros(V + 1, dtype=np.uint8)
        vs[rng.random(V + 1) < 0.05] = 2
        vo = None
        if j % 3 == 1:
            vo = np.arange(V + 1, dtype=np.uint32)
            vo[1:] = rng.permutation(np.arange(1, V + 1)).astype(np.uint32) * 3 + 7
        cnfs.append(cnf); vss.append(vs); asds.append(asd); vos.append(vo)
    check_batch(cnfs, vss, asds, vos, alone=False, ve_inprocess=inprocess, mupos=10, muneg=10)


def test_instances_stopping_at_different_rounds():
    chain = pg.Cnf.from_ints(200, [[-i, i + 1] for i in range(1, 200)])
    pure = pg.Cnf.from_ints(6, [[1, 2], [1, 3], [2, 4], [3, 5], [4, 6]])
    unsat = pg.Cnf.from_ints(6, [[1, 2], [1, -2], [-1, 3], [-1, -3], [4, 5], [-4, 6], [5, 6]])
    cnfs = [inst(3, scale=3), chain, pure, unsat, inst(4), inst(5, scale=2)]
    outs = check_batch(cnfs, electionsmin=1, mupos=10, muneg=10)
    rounds = {o.stats["rounds"] for o in outs}
    assert len(rounds) > 1


def test_instance_without_original_clauses_is_left_alone():
    learnt_only = with_learnts(inst(21), 21, frac=1.0)
    cnfs = [inst(20), learnt_only, inst(22)]
    outs = check_batch(cnfs)
    assert outs[1].cnf.num_clauses == learnt_only.num_clauses


def test_many_uneven_instances():
    rng = np.random.default_rng(5)
    cnfs = []
    for j in range(48):
        v = int(np.exp(rng.uniform(np.log(50), np.log(3000))))
        fam = j % 3
        if fam == 0:
            cnfs.append(pg.random_ksat(v, int(v * 4.26), 3, 1000 + j))
        elif fam == 1:
            cnfs.append(pg.tseitin(v, max(4, v // 20), max(1, v // 1000), 1000 + j))
        else:
            cnfs.append(pg.scale_free(v, 4 * v, 1000 + j, planted=bool(j % 2)))
    check_batch(cnfs, alone=False)


def test_plain_download_refuses_a_batch():
    with pg.Simplifier() as s:
        s.upload_batch([inst(1), inst(2)])
        s.run()
        with pytest.raises(pg.SimplifyError) as e:
            s.download()
    assert e.value.code == 5


def test_invalid_instance_is_named():
    bad = pg.Cnf.from_ints(3, [[1, 9]])
    with pg.Simplifier() as s:
        with pytest.raises(pg.SimplifyError) as e:
            s.upload_batch([inst(1), bad])
    assert e.value.code == 5 and "instance 1" in str(e.value)


def test_bulk_and_per_instance_downloads_agree():
    cnfs = [inst(60 + j, scale=1 + j % 2) for j in range(6)] + [with_learnts(inst(70), 70)]
    with pg.Simplifier() as s:
        s.upload_batch(cnfs)
        s.run()
        bulk = s.download_all()
        single = [s.download_instance(i) for i in range(len(cnfs))]
    for a, b in zip(bulk, single):
        for x, y in ((a.cnf.lits, b.cnf.lits), (a.cnf.off, b.cnf.off), (a.cnf.learnt, b.cnf.learnt),
                     (a.cnf.lbd, b.cnf.lbd), (a.cnf.usage, b.cnf.usage), (a.eliminated, b.eliminated),
                     (a.units, b.units), (a.pending_units, b.pending_units), (a.stack, b.stack),
                     (a.round_ends, b.round_ends)):
            assert np.array_equal(x, y)
        assert a.status == b.status and a.stats["clauses_out"] == b.stats["clauses_out"]


def test_download_into_pinned_buffers():
    from parafrost_gb300 import pinned
    buf = pinned.ResultBuffers()
    for seeds in ([61, 62], [63, 64, 65, 66, 67]):
        cnfs = [inst(s, scale=2).pinned() for s in seeds]
        assert all(pinned.is_pinned(c.lits) for c in cnfs)
        with pg.Simplifier() as s:
            s.upload_batch(cnfs)
            s.run()
            ref = s.download_all()
            got = s.download_all(into=buf)
        for a, b in zip(got, ref):
            for x, y in ((a.cnf.lits, b.cnf.lits), (a.cnf.off, b.cnf.off), (a.eliminated, b.eliminated),
                         (a.units, b.units), (a.stack, b.stack), (a.round_ends, b.round_ends)):
                assert np.array_equal(x, y)
        assert pinned.is_pinned(got[0].cnf.lits)


@pytest.mark.parametrize("streams", [2, 3])
def test_batch_over_several_streams(streams):
    """simplify_batch(streams=k): k runs of consecutive instances, each on its
    own context, stream and host thread; every instance as in one batch."""
    cnfs = [inst(700 + j, scale=1 + (j % 3)) for j in range(10)]
    vstates = [None] * len(cnfs)
    vstates[4] = np.zeros(cnfs[4].max_var + 1, dtype=np.uint8)
    vstates[4][1] = 1
    with pg.Simplifier() as s:
        one = s.simplify_batch(cnfs, var_states=vstates)
        many = s.simplify_batch(cnfs, var_states=vstates, streams=streams)
        again = s.simplify_batch(cnfs, var_states=vstates, streams=streams)   # the contexts are reused
    assert len(many) == len(cnfs)
    for i in range(len(cnfs)):
        assert not diff(canon(many[i]), canon(one[i])), f"instance {i}"
        assert not diff(canon(again[i]), canon(one[i])), f"instance {i}"
        assert many[i].stats["clauses_in"] == cnfs[i].num_clauses


def test_batch_over_several_streams_into_pinned_buffers():
    from parafrost_gb300 import pinned
    cnfs = [inst(800 + j, scale=2).pinned() for j in range(6)]
    bufs = [pinned.ResultBuffers() for _ in range(3)]
    with pg.Simplifier() as s:
        ref = s.simplify_batch(cnfs)
        got = s.simplify_batch(cnfs, into=bufs, streams=3)
    for a, b in zip(got, ref):
        assert not diff(canon(a), canon(b))
    assert all(pinned.is_pinned(r.cnf.lits) for r in got if r.cnf.lits.size)


def test_simplify_many_contexts_at_once():
    """pfg_simplify_many: runs of a batch uploaded into distinct contexts and
    simplified at once give every instance's result of one batch; the job's
    device time covers every context's own."""
    from parafrost_gb300.simplifier import split_runs
    cnfs = [inst(900 + j, scale=1 + (j % 2)) for j in range(9)]
    runs = split_runs([c.num_clauses for c in cnfs], 3)
    with pg.Simplifier() as s:
        ref = s.simplify_batch(cnfs)
        sims = [s] + s.peers(2)
        for sim, (b, e) in zip(sims, runs):
            sim.upload_batch(cnfs[b:e])
        stats, ms = pg.run_many(sims)
        got = []
        for sim in sims:
            got.extend(sim.download_all())
        assert ms > 0 and ms >= max(st.device_ms for st in stats) - 1e-3
        assert sum(st.clauses_processed for st in stats) == sum(int(r.stats["clauses_processed"]) for r in ref)
        # a context named twice is refused before anything runs
        for sim, (b, e) in zip(sims, runs):
            sim.upload_batch(cnfs[b:e])
        with pytest.raises(pg.SimplifyError):
            pg.run_many([sims[0], sims[0]])
        stats, ms = pg.run_many(sims)      # still uploaded: the refused call ran nothing
    for a, b in zip(got, ref):
        assert not diff(canon(a), canon(b))
