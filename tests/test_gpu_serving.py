"""GPU tests of the serving loop (pfg_server_*): continuous admission of jobs by
arena budget, batches of several slots overlapping on the device, and every
job's result equal to the one its instance gives alone."""
import time

import numpy as np
import pytest

import parafrost_gb300 as pg
from oracle import pyoracle as po
from tests.parity import canon, diff
from tests.test_gpu_variants import inst, with_learnts

pytestmark = pytest.mark.gpu


def jobs(n, base=0, scale=3):
    out = []
    for j in range(n):
        cnf = inst(base + j, scale=1 + (j % scale))
        if j % 4 == 3:
            cnf = with_learnts(cnf, base + j)
        out.append(cnf)
    return out


def check_same_as_alone(cnf, res, opts):
    ref = po.simplify(cnf, pg.options_from(**opts))
    d = diff(canon(res), canon(ref))
    assert not d, "served result differs from the oracle: " + "; ".join(d)
    with pg.Simplifier(**opts) as s:
        one = s.simplify(cnf)
    d = diff(canon(res), canon(one))
    assert not d, "served result differs from the instance alone: " + "; ".join(d)


def test_results_same_alone_and_in_the_mix():
    opts = dict(phases=3)
    cnfs = jobs(30, base=200)
    with pg.Server(slots=3, max_batch=4, **opts) as srv:
        tickets = []
        for i, cnf in enumerate(cnfs):
            tickets.append(srv.submit(cnf))
            if i % 6 == 5:
                time.sleep(0.005)   # later jobs arrive while earlier batches run
        infos = [srv.wait(t) for t in tickets]
        results = [srv.fetch(t) for t in tickets]
        st = srv.stats()
    assert all(i.rc == 0 for i in infos)
    assert st["done"] == len(cnfs) and st["batches"] >= len(cnfs) // 4
    assert max(i.batch_size for i in infos) > 1
    assert st["max_in_flight_batches"] >= 2, "no two batches were on the device at once"
    for cnf, res in zip(cnfs, results):
        check_same_as_alone(cnf, res, opts)


def test_admission_keeps_to_the_budget():
    cnfs = jobs(16, base=300)
    with pg.Server(slots=2, max_batch=64) as srv:
        est = [srv.wait(srv.submit(c)).est_bytes for c in cnfs[:4]]
    budget = int(max(est) * 2.5)
    with pg.Server(arena_bytes=budget, slots=4, max_batch=64) as srv:
        tickets = [srv.submit(c) for c in cnfs]
        infos = [srv.wait(t) for t in tickets]
        results = [srv.fetch(t) for t in tickets]
        st = srv.stats()
    assert all(i.rc == 0 for i in infos)
    assert st["peak_est_bytes"] <= budget
    # jobs are admitted in arrival order
    admits = [i.t_admit_ns for i in infos]
    assert admits == sorted(admits)
    for cnf, res in zip(cnfs, results):
        check_same_as_alone(cnf, res, {})


def test_invalid_job_is_rejected_at_submit():
    with pg.Server(slots=1) as srv:
        with pytest.raises(pg.SimplifyError) as e:
            srv.submit(pg.Cnf.from_ints(3, [[1, 7]]))
        assert e.value.code == 5
        t = srv.submit(inst(9))
        assert srv.wait(t).rc == 0


def test_unknown_ticket():
    with pg.Server(slots=1) as srv:
        with pytest.raises(pg.SimplifyError):
            srv.poll(12345)


def test_served_proofs_are_the_ones_alone():
    # proof lines per job (pfg_server_fetch_proof): byte for byte the oracle's
    # and the instance's alone, whatever batch the job ran in
    from tests.parity import proof_diff
    opts = dict(phases=3, proof=True)
    cnfs = jobs(12, base=700)
    with pg.Server(slots=2, max_batch=4, **opts) as srv:
        tickets = [srv.submit(c) for c in cnfs]
        outs = [srv.fetch(t) for t in tickets]
    assert any(len(r.proof) for r in outs)
    for i, (cnf, res) in enumerate(zip(cnfs, outs)):
        ref = po.simplify(cnf, pg.options_from(**opts))
        assert not proof_diff(res.proof, ref.proof), f"job {i}: " + proof_diff(res.proof, ref.proof)
        with pg.Simplifier(**opts) as s:
            one = s.simplify(cnf)
        assert res.proof == one.proof, f"job {i}: served proof differs from the instance alone"
