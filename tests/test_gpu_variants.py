"""GPU parity on option variants, solver-state inputs and edge cases.

Every case runs the CUDA engine through the C ABI and the oracle on the same
input and compares canonical outputs bit for bit."""
import numpy as np
import pytest

import parafrost_gb300 as pg
from tests.parity import assert_parity, canon, diff, run_both

pytestmark = pytest.mark.gpu


def inst(seed, scale=1):
    rng = np.random.default_rng(seed)
    fam = seed % 3
    if fam == 0:
        v = int(rng.integers(100, 600)) * scale
        return pg.random_ksat(v, int(v * rng.uniform(3.2, 4.4)), 3, seed)
    if fam == 1:
        return pg.tseitin(int(rng.integers(300, 2000)) * scale, int(rng.integers(20, 80)), int(rng.integers(1, 6)), seed)
    return pg.scale_free(int(rng.integers(200, 800)) * scale, int(rng.integers(800, 3000)) * scale, seed,
                         planted=bool(seed % 2))


VARIANTS = [
    dict(ere=False), dict(sub=False, veextend=False), dict(vefunction=False), dict(velitsbound=True),
    dict(lcvefast=False), dict(resolventmax=0), dict(resolventmax=3), dict(xormaxarity=2), dict(collectfreq=1),
    dict(collectfreq=0), dict(literalsmul=0.0), dict(electionsmax=6), dict(lcveclausemax=3), dict(phases=1),
    dict(phases=2, ere=False), dict(phases=8), dict(mupos=10, muneg=10), dict(eliminatedlitsmin=1),
    dict(ereclausemax=3), dict(eremaxoccurs=100), dict(submaxoccurs=100), dict(electionsmin=1000000),
    dict(ve=False, veextend=False), dict(all=True), dict(bce=True), dict(bce=True, ve=False, veextend=False),
    dict(bce=True, bcemaxoccurs=100),
]


@pytest.mark.parametrize("vi", range(len(VARIANTS)))
def test_option_variants(vi):
    opts = dict(VARIANTS[vi])
    for seed in (vi * 3 + 1, vi * 3 + 2, vi * 3 + 3):
        assert_parity(inst(seed), **opts)


def with_learnts(cnf, seed, frac=0.25):
    rng = np.random.default_rng(seed)
    n = cnf.num_clauses
    learnt = (rng.random(n) < frac).astype(np.uint8)
    # originals first, then learnts, as the solver uploads them (simplify.cu:108-109)
    order = np.concatenate([np.nonzero(learnt == 0)[0], np.nonzero(learnt == 1)[0]])
    sizes = np.diff(cnf.off)[order]
    off = np.concatenate([[0], np.cumsum(sizes)]).astype(np.uint64)
    lits = np.concatenate([cnf.clause(int(i)) for i in order]).astype(np.uint32)
    lbd = rng.integers(1, 20, n).astype(np.uint32)
    usage = rng.integers(0, 4, n).astype(np.uint8)
    return pg.Cnf(cnf.max_var, lits, off, learnt[order], lbd, usage)


@pytest.mark.parametrize("seed", range(1, 13))
@pytest.mark.parametrize("inprocess", [0, 1])
def test_learnt_clauses(seed, inprocess):
    cnf = with_learnts(inst(seed), seed)
    assert_parity(cnf, ve_inprocess=inprocess, mupos=10, muneg=10)


@pytest.mark.parametrize("seed", range(1, 9))
def test_assumptions_var_state_and_vorg(seed):
    cnf = inst(seed)
    rng = np.random.default_rng(seed + 100)
    V = cnf.max_var
    assumed = (rng.random(V + 1) < 0.05).astype(np.uint8)
    vstate = np.zeros(V + 1, dtype=np.uint8)
    vstate[rng.random(V + 1) < 0.05] = 2                  # FROZEN_M variables are never elected
    vorg = np.arange(V + 1, dtype=np.uint32)
    vorg[1:] = rng.permutation(np.arange(1, V + 1)).astype(np.uint32) * 3 + 7   # original numbering
    assert_parity(cnf, var_state=vstate, assumed=assumed, vorg=vorg)


def test_implication_chain_shrinks():
    # a chain of binary implications: every round eliminates an independent set of links
    cl = [[-i, i + 1] for i in range(1, 200)]
    cnf = pg.Cnf.from_ints(200, cl)
    res, ref = assert_parity(cnf, electionsmin=1)
    assert res.cnf.num_clauses < cnf.num_clauses // 4 and len(res.stack) > 0


def test_everything_eliminated_is_sat():
    # pure literals only: every variable is eliminated without resolvents
    cnf = pg.Cnf.from_ints(6, [[1, 2], [1, 3], [2, 4], [3, 5], [4, 6]])
    res, ref = assert_parity(cnf, electionsmin=1)
    assert res.status == ref.status


def test_too_few_elections_leaves_cnf_unchanged():
    cnf = inst(5)
    res, ref = assert_parity(cnf, electionsmin=10_000_000)
    assert res.cnf.num_clauses == cnf.num_clauses and len(res.stack) == 0


def test_conflicting_units_are_unsat():
    # x1 and its negation both follow from two binary pairs after elimination
    cnf = pg.Cnf.from_ints(6, [[1, 2], [1, -2], [-1, 3], [-1, -3], [4, 5], [-4, 6], [5, 6]])
    res, ref = assert_parity(cnf, electionsmin=1, mupos=10, muneg=10)
    assert res.status == ref.status


def test_runs_twice_identically():
    cnf = inst(7, scale=3)
    with pg.Simplifier() as s:
        a = canon(s.simplify(cnf))
        b = canon(s.simplify(cnf))
    assert not diff(a, b)


@pytest.mark.parametrize("bad", ["dup", "range", "unit", "taut"])
def test_invalid_input_is_rejected(bad):
    lits = {"dup": [[1, 2, 1]], "range": [[1, 9]], "unit": [[1]], "taut": [[1, -1]]}[bad]
    cnf = pg.Cnf.from_ints(3, lits + [[1, 2], [2, 3]])
    with pg.Simplifier() as s:
        with pytest.raises(pg.SimplifyError) as e:
            s.simplify(cnf)
    assert e.value.code == 5


def test_arena_budget_overflow_is_reported():
    cnf = pg.random_ksat(5000, 21000, 3, 1)
    with pg.Simplifier(arena_bytes=1 << 16) as s:
        with pytest.raises(pg.SimplifyError) as e:
            s.simplify(cnf)
    assert e.value.code in (2, 3)


def test_profiler_counts_match_launches():
    cnf = inst(4, scale=2)
    with pg.Simplifier() as s:
        s.profile(True)
        s.upload(cnf)
        s.profile_reset()
        st = s.run()
        rep = s.profile_report()
    assert sum(v["launches"] for v in rep.values()) == st.kernel_launches
    assert all(v["ms"] >= 0 for v in rep.values())


@pytest.mark.slow
def test_config3_scalefree_full_size():
    cnf = pg.scale_free(4_000_000, 16_000_000, seed=1, planted=True)
    assert_parity(cnf)


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_ere_duplicate_blocks(seed):
    # x_i's only resolvent is (a_i | b_i); the CNF holds blocks of copies of it
    # (originals and learnts with distinct lbd/usage, so the canonical form
    # shows which copies ERE deleted). With SUB and BVE off the first round is
    # the ERE round; blocks longer than 32 exercise the strided-lane rule.
    rng = np.random.default_rng(seed)
    clauses, learnt, lbd, usage = [], [], [], []
    nv = 0
    for k in (1, 2, 33, 40, 70, 5):
        x, a, b = nv + 1, nv + 2, nv + 3
        nv += 3
        for c in ([x, a], [-x, b]):
            clauses.append(c); learnt.append(0); lbd.append(0); usage.append(0)
        for _ in range(k):
            sa = a if rng.random() < 0.8 else -a
            clauses.append([sa, b]); learnt.append(int(rng.random() < 0.5))
            lbd.append(int(rng.integers(1, 1000))); usage.append(int(rng.integers(0, 4)))
    order = np.argsort(np.array(learnt), kind="stable")        # originals first, then learnts
    cl = [clauses[i] for i in order]
    base = pg.Cnf.from_ints(nv, cl)
    cnf = pg.Cnf(base.max_var, base.lits, base.off, np.array(learnt, dtype=np.uint8)[order],
                 np.array(lbd, dtype=np.uint32)[order], np.array(usage, dtype=np.uint8)[order])
    res, ref = assert_parity(cnf, sub=False, ve=False, veextend=False, electionsmin=1)
    assert res.stats["ere_ran"] == 1


def test_resolvents_longer_than_any_uploaded_clause():
    # scale-free instance whose ERE round merges resolvents longer than every
    # uploaded clause (it once overran the oracle's merge buffer)
    cnf = pg.generate(2, 72030, 288120, 1, 1163604499)
    assert_parity(cnf)



def test_blocked_clause_elimination_fires():
    # with BVE off BCE sees every elected variable: it must remove clauses on
    # these instances and stay equal to the oracle
    changed = 0
    for seed in range(1, 9):
        cnf = inst(seed)
        on, _ = assert_parity(cnf, bce=True, ve=False, veextend=False, mupos=10, muneg=10)
        off, _ = run_both(cnf, bce=False, ve=False, veextend=False, mupos=10, muneg=10)
        changed += on.cnf.num_clauses < off.cnf.num_clauses
    assert changed > 0
    # variable 1 is elected and (-1 | 2) is blocked by (1 | -2)
    cnf = pg.Cnf.from_ints(6, [[-1, 2], [1, -2], [3, 4], [-3, 5], [4, -5, 6], [-4, -6]])
    res, _ = assert_parity(cnf, sub=False, ve=False, veextend=False, bce=True, ere=False, electionsmin=1)
    assert res.cnf.num_clauses < cnf.num_clauses and len(res.stack) > 0
