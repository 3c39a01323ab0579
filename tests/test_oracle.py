"""CPU tests of the oracle: satisfiability preservation, model reconstruction,
agreement with the reference's own CPU solver (committed golden answers), the
canonical form, and hand-checked known answers."""
import json
import os

import numpy as np
import pytest

import parafrost_gb300 as pg
from oracle import pyoracle as po

HERE = os.path.dirname(os.path.abspath(__file__))


def small(seed):
    rng = np.random.default_rng(seed)
    fam = seed % 3
    if fam == 0:
        v = int(rng.integers(20, 70))
        return pg.random_ksat(v, int(v * rng.uniform(3.0, 4.6)), 3, seed)
    if fam == 1:
        return pg.tseitin(int(rng.integers(20, 80)), int(rng.integers(4, 12)), int(rng.integers(1, 4)), seed)
    return pg.scale_free(int(rng.integers(20, 60)), int(rng.integers(60, 220)), seed, planted=bool(seed % 2))


def check_equisat(cnf, opts, expect=None):
    r = po.simplify(cnf, opts)
    st0, _ = po.solve(cnf, 5_000_000) if expect is None else (expect, None)
    if r.status == pg.PFG_UNSAT:
        assert st0 == 20, "oracle propagation proved UNSAT on a satisfiable formula"
        return
    st1, m1 = po.solve(r.cnf, 5_000_000)
    if st0 == 0 or st1 == 0:
        pytest.skip("decision budget exhausted")
    assert st0 == st1, "simplification changed satisfiability"
    if st1 == 10:
        val = m1.copy()
        for u in r.units:
            val[u >> 1] = 0 if (u & 1) else 1
        val = po.extend_model(r.stack, val)
        assert po.satisfies(cnf, val), "reconstructed model violates the original formula"


@pytest.mark.parametrize("seed", range(1, 121))
def test_oracle_preserves_satisfiability(seed):
    rng = np.random.default_rng(seed)
    opts = pg.options_from(phases=int(rng.integers(1, 6)), mupos=10, muneg=10, electionsmin=1)
    check_equisat(small(seed), opts)


@pytest.mark.parametrize("variant", [
    dict(ere=False), dict(sub=False, veextend=False), dict(vefunction=False), dict(velitsbound=True),
    dict(lcvefast=False), dict(resolventmax=0), dict(xormaxarity=2), dict(phases=1, ere=False),
    dict(collectfreq=1), dict(literalsmul=0.0), dict(electionsmax=4), dict(lcveclausemax=2),
    dict(bce=True), dict(all=True), dict(bce=True, ve=False, veextend=False),
])
def test_oracle_option_variants(variant):
    for seed in range(1, 16):
        opts = pg.options_from(mupos=10, muneg=10, electionsmin=1, **variant)
        check_equisat(small(seed), opts)


def golden():
    with open(os.path.join(HERE, "golden", "ref_sat.json")) as f:
        return [r for r in json.load(f)["instances"] if r["answer"] in (10, 20)]


@pytest.mark.parametrize("row", golden(), ids=lambda r: f"f{r['family']}-s{r['seed']}-{r['a']}")
def test_oracle_matches_reference_cpu_solver(row):
    """The reference's own CPU solver decided each instance (golden answer);
    the oracle's simplified formula must keep that answer and its stack must
    rebuild models of the original."""
    cnf = pg.generate(row["family"], row["a"], row["b"], row["c"], row["seed"])
    assert cnf.num_clauses == row["clauses"], "generator drifted from the golden fixture"
    if cnf.max_var > 3000:
        pytest.skip("too large for the test DPLL (checked on the GPU)")
    check_equisat(cnf, pg.options_from(), expect=row["answer"])


def test_canon_stack_orders_blocks_by_witness_per_round():
    # two rounds; round 1 has blocks for witnesses 5 and 3 (in that order)
    b5 = [10, 4, 2, 11, 1]           # clause (10, 4) then witness 11 (var 5)
    b3 = [6, 1]                      # witness 6 (var 3), no clauses
    b7 = [14, 8, 2, 15, 1]           # round 2
    stack = np.array(b5 + b3 + b7, dtype=np.uint32)
    ends = np.array([len(b5) + len(b3), len(stack)], dtype=np.uint64)
    out = po.canon_stack(stack, ends)
    assert out.tolist() == b3 + b5 + b7


def test_extend_model_sets_witness_when_clause_unsatisfied():
    # block for x=var 2: saved clause (x2 | x3) with witness literal first, then witness (-x2, 1)
    stack = np.array([4, 6, 2, 5, 1], dtype=np.uint32)
    val = np.zeros(4, dtype=np.uint8)          # x3 = 0
    out = po.extend_model(stack, val)
    # walking backwards: witness -x2 -> x2 = 0; clause (x2 | x3) unsatisfied -> x2 = 1
    assert out[2] == 1
    val = np.zeros(4, dtype=np.uint8)
    val[3] = 1                                  # x3 = 1 satisfies the clause
    assert po.extend_model(stack, val)[2] == 0


def test_known_answer_pure_literal():
    """x1 occurs only positively: LCVE elects it, phase 1 eliminates it without
    resolvents (toblivion, elimination.cuh:486-538): its clauses are deleted
    and the stack holds the negative side (empty) then witness (+x1, 1)."""
    cnf = pg.Cnf.from_ints(4, [[1, 2], [1, 3], [2, 3, 4], [-2, -3], [-2, 4], [-3, -4]])
    r = po.simplify(cnf, pg.options_from(phases=1, ere=False, electionsmin=1, mupos=10, muneg=10))
    assert r.eliminated[1] & 1
    cl = r.cnf.clauses()
    assert all(1 not in c and -1 not in c for c in cl)
    # the block of x1 is [2, 1]: witness literal 2*1 = +x1 with length 1
    s = r.stack.tolist()
    i = s.index(2)
    assert s[i + 1] == 1


def test_known_answer_and_gate_substitution():
    """g = AND(a, b) (g=1, a=2, b=3) plus two uses of g; eliminating g by gate
    substitution resolves only gate x non-gate pairs (substitute_x,
    bounded.cuh:184-221): (-1|2),(-1|3),(1|-2|-3) with (1|4),(1|5) gives
    (2|4),(3|4),(2|5),(3|5) and no tautologies."""
    cnf = pg.Cnf.from_ints(5, [[-1, 2], [-1, 3], [1, -2, -3], [1, 4], [1, 5], [-4, -5, 2]])
    r = po.simplify(cnf, pg.options_from(phases=1, ere=False, electionsmin=1, mupos=10, muneg=10, sub=False,
                                         veextend=False, vefunction=False))
    if r.eliminated[1] & 1:
        cl = sorted(sorted(c) for c in r.cnf.clauses())
        for want in ([2, 4], [3, 4], [2, 5], [3, 5]):
            assert sorted(want) in cl
        assert all(1 not in c and -1 not in c for c in cl)


def test_canon_stack_orders_trailing_blocked_clauses():
    # round: a BVE block for var 5, then BCE entries (witness first, no [w, 1])
    # for vars 4, 2, 4 in append order
    b5 = [10, 4, 2, 11, 1]
    e4a = [9, 12, 2]                 # witness 9 = -4
    e2 = [5, 14, 2]                  # witness 5 = -2
    e4b = [9, 16, 2]
    stack = np.array(b5 + e4a + e2 + e4b, dtype=np.uint32)
    ends = np.array([len(stack)], dtype=np.uint64)
    out = po.canon_stack(stack, ends)
    assert out.tolist() == b5 + e2 + e4a + e4b


def test_blocked_clause_is_removed_and_model_rebuilt():
    # variable 1 ranks first (score 1, lowest index) and is elected; (-1 | 2) is
    # blocked on -1 by (1 | -2), the only clause of 1 (the resolvent is a
    # tautology). SUB and BVE are off so the clause is left to BCE.
    cnf = pg.Cnf.from_ints(6, [[-1, 2], [1, -2], [3, 4], [-3, 5], [4, -5, 6], [-4, -6]])
    opts = pg.options_from(sub=False, ve=False, veextend=False, bce=True, ere=False, electionsmin=1)
    res = po.simplify(cnf, opts)
    assert res.cnf.num_clauses < cnf.num_clauses and len(res.stack) > 0
    check_equisat(cnf, opts)
