"""DRAT proof of the simplifier (proof_en), CPU side: the oracle's proof
stream checked line by line by reverse unit propagation against the input
formula, the proof-byte guard of the resolvent counts, the text writer, and
the rejection of proofs where they have no output."""
import ctypes as C

import numpy as np
import pytest

import parafrost_gb300 as pg
from oracle import pyoracle as po
from tests.parity import decode_proof
from tests.test_writeback import small, with_units

VARIANTS = [dict(), dict(bce=True), dict(all=True), dict(mupos=10, muneg=10, electionsmin=1),
            dict(phases=1), dict(ere=False, bce=True, mupos=10, muneg=10)]


@pytest.mark.parametrize("vi", range(len(VARIANTS)))
@pytest.mark.parametrize("seed", range(1, 13))
def test_oracle_proof_lines_follow_by_unit_propagation(seed, vi):
    cnf = small(seed)
    res = po.simplify(cnf, pg.options_from(proof=True, **VARIANTS[vi]))
    bad, missing = po.check_rup(cnf, res.proof)
    assert bad == 0, f"line {bad} of the proof is not RUP"
    assert missing == 0
    # the formula after the proof's deletions and additions still implies the result
    if res.proof:
        kinds = {k for k, _ in decode_proof(res.proof)}
        assert kinds <= {"a", "d"}


@pytest.mark.parametrize("seed", range(1, 9))
def test_oracle_proof_with_learnts_and_inprocessing(seed):
    from tests.test_gpu_variants import with_learnts
    cnf = with_learnts(small(seed), seed)
    res = po.simplify(cnf, pg.options_from(proof=True, ve_inprocess=1, mupos=10, muneg=10))
    assert po.check_rup(cnf, res.proof) == (0, 0)


@pytest.mark.parametrize("seed", range(1, 7))
def test_proof_literals_use_the_original_numbering(seed):
    cnf = small(seed)
    V = cnf.max_var
    rng = np.random.default_rng(seed)
    vorg = np.zeros(V + 1, dtype=np.uint32)
    vorg[1:] = rng.permutation(np.arange(1, V + 1)).astype(np.uint32) * 7 + 1000
    res = po.simplify(cnf, pg.options_from(proof=True), vorg=vorg)
    plain = po.simplify(cnf, pg.options_from(proof=True))
    inv = {int(o): v for v, o in enumerate(vorg) if v}
    mapped = [(k, tuple(sorted((inv[l >> 1] << 1) | (l & 1) for l in lits))) for k, lits in decode_proof(res.proof)]
    direct = [(k, tuple(sorted(lits))) for k, lits in decode_proof(plain.proof)]
    assert mapped == direct


def test_proof_does_not_change_ordinary_results():
    for seed in range(1, 16):
        cnf = small(seed)
        a = po.simplify(cnf, pg.options_from(proof=True))
        b = po.simplify(cnf, pg.options_from())
        assert b.proof == b""
        assert np.array_equal(a.cnf.lits, b.cnf.lits) and np.array_equal(a.stack, b.stack)


def guard_instance(seed=3):
    """x = 1 in one clause of 50 literals and 600 clauses of 50 literals on
    disjoint variables; every other variable is kept out of the election. Its
    600 resolvents of 98 literals take 89,319 proof bytes in the instance's own
    numbering and 295,200 with 5-byte literals, over the 262,143 bytes one
    variable may add."""
    rng = np.random.default_rng(seed)
    clauses = [[1] + list(range(2, 51))]
    for _ in range(600):
        vs = rng.choice(np.arange(51, 5000), 49, replace=False)
        clauses.append([-1] + [int(v) if rng.random() < 0.5 else -int(v) for v in vs])
    cnf = pg.Cnf.from_ints(4999, clauses)
    vs = np.full(cnf.max_var + 1, 2, dtype=np.uint8)
    vs[0] = 0
    vs[1] = 0
    big = np.arange(cnf.max_var + 1, dtype=np.uint32) + (1 << 27)
    big[0] = 0
    return cnf, vs, big


GUARD_OPTS = dict(literalsmul=2.5, phases=1, electionsmin=1)


def test_proof_byte_guard_rules_out_a_variable():
    cnf, vs, big = guard_instance()
    plain = po.simplify(cnf, pg.options_from(**GUARD_OPTS), var_state=vs, vorg=big)
    small_lits = po.simplify(cnf, pg.options_from(proof=True, **GUARD_OPTS), var_state=vs)
    big_lits = po.simplify(cnf, pg.options_from(proof=True, **GUARD_OPTS), var_state=vs, vorg=big)
    assert plain.eliminated[1] & 1 and small_lits.eliminated[1] & 1
    assert not big_lits.eliminated[1]
    assert len(decode_proof(small_lits.proof)) == 600
    assert big_lits.proof == b""


def py_text(proof: bytes) -> str:
    out = []
    for kind, lits in decode_proof(proof):
        body = "".join(("-" if l & 1 else "") + str(l >> 1) + " " for l in lits)
        out.append(("d " if kind == "d" else "") + body + "0\n")
    return "".join(out)


def test_proof_text_writer():
    cnf = small(5)
    res = po.simplify(cnf, pg.options_from(proof=True, bce=True, mupos=10, muneg=10))
    assert res.proof
    assert pg.proof_text(res.proof) == py_text(res.proof)
    assert pg.proof_text(b"") == ""
    for bad in (b"x\x04\x00", b"a\x04", b"a\x84", b"d\x01\x00"):
        with pytest.raises(pg.SimplifyError):
            pg.proof_text(bad)


def test_server_proof_fetch_checks_its_arguments():
    # served jobs carry their proof (pfg_server_fetch_proof, GPU-tested in
    # test_gpu_serving.py); without a server the call is rejected, not run
    L = pg._lib.lib()
    assert L.pfg_server_fetch_proof(None, 0, None) == 5
