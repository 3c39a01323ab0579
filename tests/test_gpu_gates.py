"""GPU parity on instances built around the ITE and XOR gate detectors of BVE
(ifthenelse.cuh:50-123, xor.cuh:69-178).

Each instance defines variables as XOR gates of arity 2..5 and as ITE gates
over shared inputs, adds near misses of both (one clause of a definition
dropped, one literal's polarity flipped, a clause repeated) and random
ternary clauses around them, so the detectors find gates, fail on a missing
partner, fail after melting part of a gate, and meet duplicates. The engine
and the oracle must agree bit for bit.

The CPU tests check that the instances exercise what they are built for: the
oracle's result with XOR gates of arity up to 5 differs from the one with
arity 2 only, and the clause constructors build what they say."""
import itertools

import numpy as np
import pytest

import parafrost_gb300 as pg
from oracle import pyoracle as po


def _xor_clauses(out, ins, rng, flip=False, drop=False):
    """out = XOR(ins) as the 2^(a+1)/2 clauses over (out, ins) with an odd
    number of negations (out <-> x1 ^ ... ^ xa); `flip` negates one literal of
    one clause, `drop` leaves one clause out."""
    vs = [out] + list(ins)
    cls = []
    for signs in itertools.product((1, -1), repeat=len(vs)):
        if sum(s < 0 for s in signs) % 2 == 1:
            cls.append([s * v for s, v in zip(signs, vs)])
    if drop:
        cls.pop(int(rng.integers(len(cls))))
    if flip:
        c = cls[int(rng.integers(len(cls)))]
        q = int(rng.integers(len(c)))
        c[q] = -c[q]
    return cls


def _ite_clauses(out, c, t, e, rng, drop=False, redundant=False):
    """out = c ? t : e: (-out | -c | t), (-out | c | e), (out | -c | -t),
    (out | c | -e), optionally the two redundant clauses (-out | t | e),
    (out | -t | -e)."""
    cls = [[-out, -c, t], [-out, c, e], [out, -c, -t], [out, c, -e]]
    if redundant:
        cls += [[-out, t, e], [out, -t, -e]]
    if drop:
        cls.pop(int(rng.integers(4)))
    return cls


def gate_instance(seed, n_inputs=300, n_xor=120, n_ite=120, noise=1.5, max_arity=5):
    rng = np.random.default_rng(seed)
    nv = n_inputs
    clauses = []

    def new_var():
        nonlocal nv
        nv += 1
        return nv

    def pick(k):
        return [int(v) for v in rng.choice(np.arange(1, n_inputs + 1), size=k, replace=False)]

    for i in range(n_xor):
        arity = int(rng.integers(2, max_arity + 1))
        out = new_var()
        kind = i % 6
        cls = _xor_clauses(out, pick(arity), rng, flip=kind == 4, drop=kind == 5)
        if kind == 3:
            cls.append(list(cls[0]))
        clauses += cls
        # the gate's output is used elsewhere, so eliminating it costs resolvents
        for _ in range(int(rng.integers(1, 4))):
            a, b = pick(2)
            clauses.append([out if rng.random() < 0.5 else -out, a, -b])
    for i in range(n_ite):
        out = new_var()
        c, t, e = pick(3)
        kind = i % 5
        clauses += _ite_clauses(out, c, t, e, rng, drop=kind == 3, redundant=kind == 4)
        for _ in range(int(rng.integers(1, 4))):
            a, b = pick(2)
            clauses.append([-out if rng.random() < 0.5 else out, -a, b])
    for _ in range(int(noise * n_inputs)):
        vs = pick(3)
        clauses.append([v if rng.random() < 0.5 else -v for v in vs])
    perm = rng.permutation(len(clauses))
    return pg.Cnf.from_ints(nv, [clauses[i] for i in perm])


def _digest(res):
    lits, off, *_ = po.canon_cnf(res.cnf)
    return (lits.tobytes(), off.tobytes(), np.asarray(res.eliminated).tobytes())


def test_instances_exercise_the_xor_detector():
    cnf = gate_instance(1)
    wide = po.simplify(cnf, pg.options_from())
    narrow = po.simplify(cnf, pg.options_from(xormaxarity=2))
    assert _digest(wide) != _digest(narrow)
    assert int(np.count_nonzero(np.asarray(wide.eliminated) & 1)) > 100


def test_gate_constructors():
    whole = gate_instance(2, n_xor=60, n_ite=60)
    rng = np.random.default_rng(0)
    cls = _xor_clauses(1, [2, 3, 4], rng)
    assert len(cls) == 8 and all(sum(l < 0 for l in c) % 2 == 1 for c in cls)
    assert len(_xor_clauses(1, [2, 3], rng, drop=True)) == 3
    assert len(_ite_clauses(1, 2, 3, 4, rng, redundant=True)) == 6
    assert whole.num_clauses > 60 * 4 + 60 * 4


@pytest.mark.gpu
@pytest.mark.parametrize("seed", range(1, 9))
def test_gate_instances(seed):
    from tests.parity import assert_parity
    assert_parity(gate_instance(seed))


@pytest.mark.gpu
@pytest.mark.parametrize("opts", [dict(xormaxarity=2), dict(xormaxarity=3), dict(phases=1, ere=False),
                                  dict(lcvefast=False), dict(vefunction=False), dict(sub=False, veextend=False)])
def test_gate_instances_option_variants(opts):
    from tests.parity import assert_parity
    for seed in (11, 12):
        assert_parity(gate_instance(seed), **opts)


@pytest.mark.gpu
def test_gate_instances_batched():
    from tests.parity import canon, diff
    cnfs = [gate_instance(20 + i, n_inputs=200 + 50 * i) for i in range(6)]
    with pg.Simplifier() as s:
        outs = s.simplify_batch(cnfs)
    for cnf, res in zip(cnfs, outs):
        ref = po.simplify(cnf, pg.options_from())
        d = diff(canon(res), canon(ref))
        assert not d, "; ".join(d)
