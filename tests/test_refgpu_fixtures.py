"""Parity with the reference's own GPU simplifier.

tests/golden/refgpu/fixtures.json holds what the reference's GPU simplifier
(src/gpu, unmodified, built by oracle/ref_gpu_build.py with the cuArena
stand-in and driven by oracle/refgpu/dump_main.cpp) produced on a GB300 for
13 seeded instances (random 3-SAT up to the 20,000-variable / 85,200-clause
shape, 5-SAT, Tseitin circuits with and without root units, scale-free with
and without a planted model) under five option sets: the defaults (Luby MIS,
5 rounds, ERE), one round without ERE, sequential LCVE (-no-lcvefast) with
and without those, and -no-vefunction. Each entry lists the distinct
canonical results of three runs (tests/refgpu.py) — every entry had one.

What is compared:
  * runs with one SUB+BVE round (and runs that stopped on a conflict): the
    whole canonical result — clauses, eliminated bytes, units, pending units,
    model-stack blocks, round count;
  * runs with two or more rounds: status, eliminated bytes, units, pending
    units and round count. The reference's clauses and model stack could not
    be read back from those runs (its skip-transfer write-back, run after it
    had cached the eliminated bytes, left the host mirror holding the input
    and the stack empty), so those two fields are not compared there.
The oracle is checked on the CPU, the engine on the GPU, each against the
same fixtures."""
import json
import os

import numpy as np
import pytest

import parafrost_gb300 as pg
from oracle import pyoracle as po
from tests import refgpu

HERE = os.path.dirname(os.path.abspath(__file__))
FIX_DIR = os.path.join(HERE, "golden", "refgpu")


def load():
    with open(os.path.join(FIX_DIR, "fixtures.json")) as f:
        return json.load(f)["fixtures"]


FIXTURES = load()


def fields_of(entry):
    out = entry["outputs"][0]["canon"]
    if out["status"] == 20 or out.get("rounds", 0) <= 1:
        return refgpu.FIELDS
    return ("elim", "units", "pending", "rounds")


def input_of(entry):
    if entry["input"] == "generator":
        cnf = pg.generate(*entry["generator"])
    else:
        z = np.load(os.path.join(FIX_DIR, entry["input"]))
        cnf = pg.Cnf(int(z["max_var"]), z["lits"], z["off"], z["learnt"], z["lbd"], z["usage"])
    assert refgpu.input_digest(cnf) == entry["input_digest"], "fixture input does not regenerate"
    return cnf


def compare(got, entry):
    fields = fields_of(entry)
    for o in entry["outputs"]:
        want = o["canon"]
        if got["status"] != want["status"]:
            continue
        if got["status"] == 20 or all(got[k] == want[k] for k in fields):
            return []
    want = entry["outputs"][0]["canon"]
    if got["status"] != want["status"]:
        return [f"status {got['status']} vs {want['status']}"]
    return [d for d in refgpu.differences(got, want) if d.split(" ")[0] in fields]


SIMPLIFIED = [e for e in FIXTURES if e["input"] != "unsat-at-parse"]
IDS = [f"{e['case']}-{e['opts']}" for e in SIMPLIFIED]


def test_fixture_set_covers_the_families_and_option_sets():
    assert len(SIMPLIFIED) == 65
    assert {e["opts"] for e in SIMPLIFIED} == {"default", "p1_noere", "seq", "seq_p1_noere", "nofun"}
    full = [e for e in SIMPLIFIED if fields_of(e) == refgpu.FIELDS]
    assert len(full) >= 26
    # the reference gave one result per entry over its three runs
    assert all(len(e["outputs"]) == 1 and e["outputs"][0]["count"] == e["runs"] for e in SIMPLIFIED)


@pytest.mark.parametrize("entry", SIMPLIFIED, ids=IDS)
def test_oracle_matches_the_reference_gpu_simplifier(entry):
    cnf = input_of(entry)
    res = po.simplify(cnf, pg.options_from(**entry["engine_options"]))
    d = compare(refgpu.canon_result(res), entry)
    assert not d, "oracle differs from the reference: " + "; ".join(d)


@pytest.mark.gpu
@pytest.mark.parametrize("entry", SIMPLIFIED, ids=IDS)
def test_engine_matches_the_reference_gpu_simplifier(entry):
    cnf = input_of(entry)
    with pg.Simplifier(**entry["engine_options"]) as sim:
        res = sim.simplify(cnf)
    d = compare(refgpu.canon_result(res), entry)
    assert not d, "engine differs from the reference: " + "; ".join(d)
