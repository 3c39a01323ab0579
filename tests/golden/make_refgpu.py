"""Generates the reference-GPU golden fixtures (tests/golden/refgpu).

Runs on a GPU host after
    python -c "import __graft_entry__ as g; g.build()"
    python oracle/ref_gpu_build.py build
For every seeded instance below and every option set it writes the instance
as DIMACS, runs the reference's own GPU simplifier on it `--repeats` times
(oracle/_ref/gpu/pfref_gpu: the unmodified src/gpu sources with the
oracle/refgpu harness), and records the canonical digests of each distinct
result (tests/refgpu.py) with how often it occurred: the reference elects
with Luby MIS and appends through atomics, so a result may vary between
runs. The input is the clause database as the reference hands it to awaken
(after parsing and root propagation); for instances without unit clauses it
equals the generator's output, otherwise it is stored beside the fixtures.

It then runs the oracle (oracle/pfo.c) and the engine (libpfgpu.so) on the
same input with the same options and prints whether each equals one of the
reference's results, so one run shows the parity picture.

    python tests/golden/make_refgpu.py --out DIR [--repeats 3] [--only NAME]
"""
import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

import parafrost_gb300 as pg  # noqa: E402
from oracle import pyoracle as po  # noqa: E402
import refgpu  # noqa: E402

BIN = os.path.join(ROOT, "oracle", "_ref", "gpu", "pfref_gpu")

# (name, family, a, b, c, seed): families 0 random k-SAT (vars, clauses, k),
# 1 Tseitin circuit (gates, inputs, outputs), 2 scale-free (vars, clauses, planted)
CASES = [
    ("ksat300_s1", 0, 300, 1278, 3, 1),
    ("ksat300_s2", 0, 300, 1278, 3, 2),
    ("ksat1k", 0, 1000, 4260, 3, 3),
    ("ksat3k", 0, 3000, 12780, 3, 4),
    ("k5sat500", 0, 500, 4000, 5, 5),
    ("ksat20k", 0, 20000, 85200, 3, 1),
    ("tseitin1k", 1, 1000, 100, 0, 6),
    ("tseitin5k", 1, 5000, 300, 0, 7),
    ("tseitin2k_units", 1, 2000, 150, 20, 8),
    ("tseitin20k", 1, 20000, 1000, 0, 9),
    ("sfree2k", 2, 2000, 8000, 1, 10),
    ("sfree10k", 2, 10000, 40000, 1, 11),
    ("sfree3k_unplanted", 2, 3000, 12000, 0, 12),
]

# (name, reference CLI flags, engine options)
OPTSETS = [
    ("default", [], {}),
    ("p1_noere", ["--phases=1", "-no-ere"], {"phases": 1, "ere": False}),
    ("seq", ["-no-lcvefast"], {"lcvefast": False}),
    ("seq_p1_noere", ["-no-lcvefast", "--phases=1", "-no-ere"], {"lcvefast": False, "phases": 1, "ere": False}),
    ("nofun", ["-no-vefunction"], {"vefunction": False}),
]


def run_reference(dimacs, prefix, flags):
    t0 = time.perf_counter()
    p = subprocess.run([BIN, dimacs, prefix, *flags, "--verbose=0"], capture_output=True, text=True, timeout=600)
    dt = time.perf_counter() - t0
    if p.returncode != 0 or not os.path.exists(prefix + ".out"):
        raise RuntimeError(f"reference run failed ({p.returncode}):\n{p.stdout[-2000:]}\n{p.stderr[-2000:]}")
    inp = refgpu.read_dump(prefix + ".in", False) if os.path.exists(prefix + ".in") else None
    out = refgpu.read_dump(prefix + ".out", True)
    return inp, out, dt


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", required=True)
    ap.add_argument("--repeats", type=int, default=3)
    ap.add_argument("--only", default="")
    ap.add_argument("--no-engine", action="store_true")
    a = ap.parse_args()
    os.makedirs(a.out, exist_ok=True)
    fixtures = []
    summary = []
    tmp = tempfile.mkdtemp(prefix="refgpu_")
    for (name, fam, x, y, z, seed) in CASES:
        if a.only and a.only not in name:
            continue
        gen = pg.generate(fam, x, y, z, seed)
        dimacs = os.path.join(tmp, name + ".cnf")
        pg.write_dimacs(gen, dimacs)
        gen_digest = refgpu.input_digest(gen)
        for (oname, flags, eopts) in OPTSETS:
            outs = {}
            inp_cnf = None
            times = []
            for r in range(a.repeats):
                prefix = os.path.join(tmp, f"{name}__{oname}__{r}")
                inp, out, dt = run_reference(dimacs, prefix, flags)
                times.append(dt)
                if inp is not None and "cnf" in inp:
                    if inp_cnf is None:
                        inp_cnf = inp["cnf"]
                    elif refgpu.input_digest(inp["cnf"]) != refgpu.input_digest(inp_cnf):
                        raise RuntimeError(f"{name}: the reference saw different inputs across runs")
                if out["status"] == 20:
                    c = {"status": 20}
                else:
                    c = refgpu.canon(out["status"], out["cnf"], out["elim"], out["units"], out["pending"],
                                     out["stack"], out["rounds"])
                key = json.dumps(c, sort_keys=True)
                outs.setdefault(key, {"canon": c, "count": 0})["count"] += 1
            entry = {"case": name, "generator": [fam, x, y, z, seed], "opts": oname, "cli": flags,
                     "engine_options": eopts, "runs": a.repeats, "outputs": list(outs.values()),
                     "ref_seconds": [round(t, 3) for t in times]}
            if inp_cnf is None:
                # the reference found the conflict while parsing, before simplify
                entry["input"] = "unsat-at-parse"
                print(f"{name:20s} {oname:13s} UNSAT before simplify", flush=True)
                fixtures.append(entry)
                continue
            in_digest = refgpu.input_digest(inp_cnf)
            entry["input_digest"] = in_digest
            entry["input"] = "generator" if in_digest == gen_digest else f"{name}.npz"
            if entry["input"] != "generator":
                np.savez_compressed(os.path.join(a.out, f"{name}.npz"), max_var=inp_cnf.max_var, lits=inp_cnf.lits,
                                    off=inp_cnf.off, learnt=inp_cnf.learnt, lbd=inp_cnf.lbd, usage=inp_cnf.usage)
            # oracle and engine on the same input
            o = po.simplify(inp_cnf, pg.options_from(**eopts))
            ok_o, info_o = refgpu.matches_any(refgpu.canon_result(o), entry["outputs"])
            entry["oracle_matches"] = ok_o
            line = f"{name:20s} {oname:13s} ref distinct={len(outs)} counts={[v['count'] for v in outs.values()]} " \
                   f"oracle={'ok' if ok_o else info_o}"
            if not a.no_engine:
                with pg.Simplifier(**eopts) as s:
                    e = s.simplify(inp_cnf)
                ok_e, info_e = refgpu.matches_any(refgpu.canon_result(e), entry["outputs"])
                entry["engine_matches"] = ok_e
                line += f" engine={'ok' if ok_e else info_e}"
            print(line, flush=True)
            summary.append(line)
            fixtures.append(entry)
            with open(os.path.join(a.out, "fixtures.json"), "w") as f:
                json.dump({"bin": "oracle/_ref/gpu/pfref_gpu (reference src/gpu + oracle/refgpu)",
                           "fixtures": fixtures}, f, indent=1)
    with open(os.path.join(a.out, "summary.txt"), "w") as f:
        f.write("\n".join(summary) + "\n")


if __name__ == "__main__":
    main()
