"""Generate tests/golden/ref_sat.json: satisfiability answers of the
reference's own CPU solver on seeded instances (run in the container where
the reference sources are present; the GPU machine only reads the JSON).

For each instance (generator family, sizes, seed) the instance is written as
DIMACS and solved by oracle/_ref/parafrost (compiled from the reference's
src/cpu by oracle/ref_build.py) with `-model -modelverify`; the answer
(10 SAT / 20 UNSAT) and whether its model verified are recorded.
"""
import json
import os
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import parafrost_gb300 as pg  # noqa: E402
from oracle import ref_build  # noqa: E402


def instances():
    out = []
    for seed in range(1, 41):
        out.append({"family": 0, "a": 60 + 5 * (seed % 8), "b": int((60 + 5 * (seed % 8)) * 4.2), "c": 3, "seed": seed})
    for seed in range(1, 31):
        out.append({"family": 1, "a": 150 + 20 * (seed % 7), "b": 12 + (seed % 5), "c": 1 + seed % 4, "seed": seed})
    for seed in range(1, 31):
        out.append({"family": 2, "a": 80 + 10 * (seed % 6), "b": 300 + 40 * (seed % 6), "c": seed % 2, "seed": seed})
    # larger ones for the GPU tests
    out.append({"family": 0, "a": 2000, "b": 8520, "c": 3, "seed": 11})
    out.append({"family": 1, "a": 20000, "b": 1000, "c": 20, "seed": 5})
    out.append({"family": 2, "a": 20000, "b": 80000, "c": 1, "seed": 3})
    return out


def solve(cnf):
    with tempfile.NamedTemporaryFile("w", suffix=".cnf", delete=False) as f:
        path = f.name
    try:
        pg.write_dimacs(cnf, path)
        p = subprocess.run([ref_build.BIN, path, "-model", "-modelverify", "--verbose=1", "--timeout=120"],
                           capture_output=True, text=True, timeout=300)
        out = p.stdout
        ans = 10 if "s SATISFIABLE" in out else (20 if "s UNSATISFIABLE" in out else 0)
        verified = "VERIFIED" in out
        return ans, verified
    finally:
        os.unlink(path)


def main():
    ref_build.build()
    rows = []
    for inst in instances():
        cnf = pg.generate(inst["family"], inst["a"], inst["b"], inst["c"], inst["seed"])
        ans, ok = solve(cnf)
        rows.append(dict(inst, answer=ans, model_verified=ok, clauses=int(cnf.num_clauses)))
        print(rows[-1], flush=True)
    with open(os.path.join(HERE, "ref_sat.json"), "w") as f:
        json.dump({"solver": "reference src/cpu (oracle/_ref/parafrost)", "instances": rows}, f, indent=1)


if __name__ == "__main__":
    main()
