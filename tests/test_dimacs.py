"""Native DIMACS ingest (pfg_dimacs_read): normalisation as the reference's
parser does it (src/gpu/dimacs.cpp:226-290) and its error reports. Host code
only: runs without a GPU."""
import numpy as np
import pytest

import parafrost_gb300 as pg


def reference_rules(text):
    """The parser's rules restated in Python: (max_var, clauses, units, status)."""
    max_var, clauses, units, value = 0, [], [], {}
    toks = []
    for line in text.splitlines():
        s = line.strip()
        if not s or s[0] == "c":
            continue
        if s[0] == "p":
            max_var = int(s.split()[2])
            continue
        toks += [int(t) for t in s.split()]
    cur = []
    for t in toks:
        if t:
            cur.append(t)
            continue
        seen, out, sat = set(), [], False
        for x in cur:
            if x in seen:
                continue
            if -x in seen:
                sat = True
                continue
            seen.add(x)
            v = value.get(abs(x))
            if v is None:
                out.append(x)
            elif v == (x > 0):
                sat = True
        cur = []
        if sat:
            continue
        if not out:
            return max_var, clauses, units, 20
        if len(out) == 1:
            value[abs(out[0])] = out[0] > 0
            units.append(out[0])
            continue
        clauses.append(out)
    return max_var, clauses, units, 0


def enc(x):
    return 2 * abs(x) + (1 if x < 0 else 0)


def check(tmp_path, text):
    path = tmp_path / "f.cnf"
    path.write_text(text)
    cnf, units, status = pg.parse_dimacs(str(path))
    V, clauses, want_units, want_status = reference_rules(text)
    assert status == want_status
    assert cnf.max_var == V
    if status == 0:
        assert cnf.num_clauses == len(clauses)
        got = [cnf.clause(i).tolist() for i in range(cnf.num_clauses)]
        assert got == [[enc(x) for x in c] for c in clauses]
        assert units.tolist() == [enc(x) for x in want_units]
    return cnf, units, status


def test_plain_file_round_trips(tmp_path):
    cnf = pg.random_ksat(300, 1200, 3, 5)
    path = tmp_path / "k.cnf"
    pg.write_dimacs(cnf, str(path))
    got, units, status = pg.parse_dimacs(str(path))
    assert status == 0 and len(units) == 0
    assert np.array_equal(got.lits, cnf.lits) and np.array_equal(got.off, cnf.off)


def test_duplicates_tautologies_and_units(tmp_path):
    text = """c comment
p cnf 6 9
1 2 2 3 0
4 -4 5 0
-6 0
6 1 2 0
-6 3 4 0
1 -3
  5 0
c another comment
2 -1 2 0
5 5 0
3 -5 0
"""
    cnf, units, status = check(tmp_path, text)
    assert status == 0 and units.tolist() == [enc(-6), enc(5), enc(3)]


def test_empty_clause_and_conflicting_units(tmp_path):
    _, _, status = check(tmp_path, "p cnf 3 3\n1 2 0\n0\n2 3 0\n")
    assert status == 20
    _, _, status = check(tmp_path, "p cnf 3 3\n1 0\n-1 0\n2 3 0\n")
    assert status == 20


@pytest.mark.parametrize("seed", range(6))
def test_random_noisy_files(tmp_path, seed):
    rng = np.random.default_rng(seed)
    V = 40
    lines = [f"p cnf {V} 200"]
    for _ in range(200):
        k = int(rng.integers(1, 6))
        c = [int(x) * (1 if rng.random() < 0.5 else -1) for x in rng.integers(1, V + 1, k)]
        lines.append(" ".join(map(str, c)) + " 0")
        if rng.random() < 0.1:
            lines.append("c noise")
    check(tmp_path, "\n".join(lines) + "\n")


@pytest.mark.parametrize("text,msg", [
    ("1 2 0\n", "expected"),
    ("p cnf 0 1\n1 0\n", "variables"),
    ("p cnf 3 0\n", "clauses"),
    ("p cnf 3 1\n1 7 0\n", "too many variables"),
    ("p cnf 3 1\n1 2", "unterminated"),
    ("p dnf 3 1\n1 2 0\n", "header"),
])
def test_errors(tmp_path, text, msg):
    path = tmp_path / "bad.cnf"
    path.write_text(text)
    with pytest.raises(ValueError) as e:
        pg.parse_dimacs(str(path))
    assert msg in str(e.value)


def test_missing_file(tmp_path):
    with pytest.raises(ValueError) as e:
        pg.parse_dimacs(str(tmp_path / "nope.cnf"))
    assert "cannot open" in str(e.value)
