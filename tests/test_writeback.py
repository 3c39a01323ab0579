"""Write-back into a host solver: variable mapping (pfg_map_vars/pfg_map_lits)
and model reconstruction (pfg_extend_model), exercised on the oracle's results
(the same layout the engine downloads; the GPU tests run the engine's). A
mapped formula is solved -- by the oracle's DPLL, and by the reference's own
CPU solver when it was built here -- and its model is taken back through the
mapping and the model stack to a model of the original formula."""
import os
import re
import subprocess

import numpy as np
import pytest

import parafrost_gb300 as pg
from oracle import pyoracle as po

HERE = os.path.dirname(os.path.abspath(__file__))
REF_SOLVER = os.path.join(os.path.dirname(HERE), "oracle", "_ref", "parafrost")


def small(seed):
    rng = np.random.default_rng(seed)
    fam = seed % 3
    if fam == 0:
        v = int(rng.integers(40, 120))
        return pg.random_ksat(v, int(v * rng.uniform(3.0, 4.1)), 3, seed)
    if fam == 1:
        return pg.tseitin(int(rng.integers(60, 200)), int(rng.integers(8, 20)), int(rng.integers(1, 3)), seed)
    return pg.scale_free(int(rng.integers(60, 150)), int(rng.integers(200, 500)), seed, planted=True)


def with_units(cnf, units):
    """The mapped clauses plus the pending units as one-literal clauses."""
    ints = [cnf.clause(i).tolist() for i in range(cnf.num_clauses)] + [[int(u)] for u in units]
    lits = np.array([l for c in ints for l in c], dtype=np.uint32)
    off = np.concatenate([[0], np.cumsum([len(c) for c in ints])]).astype(np.uint64)
    return pg.Cnf(cnf.max_var, lits, off)


def solve_dpll(cnf):
    status, model = po.solve(cnf, 50_000_000)
    return status, model


def test_mapping_renumbers_active_variables():
    cnf = small(4)
    res = po.simplify(cnf, pg.options_from(mupos=10, muneg=10, electionsmin=1))
    m = pg.map_result(res)
    active = np.nonzero(res.eliminated == 0)[0]
    active = active[active > 0]
    assert m.cnf.max_var == len(active)
    assert m.old_of_new[1:].tolist() == active.tolist()
    if m.cnf.num_clauses:
        assert int((m.cnf.lits >> 1).max()) <= m.cnf.max_var and int((m.cnf.lits >> 1).min()) >= 1
        back = m.old_of_new[m.cnf.lits >> 1] * 2 + (m.cnf.lits & 1)
        assert np.array_equal(back, res.cnf.lits)


@pytest.mark.parametrize("seed", range(1, 31))
def test_model_of_mapped_formula_extends_to_the_original(seed):
    cnf = small(seed)
    res = po.simplify(cnf, pg.options_from(mupos=10, muneg=10, electionsmin=1, bce=bool(seed % 2)))
    orig_status, _ = solve_dpll(cnf)
    if int(res.status) == pg.PFG_UNSAT:
        assert orig_status == 20
        return
    m = pg.map_result(res)
    status, model = solve_dpll(with_units(m.cnf, m.units))
    assert status == orig_status
    if status == 10:
        value = pg.reconstruct_model(res, m, model)
        assert po.satisfies(cnf, value)


def reference_solve(cnf, tmp_path):
    path = tmp_path / "m.cnf"
    pg.write_dimacs(cnf, str(path))
    out = subprocess.run([REF_SOLVER, str(path), "-model", "-modelprint", "-quiet"], capture_output=True,
                         text=True, timeout=300).stdout
    out = re.sub(r"\x1b\[[0-9;]*m", "", out)
    status = 10 if "s SATISFIABLE" in out else (20 if "s UNSATISFIABLE" in out else 0)
    model = np.zeros(cnf.max_var + 1, dtype=np.uint8)
    for line in out.splitlines():
        if line.startswith("v"):
            for tok in line[1:].split():
                x = int(tok)
                if x > 0:
                    model[x] = 1
    return status, model


@pytest.mark.skipif(not os.path.exists(REF_SOLVER), reason="the reference's CPU solver was not built here")
@pytest.mark.parametrize("seed", range(1, 13))
def test_reference_solver_on_the_mapped_formula(seed, tmp_path):
    cnf = small(seed) if seed % 4 else pg.random_ksat(3000, 10500, 3, seed)
    res = po.simplify(cnf, pg.options_from())
    orig, _ = reference_solve(cnf, tmp_path)
    assert orig in (10, 20)
    if int(res.status) == pg.PFG_UNSAT:
        assert orig == 20
        return
    m = pg.map_result(res)
    mapped = with_units(m.cnf, m.units)
    if mapped.num_clauses == 0:
        status, model = 10, np.zeros(mapped.max_var + 1, dtype=np.uint8)
    else:
        status, model = reference_solve(mapped, tmp_path)
    assert status == orig
    if status == 10:
        value = pg.reconstruct_model(res, m, model)
        assert po.satisfies(cnf, value)


def test_extend_model_matches_the_oracle():
    import ctypes as C
    cnf = small(7)
    res = po.simplify(cnf, pg.options_from(mupos=10, muneg=10, electionsmin=1))
    rng = np.random.default_rng(7)
    value = rng.integers(0, 2, cnf.max_var + 1).astype(np.uint8)
    want = po.extend_model(res.stack, value)
    got = value.copy()
    st = np.ascontiguousarray(res.stack, dtype=np.uint32)
    assert pg._lib.lib().pfg_extend_model(len(st), st.ctypes.data_as(C.POINTER(C.c_uint32)), cnf.max_var,
                                          got.ctypes.data_as(C.POINTER(C.c_uint8))) == 0
    assert np.array_equal(got[1:], want[1:])
