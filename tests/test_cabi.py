"""The C ABI used from C and C++ rather than Python.

tests/cabi/header_c.c compiles include/pfgpu.h as C99; tests/cabi/pfg_solve.cpp
is a C++ host of the library that runs the whole write-back sequence a
solver's simplify call site runs (DIMACS ingest, root units, pfg_create /
pfg_upload / pfg_simplify / pfg_result_sizes_get / pfg_download / pfg_destroy,
one batch, one served job, variable mapping, an external solver on the mapped
formula, model extension and a check of the model against the original
formula). On the GPU its simplify result must equal the Python path's, and
its end-to-end answer the reference CPU solver's on the original formula."""
import os
import re
import subprocess

import numpy as np
import pytest

import parafrost_gb300 as pg
from parafrost_gb300 import build as ebuild
from tests import refgpu

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
INCLUDE = os.path.join(ROOT, "include")
CALLER = os.path.join(HERE, "cabi", "pfg_solve.cpp")
OUT = os.path.join(ebuild.BUILD_DIR, "pfg_solve")
REF_SOLVER = os.path.join(ROOT, "oracle", "_ref", "parafrost")


def build_caller() -> str:
    os.makedirs(ebuild.BUILD_DIR, exist_ok=True)
    if not os.path.exists(OUT) or os.path.getmtime(OUT) < max(os.path.getmtime(CALLER), os.path.getmtime(ebuild.LIB)):
        subprocess.check_call(["g++", "-std=c++17", "-O2", "-Wall", "-I", INCLUDE, CALLER, "-L", ebuild.HERE,
                               "-lpfgpu", f"-Wl,-rpath,{ebuild.HERE}", "-o", OUT + ".tmp"])
        os.replace(OUT + ".tmp", OUT)
    return OUT


def test_header_compiles_as_c99(tmp_path):
    obj = tmp_path / "h.o"
    subprocess.check_call(["gcc", "-std=c99", "-Wall", "-Werror", "-pedantic", "-I", INCLUDE, "-c",
                           os.path.join(HERE, "cabi", "header_c.c"), "-o", str(obj)])
    syms = subprocess.run(["nm", str(obj)], capture_output=True, text=True).stdout
    assert "U pfg_default_options" in syms and "U pfg_abi_sizes" in syms


def test_cpp_caller_builds_and_links():
    exe = build_caller()
    deps = subprocess.run(["ldd", exe], capture_output=True, text=True).stdout
    assert "libpfgpu.so" in deps


def ref_status(path):
    out = subprocess.run([REF_SOLVER, path, "-quiet"], capture_output=True, text=True, timeout=120).stdout
    out = re.sub(r"\x1b\[[0-9;]*m", "", out)
    return 10 if "s SATISFIABLE" in out else (20 if "s UNSATISFIABLE" in out else 0)


CASES = [
    ("ksat", lambda: pg.random_ksat(2000, 8000, 3, 5), []),
    ("ksat_threshold", lambda: pg.random_ksat(150, 640, 3, 6), []),
    ("tseitin_units", lambda: pg.tseitin(3000, 150, 0, 7), [3100, -3050, 3001]),
    ("scalefree", lambda: pg.scale_free(3000, 12000, 8, planted=True), []),
]


@pytest.mark.gpu
@pytest.mark.parametrize("name,make,units", CASES, ids=[c[0] for c in CASES])
def test_cpp_caller_end_to_end(name, make, units, tmp_path):
    exe = build_caller()
    cnf = make()
    path = str(tmp_path / "in.cnf")
    pg.write_dimacs(cnf, path, extra_units=units)
    solver = [REF_SOLVER, "-model", "-modelprint", "-quiet"] if os.path.exists(REF_SOLVER) else []
    p = subprocess.run([exe, path, str(tmp_path), *solver], capture_output=True, text=True, timeout=300)
    assert p.returncode == 0, p.stdout + p.stderr
    lines = [l for l in p.stdout.splitlines() if l.startswith("result")]
    assert not any("FAILED" in l for l in lines), "\n".join(lines)
    for step in ("batch_instance_0", "batch_instance_1", "server_job"):
        assert f"result {step} ok" in lines
    status = int(next(l for l in lines if l.startswith("result status")).split()[2])
    # the C++ simplify result equals the Python path on the same upload
    if os.path.exists(tmp_path / "simp.out"):
        inp = refgpu.read_dump(str(tmp_path / "simp.in"), False)["cnf"]
        out = refgpu.read_dump(str(tmp_path / "simp.out"), True)
        with pg.Simplifier() as sim:
            res = sim.simplify(inp)
        mine = refgpu.canon(out["status"], out["cnf"], out["elim"], out["units"], out["pending"], out["stack"],
                            out["rounds"])
        assert not refgpu.differences(mine, refgpu.canon_result(res))
    if solver:
        assert status == ref_status(path), "end-to-end answer differs from the reference solver's"
        if status == 10:
            assert "result model_verified ok" in lines
