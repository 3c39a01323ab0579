"""CPU tests of the C ABI: the library loads and exports every entry point
include/pfgpu.h declares, struct layouts match, options and generators behave."""
import ctypes as C
import os
import re

import numpy as np
import pytest

import parafrost_gb300 as pg
from parafrost_gb300 import _abi, _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    src = open(os.path.join(ROOT, "include", "pfgpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(pfg_[a-z_]+)\s*\(", src)))


def test_library_exports_every_declared_entry_point():
    L = C.CDLL(_lib.LIB_PATH)
    names = declared_functions()
    assert len(names) >= 15
    for n in names:
        assert hasattr(L, n), f"{n} declared in include/pfgpu.h but not exported"
    assert set(_lib.EXPORTED) == set(names)


def test_struct_layouts_match_the_library():
    L = _lib.lib()
    a, b, c = C.c_size_t(), C.c_size_t(), C.c_size_t()
    L.pfg_abi_sizes(C.byref(a), C.byref(b), C.byref(c))
    assert a.value == C.sizeof(_abi.PfgOptions)
    assert b.value == C.sizeof(_abi.PfgStats)
    assert c.value == C.sizeof(_abi.PfgResultSizes)


def test_default_options_are_the_reference_defaults():
    L = _lib.lib()
    o = _abi.PfgOptions()
    L.pfg_default_options(C.byref(o))
    assert _abi.options_dict(o) == _abi.options_dict(_abi.default_options())
    # options.cpp:24-43 and options.cu:33-60
    assert (o.phases, o.shrink_rate, o.lcve_min_vars, o.lcve_max_occurs, o.lcve_clause_max) == (5, 2, 2, 3000, 30000)
    assert (o.phase_lits_min, o.mu_pos, o.mu_neg, o.ve_clause_max, o.xor_max_arity) == (500, 32, 32, 100, 10)
    assert (o.ve_en, o.ve_plus_en, o.sub_en, o.ere_en, o.bce_en, o.ve_fun_en, o.ve_lbound_en) == (1, 1, 1, 1, 0, 1, 0)


@pytest.mark.parametrize("kw,expect", [
    (dict(ve=False), dict(ve_en=1)),                                   # ve_en = ve || veextend
    (dict(ve=False, veextend=False), dict(ve_en=0, phases=1)),         # phases > 1 && !ve -> 1
    (dict(ve=False, veextend=False, sub=False), dict(phases=0)),       # nothing to run
    (dict(phases=0), dict(phases=1)),                                  # at least one phase
    (dict(all=True, ve=False, veextend=False), dict(ve_en=1, ere_en=1, bce_en=1)),
    (dict(ereclausemax=400), dict(ere_clause_max=250)),                # SH_MAX_ERE_OUT clamp
])
def test_option_folding(kw, expect):
    L = _lib.lib()
    o = _abi.options_from(**kw)
    L.pfg_resolve_options(C.byref(o))
    for k, v in expect.items():
        assert getattr(o, k) == v, (kw, k)


def test_cli_names_cover_every_option():
    assert set(_abi.CLI_NAMES.values()) | {"ve_inprocess"} >= {f[0] for f in _abi.PfgOptions._fields_ if f[0] != "_pad"}
    with pytest.raises(KeyError):
        _abi.options_from(not_an_option=1)


@pytest.mark.parametrize("family,a,b,c", [(0, 300, 1200, 3), (1, 500, 30, 5), (2, 400, 1500, 0), (2, 400, 1500, 1)])
def test_generators_are_seeded_and_well_formed(family, a, b, c):
    x = pg.generate(family, a, b, c, 7)
    y = pg.generate(family, a, b, c, 7)
    z = pg.generate(family, a, b, c, 8)
    assert np.array_equal(x.lits, y.lits) and np.array_equal(x.off, y.off)
    assert not (len(x.lits) == len(z.lits) and np.array_equal(x.lits, z.lits))
    sizes = np.diff(x.off)
    assert sizes.min() >= 2
    v = x.lits >> 1
    assert v.min() >= 1 and v.max() <= x.max_var
    for i in range(x.num_clauses):
        cv = v[x.off[i]:x.off[i + 1]]
        assert len(np.unique(cv)) == len(cv)


def test_tseitin_clause_mix():
    cnf = pg.tseitin(20000, 1000, 0, seed=3)     # no asserted outputs: nothing propagated
    per_gate = cnf.num_clauses / 20000
    assert 3.2 < per_gate < 3.4                   # 0.4*3 + 0.3*3 + 0.3*4 = 3.3
    assert 8.3 < cnf.num_literals / 20000 < 8.7   # 8.5 literals per gate


def test_planted_scalefree_is_satisfied_by_construction():
    from oracle import pyoracle as po
    cnf = pg.scale_free(200, 900, seed=4, planted=True)
    st, model = po.solve(cnf, 2_000_000)
    assert st == 10


def test_invalid_generator_arguments():
    with pytest.raises(ValueError):
        pg.generate(9, 1, 1, 1, 1)


def test_pinned_arrays_fall_back_without_a_device():
    from parafrost_gb300 import pinned
    a = pinned.empty(10, np.uint32)
    a[:] = np.arange(10)
    assert a.dtype == np.uint32 and a.sum() == 45
    b = pinned.copy(np.arange(5, dtype=np.uint64))
    assert b.tolist() == [0, 1, 2, 3, 4]
    buf = pinned.ResultBuffers()
    assert buf.get("lits", 7).size == 7 and buf.get("lits", 3).size == 3


def test_tuning_struct_layout():
    # pfg_tuning: seven uint32 knobs and nine reserved words, in header order
    src = open(os.path.join(ROOT, "include", "pfgpu.h")).read()
    body = src[src.index("typedef struct pfg_tuning {"):src.index("} pfg_tuning;")]
    names = re.findall(r"uint32_t\s+([a-z_0-9]+)", body)
    assert names == [f[0] for f in _abi.PfgTuning._fields_]
    assert C.sizeof(_abi.PfgTuning) == 64
