"""Parity of the CUDA engine with the oracle (bit-exact canonical outputs).

Every test calls the engine through the C ABI (libpfgpu.so via ctypes) and
compares the canonical simplified CNF, eliminated-variable bytes, units and
model-reconstruction stack with the oracle on the same seeded input.
"""
import numpy as np
import pytest

import parafrost_gb300 as pg
from tests.parity import assert_parity

pytestmark = pytest.mark.gpu


def small_instance(seed):
    rng = np.random.default_rng(seed)
    fam = seed % 3
    if fam == 0:
        v = int(rng.integers(50, 400))
        return pg.random_ksat(v, int(v * rng.uniform(3.0, 4.5)), int(rng.integers(3, 5)), seed)
    if fam == 1:
        return pg.tseitin(int(rng.integers(100, 1500)), int(rng.integers(10, 60)), int(rng.integers(1, 8)), seed)
    return pg.scale_free(int(rng.integers(80, 600)), int(rng.integers(300, 2400)), seed)


@pytest.mark.parametrize("seed", range(1, 31))
def test_small_families_default_options(seed):
    assert_parity(small_instance(seed))


@pytest.mark.parametrize("seed", range(31, 51))
def test_small_families_aggressive(seed):
    # low freezing temperatures and minimum elections exercise more BVE/SUB rounds
    assert_parity(small_instance(seed), phases=5, mupos=10, muneg=10, electionsmin=1)


def test_config1_random_3sat_full_size():
    cnf = pg.random_ksat(20000, 85200, 3, seed=1)
    assert_parity(cnf, phases=1, ere=False)
    assert_parity(cnf)


def test_config2_tseitin_full_size():
    # 1M gates, 50k inputs, 1k outputs: ~3.25M clauses, 5 rounds of gate-definition BVE
    cnf = pg.tseitin(1_000_000, 50_000, 1_000, seed=1)
    res, ref = assert_parity(cnf)
    assert res.stats["rounds"] == 5 and res.cnf.num_clauses < cnf.num_clauses // 5


def test_config3_scalefree_reduced():
    # the scale-free family at 1/10 of its full size (planted model: all rounds run)
    cnf = pg.scale_free(400_000, 1_600_000, seed=1, planted=True)
    assert_parity(cnf)
