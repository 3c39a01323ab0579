"""The allocation-free device write-back, pfg_download_device_noalloc.

Called through the C ABI with device buffers owned by the test, it must give
exactly the clauses pfg_download gives, on two calls in a row and after
other contexts have used the device. This file is collected last on purpose:
it must pass both alone and after the rest of the suite."""
import ctypes as C

import numpy as np
import pytest

import parafrost_gb300 as pg
from parafrost_gb300 import _abi
from tests.test_gpu_variants import inst, with_learnts

pytestmark = pytest.mark.gpu


def device_download(sim, want=("lits", "off", "learnt", "lbd", "usage")):
    import torch
    sz = _abi.PfgResultSizes()
    assert sim.lib.pfg_result_sizes_get(sim._ctx, C.byref(sz)) == 0
    nc, nl = int(sz.clauses), int(sz.literals)
    # pre-filled with a pattern, so a word the call fails to write shows up
    bufs = {
        "lits": torch.full((max(nl, 1),), 0x55555555, dtype=torch.int32, device="cuda"),
        "off": torch.full((nc + 1,), -1, dtype=torch.int64, device="cuda"),
        "learnt": torch.full((max(nc, 1),), 0xAA, dtype=torch.uint8, device="cuda"),
        "lbd": torch.full((max(nc, 1),), -1, dtype=torch.int32, device="cuda"),
        "usage": torch.full((max(nc, 1),), 0xAA, dtype=torch.uint8, device="cuda"),
    }
    ptr = {k: (bufs[k].data_ptr() if k in want else None) for k in bufs}
    rc = sim.lib.pfg_download_device_noalloc(sim._ctx, ptr["lits"], ptr["off"], ptr["learnt"], ptr["lbd"],
                                             ptr["usage"])
    assert rc == 0, sim.lib.pfg_last_error(sim._ctx)
    return {
        "lits": bufs["lits"].cpu().numpy().view(np.uint32)[:nl],
        "off": bufs["off"].cpu().numpy().view(np.uint64),
        "learnt": bufs["learnt"].cpu().numpy()[:nc],
        "lbd": bufs["lbd"].cpu().numpy().view(np.uint32)[:nc],
        "usage": bufs["usage"].cpu().numpy()[:nc],
    }


def expected(res):
    c = res.cnf
    return {"lits": c.lits, "off": c.off, "learnt": c.learnt, "lbd": c.lbd, "usage": c.usage}


@pytest.mark.parametrize("seed", [3, 4, 5])
def test_same_clauses_as_download_on_two_calls(seed):
    cnf = with_learnts(inst(seed, scale=2), seed)
    with pg.Simplifier(mupos=10, muneg=10) as sim:
        sim.upload(cnf)
        sim.run()
        want = expected(sim.download())
        for _ in range(2):
            got = device_download(sim)
            for k in want:
                assert np.array_equal(got[k], want[k]), f"{k} differs from pfg_download"


def test_before_simplify_and_with_missing_outputs():
    cnf = with_learnts(inst(7), 7)
    with pg.Simplifier() as sim:
        sim.upload(cnf)
        got = device_download(sim, want=("lits", "off"))
        # the upload sorts the literals of every clause (prep_cnf_k)
        sorted_lits = np.concatenate([np.sort(cnf.clause(i)) for i in range(cnf.num_clauses)])
        assert np.array_equal(got["lits"], sorted_lits) and np.array_equal(got["off"], cnf.off)
        sim.run()
        want = expected(sim.download())
        got = device_download(sim, want=("learnt", "usage"))
        assert np.array_equal(got["learnt"], want["learnt"]) and np.array_equal(got["usage"], want["usage"])


def test_store_beyond_the_scratch_is_rejected():
    cnf = pg.random_ksat(400_000, 1_704_000, 3, 1)
    with pg.Simplifier() as sim:
        sim.upload(cnf)
        rc = sim.lib.pfg_download_device_noalloc(sim._ctx, None, None, None, None, None)
        assert rc == 5
        assert b"at most" in sim.lib.pfg_last_error(sim._ctx)


def test_batch_context_is_rejected():
    with pg.Simplifier() as sim:
        sim.upload_batch([inst(1), inst(2)])
        assert sim.lib.pfg_download_device_noalloc(sim._ctx, None, None, None, None, None) == 5


def test_second_call_allocates_no_device_memory():
    """Device memory in use is the same before and after a call: the caller's
    buffers are made first, one call warms the module up, then the free bytes
    the driver reports and torch's allocator counters must not move."""
    import torch
    cnf = with_learnts(inst(4, scale=2), 4)
    with pg.Simplifier() as sim:
        sim.upload(cnf)
        sim.run()
        want = expected(sim.download())
        sz = _abi.PfgResultSizes()
        assert sim.lib.pfg_result_sizes_get(sim._ctx, C.byref(sz)) == 0
        nc, nl = int(sz.clauses), int(sz.literals)
        lits = torch.empty(max(nl, 1), dtype=torch.int32, device="cuda")
        off = torch.empty(nc + 1, dtype=torch.int64, device="cuda")

        def call():
            return sim.lib.pfg_download_device_noalloc(sim._ctx, lits.data_ptr(), off.data_ptr(), None, None, None)

        assert call() == 0, sim.lib.pfg_last_error(sim._ctx)
        torch.cuda.synchronize()
        free0 = torch.cuda.mem_get_info()[0]
        alloc0, reserved0 = torch.cuda.memory_allocated(), torch.cuda.memory_reserved()
        assert call() == 0, sim.lib.pfg_last_error(sim._ctx)
        torch.cuda.synchronize()
        assert torch.cuda.mem_get_info()[0] == free0, "free device memory changed across the call"
        assert torch.cuda.memory_allocated() == alloc0 and torch.cuda.memory_reserved() == reserved0
        assert np.array_equal(lits.cpu().numpy().view(np.uint32)[:nl], want["lits"])
        assert np.array_equal(off.cpu().numpy().view(np.uint64), want["off"])
