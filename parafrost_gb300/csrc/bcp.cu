// Device unit propagation of the units produced by SUB/BVE.
//
// Replaces Solver::prop (src/gpu/elimbcp.cu:144-215): a BFS over falsified
// literals whose frontier lives on the device; one warp scans one frontier
// literal's occurrence list. Assignments are claimed with atomicCAS, so the
// fixpoint (and a conflict) is independent of the schedule. Every level is a
// kernel launch; the host reads the frontier size only every 1, 2, 4 .. 64
// levels, and the level loop is bounded.
#include "engine.cuh"

namespace pfg {
namespace {

constexpr uint8_t BCP_UNSET = 0, BCP_TRUE = 1, BCP_FALSE = 2;

PFG_D uint32_t litval(const uint8_t* st, uint32_t lit) {
    const uint8_t s = st[ABSV(lit)];
    if (s == BCP_UNSET) return BCP_UNSET;
    const bool sat = SIGNL(lit) ? (s == BCP_FALSE) : (s == BCP_TRUE);
    return sat ? BCP_TRUE : BCP_FALSE;
}

PFG_D void assign_unit(uint8_t* st, uint8_t* elim, uint32_t unit, uint32_t* front_next, DevCounters* dc,
                       uint32_t* trail, uint32_t trail_cap, uint32_t V) {
    const uint32_t v = ABSV(unit);
    if (v == 0 || v > V) { atomicOr(&dc->err, ERR_BAD_LIT); return; }
    const uint8_t desired = SIGNL(unit) ? BCP_FALSE : BCP_TRUE;
    // byte-granular CAS through the containing word
    unsigned int* word = (unsigned int*)((uintptr_t)(st + v) & ~(uintptr_t)3);
    const unsigned int shift = (unsigned int)(((uintptr_t)(st + v) & 3u) * 8u);
    unsigned int old = *((volatile unsigned int*)word);
    for (int it = 0; it < 64; it++) {  // bounded: 4 bytes can change at most 4 times
        const uint8_t cur = (uint8_t)((old >> shift) & 0xFFu);
        if (cur != BCP_UNSET) {
            if (cur != desired) dc->conflict = 1;
            return;
        }
        const unsigned int nw = (old & ~(0xFFu << shift)) | ((unsigned int)desired << shift);
        const unsigned int prev = atomicCAS(word, old, nw);
        if (prev == old) {
            elim[v] |= FORCED_MASK;
            const uint32_t t = atomicAdd(&dc->ntrail, 1u);
            if (t < trail_cap) trail[t] = unit; else atomicOr(&dc->err, ERR_UNITS_OVERFLOW);
            front_next[atomicAdd(&dc->bcp_next, 1u)] = FLIPL(unit);
            return;
        }
        old = prev;
    }
}

__global__ void bcp_seed_k(uint8_t* st, uint8_t* elim, const uint32_t* units, uint32_t nunits, uint32_t* front,
                           DevCounters* dc, uint32_t* trail, uint32_t trail_cap, uint32_t V) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < nunits; i += gridDim.x * blockDim.x)
        assign_unit(st, elim, units[i], front, dc, trail, trail_cap, V);
}

__global__ void bcp_advance_k(DevCounters* dc) {
    dc->bcp_curr = dc->bcp_next;
    dc->bcp_next = 0;
    dc->bcp_level++;
}

// warp per frontier literal, lanes stride its occurrence list
__global__ void bcp_propagate_k(const ClsHdr* hdr, const uint32_t* lits, const uint32_t* ot_off,
                                const uint32_t* ot_size, const uint32_t* ot_ids, uint8_t* st, uint8_t* elim,
                                const uint32_t* front_a, uint32_t* front_b, DevCounters* dc,
                                uint32_t* trail, uint32_t trail_cap, uint32_t V) {
    if (dc->conflict) return;
    const uint32_t level = dc->bcp_level;
    const uint32_t* cur = (level & 1u) ? front_b : (uint32_t*)front_a;
    uint32_t* nxt = (level & 1u) ? (uint32_t*)front_a : front_b;
    const uint32_t n = dc->bcp_curr;
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
    const unsigned lane = threadIdx.x & 31u;
    for (uint32_t fi = warp; fi < n; fi += nwarps) {
        const uint32_t f = cur[fi];
        const uint32_t o = ot_off[f], sz = ot_size[f];
        for (uint32_t j = lane; j < sz; j += 32) {
            const ClsHdr h = hdr[ot_ids[o + j]];
            if (m_deleted(h.meta)) continue;
            uint32_t unit = 0;
            int nunset = 0;
            bool sat = false;
            for (uint32_t k = 0; k < h.size; k++) {
                const uint32_t l = lits[h.off + k];
                const uint32_t ve = litval(st, l);
                if (ve == BCP_TRUE) { sat = true; break; }
                if (ve == BCP_UNSET) { unit = l; if (++nunset > 1) break; }
            }
            if (sat) continue;
            if (!nunset) dc->conflict = 1;
            else if (nunset == 1) assign_unit(st, elim, unit, nxt, dc, trail, trail_cap, V);
        }
    }
}

__global__ void bcp_apply_k(ClsHdr* hdr, uint32_t* lits, uint64_t ncls, const uint8_t* st) {
    for (uint64_t c = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; c < ncls; c += (uint64_t)gridDim.x * blockDim.x) {
        ClsHdr h = hdr[c];
        if (m_deleted(h.meta)) continue;
        uint32_t* l = lits + h.off;
        uint32_t sig = 0, n = 0;
        bool sat = false;
        for (uint32_t k = 0; k < h.size; k++) {
            const uint32_t lit = l[k];
            const uint32_t ve = litval(st, lit);
            if (ve == BCP_TRUE) { sat = true; break; }
            if (ve == BCP_FALSE) continue;
            l[n++] = lit;
            sig |= MAPHASH(lit);
        }
        if (sat) hdr[c].meta = m_set_st(h.meta, ST_DELETED);
        else { hdr[c].sig = sig; hdr[c].size = n; }
    }
}

}  // namespace

// Returns false on a CUDA/engine error; `ok` = false on a conflict (UNSAT).
bool bcp_prop(Ctx& c, bool& ok) {
    ok = true;
    if (!c.nUnits) return true;
    cudaMemsetAsync(c.bstate, 0, c.V + 1, c.s);
    cudaMemsetAsync(&c.dc->conflict, 0, sizeof(uint32_t), c.s);
    cudaMemsetAsync(&c.dc->bcp_curr, 0, 3 * sizeof(uint32_t), c.s);
    const uint32_t trail_before = c.hc->ntrail;
    // seed: assigned literals go to front_a through bcp_next, then advance to level 0
    PFG_LAUNCH(K_BCP, bcp_seed_k, grid_for(c.nUnits, 256), 256, 0, c.s, c.bstate, c.elim, c.units, (uint32_t)c.nUnits, c.front_a,
                                                        c.dc, c.trail, c.trail_cap, c.V);
    PFG_LAUNCH(K_BCP, bcp_advance_k, 1, 1, 0, c.s, c.dc);   // curr = seeded, level = 1
    // make level parity start at 0 with the seeds in front_a
    cudaMemsetAsync(&c.dc->bcp_level, 0, sizeof(uint32_t), c.s);
    const unsigned grid = 152 * 8;
    uint32_t levels = 0;
    const uint32_t max_levels = c.V + 2;   // every level assigns at least one new variable
    for (int batch = 1;; batch = std::min(batch << 1, 64)) {
        for (int b = 0; b < batch; b++) {
            PFG_LAUNCH(K_BCP, bcp_propagate_k, grid, 256, 0, c.s, c.hdr, c.lits, c.ot_off, c.ot_size, c.ot_ids, c.bstate, c.elim,
                                                   c.front_a, c.front_b, c.dc, c.trail, c.trail_cap, c.V);
            PFG_LAUNCH(K_BCP, bcp_advance_k, 1, 1, 0, c.s, c.dc);
        }
        levels += batch;
        sync_counters(c);
        if (!c.err.empty()) return false;
        if (c.hc->conflict || !c.hc->bcp_curr) break;
        if (levels > max_levels) { c.err = "device unit propagation did not converge"; c.simpstate = PFG_TIMEOUT; return false; }
    }
    if (c.hc->err) { c.err = "device error during unit propagation"; return false; }
    if (c.hc->conflict) { ok = false; return true; }
    PFG_LAUNCH(K_BCP, bcp_apply_k, grid_for(c.ncls, 256), 256, 0, c.s, c.hdr, c.lits, c.ncls, c.bstate);
    (void)trail_before;
    return cuda_ok(c, cudaGetLastError(), "bcp");
}

}  // namespace pfg
