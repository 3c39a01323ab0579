// Device unit propagation of the units produced by SUB/BVE.
//
// Replaces Solver::prop (src/gpu/elimbcp.cu:144-215): a BFS over falsified
// literals whose frontier lives on the device; one warp scans one frontier
// literal's occurrence list, and the lists longer than BCP_LONG (hub literals
// of skewed instances) are spread over every thread of the grid instead, so
// one long list does not hold up its level. Assignments are claimed with atomicCAS, so the
// fixpoint (and a conflict) is independent of the schedule. Every level is a
// kernel launch; the host reads the frontier size only every 1, 2, 4 .. 64
// levels, and the level loop is bounded. With several instances, each one
// seeds from its own unit region, records its own trail and conflict, and a
// conflicting instance is left unchanged (its clauses are not rewritten), as
// the reference leaves the CNF of an instance whose propagation conflicted.
#include "engine.cuh"

namespace pfg {
namespace {

constexpr uint8_t BCP_UNSET = 0, BCP_TRUE = 1, BCP_FALSE = 2;

struct BK {
    uint8_t* st;
    uint8_t* elim;
    const uint32_t* vinst;
    const unsigned long long* tbase;
    const uint32_t* tcap;
    uint32_t* tcount;
    uint32_t* conflict;
    uint32_t* trail;
    DevCounters* dc;
    const uint32_t* ot_size;
    uint32_t* long_next;     // frontier literals with long lists, next level
    uint32_t V;
};

constexpr uint32_t BCP_LONG = 1024;   // lists longer than this are split over the grid

PFG_D uint32_t litval(const uint8_t* st, uint32_t lit) {
    const uint8_t s = st[ABSV(lit)];
    if (s == BCP_UNSET) return BCP_UNSET;
    const bool sat = SIGNL(lit) ? (s == BCP_FALSE) : (s == BCP_TRUE);
    return sat ? BCP_TRUE : BCP_FALSE;
}

PFG_D void set_conflict(const BK& k, uint32_t inst) {
    k.conflict[inst] = 1;
    k.dc->conflict = 1;
}

PFG_D void assign_unit(const BK& k, uint32_t unit, uint32_t* front_next) {
    const uint32_t v = ABSV(unit);
    if (v == 0 || v > k.V) { atomicOr(&k.dc->err, ERR_BAD_LIT); return; }
    const uint32_t inst = k.vinst[v];
    const uint8_t desired = SIGNL(unit) ? BCP_FALSE : BCP_TRUE;
    // byte-granular CAS through the containing word
    unsigned int* word = (unsigned int*)((uintptr_t)(k.st + v) & ~(uintptr_t)3);
    const unsigned int shift = (unsigned int)(((uintptr_t)(k.st + v) & 3u) * 8u);
    unsigned int old = *((volatile unsigned int*)word);
    for (int it = 0; it < 64; it++) {  // bounded: 4 bytes can change at most 4 times
        const uint8_t cur = (uint8_t)((old >> shift) & 0xFFu);
        if (cur != BCP_UNSET) {
            if (cur != desired) set_conflict(k, inst);
            return;
        }
        const unsigned int nw = (old & ~(0xFFu << shift)) | ((unsigned int)desired << shift);
        const unsigned int prev = atomicCAS(word, old, nw);
        if (prev == old) {
            k.elim[v] |= FORCED_MASK;
            const uint32_t t = atomicAdd(&k.tcount[inst], 1u);
            if (t < k.tcap[inst]) k.trail[k.tbase[inst] + t] = unit; else atomicOr(&k.dc->err, ERR_UNITS_OVERFLOW);
            const uint32_t f = FLIPL(unit);
            if (k.ot_size[f] > BCP_LONG) k.long_next[atomicAdd(&k.dc->bcp_lnext, 1u)] = f;
            else front_next[atomicAdd(&k.dc->bcp_next, 1u)] = f;
            return;
        }
        old = prev;
    }
}

// grid.y walks the instances, grid.x strides the units of one instance
__global__ void bcp_seed_k(BK k, const uint32_t* units, const unsigned long long* ubase, const uint32_t* ucount,
                           const uint8_t* bcp, uint32_t ninst, uint32_t* front) {
    for (uint32_t i = blockIdx.y; i < ninst; i += gridDim.y) {
        if (!bcp[i]) continue;
        const uint32_t n = ucount[i];
        const uint32_t* u = units + ubase[i];
        for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x)
            assign_unit(k, u[j], front);
    }
}

__global__ void bcp_advance_k(DevCounters* dc) {
    dc->bcp_curr = dc->bcp_next;
    dc->bcp_next = 0;
    dc->bcp_lcurr = dc->bcp_lnext;
    dc->bcp_lnext = 0;
    dc->bcp_level++;
}

// warp per frontier literal, lanes stride its occurrence list
constexpr uint32_t BCP_GROUP = 32;
constexpr unsigned FULL = 0xFFFFFFFFu;

// exclusive prefix sum of v over the warp; the warp's sum in `total`
PFG_D uint32_t bcp_warp_scan(uint32_t v, uint32_t lane, uint32_t& total) {
    uint32_t incl = v;
#pragma unroll
    for (uint32_t d = 1; d < 32; d <<= 1) {
        const uint32_t t = __shfl_up_sync(FULL, incl, d);
        if (lane >= d) incl += t;
    }
    total = __shfl_sync(FULL, incl, 31);
    return incl - v;
}

constexpr uint32_t BCP_HEAD = 4;

// one clause of a falsified literal's list: conflict, unit or nothing
PFG_D void bcp_clause(const BK& k, const ClsHdr* hdr, const uint32_t* lits, uint32_t cid, uint32_t inst,
                      uint32_t* nxt) {
    const ClsHdr h = hdr[cid];
    if (m_deleted(h.meta)) return;
    uint32_t unit = 0;
    int nunset = 0;
    bool sat = false;
    // the first BCP_HEAD literals and their values are loaded together
    const uint32_t* cl = lits + h.off;
    uint32_t hl[BCP_HEAD];
    uint32_t hv[BCP_HEAD];
#pragma unroll
    for (uint32_t q = 0; q < BCP_HEAD; q++) hl[q] = q < h.size ? cl[q] : 0u;
#pragma unroll
    for (uint32_t q = 0; q < BCP_HEAD; q++) hv[q] = q < h.size ? litval(k.st, hl[q]) : BCP_FALSE;
#pragma unroll
    for (uint32_t q = 0; q < BCP_HEAD; q++) {
        if (hv[q] == BCP_TRUE) sat = true;
        else if (hv[q] == BCP_UNSET) { unit = hl[q]; nunset++; }
    }
    for (uint32_t q = BCP_HEAD; q < h.size && !sat && nunset < 2; q++) {
        const uint32_t l = cl[q];
        const uint32_t ve = litval(k.st, l);
        if (ve == BCP_TRUE) { sat = true; break; }
        if (ve == BCP_UNSET) { unit = l; nunset++; }
    }
    if (sat) return;
    if (!nunset) set_conflict(k, inst);
    else if (nunset == 1) assign_unit(k, unit, nxt);
}

__global__ void bcp_propagate_k(BK k, const ClsHdr* hdr, const uint32_t* lits, const uint32_t* ot_off,
                                const uint32_t* ot_size, const uint32_t* ot_ids, const uint32_t* front_a,
                                uint32_t* front_b, const uint32_t* long_a, uint32_t* long_b) {
    DevCounters* dc = k.dc;
    const uint32_t level = dc->bcp_level;
    const uint32_t* cur = (level & 1u) ? front_b : (uint32_t*)front_a;
    uint32_t* nxt = (level & 1u) ? (uint32_t*)front_a : front_b;
    const uint32_t* lcur = (level & 1u) ? long_b : (uint32_t*)long_a;
    k.long_next = (level & 1u) ? (uint32_t*)long_a : long_b;
    const uint32_t n = dc->bcp_curr;
    const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t nthreads = gridDim.x * blockDim.x;
    const uint32_t group = tid / BCP_GROUP;
    const uint32_t ngroups = nthreads / BCP_GROUP;
    const uint32_t lane = threadIdx.x % BCP_GROUP;
    for (uint32_t fi = group; fi < n; fi += ngroups) {
        const uint32_t f = cur[fi];
        const uint32_t inst = k.vinst[ABSV(f)];
        if (k.conflict[inst]) continue;       // this instance is UNSAT: stop propagating it
        const uint32_t o = ot_off[f], sz = ot_size[f];
        for (uint32_t j = lane; j < sz; j += BCP_GROUP) bcp_clause(k, hdr, lits, ot_ids[o + j], inst, nxt);
    }
    // Long lists: the grid strides over their concatenation, so the entries of
    // many long lists spread over all threads (starting every list at thread 0
    // gave the first threads an entry of every list and left the rest idle). A
    // warp reads 32 lists' bounds at once; the concatenation offsets come from
    // the list sizes alone, so every thread computes the same ones.
    const uint32_t nl = dc->bcp_lcurr;
    const uint32_t wlane = threadIdx.x & 31u;
    uint64_t base = 0;
    for (uint32_t l0 = 0; l0 < nl; l0 += 32) {
        const uint32_t li = l0 + wlane;
        uint32_t o = 0, sz = 0, inst = 0;
        if (li < nl) {
            const uint32_t f = lcur[li];
            inst = k.vinst[ABSV(f)];
            o = ot_off[f];
            sz = ot_size[f];
        }
        uint32_t tot;
        const uint32_t start = bcp_warp_scan(sz, wlane, tot);
        const uint32_t cnt = min(32u, nl - l0);
        for (uint32_t q = 0; q < cnt; q++) {
            const uint32_t qo = __shfl_sync(FULL, o, q), qs = __shfl_sync(FULL, sz, q);
            const uint32_t qst = __shfl_sync(FULL, start, q), qi = __shfl_sync(FULL, inst, q);
            if (k.conflict[qi]) continue;       // this instance is UNSAT: stop propagating it
            const uint32_t rot = (uint32_t)((base + qst) % nthreads);
            for (uint32_t j = (tid + nthreads - rot) % nthreads; j < qs; j += nthreads)
                bcp_clause(k, hdr, lits, ot_ids[qo + j], qi, nxt);
        }
        base += tot;
    }
}

// strip false literals, delete satisfied clauses of the propagating, conflict-free
// instances, and count the live clauses and literals that remain (totals, and
// per instance when there are several), as the count after prop() does
__global__ void bcp_apply_k(ClsHdr* hdr, uint32_t* lits, uint64_t ncls, const uint8_t* st, const uint32_t* vinst,
                            const uint8_t* bcp, const uint32_t* conflict, int multi, unsigned long long* icnt,
                            DevCounters* dc) {
    const unsigned lane = threadIdx.x & 31u;
    uint64_t b, e;
    warp_chunk(ncls, b, e);   // contiguous, so the per-instance counts are run totals
    unsigned long long nc = 0, nl = 0;
    InstRun run;
    for (uint64_t c0 = b; c0 < e; c0 += 32) {
        const uint64_t c = c0 + lane;
        ClsHdr h{0, 0, 0, 0};
        uint32_t inst = 0xFFFFFFFFu;
        if (c < e) h = hdr[c];
        if (c < e && !m_deleted(h.meta)) {
            uint32_t* l = lits + h.off;
            inst = vinst[ABSV(l[0])];
            if (h.size && bcp[inst] && !conflict[inst]) {
                uint32_t sig = 0, n = 0;
                bool sat = false;
                for (uint32_t q = 0; q < h.size; q++) {
                    const uint32_t lit = l[q];
                    const uint32_t ve = litval(st, lit);
                    if (ve == BCP_TRUE) { sat = true; break; }
                    if (ve == BCP_FALSE) continue;
                    if (n != q) l[n] = lit;      // only a clause that lost a literal is rewritten
                    n++;
                    sig |= MAPHASH(lit);
                }
                if (sat) { hdr[c].meta = m_set_st(h.meta, ST_DELETED); inst = 0xFFFFFFFFu; }
                else if (n != h.size) { hdr[c].sig = sig; hdr[c].size = n; h.size = n; }
            }
        }
        const bool live = inst != 0xFFFFFFFFu;
        if (live) { nc++; nl += h.size; }
        if (multi) inst_run_add(run, live, inst, live ? h.size : 0u, icnt, lane);
    }
    if (multi) inst_run_flush(run, icnt, lane);
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) {
        nc += __shfl_down_sync(0xFFFFFFFFu, nc, d);
        nl += __shfl_down_sync(0xFFFFFFFFu, nl, d);
    }
    if ((threadIdx.x & 31u) == 0 && (nc || nl)) {
        atomicAdd(&dc->live_cls, nc);
        atomicAdd(&dc->live_lits, nl);
    }
}

}  // namespace

// Propagates the units of the instances flagged in di.bcp (their counts are in
// dout.ucount). Returns false on a CUDA/engine error; conflicts are reported
// per instance in dout.conflict.
bool bcp_prop(Ctx& c) {
    cudaMemsetAsync(c.bstate, 0, c.V + 1, c.s);
    cudaMemsetAsync(&c.dc->conflict, 0, sizeof(uint32_t), c.s);
    cudaMemsetAsync(c.dout.conflict, 0, c.ninst * sizeof(uint32_t), c.s);
    cudaMemsetAsync(&c.dc->bcp_curr, 0, 3 * sizeof(uint32_t), c.s);
    cudaMemsetAsync(&c.dc->bcp_lcurr, 0, 2 * sizeof(uint32_t), c.s);
    BK k;
    k.st = c.bstate; k.elim = c.elim; k.vinst = c.vinst;
    k.tbase = c.di.tbase; k.tcap = c.di.tcap; k.tcount = c.dout.tcount;
    k.conflict = c.dout.conflict; k.trail = c.trail; k.dc = c.dc; k.V = c.V;
    k.ot_size = c.ot_size; k.long_next = c.long_a;
    uint64_t maxu = 0;
    for (uint32_t i = 0; i < c.ninst; i++)
        if (c.hi.bcp[i]) maxu = std::max<uint64_t>(maxu, c.ih[i].nUnits);
    // seed: assigned literals go to front_a through bcp_next, then advance
    const dim3 sgrid(grid_for(maxu, 256, 8), std::min<uint32_t>(c.ninst, 65535u));
    PFG_LAUNCH(K_BCP, bcp_seed_k, sgrid, 256, 0, c.s, k, c.units, c.di.ubase, c.dout.ucount, c.di.bcp, c.ninst,
               c.front_a);
    PFG_LAUNCH(K_BCP, bcp_advance_k, 1, 1, 0, c.s, c.dc);
    // make level parity start at 0 with the seeds in front_a
    cudaMemsetAsync(&c.dc->bcp_level, 0, sizeof(uint32_t), c.s);
    const unsigned grid = sm_count() * tuned(c.tune.bcp_blocks_per_sm, BCP_BLOCKS_PER_SM);
    uint32_t levels = 0;
    // every level assigns at least one new variable, so V + 2 levels always suffice
    const uint32_t max_levels = c.lim_bcp_levels ? c.lim_bcp_levels : c.V + 2;
    const bool single = c.ninst == 1;
    for (int batch = 1;; batch = std::min(batch << 1, 64)) {
        for (int b = 0; b < batch; b++) {
            PFG_LAUNCH(K_BCP, bcp_propagate_k, grid, 256, 0, c.s, k, c.hdr, c.lits, c.ot_off, c.ot_size, c.ot_ids,
                       c.front_a, c.front_b, c.long_a, c.long_b);
            PFG_LAUNCH(K_BCP, bcp_advance_k, 1, 1, 0, c.s, c.dc);
        }
        levels += batch;
        sync_counters(c);
        if (!c.err.empty()) return false;
        if ((single && c.hc->conflict) || !(c.hc->bcp_curr | c.hc->bcp_lcurr)) break;
        if (levels > max_levels) { c.err = "device unit propagation did not converge"; c.simpstate = PFG_TIMEOUT; return false; }
    }
    if (c.hc->err) { c.err = "device error during unit propagation"; return false; }
    // rewrite (conflict-free instances) and count: the live counts land in the
    // counters and dout.cnt as count_live leaves them
    const int multi = c.ninst > 1;
    cudaMemsetAsync(&c.dc->live_cls, 0, 2 * sizeof(unsigned long long), c.s);
    if (multi) cudaMemsetAsync(c.dout.cnt, 0, 2 * c.ninst * sizeof(unsigned long long), c.s);
    // byte model of the rewrite, which also does the count: 4 (L + C), booked
    // with the kernel under the propagation group
    c.prof.bytes[K_BCP] += 4 * (c.numLiterals + c.numClauses);
    if (c.ncls)
        PFG_LAUNCH(K_BCP, bcp_apply_k, grid_for(c.ncls, 256, 8), 256, 0, c.s, c.hdr, c.lits, c.ncls, c.bstate, c.vinst,
                   c.di.bcp, c.dout.conflict, multi, c.dout.cnt, c.dc);
    if (!multi)
        cudaMemcpyAsync(c.dout.cnt, &c.dc->live_cls, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToDevice, c.s);
    return cuda_ok(c, cudaGetLastError(), "bcp");
}

}  // namespace pfg
