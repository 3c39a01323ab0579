// Live-clause counting and clause-store compaction.
//
// Replaces cnt_cls_lits + the host block reduction (count.cu:83-131,171) and
// cuMM::compactCNF (recycle.cu:34-103): live clauses are kept in order,
// packed into freshly sized arrays, and the reference's bucket accounting of
// every instance still in the round loop is reset to 3 * clauses + literals
// (recycle.cu:71) with the capacities of reallocCNF (cnf.cu:129-139).
#include "engine.cuh"

namespace pfg {
namespace {

// Totals, and with several instances the counts per instance (the instance of
// a clause is the instance of its literals); a warp takes a contiguous chunk
// of clause ids so that its per-instance counts are run totals (InstRun).
__global__ void count_k(const ClsHdr* __restrict__ hdr, const uint32_t* __restrict__ lits, uint64_t ncls,
                        const uint32_t* __restrict__ vinst, int multi, unsigned long long* icnt, DevCounters* dc) {
    const unsigned lane = threadIdx.x & 31u;
    uint64_t b, e;
    warp_chunk(ncls, b, e);
    unsigned long long nc = 0, nl = 0;
    InstRun r;
    for (uint64_t c0 = b; c0 < e; c0 += 32) {
        const uint64_t c = c0 + lane;
        bool live = false;
        uint32_t sz = 0, inst = 0xFFFFFFFFu;
        if (c < e) {
            const ClsHdr h = hdr[c];
            live = !m_deleted(h.meta);
            if (live) {
                sz = h.size;
                if (multi) inst = vinst[ABSV(lits[h.off])];
            }
        }
        if (live) { nc++; nl += sz; }
        if (multi) inst_run_add(r, live, inst, sz, icnt, lane);
    }
    if (multi) inst_run_flush(r, icnt, lane);
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) {
        nc += __shfl_down_sync(0xFFFFFFFFu, nc, d);
        nl += __shfl_down_sync(0xFFFFFFFFu, nl, d);
    }
    if (lane == 0 && (nc || nl)) {
        atomicAdd(&dc->live_cls, nc);
        atomicAdd(&dc->live_lits, nl);
    }
}

__global__ void live_flags_k(const ClsHdr* __restrict__ hdr, uint64_t ncls, uint32_t* flag, unsigned long long* sz) {
    for (uint64_t c = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; c < ncls; c += (uint64_t)gridDim.x * blockDim.x) {
        const ClsHdr h = hdr[c];
        const bool live = !m_deleted(h.meta);
        flag[c] = live ? 1u : 0u;
        sz[c] = live ? h.size : 0ull;
    }
}

// thread per clause: copy header and literals into the new store (clauses are short)
__global__ void compact_k(const ClsHdr* __restrict__ hdr, const uint32_t* __restrict__ lits, uint64_t ncls,
                          const uint32_t* __restrict__ pos, const unsigned long long* __restrict__ loff,
                          ClsHdr* nhdr, uint32_t* nlits, const uint8_t* __restrict__ cnew, uint8_t* ncnew) {
    for (uint64_t c = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; c < ncls; c += (uint64_t)gridDim.x * blockDim.x) {
        const ClsHdr h = hdr[c];
        if (m_deleted(h.meta)) continue;
        const uint64_t o = loff[c];
        for (uint32_t k = 0; k < h.size; k++) nlits[o + k] = lits[h.off + k];
        ClsHdr nh = h;
        nh.off = (uint32_t)o;
        nhdr[pos[c]] = nh;
        ncnew[pos[c]] = cnew[c];
    }
}

// One word per 32 old clause ids for the table update after a compaction:
// live bits, kept bits (live and not flagged in the drop bytes), and the new id
// of the word's first live clause (the exclusive scan of the live flags).
__global__ void drop_bits_k(const ClsHdr* __restrict__ hdr, const uint8_t* __restrict__ drop,
                            const uint32_t* __restrict__ pos, uint64_t n, uint4* bits) {
    const uint64_t nw = (n + 31) / 32;
    const unsigned lane = threadIdx.x & 31u;
    const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    for (uint64_t w = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < nw; w += nwarps) {
        const uint64_t c = w * 32 + lane;
        bool live = false, keep = false;
        if (c < n) {
            live = !m_deleted(hdr[c].meta);
            keep = live && !drop[c];
        }
        const unsigned lb = __ballot_sync(0xFFFFFFFFu, live), kb = __ballot_sync(0xFFFFFFFFu, keep);
        if (lane == 0) bits[w] = make_uint4(lb, kb, pos[w * 32], 0u);
    }
}

}  // namespace

void count_live(Ctx& c) {
    cudaMemsetAsync(&c.dc->live_cls, 0, 2 * sizeof(unsigned long long), c.s);
    const int multi = c.ninst > 1;
    if (multi) cudaMemsetAsync(c.dout.cnt, 0, 2 * c.ninst * sizeof(unsigned long long), c.s);
    c.prof.bytes[K_COUNT] += 8 * c.ncls;
    if (c.ncls)
        PFG_LAUNCH(K_COUNT, count_k, grid_for(c.ncls, 256, 8), 256, 0, c.s, c.hdr, c.lits, c.ncls, c.vinst, multi,
                   c.dout.cnt, c.dc);
    if (!multi)
        cudaMemcpyAsync(c.dout.cnt, &c.dc->live_cls, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToDevice, c.s);
}

bool compact_cnf(Ctx& c) {
    // capacities of reallocCNF (cnf.cu:129-139) for every instance still in the
    // loop; stopped instances only keep their live clauses
    uint64_t clsCap = 0, litsCap = 0;
    for (uint32_t i = 0; i < c.ninst; i++) {
        InstHost& h = c.ih[i];
        const uint64_t addCls = (h.active && c.o.ve_en) ? h.numClauses : 0;
        const uint64_t addLits = (h.active && c.o.ve_en) ? (uint64_t)((double)h.orig_lits * c.o.lits_mul) : 0;
        clsCap += h.numClauses + addCls;
        litsCap += h.numLiterals + NBUCKETS * addCls + addLits;   // data_cap - 3 * live clauses
        if (h.active) {
            unsigned long long* acc = c.hi.acc + 4 * i;
            acc[0] = h.numClauses;
            acc[1] = h.numClauses * NBUCKETS + h.numLiterals;
            acc[2] = h.numClauses + addCls;
            acc[3] = acc[2] * NBUCKETS + h.numLiterals + addLits;
        }
    }
    const uint64_t phys_lits = litsCap + 64;
    if (phys_lits > 0xFFFFFFF0ull || clsCap > 0xFFFFFFF0ull) {
        c.simpstate = PFG_CNFALLOC_FAIL;
        c.err = "clause store exceeds 2^32 entries";
        return false;
    }
    ClsHdr* nhdr = nullptr;
    uint32_t* nlits = nullptr;
    uint8_t* ncnew = nullptr;
    if (!dalloc_t(c, &nhdr, clsCap + 1) || !dalloc_t(c, &nlits, phys_lits) || !dalloc_t(c, &ncnew, clsCap + 1)) {
        dfree(c, nhdr); dfree(c, nlits); dfree(c, ncnew);
        c.simpstate = PFG_CNFALLOC_FAIL;
        return false;
    }
    const uint64_t n = c.ncls;
    uint32_t* pos = nullptr;
    unsigned long long* loff = nullptr;
    if (!dalloc_t(c, &pos, n + 1) || !dalloc_t(c, &loff, n + 1)) {
        dfree(c, nhdr); dfree(c, nlits); dfree(c, ncnew); dfree(c, pos); dfree(c, loff);
        c.simpstate = PFG_CNFALLOC_FAIL;
        return false;
    }
    if (!ensure_tmp(c, scan_temp_bytes(n))) return false;
    PFG_LAUNCH(K_COMPACT, live_flags_k, grid_for(n, 256), 256, 0, c.s, c.hdr, n, pos, loff);
    exclusive_scan_u32(pos, pos, n, 0u, nullptr, c.tmp, c.s);
    exclusive_scan_u64(loff, loff, n, 0ull, nullptr, c.tmp, c.s);
    cudaMemsetAsync(ncnew, 0, clsCap + 1, c.s);
    PFG_LAUNCH(K_COMPACT, compact_k, grid_for(n, 256), 256, 0, c.s, c.hdr, c.lits, n, pos, loff, nhdr, nlits, c.cnew,
               ncnew);
    // the occurrence-table update keeps and renumbers its entries through
    // these words (the drop bytes, c.cnew, are on the old ids)
    dfree(c, c.cbits);
    c.cbits = nullptr;
    if (c.ot_valid) {
        const uint64_t nw = (n + 31) / 32;
        if (!dalloc_t(c, &c.cbits, nw + 1)) {
            dfree(c, nhdr); dfree(c, nlits); dfree(c, ncnew); dfree(c, pos); dfree(c, loff);
            c.simpstate = PFG_CNFALLOC_FAIL;
            return false;
        }
        cudaMemsetAsync(c.cbits, 0, (nw + 1) * sizeof(uint4), c.s);
        if (n)
            PFG_LAUNCH(K_COMPACT, drop_bits_k, grid_for(nw * 32, 256), 256, 0, c.s, c.hdr, c.cnew, pos, n, c.cbits);
    }
    dfree(c, pos);
    dfree(c, loff);
    c.prof.bytes[K_COMPACT] += 8 * (c.numLiterals + c.numClauses);
    dfree(c, c.hdr); dfree(c, c.lits);
    dfree(c, c.cnew);
    c.hdr = nhdr; c.lits = nlits; c.cnew = ncnew;
    c.hdr_cap = clsCap + 1; c.lits_cap = phys_lits;
    c.ncls = c.numClauses;
    c.lits_used = c.numLiterals;
    push_inst_in(c);
    return cuda_ok(c, cudaGetLastError(), "compact_cnf");
}

}  // namespace pfg
