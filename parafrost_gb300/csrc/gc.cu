// Live-clause counting and clause-store compaction.
//
// Replaces cnt_cls_lits + the host block reduction (count.cu:83-131,171) and
// cuMM::compactCNF (recycle.cu:34-103): live clauses are kept in order,
// packed into freshly sized arrays, and the reference's bucket accounting is
// reset to 3 * clauses + literals (recycle.cu:71).
#include "engine.cuh"

namespace pfg {
namespace {

__global__ void count_k(const ClsHdr* __restrict__ hdr, uint64_t ncls, DevCounters* dc) {
    unsigned long long nc = 0, nl = 0;
    for (uint64_t c = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; c < ncls; c += (uint64_t)gridDim.x * blockDim.x) {
        const ClsHdr h = hdr[c];
        if (!m_deleted(h.meta)) { nc++; nl += h.size; }
    }
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
                          ClsHdr* nhdr, uint32_t* nlits) {
    for (uint64_t c = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; c < ncls; c += (uint64_t)gridDim.x * blockDim.x) {
        const ClsHdr h = hdr[c];
        if (m_deleted(h.meta)) continue;
        const uint64_t o = loff[c];
        for (uint32_t k = 0; k < h.size; k++) nlits[o + k] = lits[h.off + k];
        ClsHdr nh = h;
        nh.off = (uint32_t)o;
        nhdr[pos[c]] = nh;
    }
}

}  // namespace

void count_live(Ctx& c) {
    cudaMemsetAsync(&c.dc->live_cls, 0, 2 * sizeof(unsigned long long), c.s);
    c.prof.bytes[K_COUNT] += 8 * c.ncls;
    if (c.ncls) {
        PFG_LAUNCH(K_COUNT, count_k, grid_for(c.ncls, 256, 8), 256, 0, c.s, c.hdr, c.ncls, c.dc);
    }
}

bool compact_cnf(Ctx& c) {
    // capacities of the new store (cnf.cu:129-139)
    const uint64_t addCls = c.o.ve_en ? c.numClauses : 0;
    const uint64_t addLits = c.o.ve_en ? (uint64_t)((double)c.orig_lits * c.o.lits_mul) : 0;
    const uint64_t clsCap = c.numClauses + addCls, litsCap = c.numLiterals + addLits;
    const uint64_t data_cap = clsCap * NBUCKETS + litsCap;
    // physical literal words: data_cap minus the header buckets of the clauses kept
    const uint64_t phys_lits = data_cap - NBUCKETS * c.numClauses + 64;
    if (phys_lits > 0xFFFFFFF0ull) { c.simpstate = PFG_CNFALLOC_FAIL; c.err = "clause store exceeds 2^32 literals"; return false; }
    ClsHdr* nhdr = nullptr;
    uint32_t* nlits = nullptr;
    if (!dalloc_t(c, &nhdr, clsCap + 1) || !dalloc_t(c, &nlits, phys_lits)) {
        dfree(c, nhdr); dfree(c, nlits);
        c.simpstate = PFG_CNFALLOC_FAIL;
        return false;
    }
    const uint64_t n = c.ncls;
    uint32_t* pos = nullptr;
    unsigned long long* loff = nullptr;
    if (!dalloc_t(c, &pos, n + 1) || !dalloc_t(c, &loff, n + 1)) {
        dfree(c, nhdr); dfree(c, nlits); dfree(c, pos); dfree(c, loff);
        c.simpstate = PFG_CNFALLOC_FAIL;
        return false;
    }
    if (!ensure_tmp(c, scan_temp_bytes(n))) return false;
    PFG_LAUNCH(K_COMPACT, live_flags_k, grid_for(n, 256), 256, 0, c.s, c.hdr, n, pos, loff);
    exclusive_scan_u32(pos, pos, n, 0u, nullptr, c.tmp, c.s);
    exclusive_scan_u64(loff, loff, n, 0ull, nullptr, c.tmp, c.s);
    PFG_LAUNCH(K_COMPACT, compact_k, grid_for(n, 256), 256, 0, c.s, c.hdr, c.lits, n, pos, loff, nhdr, nlits);
    dfree(c, pos); dfree(c, loff);
    c.prof.bytes[K_COMPACT] += 8 * (c.numLiterals + c.numClauses);
    dfree(c, c.hdr); dfree(c, c.lits);
    c.hdr = nhdr; c.lits = nlits;
    c.hdr_cap = clsCap + 1; c.lits_cap = phys_lits;
    c.ncls = c.numClauses;
    c.lits_used = c.numLiterals;
    c.cs_cap = clsCap;
    c.data_cap = data_cap;
    c.data_size = c.numClauses * NBUCKETS + c.numLiterals;
    return cuda_ok(c, cudaGetLastError(), "compact_cnf");
}

}  // namespace pfg
