// Shared device definitions of the GB300 CNF inprocessing engine.
//
// Clause store (structure of arrays, replaces SCLAUSE + S_REF, src/gpu/sclause.cuh:37,
// src/gpu/cnf.cuh:35):
//   ClsHdr hdr[c]  = {off, size, sig, meta}: one 16-byte vector load per clause
//   lits[off .. off+size)  literals 2v|s, ascending inside a clause
// meta packs the reference's header bits: status (2), molten (1), added (1),
// usage (2), lbd (26).
// Clause ids follow the reference's ref order (upload order, then resolvents in
// elected order), so every ordering tie-break of the reference holds.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#define PFG_HD __host__ __device__ __forceinline__
#define PFG_D __device__ __forceinline__

namespace pfg {

// clause status (src/gpu/constants.hpp:69-71)
constexpr uint32_t ST_ORIGINAL = 0u;
constexpr uint32_t ST_LEARNT = 1u;
constexpr uint32_t ST_DELETED = 2u;
// eliminated-variable bits (src/gpu/constants.cuh:34-36)
constexpr uint8_t MELTING_MASK = 0x01u;
constexpr uint8_t ADDING_MASK = 0x02u;
constexpr uint8_t FORCED_MASK = 0x04u;
// BVE type word (src/gpu/constants.cuh:38-63)
constexpr uint32_t RES_MASK = 1u;
constexpr uint32_t AOIX_MASK = 2u;
constexpr uint32_t CORE_MASK = 3u;
constexpr uint32_t ADDEDCLS_MAX = 0x3FFFu;
constexpr uint32_t ADDEDLITS_MAX = 0xFFFFu;
// reference arena accounting: a clause occupies 3 header buckets + its literals
constexpr uint32_t NBUCKETS = 3u;
// kernel limits of an EXTSHMEM build (the reference's install.sh enables it on cc >= 7)
constexpr uint32_t SH_MAX_BVE_OUT1 = 250u;
constexpr uint32_t SH_MAX_ERE_OUT = 250u;
constexpr uint32_t SUB_MAX_CL_SIZE = 1000u;
constexpr uint32_t LBD_TIER1 = 2u;
constexpr uint32_t USAGET3 = 1u;
constexpr uint32_t NOREF = 0xFFFFFFFFu;
constexpr uint32_t ERE_LANES = 32u;  // blockDim.x of the reference's ere_k
// DRAT proof (src/gpu/constants.cuh:46, constants.hpp:45-46)
constexpr uint32_t ADDEDPROOF_MAX = 0x3FFFFu;   // proof bytes one variable may add
constexpr uint8_t PROOF_ADDED = 97u;            // 'a'
constexpr uint8_t PROOF_DELETED = 100u;         // 'd'

struct __align__(16) ClsHdr {
    uint32_t off;
    uint32_t size;
    uint32_t sig;
    uint32_t meta;
};

PFG_HD uint32_t m_st(uint32_t m) { return m & 3u; }
PFG_HD bool m_orig(uint32_t m) { return (m & 3u) == ST_ORIGINAL; }
PFG_HD bool m_learnt(uint32_t m) { return (m & ST_LEARNT) != 0; }
PFG_HD bool m_deleted(uint32_t m) { return (m & ST_DELETED) != 0; }
PFG_HD bool m_molten(uint32_t m) { return (m >> 2) & 1u; }
PFG_HD uint32_t m_usage(uint32_t m) { return (m >> 4) & 3u; }
PFG_HD uint32_t m_lbd(uint32_t m) { return m >> 6; }
PFG_HD uint32_t m_make(uint32_t st, uint32_t molten, uint32_t added, uint32_t usage, uint32_t lbd) {
    return st | (molten << 2) | (added << 3) | (usage << 4) | (lbd << 6);
}
PFG_HD uint32_t m_set_st(uint32_t m, uint32_t st) { return (m & ~3u) | st; }
PFG_HD uint32_t m_set_molten(uint32_t m, uint32_t f) { return (m & ~4u) | (f << 2); }

PFG_HD uint32_t ABSV(uint32_t l) { return l >> 1; }
PFG_HD uint32_t SIGNL(uint32_t l) { return l & 1u; }
PFG_HD uint32_t FLIPL(uint32_t l) { return l ^ 1u; }
PFG_HD uint32_t MAPHASH(uint32_t l) { return 1u << (l & 31u); }
PFG_HD bool SUBSIG(uint32_t a, uint32_t b) { return !(a & ~b); }

// Device counters shared between kernels and the host (one pinned mirror);
// per-instance counters live in the engine's InstOut arrays.
struct DevCounters {
    unsigned long long live_cls;   // live clauses (count kernel)
    unsigned long long live_lits;
    unsigned long long err_info;   // first error detail
    uint32_t err;                  // error flags (ERR_*)
    uint32_t nwork;                // MIS worklist size
    uint32_t nwin;                 // winners in the current MIS round
    uint32_t nelected;
    uint32_t nfrozen;
    uint32_t conflict;             // BCP conflict flag
    uint32_t bcp_curr, bcp_next, bcp_level;
    uint32_t bcp_lcurr, bcp_lnext;           // frontier literals with long lists
    uint32_t big_lists;
    uint32_t nbig_sub, nbig_ve1, nbig_ve3;   // variables too large for the warp stage
    unsigned long long ve_cls, ve_lits;      // store size after the last BVE emission
    uint32_t sort_warp;                      // lists sorted by one warp each
    unsigned long long pf_words;             // proof line words reserved in the running pass
    unsigned long long pf_need;              // proof words BVE emission needs
    uint32_t pf_blocks;                      // proof blocks reserved in the running pass
    uint32_t mis_done;                       // a MIS round found nothing undecided: later rounds return at once
    uint32_t steal[4];                       // next variable of the warp kernels (SUB, BVE 1, BVE 3)
    uint32_t ot_long;                        // lists the list passes hand to whole blocks
    unsigned long long vol_ve[2], vol_ere[2];   // clauses, literals on the elected lists (byte model)
};

// Per-instance clause and literal counts from a warp walking a contiguous
// chunk of clause ids 32 at a time. The store keeps an instance's clauses in
// runs, so while a whole step lies in one instance the warp only adds to a
// running total, which goes to that instance's counters when the run ends; a
// step that mixes instances is added per instance. A dead lane (deleted
// clause, or past the chunk) takes the step's first live instance, or the
// running one. Every lane of the warp calls it with warp-uniform control.
struct InstRun {
    uint32_t run = 0xFFFFFFFFu;              // warp-uniform
    unsigned long long ra = 0, rb = 0;       // clauses, literals of the run
};

PFG_D void inst_run_flush(InstRun& r, unsigned long long* icnt, unsigned lane) {
    if (lane == 0 && r.run != 0xFFFFFFFFu && (r.ra || r.rb)) {
        atomicAdd(&icnt[2 * (uint64_t)r.run], r.ra);
        atomicAdd(&icnt[2 * (uint64_t)r.run + 1], r.rb);
    }
    r.run = 0xFFFFFFFFu;
    r.ra = r.rb = 0;
}

PFG_D void inst_run_add(InstRun& r, bool live, uint32_t inst, uint32_t sz, unsigned long long* icnt,
                        unsigned lane) {
    constexpr uint32_t NONE = 0xFFFFFFFFu;
    const unsigned lb = __ballot_sync(0xFFFFFFFFu, live);
    const uint32_t first = lb ? __shfl_sync(0xFFFFFFFFu, inst, __ffs(lb) - 1) : r.run;
    const uint32_t key = live ? inst : first;
    if (r.run != NONE && __all_sync(0xFFFFFFFFu, key == r.run)) {
        r.ra += __reduce_add_sync(0xFFFFFFFFu, live ? 1u : 0u);
        r.rb += __reduce_add_sync(0xFFFFFFFFu, live ? sz : 0u);
        return;
    }
    inst_run_flush(r, icnt, lane);
    const unsigned peers = __match_any_sync(0xFFFFFFFFu, key);
    const unsigned ca = __reduce_add_sync(peers, live ? 1u : 0u);
    const unsigned cb = __reduce_add_sync(peers, live ? sz : 0u);
    if (peers == 0xFFFFFFFFu) {              // the whole step is one instance: a new run
        if (key != NONE) { r.run = key; r.ra = ca; r.rb = cb; }
    } else if (key != NONE && ca && (int)lane == __ffs(peers) - 1) {
        atomicAdd(&icnt[2 * (uint64_t)key], (unsigned long long)ca);
        atomicAdd(&icnt[2 * (uint64_t)key + 1], (unsigned long long)cb);
    }
}

// [b, e): the contiguous chunk of n items of the calling warp, 32-aligned
PFG_D void warp_chunk(uint64_t n, uint64_t& b, uint64_t& e) {
    const uint64_t warp = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    const uint64_t per = ((n + nwarps - 1) / nwarps + 31) & ~31ull;
    b = warp * per;
    e = b + per < n ? b + per : n;
}

constexpr uint32_t ERR_UNITS_OVERFLOW = 1u;
constexpr uint32_t ERR_STACK_OVERFLOW = 2u;
constexpr uint32_t ERR_SLOT_MISMATCH = 4u;
constexpr uint32_t ERR_BAD_LIT = 8u;
constexpr uint32_t ERR_OT_OVERFLOW = 16u;
constexpr uint32_t ERR_PROOF_OVERFLOW = 32u;

}  // namespace pfg
