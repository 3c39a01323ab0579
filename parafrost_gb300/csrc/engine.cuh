// Engine context and pass launchers (host side).
//
// One context = one device-resident CNF instance on one GPU stream. The
// round driver in engine.cu mirrors Solver::simplifying
// (src/gpu/simplify.cu:136-241); each pass lives in its own translation unit.
#pragma once

#include <string>
#include <vector>

#include "common.cuh"
#include "pfgpu.h"
#include "prims.cuh"

namespace pfg {

struct Ctx {
    pfg_options o{};
    int device = 0;
    cudaStream_t s = nullptr;
    cudaEvent_t ev_begin = nullptr, ev_end = nullptr, ev_a = nullptr, ev_b = nullptr;
    std::string err;
    uint64_t launches = 0;
    bool uploaded = false;
    bool simplified = false;

    // instance
    uint32_t V = 0;
    uint64_t nlist = 0;  // 2V + 2 literal lists

    // clause store
    ClsHdr* hdr = nullptr;
    uint32_t* lits = nullptr;
    uint64_t hdr_cap = 0, lits_cap = 0;
    uint64_t ncls = 0;                 // clauses in the array (cnf->size())
    uint64_t lits_used = 0;            // packed literal words in use
    uint64_t data_size = 0, data_cap = 0, cs_cap = 0;  // reference bucket accounting
    uint64_t orig_cls = 0, orig_lits = 0;
    uint64_t numClauses = 0, numLiterals = 0;

    // occurrence table (CSR)
    uint32_t* hist = nullptr;    // nlist
    uint32_t* ot_off = nullptr;  // nlist + 1
    uint32_t* ot_size = nullptr; // nlist
    uint32_t* ot_fill = nullptr; // nlist (fill cursors)
    uint32_t* ot_ids = nullptr;
    uint64_t ot_cap = 0;
    // big-list sort scratch
    uint32_t* big_lists = nullptr;   // nlist (worst case)
    uint32_t* mid_desc = nullptr;    // descriptors (offset, size) pairs
    uint64_t mid_desc_cap = 0;
    uint4* big_keys = nullptr; uint4* big_keys_alt = nullptr;
    uint32_t* big_ids = nullptr; uint32_t* big_ids_alt = nullptr;
    uint64_t big_cap = 0;

    // per variable
    uint8_t* elim = nullptr;     // V+1 eliminated bytes
    uint8_t* vstate = nullptr;   // V+1
    uint8_t* assumed = nullptr;  // V+1 or null
    uint8_t* frozen = nullptr;   // V+1
    uint8_t* mstate = nullptr;   // V+1
    uint8_t* flag8 = nullptr;    // V+1 scratch flags
    uint32_t* vorg = nullptr;    // V+1
    uint32_t* scores = nullptr;  // V+1
    uint32_t* keys_a = nullptr;  // V+1 sort keys
    uint32_t* keys_b = nullptr;
    uint32_t* eligible = nullptr;    // V+1
    uint32_t* eligible_b = nullptr;  // V+1
    uint32_t* rank = nullptr;    // V+1
    uint32_t* varcore = nullptr; // V+1
    uint32_t* elected = nullptr; // V+1
    uint32_t* work = nullptr;    // V+1 MIS worklist
    uint32_t* work_b = nullptr;  // V+1
    uint32_t* vscan = nullptr;   // V+2 scan scratch
    uint8_t* winv = nullptr;     // V+1 MIS round winners
    uint4* ckeys = nullptr;      // per-clause sort key (size, first, last, sig)
    uint64_t ckeys_cap = 0;
    uint32_t nelected = 0;
    bool varcore_on = false;

    // BVE per elected index
    uint32_t* type = nullptr;
    uint32_t* ucnt = nullptr;
    unsigned long long* rpos = nullptr;
    unsigned long long* rref = nullptr;

    // units, trail and model stack
    uint32_t* units = nullptr; uint32_t units_cap = 0;
    uint32_t* trail = nullptr; uint32_t trail_cap = 0;
    uint32_t* stack = nullptr; uint64_t stack_cap = 0;
    std::vector<uint64_t> round_ends;
    uint64_t nUnits = 0;

    // BCP
    uint8_t* bstate = nullptr;
    uint32_t* front_a = nullptr;
    uint32_t* front_b = nullptr;

    // counters
    DevCounters* dc = nullptr;   // device
    DevCounters* hc = nullptr;   // pinned host mirror

    // scratch
    void* tmp = nullptr; size_t tmp_cap = 0;
    uint32_t* tmp_u32 = nullptr; uint64_t tmp_u32_cap = 0;   // generic u32 scratch

    // per-kernel profiler (launch counts always; CUDA-event timing when enabled)
    Profiler prof;

    // round state
    int phase = 0, multiplier = 0, simpstate = 0, status = PFG_UNKNOWN;
    uint32_t mis_rounds = 0;
    pfg_stats stats{};
    double pass_ms[8] = {0};
};

// ---- memory helpers (engine.cu) ----
bool dalloc(Ctx& c, void** p, size_t bytes);
void dfree(Ctx& c, void* p);
template <typename T>
inline bool dalloc_t(Ctx& c, T** p, size_t count) { return dalloc(c, (void**)p, count * sizeof(T)); }
bool ensure_tmp(Ctx& c, size_t bytes);
bool ensure_tmp_u32(Ctx& c, uint64_t count);
void sync_counters(Ctx& c);     // D2H copy of counters + stream sync
bool cuda_ok(Ctx& c, cudaError_t e, const char* what);

// ---- passes ----
// occurrence table (ot.cu)
bool ot_build(Ctx& c);          // histogram + CSR offsets + unsorted fill (clause order irrelevant)
bool ot_sort(Ctx& c, bool by_id);  // sort every list by OLIST_CMP (key.cuh:67-85) or by clause id
// counting + compaction (gc.cu)
void count_live(Ctx& c);        // counters live_cls/live_lits (needs sync to read)
bool compact_cnf(Ctx& c);       // Solver::reallocCNF(true) (cnf.cu:129-144, recycle.cu:60)
// device BCP (bcp.cu): returns false on conflict
bool bcp_prop(Ctx& c, bool& ok);
// LCVE (lcve.cu): returns number elected
bool lcve(Ctx& c);
// SUB, BVE, ERE (elim.cu)
void sub_pass(Ctx& c);
bool ve_pass(Ctx& c);
void ere_pass(Ctx& c);

}  // namespace pfg
