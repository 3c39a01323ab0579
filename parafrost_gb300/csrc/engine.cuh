// Engine context and pass launchers (host side).
//
// One context holds n >= 1 independent CNF instances in one device clause
// store on one GPU stream. Instance i owns the global variables
// voff[i]+1 .. voff[i+1] (its local variable v is global voff[i] + v), so the
// instances share no clause and every pass runs once over all of them. All
// state the reference keeps per Solver (round counter, stop-rule differences,
// arena accounting, units, trail, model stack) is kept per instance, so each
// instance's result is the one a run of that instance alone gives. The round
// driver in engine.cu mirrors Solver::simplifying (src/gpu/simplify.cu:136-241);
// each pass lives in its own translation unit.
#pragma once

#include <algorithm>
#include <string>
#include <vector>

#include "common.cuh"
#include "pfgpu.h"
#include "prims.cuh"

namespace pfg {

// Host-side state of one instance (the reference's per-Solver simplifier state).
struct InstHost {
    uint32_t V = 0;                 // variables of the instance
    uint32_t voff = 0;              // global variable = local variable + voff
    uint64_t orig_cls = 0, orig_lits = 0;       // original (non-learnt) clauses at upload
    uint64_t cls_in = 0, lits_in = 0;
    uint64_t numClauses = 0, numLiterals = 0;   // live clauses / literals
    int status = PFG_UNKNOWN;
    bool active = false;            // still in the round loop
    bool varcore_on = false;        // function-table gates enabled (vars->varcore != NULL)
    bool ere_ran = false;
    int mode = 0;                   // this round: 0 idle, 1 SUB+BVE, 2 ERE
    int64_t cdiff = 0, ldiff = 0, clsbefore = 0, litsbefore = 0;
    uint64_t nUnits = 0;            // units produced by its last round, not yet propagated
    uint32_t rounds = 0;
    uint32_t nelected = 0;
    uint64_t processed_cls = 0, processed_lits = 0, resolvents = 0;
    std::vector<uint32_t> pending;  // units left unpropagated when it stopped
    std::vector<uint64_t> round_ends;
    std::vector<uint8_t> proof;     // binary DRAT lines of its passes (proof_en)
};

// Per-instance kernel inputs, written by the host (one allocation, mirrored in
// pinned host memory with the same layout).
struct InstIn {
    uint32_t* voff = nullptr;              // n+1
    uint32_t* seg = nullptr;               // n+1: first index of each instance in the BVE set
    uint32_t* ucap = nullptr;              // n: unit region capacity
    uint32_t* tcap = nullptr;              // n: trail region capacity
    unsigned long long* ubase = nullptr;   // n
    unsigned long long* tbase = nullptr;   // n
    unsigned long long* sbase = nullptr;   // n: model-stack region
    unsigned long long* scap = nullptr;    // n
    unsigned long long* acc = nullptr;     // 4n: reference accounting vncls, vdata, cs_cap, data_cap
    uint8_t* active = nullptr;             // n: its variables may be elected this round
    uint8_t* vc_on = nullptr;              // n: function-table gates on
    uint8_t* bcp = nullptr;                // n: propagates its units this round
    uint8_t* mode = nullptr;               // n: 1 SUB+BVE, 2 ERE this round
};

// Per-instance kernel outputs, written by the device.
struct InstOut {
    uint32_t* conflict = nullptr;          // n
    uint32_t* ucount = nullptr;            // n: units in its region
    uint32_t* tcount = nullptr;            // n: trail length
    uint32_t* nelect = nullptr;            // n: elected variables
    uint32_t* nfrozen = nullptr;           // n
    uint32_t* fbase = nullptr;             // n+1: frozen-scan value at the instance's first variable
    unsigned long long* scount = nullptr;  // n: model-stack words
    unsigned long long* cnt = nullptr;     // 2n: live clauses, live literals
    unsigned long long* add = nullptr;     // 2n: clauses, literals added by the last BVE
};

size_t inst_in_layout(uint32_t n, char* base, InstIn* p);    // returns bytes; base may be null
size_t inst_out_layout(uint32_t n, char* base, InstOut* p);

struct Ctx {
    pfg_options o{};
    pfg_tuning tune{};               // launch shapes (zero: built-in), kept across uploads
    int device = 0;
    cudaStream_t s = nullptr;
    cudaStream_t s_copy = nullptr;   // write-back copies that overlap the last write-back kernels
    cudaEvent_t ev_copy = nullptr;
    cudaEvent_t ev_begin = nullptr, ev_end = nullptr;
    Profiler pass_clock;          // event pairs around the passes of a call (pass_ms of the stats)
    std::string err;
    uint64_t launches = 0;
    bool uploaded = false;
    bool simplified = false;

    // instances (the single-instance API is n = 1)
    uint32_t ninst = 0;
    std::vector<InstHost> ih;
    InstIn di, hi;                  // device / pinned host mirror
    InstOut dout, hout;
    void* in_blob_h = nullptr; void* out_blob_h = nullptr;
    size_t in_bytes = 0, out_bytes = 0;
    uint32_t* vinst = nullptr;      // V+1: instance of a global variable
    int phase = 0, multiplier = 0;  // shared by every instance still in the loop

    // union of all instances
    uint32_t V = 0;
    uint64_t nlist = 0;  // 2V + 2 literal lists

    // clause store
    ClsHdr* hdr = nullptr;
    uint32_t* lits = nullptr;
    uint64_t hdr_cap = 0, lits_cap = 0;
    uint64_t ncls = 0;                 // clauses in the array (deleted ones included)
    uint64_t lits_used = 0;            // packed literal words in use
    uint64_t numClauses = 0, numLiterals = 0;   // live totals over all instances

    // occurrence table (CSR)
    uint32_t* hist = nullptr;    // nlist
    uint32_t* ot_off = nullptr;  // nlist + 1
    uint32_t* ot_size = nullptr; // nlist
    uint32_t* ot_fill = nullptr; // nlist (fill cursors)
    uint32_t* ot_ids = nullptr;
    uint64_t ot_cap = 0;
    // Between rounds the table is updated instead of rebuilt: a clause whose
    // literals were replaced in place (substitution) or that was added (a
    // resolvent) is flagged in cnew; every other change either deletes a clause
    // or removes it from the one list it left (SUB strengthening, updateOL).
    bool ot_valid = false;           // lists hold every live clause except those flagged in cnew
    uint8_t* cnew = nullptr;         // hdr_cap
    uint32_t* ot_ids2 = nullptr;     // second id array / offsets of the update
    uint64_t ot_cap2 = 0;
    uint32_t* ot_off2 = nullptr;     // nlist + 1
    // the last compaction, on the old clause ids, one word per 32 ids: bits of
    // the live clauses, bits of the kept ones (live and not flagged), and the
    // live clauses before the word's first id (its new id is that plus the
    // live bits below it); read by the table update, ~1 bit per clause
    uint4* cbits = nullptr;
    // big-list sort scratch
    uint32_t* big_lists = nullptr;   // nlist (worst case)
    uint32_t* mid_desc = nullptr;    // descriptors (offset, size) pairs
    uint32_t* warp_desc = nullptr;   // descriptors of the lists sorted by one warp
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
    uint32_t* vorg = nullptr;    // V+1: original (instance-local) variable
    uint32_t* scores = nullptr;  // V+1
    uint32_t* keys_a = nullptr;  // V+1 sort keys
    uint32_t* keys_b = nullptr;
    uint32_t* eligible = nullptr;    // V+1
    uint32_t* eligible_b = nullptr;  // V+1
    uint32_t* rank = nullptr;    // V+1
    uint32_t* varcore = nullptr; // V+1
    uint32_t* fcut = nullptr;    // n: largest frozen variable with varcore < 12, per instance
    uint32_t* elected = nullptr; // V+1
    uint32_t* work = nullptr;    // V+1 MIS worklist
    uint32_t* work_b = nullptr;  // V+1
    uint32_t* vscan = nullptr;   // V+2 scan scratch
    uint8_t* winv = nullptr;     // V+1 MIS round winners / BVE slot-fits flags
    uint4* ckeys = nullptr;      // per-clause sort key (size, first, last, sig)
    uint64_t ckeys_cap = 0;
    uint32_t nelected = 0;

    // BVE per index of the SUB+BVE set
    uint32_t* type = nullptr;
    uint32_t* ucnt = nullptr;
    unsigned long long* rpos = nullptr;   // clauses added (scan)
    unsigned long long* rref = nullptr;   // buckets added (scan)
    unsigned long long* rslot = nullptr;  // physical first clause slot
    unsigned long long* rlit = nullptr;   // physical first literal word
    uint32_t* veset = nullptr;            // SUB+BVE set (elected of instances in mode 1)
    uint32_t* ereset = nullptr;           // ERE set (elected of instances in mode 2)
    uint32_t nve = 0, nere = 0;

    // units, trail and model stack (one region per instance)
    uint32_t* units = nullptr; uint64_t units_total = 0;
    uint32_t* trail = nullptr; uint64_t trail_total = 0;
    uint32_t* stack = nullptr; uint64_t stack_total = 0;

    // BCP
    uint8_t* bstate = nullptr;
    uint32_t* front_a = nullptr;
    uint32_t* front_b = nullptr;
    uint32_t* long_a = nullptr;   // frontier literals whose lists are split over the grid
    uint32_t* long_b = nullptr;

    // counters
    DevCounters* dc = nullptr;   // device
    DevCounters* hc = nullptr;   // pinned host mirror

    // scratch
    void* tmp = nullptr; size_t tmp_cap = 0;
    uint32_t* tmp_u32 = nullptr; uint64_t tmp_u32_cap = 0;   // generic u32 scratch

    // DRAT proof (proof_en): a pass writes its lines into pf_w in blocks, each
    // block recorded in pf_b as {variable << 32 | sequence, first word}; a line
    // is a header word (bit 31 = deletion, low bits = length) followed by its
    // literals in original numbering, a zero word is padding. After the pass
    // the host orders the blocks by key and appends the lines, as bytes, to
    // the proof of the variable's instance.
    uint32_t* pf_w = nullptr; unsigned long long pf_wcap = 0;
    ulonglong2* pf_b = nullptr; uint32_t pf_bcap = 0;
    uint8_t* lbyte = nullptr;    // 2V+2: proof bytes of each literal (7-bit groups of its original)
    std::vector<uint32_t> pf_hw;
    std::vector<ulonglong2> pf_hb;

    // per-kernel profiler (launch counts always; CUDA-event timing when enabled)
    Profiler prof;

    // round state
    int simpstate = 0;
    uint32_t mis_rounds = 0;
    // host-side bounds of the device loops (0: the built-in bound from V)
    uint32_t lim_bcp_levels = 0, lim_mis_rounds = 0;
    pfg_stats stats{};

    // batch write-back (built on the first per-instance call): live clauses packed
    // on the device, grouped by instance, literals back in instance numbering and
    // offsets relative to the instance; each instance is copied from there
    // straight into the caller's buffers
    bool cache_ready = false;
    uint32_t* pk_lits = nullptr;
    unsigned long long* pk_roff = nullptr;
    uint8_t* pk_learnt = nullptr;
    uint8_t* pk_usage = nullptr;
    uint32_t* pk_lbd = nullptr;
    std::vector<uint64_t> cache_cls_base;       // n+1: first packed clause of each instance
    std::vector<uint64_t> cache_lit_base;       // n+1: first packed literal of each instance
    std::vector<uint64_t> cache_elim_cnt, cache_forced_cnt;
};

// ---- launch shapes: the built-in choices of the pfg_tuning fields left zero ----
constexpr uint32_t VE3_TICKET = 16;
constexpr uint32_t MIS_THREADS = 128;
constexpr uint32_t LIST_THREADS = 256;
constexpr uint32_t BCP_BLOCKS_PER_SM = 8;
unsigned sm_count();            // SMs of the current device (read once)
bool profiling(pfg_ctx* o);     // per-kernel timing on (engine.cu)
void set_error(pfg_ctx* o, const std::string& e);
inline unsigned tuned(uint32_t v, uint32_t dflt) { return v ? v : dflt; }

// ---- memory helpers (engine.cu) ----
bool dalloc(Ctx& c, void** p, size_t bytes);
void dfree(Ctx& c, void* p);
template <typename T>
inline bool dalloc_t(Ctx& c, T** p, size_t count) { return dalloc(c, (void**)p, count * sizeof(T)); }
bool ensure_tmp(Ctx& c, size_t bytes);
bool ensure_tmp_u32(Ctx& c, uint64_t count);
void sync_counters(Ctx& c);     // D2H copy of counters + stream sync
bool stream_sync(Ctx& c, const char* what);   // closes the profiler's open span, then waits for c.s
void push_inst_in(Ctx& c);      // H2D copy of the per-instance inputs
void pull_inst_out(Ctx& c);     // D2H copy of the per-instance outputs and counters + sync
bool cuda_ok(Ctx& c, cudaError_t e, const char* what);

// ---- passes ----
// occurrence table (ot.cu)
bool ot_build(Ctx& c);          // histogram + CSR offsets + unsorted fill (clause order irrelevant)
// sort lists by OLIST_CMP (key.cuh:67-85) or by clause id: all of them, or the two
// lists of every variable in vlist[0..nv)
// keys_ready: the clause keys of the previous ot_sort call still hold (no
// clause changed since), so they are not made again
bool ot_sort(Ctx& c, bool by_id, const uint32_t* vlist = nullptr, uint32_t nv = 0, bool keys_ready = false);
bool ot_filter(Ctx& c, const uint8_t* assigned);   // drop what unit propagation removed from the lists
// Incremental table between rounds: ot_prune drops deleted and flagged clauses and
// the lists of eliminated variables (run before a compaction, on the old ids);
// ot_update then moves the kept entries into a fresh CSR (through cbits when the
// store was compacted) and appends the flagged clauses.
bool ot_prune(Ctx& c);
bool ot_update(Ctx& c);
// counting + compaction (gc.cu)
void count_live(Ctx& c);        // totals into counters, per instance into dout.cnt (read after a sync)
bool compact_cnf(Ctx& c);       // Solver::reallocCNF(true) (cnf.cu:129-144, recycle.cu:60); keeps cbits when ot_valid
// device BCP (bcp.cu) of the instances flagged in di.bcp; conflicts land in dout.conflict
bool bcp_prop(Ctx& c);
// LCVE (lcve.cu) over the active instances; per-instance counts in dout.nelect
bool lcve(Ctx& c);
// SUB, BVE, ERE (elim.cu) over c.veset / c.ereset
bool sub_pass(Ctx& c);
bool ve_pass(Ctx& c);
bool ere_pass(Ctx& c);
bool bce_pass(Ctx& c);   // blocked clause elimination over the surviving elected variables
// DRAT proof of a pass (engine.cu): room for `words` line words before the pass,
// then the pass's blocks appended to the instances' proofs
bool proof_prepare(Ctx& c, unsigned long long words);
bool proof_collect(Ctx& c);
PFG_HD uint32_t varint_len(uint32_t x) {
    uint32_t n = 1;
    while (x >= 0x80u) { x >>= 7; n++; }
    return n;
}

// device helper: instance of a global variable (binary search over voff[0..n])
PFG_D uint32_t inst_search(const uint32_t* voff, uint32_t n, uint32_t v) {
    uint32_t lo = 0, hi = n;   // largest i < n with voff[i] < v
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (voff[mid] < v) lo = mid; else hi = mid;
    }
    return lo;
}

}  // namespace pfg
