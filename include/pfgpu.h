/*
 * pfgpu.h - C ABI of the GB300-native CNF inprocessing engine.
 *
 * This header is the drop-in boundary for ParaFROST's GPU simplify phase.
 * The reference has no C ABI for this path: its boundary is the C++ member
 * function `void Solver::simplify(const bool& skip_transfer_to_host)`
 * (src/gpu/solver.hpp:772, src/gpu/simplify.cu:57) whose body
 * (`Solver::simplifying`, src/gpu/simplify.cu:136-241) uploads the clause
 * database (`awaken`, simplify.cu:77-134), runs the round loop
 * (simplify.cu:163-186) and writes results back (simplify.cu:190-240).
 * The entry points below replace that body: a host adapter inside
 * `Solver::simplifying` calls pfg_upload after its rootify/shrinkTop, then
 * pfg_simplify, pfg_result_sizes_get and pfg_download, and writes the
 * clauses, units, eliminated variables and model stack back into the solver.
 *
 * Conventions
 *  - Literals use the reference's internal encoding: lit = 2*v | sign,
 *    v in [1, max_var] (src/gpu/constants.hpp:72-80).
 *  - The caller owns every host buffer; the engine owns all device memory
 *    (it replaces cuMM/cuArena, src/gpu/memory.cuh:54-180).
 *  - No entry point exits, traps or throws. Calls on one context must come
 *    from one host thread; contexts are independent.
 *  - Return codes mirror the reference's `simpstate` values
 *    (src/gpu/constants.cuh:28-31) plus engine-specific codes.
 */
#ifndef PFGPU_H
#define PFGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* return codes: 0..3 keep the reference's simpstate meaning */
#define PFG_OK             0  /* AWAKEN_SUCC                                  */
#define PFG_AWAKEN_FAIL    1  /* AWAKEN_FAIL  (device pool could not be made) */
#define PFG_CNFALLOC_FAIL  2  /* CNFALLOC_FAIL (clause store does not fit)    */
#define PFG_OTALLOC_FAIL   3  /* OTALLOC_FAIL  (occurrence table does not fit)*/
#define PFG_TIMEOUT        4  /* a bounded device-side loop gave up           */
#define PFG_INVALID        5  /* invalid argument or input                    */
#define PFG_CUDA_ERROR     6  /* a CUDA runtime call failed                   */
#define PFG_PENDING        7  /* serving: the job has not finished yet        */

/* solver status after pfg_simplify (same values as the reference CLI/IPASIR) */
#define PFG_UNKNOWN        0
#define PFG_SAT           10  /* every clause was removed                       */
#define PFG_UNSAT         20  /* device unit propagation found a conflict       */

/*
 * Simplifier options. Names in comments are the reference's CLI option names
 * and defaults (src/gpu/options.cpp:24-43, src/gpu/options.cu:33-60); the
 * folding rules of OPTION::init (options.cpp:274-299) are applied by
 * pfg_resolve_options().
 */
typedef struct pfg_options {
    int32_t  phases;          /* "phases"            5     */
    int32_t  shrink_rate;     /* "collectfreq"       2     */
    int32_t  lcve_fast;       /* "lcvefast"          1 (Luby MIS) */
    uint32_t lcve_min_vars;   /* "electionsmin"      2     */
    uint32_t lcve_max_occurs; /* "electionsmax"      3000  */
    int32_t  lcve_clause_max; /* "lcveclausemax"     30000 */
    uint32_t phase_lits_min;  /* "eliminatedlitsmin" 500   */
    uint32_t mu_pos;          /* "mupos"             32    */
    uint32_t mu_neg;          /* "muneg"             32    */
    double   lits_mul;        /* "literalsmul"       1.0   */
    uint8_t  ve_en;           /* "ve"                1     */
    uint8_t  ve_plus_en;      /* "veextend"          1     */
    uint8_t  sub_en;          /* "sub"               1     */
    uint8_t  ere_en;          /* "ere"               1     */
    uint8_t  bce_en;          /* "bce"               0     */
    uint8_t  all_en;          /* "all"               0     */
    uint8_t  ve_fun_en;       /* "vefunction"        1     */
    uint8_t  ve_lbound_en;    /* "velitsbound"       0     */
    uint8_t  proof_en;        /* "proof"             0: emit the binary DRAT lines of
                                 SUB, BVE, BCE and ERE (pfg_download_proof)           */
    uint8_t  ve_inprocess;    /* 1 when Solver::stats.sigma.calls > 1: BVE counts only
                                 original clauses (in_ve_k_1, bounded.cuh:397)       */
    uint8_t  _pad[6];
    uint32_t ve_clause_max;   /* "resolventmax"      100   */
    uint32_t xor_max_arity;   /* "xormaxarity"       10    */
    uint32_t sub_max_occurs;  /* "submaxoccurs"      3000  */
    uint32_t ere_max_occurs;  /* "eremaxoccurs"      3000  */
    uint32_t ere_clause_max;  /* "ereclausemax"      250 (clamped to 250)  */
    uint32_t bce_max_occurs;  /* "bcemaxoccurs"      3000  */
} pfg_options;

/* Per-call statistics (the reference's stats.sigma / inf counters). */
typedef struct pfg_stats {
    int32_t  status;          /* PFG_UNKNOWN / PFG_SAT / PFG_UNSAT                 */
    int32_t  rounds;          /* SUB+BVE rounds executed (reference `phase`)       */
    int32_t  ere_ran;         /* 1 if the final ERE pass ran                       */
    int32_t  simpstate;       /* reference simpstate at exit                       */
    uint64_t clauses_in;      /* live clauses uploaded                              */
    uint64_t literals_in;
    uint64_t clauses_out;     /* live clauses after simplification                  */
    uint64_t literals_out;
    uint64_t clauses_processed; /* sum over rounds of live clauses entering SUB+BVE */
    uint64_t literals_processed;
    uint64_t eliminated;      /* variables eliminated (MELTING bit, not FORCED)     */
    uint64_t forced;          /* variables assigned by device unit propagation      */
    uint64_t resolvents;      /* clauses added by BVE                               */
    uint64_t stack_words;     /* model-reconstruction words produced                */
    double   device_ms;       /* cudaEvent time of all rounds (upload/download excluded) */
    double   pass_ms[8];      /* per pass: ot, bcp, lcve, sub, ve, ere, gc/count, other */
    uint64_t alg_bytes;       /* algorithmic bytes of all rounds (4-byte literal and clause words each pass must move);
                                 the elected lists' term 8(L_E + C_E) takes a pass of its own and is counted only
                                 while the profiler is on (pfg_profile_enable) */
    uint64_t kernel_launches; /* kernels launched by pfg_simplify                   */
} pfg_stats;

/* Sizes of the results of the last pfg_simplify call. */
typedef struct pfg_result_sizes {
    uint64_t clauses;         /* live clauses in the simplified CNF                */
    uint64_t literals;        /* their literals                                     */
    uint64_t units;           /* units assigned on the device (set, sorted)         */
    uint64_t pending_units;   /* units produced by the last round and not propagated */
    uint64_t stack_words;     /* model-reconstruction stack words                   */
    uint64_t rounds;          /* entries of round_ends                              */
    uint32_t max_var;
    uint32_t _pad;
    uint64_t proof_bytes;     /* binary DRAT bytes (proof_en)                       */
} pfg_result_sizes;

typedef struct pfg_ctx pfg_ctx;

/* sizeof of the ABI structs as compiled into the library (FFI layout check). */
void pfg_abi_sizes(size_t* options, size_t* stats, size_t* result_sizes);

/* Fill `o` with the reference defaults. */
void pfg_default_options(pfg_options* o);

/* Apply OPTION::init's folding rules (src/gpu/options.cpp:283-297). */
void pfg_resolve_options(pfg_options* o);

/*
 * Create a context on the current CUDA device with a device pool of
 * `arena_bytes` (0 = size it from the free device memory, as
 * cuMM::initDeviceArena does, src/gpu/memory.cu:99-176).
 * Replaces: Solver::optSimp + cuMM::init (simplify.cu:243, memory.cu:99).
 */
int  pfg_create(pfg_ctx** ctx, const pfg_options* opts, size_t arena_bytes);

/*
 * Upload one CNF instance (host buffers, internal literal encoding).
 *   lits[cls_off[i] .. cls_off[i+1])  literals of clause i (any order, no duplicates,
 *                                     size >= 2);
 *   cls_learnt[i]  0 = original, 1 = learnt (nullable: all original)
 *   cls_lbd[i], cls_usage[i]  learnt metadata (nullable)
 *   var_state[v]   non-zero VSTATE.state excludes v from elections (nullable)
 *   assumed[v]     non-zero excludes v from elections (nullable)
 *   vorg[v]        original variable of v used in the model stack (nullable: identity)
 * Clause order is preserved: originals are expected first, then learnts, as
 * Solver::extractCNF appends them (simplify.cu:108-109, cnf.cu:176-184).
 * Replaces: Solver::awaken (simplify.cu:77-134): extractCNF/reflectCNF and
 * prepareCNFAsync (cnf.cu:108).
 */
int  pfg_upload(pfg_ctx* ctx, uint32_t max_var, uint64_t num_clauses,
                const uint32_t* lits, const uint64_t* cls_off,
                const uint8_t* cls_learnt, const uint32_t* cls_lbd,
                const uint8_t* cls_usage, const uint8_t* var_state,
                const uint8_t* assumed, const uint32_t* vorg);

/*
 * Run simplification rounds until the reference's stop rule
 * (Solver::stop, solver.hpp:748-753).
 * Replaces: the round loop of Solver::simplifying (simplify.cu:159-186).
 */
int  pfg_simplify(pfg_ctx* ctx, pfg_stats* stats);

/*
 * Simplify k uploaded contexts at once: ctxs[0] on the calling thread,
 * ctxs[1..k) on host threads of their own, every context on its own stream,
 * so one context's kernels use the GPU while another waits on the host or
 * runs a narrow pass. The contexts must be distinct and on one device.
 * stats[j] is what pfg_simplify(ctxs[j], ...) gives; *device_ms (nullable)
 * is the device time of the whole job, from an event every stream waits on
 * before its first kernel to the last context's end. Every context runs;
 * the result is the first code other than PFG_OK in context order.
 * Replaces: nothing in the reference (one instance per solver): it runs a
 * batch cut into runs of instances (pfg_batch_upload per context) as one job.
 */
int  pfg_simplify_many(pfg_ctx* const* ctxs, uint32_t k, pfg_stats* stats, float* device_ms);

/* Sizes needed by pfg_download. */
int  pfg_result_sizes_get(pfg_ctx* ctx, pfg_result_sizes* sizes);

/*
 * Copy results to host buffers sized by pfg_result_sizes_get (any pointer
 * may be NULL to skip that item).
 *   lits/cls_off/cls_learnt/cls_lbd/cls_usage: simplified CNF in clause order
 *       (Solver::cacheCNF, cnf.cu:200-236)
 *   eliminated[max_var+1]: MELTING 0x1 | ADDING 0x2 | FORCED 0x4 bytes
 *       (Solver::cacheEliminated, transfer.cu:69)
 *   units: literals assigned by device propagation, sorted ascending
 *       (what Solver::prop enqueues on the host trail, elimbcp.cu:193-203)
 *   pending_units: units produced in the last round that no later round
 *       propagated (the reference leaves them in vars->units)
 *   stack: model-reconstruction words [lit_w, l2..lk, k]* [w, 1] in original
 *       variable numbering (Solver::cacheResolved, transfer.cu:83)
 *   round_ends[r]: stack length after round r
 */
int  pfg_download(pfg_ctx* ctx, uint32_t* lits, uint64_t* cls_off,
                  uint8_t* cls_learnt, uint32_t* cls_lbd, uint8_t* cls_usage,
                  uint8_t* eliminated, uint32_t* units, uint32_t* pending_units,
                  uint32_t* stack, uint64_t* round_ends);

/*
 * Batched simplification: n independent instances in one device clause store,
 * every pass launched once for all of them. Each instance keeps its own round
 * counter, stop rule, capacities and results, so its output is the one a
 * single pfg_upload/pfg_simplify of that instance gives. pfg_upload is the
 * n = 1 case. (No counterpart in the reference, which simplifies one CNF.)
 */
typedef struct pfg_instance {
    uint32_t        max_var;
    uint32_t        _pad;
    uint64_t        num_clauses;
    const uint32_t* lits;
    const uint64_t* cls_off;
    const uint8_t*  cls_learnt;   /* nullable */
    const uint32_t* cls_lbd;      /* nullable */
    const uint8_t*  cls_usage;    /* nullable */
    const uint8_t*  var_state;    /* nullable */
    const uint8_t*  assumed;      /* nullable */
    const uint32_t* vorg;         /* nullable: identity */
} pfg_instance;

int  pfg_batch_upload(pfg_ctx* ctx, uint32_t n, const pfg_instance* instances);
/* number of instances of the last upload */
uint32_t pfg_batch_size(pfg_ctx* ctx);
/* statistics of instance i of the last pfg_simplify (totals come from pfg_simplify itself) */
int  pfg_batch_stats(pfg_ctx* ctx, uint32_t i, pfg_stats* stats);
int  pfg_batch_result_sizes(pfg_ctx* ctx, uint32_t i, pfg_result_sizes* sizes);
int  pfg_batch_download(pfg_ctx* ctx, uint32_t i, uint32_t* lits, uint64_t* cls_off,
                        uint8_t* cls_learnt, uint32_t* cls_lbd, uint8_t* cls_usage,
                        uint8_t* eliminated, uint32_t* units, uint32_t* pending_units,
                        uint32_t* stack, uint64_t* round_ends);
/* The same for all instances at once: sizes[0..n), then every output holds the
   instances back to back in instance order, each part laid out as
   pfg_batch_download writes it (cls_off: clauses + 1 entries from 0,
   eliminated: max_var + 1 entries). One copy per output instead of one per
   instance and output. */
int  pfg_batch_result_sizes_all(pfg_ctx* ctx, pfg_result_sizes* sizes);
int  pfg_batch_download_all(pfg_ctx* ctx, uint32_t* lits, uint64_t* cls_off,
                            uint8_t* cls_learnt, uint32_t* cls_lbd, uint8_t* cls_usage,
                            uint8_t* eliminated, uint32_t* units, uint32_t* pending_units,
                            uint32_t* stack, uint64_t* round_ends);

/*
 * DRAT proof of the last pfg_simplify (proof_en), size in
 * pfg_result_sizes.proof_bytes: the binary lines the reference's device passes
 * write (src/gpu/proof.cu, proofutils.cuh) -- clauses strengthened by SUB
 * added and clauses it subsumed deleted, clauses substituted and resolvents
 * (units included) added by BVE, blocked clauses deleted by BCE, redundant
 * clauses deleted by ERE -- with literals in original variable numbering
 * (vorg). A line is 'a' (97) or 'd' (100), then every literal 2v+s in 7-bit
 * groups, low group first, the high bit set on all groups but the last, then
 * a zero byte. The reference appends the lines of a pass in the order its
 * threads get to them; here the passes of a round follow each other (SUB, BVE
 * substitutions, BVE resolvents, BCE, ERE) and inside a pass the lines of the
 * variables come in variable order, each variable's in the reference's order.
 * Replaces: cuPROOF::cacheProof / writeProof (src/gpu/proof.cu:184-246).
 */
int  pfg_download_proof(pfg_ctx* ctx, uint8_t* out);
int  pfg_batch_download_proof(pfg_ctx* ctx, uint32_t i, uint8_t* out);
/* Text form of a binary proof (the reference's non-binary writer,
   cuPROOF::writeClause, src/gpu/proof.cu:130-160): "d " before deletions,
   signed decimal literals each followed by a space, then "0\n". *len gets the
   text length; `out` (may be NULL) receives min(cap, *len) bytes. PFG_INVALID
   on a malformed stream. */
int  pfg_proof_text(const uint8_t* bin, uint64_t n, char* out, uint64_t cap, uint64_t* len);

/*
 * The simplified CNF of a one-instance context written straight into
 * caller-owned DEVICE buffers (sizes from pfg_result_sizes_get; any pointer
 * may be NULL), allocating no device or host memory. No counterpart in the
 * reference, whose write-back always goes through host buffers (cacheCNF,
 * src/gpu/cnf.cu:200-236).
 *
 * For callers that pass the clauses on to another GPU stage and cannot
 * allocate while doing so: a serving loop that has reserved the device's
 * memory for its own arena (an allocation would fail or eat into another
 * job's share), or code that must not stall on the device-wide
 * synchronisation cudaMalloc/cudaFree bring while other streams are busy.
 * pfg_download allocates packing buffers on every call.
 *
 * Scratch is one static 16 MiB device array per device, enough for a clause
 * store of about 1.3 million slots (live or deleted); a larger store is
 * rejected with PFG_INVALID and pfg_last_error says the limit. Every device
 * that loads the library holds the array until the process exits, whether or
 * not this call is used. Each call looks the array's address up with
 * cudaGetSymbolAddress in the current context; the first call on a device
 * may load the module, so make that first call before any stream capture.
 * The context's device must be the current device (PFG_CUDA_ERROR
 * otherwise). No scratch word
 * has to start at zero (each call writes every word before reading it). Calls
 * that overlap in time on one device -- from two threads, or on two contexts
 * whose streams run at once -- share the array and corrupt each other's
 * output: run them one after another. Returns once its work on the context's
 * stream has finished.
 */
int  pfg_download_device_noalloc(pfg_ctx* ctx, uint32_t* d_lits, uint64_t* d_cls_off,
                                 uint8_t* d_cls_learnt, uint32_t* d_cls_lbd,
                                 uint8_t* d_cls_usage);

/*
 * Serving: a request loop for simplification jobs that arrive over time (no
 * counterpart in the reference). Jobs are queued by pfg_server_submit (the
 * server copies the instance) and admitted in arrival order while their
 * estimated device footprint fits the server's arena budget. `slots` worker
 * threads each own a context and stream; a free worker takes every admitted
 * job that is waiting (up to `max_batch`) and simplifies them as one batch
 * (pfg_batch_upload), so jobs that arrive while other batches are on the GPU
 * start as soon as a slot and memory free up, and the batches of different
 * slots overlap on the device. Each job's result is the one it gives alone.
 */
typedef struct pfg_server pfg_server;

typedef struct pfg_job_info {
    int32_t  rc;              /* PFG_OK or the error of the job's batch      */
    int32_t  status;          /* PFG_UNKNOWN / PFG_SAT / PFG_UNSAT           */
    uint32_t batch_size;      /* jobs in the batch that ran it               */
    uint32_t slot;            /* worker that ran it                          */
    uint64_t est_bytes;       /* device footprint charged at admission       */
    uint64_t t_submit_ns;     /* steady-clock times                          */
    uint64_t t_admit_ns;
    uint64_t t_done_ns;
    uint64_t clauses_processed;
    pfg_result_sizes sizes;   /* buffer sizes for pfg_server_fetch           */
} pfg_job_info;

typedef struct pfg_server_stats {
    uint64_t submitted, admitted, done, batches;
    uint64_t max_in_flight_batches;   /* most batches on the device at once   */
    uint64_t max_jobs_in_flight;
    uint64_t peak_est_bytes;          /* most device bytes charged at once    */
    uint64_t budget_bytes;
} pfg_server_stats;

int  pfg_server_create(pfg_server** server, const pfg_options* opts, size_t arena_bytes,
                       uint32_t slots, uint32_t max_batch);
/* queue one job; the instance is copied, the caller's buffers may be reused at once */
int  pfg_server_submit(pfg_server* server, const pfg_instance* job, uint64_t* ticket);
/* PFG_OK and `info` once the job is done, PFG_PENDING while it is queued or
   running (waits up to wait_ms first), PFG_INVALID for an unknown ticket */
int  pfg_server_poll(pfg_server* server, uint64_t ticket, int32_t wait_ms, pfg_job_info* info);
/* copy the result of a finished job (buffers sized by info.sizes, any may be
   NULL) and forget the job; outputs as pfg_download */
int  pfg_server_fetch(pfg_server* server, uint64_t ticket, uint32_t* lits, uint64_t* cls_off,
                      uint8_t* cls_learnt, uint32_t* cls_lbd, uint8_t* cls_usage,
                      uint8_t* eliminated, uint32_t* units, uint32_t* pending_units,
                      uint32_t* stack, uint64_t* round_ends);
/* copy the binary DRAT proof of a finished job (info.sizes.proof_bytes bytes;
   nothing without proof_en) and keep the job: call it before pfg_server_fetch.
   The lines are the ones pfg_batch_download_proof gives for the instance, so
   the same as the instance simplified alone. */
int  pfg_server_fetch_proof(pfg_server* server, uint64_t ticket, uint8_t* out);
int  pfg_server_stats_get(pfg_server* server, pfg_server_stats* stats);
/* finish every queued job, stop the workers and free everything */
void pfg_server_destroy(pfg_server* server);
const char* pfg_server_last_error(pfg_server* server);

/*
 * DIMACS ingest (Solver::parse / toClause, src/gpu/dimacs.cpp:41-290): the file
 * is memory-mapped and normalised as the reference does while parsing --
 * repeated literals dropped, tautologies dropped, literals of unit clauses read
 * earlier applied, one-literal clauses returned as units, an empty clause
 * reported as PFG_UNSAT. The clauses come out in the layout pfg_upload takes.
 */
typedef struct pfg_dimacs pfg_dimacs;
typedef struct pfg_dimacs_info {
    uint32_t max_var;          /* from the header                                  */
    int32_t  status;           /* PFG_UNKNOWN, or PFG_UNSAT (empty clause, conflict) */
    uint64_t header_clauses;
    uint64_t num_clauses;      /* clauses of two or more literals                  */
    uint64_t num_literals;
    uint64_t num_units;
} pfg_dimacs_info;

/* *out is always set (free it with pfg_dimacs_free); on PFG_INVALID
   pfg_dimacs_error says why */
int  pfg_dimacs_read(const char* path, pfg_dimacs** out);
int  pfg_dimacs_get_info(pfg_dimacs* d, pfg_dimacs_info* info);
/* lits[num_literals], cls_off[num_clauses + 1], units[num_units]; any may be NULL */
int  pfg_dimacs_copy(pfg_dimacs* d, uint32_t* lits, uint64_t* cls_off, uint32_t* units);
const char* pfg_dimacs_error(pfg_dimacs* d);
void pfg_dimacs_free(pfg_dimacs* d);

/*
 * Write-back helpers for the host solver (host code, no device work).
 * pfg_map_vars: VMAP::initiate (src/gpu/vmap.hpp:61-72) -- variables whose
 * eliminated byte is 0 are renumbered 1..*new_max_var in increasing order
 * (new_of_old[max_var + 1], 0 for dropped ones; old_of_new[max_var + 1] may be
 * NULL). pfg_map_lits: mapLit (vmap.hpp:44) over n literals; PFG_INVALID if
 * one belongs to a dropped variable. pfg_extend_model: MODEL::extend
 * (src/gpu/model.cpp:101-160) over the model stack, value[1..max_var] in
 * {0, 1} on entry and on return.
 */
int  pfg_map_vars(uint32_t max_var, const uint8_t* eliminated, uint32_t* new_of_old, uint32_t* old_of_new,
                  uint32_t* new_max_var);
int  pfg_map_lits(const uint32_t* new_of_old, uint32_t max_var, uint64_t n, const uint32_t* in, uint32_t* out);
int  pfg_extend_model(uint64_t nstack, const uint32_t* stack, uint32_t max_var, uint8_t* value);

/* Page-locked host memory for input and result buffers (cuMM::allocPinned,
   src/gpu/memory.cu:505-523): uploads from and downloads into it are direct
   DMA transfers. NULL when it cannot be allocated. */
void* pfg_host_alloc(size_t bytes);
void  pfg_host_free(void* p);

/* Release all device memory of the context. Replaces Solver::freeSimp (simplify.cu:254). */
void pfg_destroy(pfg_ctx* ctx);

/* Last CUDA or engine error message of the context (never NULL). */
const char* pfg_last_error(pfg_ctx* ctx);

/* Number of this library's kernels launched since the context was created. */
uint64_t pfg_kernel_launches(pfg_ctx* ctx);

/*
 * Per-kernel profiling of pfg_simplify. Launch counts are always kept; with
 * profiling enabled every launch is also bracketed by CUDA events on the
 * context's stream. Kernel groups are numbered 0 .. pfg_profile_count()-1;
 * alg_bytes is the algorithmic byte count of the group (the literal and
 * clause words its passes must read or write, 4 bytes each).
 */
int  pfg_profile_enable(pfg_ctx* ctx, int on);
void pfg_profile_reset(pfg_ctx* ctx);
int  pfg_profile_count(void);
const char* pfg_profile_name(int id);
int  pfg_profile_get(pfg_ctx* ctx, int id, uint64_t* launches, double* ms, uint64_t* alg_bytes);

/*
 * Launch shapes per pass, and the autotuner that picks them. Replaces the
 * reference's launch-configuration macros, which size grids from the device
 * properties alone (OPTIMIZEBLOCKS, OPTIMIZEBLOCKSELIM, OPTIMIZEBLOCKSERE,
 * OPTIMIZEBLOCKS2, OPTIMIZESHARED, src/gpu/grid.cuh:137-232, and the
 * veminthreads-style options, src/gpu/options.cu:36-47). A zero field means
 * the built-in choice (shown in brackets). No field changes any result: the
 * passes are schedule-independent, only their speed moves.
 */
typedef struct pfg_tuning {
    uint32_t sub_blocks_per_sm;  /* SUB warp kernel: blocks per SM of its persistent grid [all the SM holds] */
    uint32_t ve1_blocks_per_sm;  /* BVE phase 1 warp kernel, likewise [all] */
    uint32_t ve3_blocks_per_sm;  /* BVE phase 3 warp kernel, likewise [all] */
    uint32_t ve3_ticket;         /* variables per work-stealing draw in BVE phase 3 [16] */
    uint32_t mis_threads;        /* block size of the MIS round kernels (multiple of 32, <= 1024) [128] */
    uint32_t list_threads;       /* block size of the occurrence-list passes (multiple of 32, <= 1024) [256] */
    uint32_t bcp_blocks_per_sm;  /* blocks per SM of each propagation level [8] */
    uint32_t _reserved[9];
} pfg_tuning;

/* The context's launch shapes (kept across uploads). Set rejects a field out
 * of range with PFG_INVALID and changes nothing then. */
int pfg_tuning_get(pfg_ctx* ctx, pfg_tuning* out);
int pfg_tuning_set(pfg_ctx* ctx, const pfg_tuning* t);

/*
 * Bounds of the two host-driven device loops of a simplify call: levels of
 * device unit propagation (the loop of Solver::prop, src/gpu/elimbcp.cu:168-177)
 * and Luby MIS rounds of one election (the loop of Solver::LCVE,
 * src/gpu/lcve.cu:356-363). The reference loops until they converge; the
 * engine gives up beyond a bound and pfg_simplify returns PFG_TIMEOUT with
 * pfg_last_error naming the loop. 0 (the default) keeps the built-in bounds,
 * max_var + 2 levels and (candidates + 2) rounds, which a correct run never
 * reaches. A caller with a latency budget may set lower ones; a context that
 * returned PFG_TIMEOUT holds a partial result and takes a new upload (or
 * pfg_destroy). Kept across uploads.
 */
int pfg_set_loop_limits(pfg_ctx* ctx, uint32_t max_bcp_levels, uint32_t max_mis_rounds);

/*
 * Measured choice of the launch shapes on the caller's instances: every trial
 * uploads the n instances, simplifies them with per-kernel timing and reads
 * each tuned pass's own kernel time; the knobs of different passes are swept
 * together (one trial per candidate), then the BVE phase 3 ticket with the
 * best grid. `repeats` trials per candidate, the fastest counts. The best
 * shapes are set on the context and written to *out (if not NULL). The
 * context holds the last trial's result afterwards: upload again before the
 * next simplify. Profiling is left as it was.
 */
int pfg_autotune(pfg_ctx* ctx, uint32_t n, const pfg_instance* instances, uint32_t repeats, pfg_tuning* out);

/*
 * Host-side synthetic CNF generators (the seeded families used by the
 * benchmark and the tests). They write into caller buffers; call once with
 * lits == NULL to get the sizes.
 *   family 0: uniform random k-SAT   (a = vars, b = clauses, c = k)
 *   family 1: Tseitin circuit        (a = gates, b = primary inputs, c = outputs)
 *   family 2: scale-free CNF         (a = vars, b = clauses, c = 1: planted model)
 */
int  pfg_generate(int family, uint64_t a, uint64_t b, uint64_t c, uint64_t seed,
                  uint32_t* max_var, uint64_t* num_clauses, uint64_t* num_lits,
                  uint32_t* lits, uint64_t* cls_off);

#ifdef __cplusplus
}
#endif

#endif /* PFGPU_H */
