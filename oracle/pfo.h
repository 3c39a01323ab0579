/*
 * pfo.h - oracle for the GPU simplify path (TEST INFRASTRUCTURE ONLY).
 *
 * A sequential CPU restatement of ParaFROST's GPU simplification round
 * (src/gpu/simplify.cu:136-241 and the kernels it calls). Only tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg may load it, and
 * only as the checker or the timed CPU baseline; the product never calls it.
 *
 * Parity status: the reference GPU simplifier cannot be built or run in this
 * environment (its cuArena dependency is an empty submodule) and the
 * reference ships no tests or golden vectors for this path, so this oracle is
 * pinned against the reference's CPU solver on properties (model validity and
 * satisfiability agreement), not bit-for-bit: parity unpinned.
 *
 * Where the reference is nondeterministic (atomic append orders), the oracle
 * follows one legal schedule of the reference's kernels:
 *   - warps append in ascending thread index (elected variables in
 *     (MIS round, rank) order; frozen variables in ascending id);
 *   - a kernel's threads run one after another in thread-index order.
 */
#ifndef PFO_H
#define PFO_H

#include <stdint.h>
#include "../include/pfgpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct pfo_round {
    uint32_t elected;        /* variables elected by LCVE                 */
    uint32_t mis_rounds;     /* Luby MIS rounds                            */
    uint32_t eliminated;     /* variables eliminated by BVE this round     */
    uint32_t units;          /* units produced (SUB + BVE)                 */
    uint32_t resolvents;     /* clauses added by BVE                       */
    uint64_t clauses_before; /* live clauses entering SUB                  */
    uint64_t literals_before;
    uint64_t clauses_after;  /* live clauses after BVE                     */
    uint64_t literals_after;
} pfo_round;

typedef struct pfo_result {
    int32_t  status;         /* PFG_UNKNOWN / PFG_SAT / PFG_UNSAT          */
    int32_t  simpstate;
    int32_t  rounds;
    int32_t  ere_ran;
    uint32_t max_var;
    uint64_t ncls, nlits;
    uint32_t* lits;          /* simplified CNF in clause order             */
    uint64_t* cls_off;       /* ncls + 1                                   */
    uint8_t*  cls_learnt;
    uint32_t* cls_lbd;
    uint8_t*  cls_usage;
    uint8_t*  eliminated;    /* max_var + 1                                */
    uint64_t  nunits;
    uint32_t* units;         /* propagated units (sorted set)              */
    uint64_t  npending;
    uint32_t* pending;       /* units left after the last round (sorted)   */
    uint64_t  nstack;
    uint32_t* stack;         /* model-reconstruction stack                 */
    uint64_t  nround_ends;
    uint64_t* round_ends;    /* stack length after each round              */
    uint64_t  nround_stats;
    pfo_round* round_stats;
    uint64_t  nproof;
    uint8_t*  proof;         /* binary DRAT lines of the simplifier (proof_en)  */
} pfo_result;

/* Run one Solver::simplify call on the given clause database. */
int pfo_simplify(const pfg_options* opts, uint32_t max_var, uint64_t ncls,
                 const uint32_t* lits, const uint64_t* cls_off,
                 const uint8_t* cls_learnt, const uint32_t* cls_lbd,
                 const uint8_t* cls_usage, const uint8_t* var_state,
                 const uint8_t* assumed, const uint32_t* vorg,
                 pfo_result** out);

void pfo_free(pfo_result* r);

/*
 * Canonical form for comparisons (both the oracle's and the engine's output
 * go through it): clauses sorted lexicographically by (size, literals...,
 * learnt, lbd, usage); the stack split into per-variable blocks and, inside
 * each round, the blocks sorted by witness variable. Writes into
 * caller-allocated arrays of the same sizes as the inputs.
 */
int pfo_canon_cnf(uint64_t ncls, const uint32_t* lits, const uint64_t* off,
                  const uint8_t* learnt, const uint32_t* lbd, const uint8_t* usage,
                  uint32_t* out_lits, uint64_t* out_off, uint8_t* out_learnt,
                  uint32_t* out_lbd, uint8_t* out_usage);

int pfo_canon_stack(uint64_t nstack, const uint32_t* stack, uint64_t nrounds,
                    const uint64_t* round_ends, uint32_t* out_stack);

/*
 * Extend an assignment of the simplified formula to the original variables
 * by walking the stack backwards (src/gpu/model.cpp:101-135). `value[v]` is
 * 0/1 for v in [1, max_var]; updated in place.
 */
void pfo_extend_model(uint64_t nstack, const uint32_t* stack, uint8_t* value);

/*
 * RUP check of a binary DRAT proof (test helper): every added line must follow
 * by unit propagation from the formula plus the earlier lines, minus deleted
 * clauses. Returns 0 when every line checks, else the 1-based number of the
 * first line that does not (or is malformed); *missing_deletions counts
 * deletions of clauses that were not present.
 */
int64_t pfo_check_rup(uint32_t V, uint64_t ncls, const uint32_t* lits, const uint64_t* off,
                      const uint8_t* proof, uint64_t nproof, uint64_t* missing_deletions);

/*
 * Small DPLL solver for the tests (two watched literals). Returns 10 (SAT,
 * model written to value[1..V]), 20 (UNSAT) or 0 (decision budget spent).
 */
int pfo_solve(uint32_t V, uint64_t ncls, const uint32_t* lits, const uint64_t* off,
              uint8_t* value, uint64_t max_decisions);

#ifdef __cplusplus
}
#endif

#endif
