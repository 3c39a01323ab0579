// Least-constrained variable elections (LCVE).
//
// Replaces Solver::varReorder + Solver::LCVE (src/gpu/lcve.cu:221-417):
//   - scores ps*ns (uint32, assign_scores :221) ordered by (score, var) with the
//     engine's stable radix sort instead of thrust::sort with GPU_LCV_CMP; the
//     parallel elections order only their candidates, which keeps their
//     relative order, the only one the rounds read;
//   - the Luby-style MIS (mis_init_k/mis_round_k/mis_freeze_k :143-209) runs on
//     a shrinking worklist kept in rank order, so winners are appended in
//     (round, rank) order -- one legal order of the reference's atomic appends;
//   - frozen variables get their function-table index from a scan in
//     ascending variable order (mis_collect_k + mapfrozen_k :211-260).
// The sequential lcve_k (:63-98, option lcvefast=0) runs on one thread per
// instance, as in the reference, over occurrence lists sorted by clause id.
// With several instances the global (score, var) order restricted to one
// instance is that instance's own order, neighbours never cross instances, and
// the elected list is grouped by instance, so every instance elects exactly
// what it elects alone.
#include "engine.cuh"

namespace pfg {
namespace {

constexpr uint8_t MIS_NONE = 0, MIS_UNDECIDED = 1, MIS_ELECTED = 2, MIS_FROZEN = 3;
// rank[v] is v's place in the (score, var) order while v is undecided and
// NO_RANK otherwise (not a candidate, elected or frozen), so "an undecided
// neighbour of smaller rank" is one load per neighbour: rank[u] < r
constexpr uint32_t NO_RANK = 0xFFFFFFFFu;

// keys/vals (the sort's input over every variable) only when given
__global__ void scores_k(const uint32_t* hist, uint32_t V, uint32_t* scores, uint32_t* keys, uint32_t* vals,
                         DevCounters* dc) {
    uint32_t mx = 0;
    for (uint32_t v = 1 + blockIdx.x * blockDim.x + threadIdx.x; v <= V; v += gridDim.x * blockDim.x) {
        const uint32_t s = hist[2 * v] * hist[2 * v + 1];   // uint32 product, as assign_scores
        scores[v] = s;
        if (keys) {
            keys[v - 1] = s;
            vals[v - 1] = v;
        }
        mx = max(mx, s);
    }
    for (int d = 16; d > 0; d >>= 1) mx = max(mx, __shfl_down_sync(0xFFFFFFFFu, mx, d));
    if ((threadIdx.x & 31u) == 0 && mx) atomicMax(&dc->nfrozen, mx);   // nfrozen reused as max score here
}

// A variable that occurs in a live clause longer than lcveclausemax is never a
// candidate (mis_init_k, lcve.cu:150-173); one pass over the clauses marks them.
__global__ void oversize_mark_k(const ClsHdr* __restrict__ hdr, const uint32_t* __restrict__ lits, uint64_t ncls,
                                int maxcsize, uint8_t* mark) {
    for (uint64_t c = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; c < ncls; c += (uint64_t)gridDim.x * blockDim.x) {
        const ClsHdr h = hdr[c];
        if (m_deleted(h.meta) || (int)h.size <= maxcsize) continue;
        for (uint32_t k = 0; k < h.size; k++) mark[ABSV(lits[h.off + k])] = 1;
    }
}

// The candidates of an election (mis_init_k, lcve.cu:150-173), in variable
// order: flag (cand[v], cand[0] stays clear), state and no rank yet; the
// largest candidate score goes to cmax (the key width of the sort that orders
// only the candidates).
__global__ void cand_k(uint32_t V, const uint32_t* scores, uint8_t* mstate, uint32_t* rank, const uint8_t* vstate,
                       const uint8_t* assumed, const uint32_t* hist, const uint8_t* oversized, uint32_t pmax,
                       uint32_t nmax, uint32_t maxoccurs, uint8_t* cand, const uint32_t* vinst,
                       const uint8_t* active, uint32_t* cmax) {
    uint32_t mx = 0;
    for (uint32_t v = 1 + blockIdx.x * blockDim.x + threadIdx.x; v <= V; v += gridDim.x * blockDim.x) {
        uint8_t st = MIS_NONE;
        if (active[vinst[v]] && !vstate[v] && !(assumed && assumed[v])) {
            const uint32_t p = 2 * v, n = p | 1;
            const uint32_t ps = hist[p], ns = hist[n];
            if ((ps || ns) && ps <= maxoccurs && ns <= maxoccurs && !(ps >= pmax && ns >= nmax) && !oversized[v])
                st = MIS_UNDECIDED;
        }
        mstate[v] = st;
        rank[v] = NO_RANK;
        cand[v] = st == MIS_UNDECIDED;
        if (st == MIS_UNDECIDED) mx = max(mx, scores[v]);
    }
    for (int d = 16; d > 0; d >>= 1) mx = max(mx, __shfl_down_sync(0xFFFFFFFFu, mx, d));
    if ((threadIdx.x & 31u) == 0 && mx) atomicMax(cmax, mx);
}

__global__ void cand_keys_k(const uint32_t* cands, uint32_t n, const uint32_t* scores, uint32_t* keys) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        keys[i] = scores[cands[i]];
}

// rank = place in the candidates' (score, var) order
__global__ void cand_rank_k(const uint32_t* cands, uint32_t n, uint32_t* rank) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        rank[cands[i]] = i;
}

// The first MIS_HEAD literals of a clause are loaded together, then their
// ranks: independent loads in flight instead of one dependent chain per
// literal (most clauses are that short). The candidate's own rank is r, never
// below it.
constexpr uint32_t MIS_HEAD = 4;

PFG_D bool blocked(const ClsHdr* hdr, const uint32_t* lits, const uint32_t* ot_off, const uint32_t* ot_size,
                   const uint32_t* ot_ids, uint32_t lit, uint32_t r, const uint32_t* rank) {
    const uint32_t o = ot_off[lit], n = ot_size[lit];
    ClsHdr next = n ? hdr[ot_ids[o]] : ClsHdr{0, 0, 0, 0};
    for (uint32_t i = 0; i < n; i++) {
        const ClsHdr h = next;
        if (i + 1 < n) next = hdr[ot_ids[o + i + 1]];   // in flight while h is checked
        if (m_deleted(h.meta)) continue;
        const uint32_t* l = lits + h.off;
        uint32_t u[MIS_HEAD];
        uint32_t rk[MIS_HEAD];
#pragma unroll
        for (uint32_t q = 0; q < MIS_HEAD; q++) u[q] = q < h.size ? ABSV(l[q]) : 0u;
#pragma unroll
        for (uint32_t q = 0; q < MIS_HEAD; q++) rk[q] = q < h.size ? rank[u[q]] : NO_RANK;
#pragma unroll
        for (uint32_t q = 0; q < MIS_HEAD; q++)
            if (rk[q] < r) return true;
        for (uint32_t k = MIS_HEAD; k < h.size; k++)
            if (rank[ABSV(l[k])] < r) return true;
    }
    return false;
}

PFG_D void freeze_list(const ClsHdr* hdr, const uint32_t* lits, const uint32_t* ot_off, const uint32_t* ot_size,
                       const uint32_t* ot_ids, uint32_t lit, uint32_t cand, uint8_t* frozen, uint8_t* mstate,
                       uint32_t* rank) {
    const uint32_t o = ot_off[lit], n = ot_size[lit];
    ClsHdr next = n ? hdr[ot_ids[o]] : ClsHdr{0, 0, 0, 0};
    for (uint32_t i = 0; i < n; i++) {
        const ClsHdr h = next;
        if (i + 1 < n) next = hdr[ot_ids[o + i + 1]];
        if (m_deleted(h.meta)) continue;
        const uint32_t* l = lits + h.off;
        uint32_t u[MIS_HEAD];
        uint8_t st[MIS_HEAD];
#pragma unroll
        for (uint32_t q = 0; q < MIS_HEAD; q++) u[q] = q < h.size ? ABSV(l[q]) : cand;
#pragma unroll
        for (uint32_t q = 0; q < MIS_HEAD; q++) st[q] = u[q] != cand ? mstate[u[q]] : MIS_NONE;
#pragma unroll
        for (uint32_t q = 0; q < MIS_HEAD; q++) {
            if (u[q] == cand) continue;
            frozen[u[q]] = 1;
            if (st[q] == MIS_UNDECIDED) { mstate[u[q]] = MIS_FROZEN; rank[u[q]] = NO_RANK; }
        }
        for (uint32_t k = MIS_HEAD; k < h.size; k++) {
            const uint32_t v = ABSV(l[k]);
            if (v != cand) {
                frozen[v] = 1;
                if (mstate[v] == MIS_UNDECIDED) { mstate[v] = MIS_FROZEN; rank[v] = NO_RANK; }
            }
        }
    }
}

// var-order round kernels: every variable checks its own state (coalesced)
__global__ void mis_win3_k(uint32_t V, const ClsHdr* hdr, const uint32_t* lits, const uint32_t* ot_off,
                           const uint32_t* ot_size, const uint32_t* ot_ids, const uint32_t* rank,
                           const uint8_t* mstate, uint8_t* winv, uint32_t* undecided, const uint32_t* done) {
    if (*done) return;   // an earlier round of this batch converged
    uint32_t cnt = 0;
    for (uint32_t v = 1 + blockIdx.x * blockDim.x + threadIdx.x; v <= V; v += gridDim.x * blockDim.x) {
        if (mstate[v] != MIS_UNDECIDED) continue;
        cnt++;
        const uint32_t r = rank[v];
        winv[v] = !(blocked(hdr, lits, ot_off, ot_size, ot_ids, 2 * v, r, rank) ||
                    blocked(hdr, lits, ot_off, ot_size, ot_ids, 2 * v + 1, r, rank));
    }
    for (int d = 16; d > 0; d >>= 1) cnt += __shfl_down_sync(0xFFFFFFFFu, cnt, d);
    if ((threadIdx.x & 31u) == 0 && cnt) atomicAdd(undecided, cnt);
}

// First MIS round through clause minima: with every candidate undecided, a
// candidate is blocked exactly when one of its live clauses holds an undecided
// variable of smaller rank, i.e. when the clause's smallest undecided rank is
// below its own. One pass over the clauses records that minimum (a deleted
// clause gets none); the candidates then read one word per occurrence instead
// of the clause's header, literals and their states.
__global__ void clause_min_k(const ClsHdr* __restrict__ hdr, const uint32_t* __restrict__ lits, uint64_t ncls,
                             const uint32_t* __restrict__ rank, uint32_t* cmin) {
    for (uint64_t c = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; c < ncls; c += (uint64_t)gridDim.x * blockDim.x) {
        const ClsHdr h = hdr[c];
        uint32_t m = 0xFFFFFFFFu;
        if (!m_deleted(h.meta)) {
            const uint32_t* l = lits + h.off;
            for (uint32_t k = 0; k < h.size; k++) m = min(m, rank[ABSV(l[k])]);
        }
        cmin[c] = m;
    }
}

PFG_D bool blocked_min(const uint32_t* ot_off, const uint32_t* ot_size, const uint32_t* ot_ids, const uint32_t* cmin,
                       uint32_t lit, uint32_t r) {
    const uint32_t o = ot_off[lit], n = ot_size[lit];
    for (uint32_t i = 0; i < n; i++)
        if (cmin[ot_ids[o + i]] < r) return true;
    return false;
}

// the outcome is also kept by rank (winr), the index a clause minimum holds
__global__ void mis_win_min_k(uint32_t V, const uint32_t* ot_off, const uint32_t* ot_size, const uint32_t* ot_ids,
                              const uint32_t* cmin, const uint32_t* rank, const uint8_t* mstate, uint8_t* winv,
                              uint8_t* winr, uint32_t* undecided) {
    uint32_t cnt = 0;
    for (uint32_t v = 1 + blockIdx.x * blockDim.x + threadIdx.x; v <= V; v += gridDim.x * blockDim.x) {
        if (mstate[v] != MIS_UNDECIDED) continue;
        cnt++;
        const uint32_t r = rank[v];
        const bool win = !(blocked_min(ot_off, ot_size, ot_ids, cmin, 2 * v, r) ||
                           blocked_min(ot_off, ot_size, ot_ids, cmin, 2 * v + 1, r));
        winv[v] = win;
        winr[r] = win;
    }
    for (int d = 16; d > 0; d >>= 1) cnt += __shfl_down_sync(0xFFFFFFFFu, cnt, d);
    if ((threadIdx.x & 31u) == 0 && cnt) atomicAdd(undecided, cnt);
}

// First MIS round, applied through the same clause minima: a winner is the
// smallest undecided variable of every clause it is in, so a live clause holds
// a winner exactly when its minimum-rank variable won, and then every other
// variable of the clause is its neighbour and is frozen (freeze_list over the
// winner's lists reaches the same clauses). No other variable of such a clause
// is a winner, so the freezing never meets an election.
__global__ void mis_apply_min_k(const ClsHdr* __restrict__ hdr, const uint32_t* __restrict__ lits, uint64_t ncls,
                                const uint32_t* __restrict__ cmin, const uint32_t* __restrict__ eligible,
                                const uint8_t* __restrict__ winr, uint8_t* frozen, uint8_t* mstate, uint32_t* rank) {
    for (uint64_t c = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; c < ncls; c += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t m = cmin[c];
        if (m == NO_RANK || !winr[m]) continue;
        const uint32_t u = eligible[m];
        const ClsHdr h = hdr[c];
        const uint32_t* l = lits + h.off;
        for (uint32_t k = 0; k < h.size; k++) {
            const uint32_t v = ABSV(l[k]);
            if (v == u) continue;
            frozen[v] = 1;
            if (mstate[v] == MIS_UNDECIDED) { mstate[v] = MIS_FROZEN; rank[v] = NO_RANK; }
        }
    }
}

__global__ void mis_elect_k(uint32_t V, const uint8_t* winv, uint32_t r, uint32_t* mround, uint8_t* mstate,
                            uint32_t* rank, const uint32_t* undecided) {
    if (*undecided == 0) return;
    for (uint32_t v = 1 + blockIdx.x * blockDim.x + threadIdx.x; v <= V; v += gridDim.x * blockDim.x) {
        if (mstate[v] != MIS_UNDECIDED || !winv[v]) continue;
        mstate[v] = MIS_ELECTED;
        rank[v] = NO_RANK;
        mround[v] = r;
    }
}

__global__ void mis_apply3_k(uint32_t V, const uint8_t* winv, uint32_t r, uint32_t* mround, const ClsHdr* hdr,
                             const uint32_t* lits, const uint32_t* ot_off, const uint32_t* ot_size,
                             const uint32_t* ot_ids, uint8_t* frozen, uint8_t* mstate, uint32_t* rank,
                             const uint32_t* undecided, uint32_t* done) {
    if (*undecided == 0) {   // nothing was undecided: no winner, and the rounds left have nothing to do
        if (blockIdx.x == 0 && threadIdx.x == 0) *done = 1;
        return;
    }
    for (uint32_t v = 1 + blockIdx.x * blockDim.x + threadIdx.x; v <= V; v += gridDim.x * blockDim.x) {
        if (mstate[v] != MIS_UNDECIDED || !winv[v]) continue;
        mstate[v] = MIS_ELECTED;
        rank[v] = NO_RANK;
        mround[v] = r;
        freeze_list(hdr, lits, ot_off, ot_size, ot_ids, 2 * v, v, frozen, mstate, rank);
        freeze_list(hdr, lits, ot_off, ot_size, ot_ids, 2 * v + 1, v, frozen, mstate, rank);
    }
}

__global__ void elected_flags_k(const uint32_t* work, uint32_t nwork, const uint8_t* mstate, uint8_t* flag) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < nwork; i += gridDim.x * blockDim.x)
        flag[i] = mstate[work[i]] == MIS_ELECTED;
}

__global__ void round_keys_k(const uint32_t* elected, uint32_t n, const uint32_t* mround, uint32_t* keys) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        keys[i] = mround[elected[i]];
}

__global__ void frozen_u32_k(const uint8_t* frozen, uint32_t V, uint32_t* out) {
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v <= V; v += gridDim.x * blockDim.x)
        out[v] = (v >= 1 && frozen[v]) ? 1u : 0u;
}

// fbase[i] = frozen variables before instance i (fbase[n] = all of them)
__global__ void frozen_base_k(const uint32_t* pos, const uint32_t* voff, uint32_t ninst, uint32_t* fbase) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i <= ninst; i += gridDim.x * blockDim.x)
        fbase[i] = pos[voff[i] + 1];
}

// function-table index of a frozen variable: its rank among its instance's frozen variables
__global__ void varcore_k(const uint8_t* frozen, uint32_t V, const uint32_t* pos, const uint32_t* vinst,
                          const uint32_t* fbase, uint32_t* varcore) {
    for (uint32_t v = 1 + blockIdx.x * blockDim.x + threadIdx.x; v <= V; v += gridDim.x * blockDim.x)
        if (frozen[v]) varcore[v] = pos[v] - fbase[vinst[v]];
}

// largest frozen variable of each instance inside the function-table core
// (varcore < MAXFUNVAR): a neighbour above it cannot be mapped by find_fun_gate
__global__ void fcut_k(const uint8_t* frozen, const uint32_t* varcore, uint32_t V, const uint32_t* vinst,
                       uint32_t* fcut) {
    for (uint32_t v = 1 + blockIdx.x * blockDim.x + threadIdx.x; v <= V; v += gridDim.x * blockDim.x)
        if (frozen[v] && varcore[v] < 12u) atomicMax(&fcut[vinst[v]], v);
}

// per-instance counts of a variable list (warp-aggregated over equal instances)
__global__ void inst_count_k(const uint32_t* list, uint32_t n, const uint32_t* vinst, uint32_t* cnt) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t inst = vinst[list[i]];
        const unsigned peers = __match_any_sync(__activemask(), inst);
        if ((int)(threadIdx.x & 31u) == __ffs(peers) - 1) atomicAdd(&cnt[inst], (uint32_t)__popc(peers));
    }
}

__global__ void inst_keys_k(const uint32_t* list, uint32_t n, const uint32_t* vinst, const uint32_t* mround,
                            int rbits, uint32_t* keys) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t v = list[i];
        keys[i] = (vinst[v] << rbits) | (mround ? mround[v] : 0u);
    }
}

// sequential lcve_k (lcve.cu:63-98): one thread per instance walks the
// instance's segment [voff[i], voff[i+1]) of the eligible order
__global__ void lcve_seq_k(const uint32_t* eligible, const uint32_t* voff, const uint8_t* active, uint32_t ninst,
                           uint8_t* eflag, uint32_t* flist, uint8_t* frozen, const uint8_t* vstate,
                           const uint8_t* assumed, const uint32_t* hist, const ClsHdr* hdr, const uint32_t* lits,
                           const uint32_t* ot_off, const uint32_t* ot_size, const uint32_t* ot_ids, uint32_t pmax,
                           uint32_t nmax, uint32_t maxoccurs, int maxcsize, uint32_t* nelect, uint32_t* nfrozen) {
    for (uint32_t inst = blockIdx.x * blockDim.x + threadIdx.x; inst < ninst; inst += gridDim.x * blockDim.x) {
        const uint32_t b = voff[inst], e = voff[inst + 1];
        uint32_t tail = b, ne = 0;
        if (active[inst]) {
            for (uint32_t ei = b; ei < e; ei++) {
                const uint32_t cand = eligible[ei];
                if (frozen[cand]) continue;
                if (vstate[cand]) continue;
                if (assumed && assumed[cand]) continue;
                const uint32_t p = 2 * cand, n = p | 1;
                const uint32_t ps = hist[p], ns = hist[n];
                if (!ps && !ns) continue;
                if (ps > maxoccurs || ns > maxoccurs) break;
                if (ps >= pmax && ns >= nmax) break;
                bool okp = true;
                for (int side = 0; side < 2 && okp; side++) {
                    const uint32_t lit = side ? n : p;
                    const uint32_t saved = tail;
                    const uint32_t o = ot_off[lit], sz = ot_size[lit];
                    for (uint32_t i = 0; i < sz; i++) {
                        const ClsHdr h = hdr[ot_ids[o + i]];
                        if (m_deleted(h.meta)) continue;
                        if ((int)h.size > maxcsize) {
                            for (uint32_t q = saved; q < tail; q++) frozen[flist[q]] = 0;
                            tail = saved;
                            okp = false;
                            break;
                        }
                        for (uint32_t k = 0; k < h.size; k++) {
                            const uint32_t u = ABSV(lits[h.off + k]);
                            if (!frozen[u] && u != cand) { frozen[u] = 1; flist[tail++] = u; }
                        }
                    }
                }
                if (okp) { eflag[ei] = 1; ne++; }
            }
        }
        nelect[inst] = ne;
        nfrozen[inst] = tail - b;
    }
}

// varcore[flist[j]] = j within each instance's frozen list (mapfrozen_k, lcve.cu:253)
__global__ void mapfrozen_k(const uint32_t* flist, uint32_t V, const uint32_t* voff, const uint32_t* vinst,
                            const uint32_t* nfrozen, uint32_t* varcore) {
    for (uint32_t idx = blockIdx.x * blockDim.x + threadIdx.x; idx < V; idx += gridDim.x * blockDim.x) {
        const uint32_t inst = vinst[idx + 1];
        const uint32_t j = idx - voff[inst];
        if (j < nfrozen[inst]) varcore[flist[idx]] = j;
    }
}

}  // namespace


bool lcve(Ctx& c) {
    const uint32_t V = c.V;
    const uint32_t ninst = c.ninst;
    // scores (and, for the sequential elections, the sort input over every variable)
    cudaMemsetAsync(&c.dc->nfrozen, 0, sizeof(uint32_t), c.s);
    PFG_LAUNCH(K_LCVE, scores_k, grid_for(V, 256), 256, 0, c.s, c.hist, V, c.scores,
               c.o.lcve_fast ? nullptr : c.keys_a, c.o.lcve_fast ? nullptr : c.eligible, c.dc);
    if (!ensure_tmp(c, std::max(radix_temp_bytes(V), scan_temp_bytes(V + 1)))) return false;
    int ibits = 0;
    while (ibits < 32 && ((ninst - 1) >> ibits)) ibits += 8;
    const uint32_t maxoccurs = c.o.lcve_max_occurs;
    const uint32_t pmax = c.o.mu_pos << c.multiplier;
    const uint32_t nmax = c.o.mu_neg << c.multiplier;
    const int maxcsize = c.o.lcve_clause_max;
    bool any_vc = false;
    for (uint32_t i = 0; i < ninst; i++) any_vc |= c.ih[i].active && c.ih[i].varcore_on;
    cudaMemsetAsync(c.frozen, 0, V + 1, c.s);
    cudaMemsetAsync(c.dout.nelect, 0, ninst * sizeof(uint32_t), c.s);
    cudaMemsetAsync(c.dout.nfrozen, 0, ninst * sizeof(uint32_t), c.s);
    c.nelected = 0;
    c.mis_rounds = 0;
    if (c.o.lcve_fast) {
        // winv is free until the rounds start: it holds the oversize marks here
        cudaMemsetAsync(c.winv, 0, V + 1, c.s);
        c.prof.bytes[K_LCVE] += 4 * (c.numLiterals + c.numClauses);   // byte model of the clause-size pass
        PFG_LAUNCH(K_LCVE, oversize_mark_k, grid_for(c.ncls, 256), 256, 0, c.s, c.hdr, c.lits, c.ncls, maxcsize,
                   c.winv);
        // Only the candidates are put in (score, var) order: the rounds compare
        // ranks of candidates alone, and the candidates taken in variable order
        // and sorted stably by score are in the order they have among all
        // variables sorted by (score, var) (assign_scores + thrust::sort,
        // lcve.cu:221-300). A candidate's rank is its place in c.work.
        cudaMemsetAsync(&c.dc->nfrozen, 0, sizeof(uint32_t), c.s);
        PFG_LAUNCH(K_LCVE, cand_k, grid_for(V, 256), 256, 0, c.s, V, c.scores, c.mstate, c.rank, c.vstate,
                   c.assumed, c.hist, c.winv, pmax, nmax, maxoccurs, c.flag8, c.vinst, c.di.active, &c.dc->nfrozen);
        cudaMemsetAsync(c.flag8, 0, 1, c.s);   // variable 0
        select_flagged(nullptr, c.flag8, c.work, V + 1, &c.dc->nwork, c.vscan, c.tmp, c.s);   // the flagged v
        sync_counters(c);
        const uint32_t nwork = c.hc->nwork;
        const uint32_t cmax = c.hc->nfrozen;    // nfrozen reused as the largest candidate score
        int cbits = 0;
        while (cbits < 32 && (cmax >> cbits)) cbits += 8;
        if (nwork > 1 && cbits) {
            PFG_LAUNCH(K_LCVE, cand_keys_k, grid_for(nwork, 256), 256, 0, c.s, c.work, nwork, c.scores, c.keys_a);
            const int which = radix_sort_pairs(c.keys_a, c.work, c.keys_b, c.eligible_b, nwork, 0, cbits, c.tmp, c.s);
            if (which) cudaMemcpyAsync(c.work, c.eligible_b, nwork * sizeof(uint32_t), cudaMemcpyDeviceToDevice, c.s);
        }
        if (nwork) PFG_LAUNCH(K_LCVE, cand_rank_k, grid_for(nwork, 256), 256, 0, c.s, c.work, nwork, c.rank);
        // Rounds run without compaction; each winner records its round. The host
        // reads the undecided count only every 1, 2, 4 .. 16 rounds.
        uint32_t* mround = c.scores;     // scores are dead once the order is sorted
        const unsigned mt = tuned(c.tune.mis_threads, MIS_THREADS);
        uint32_t r = 0;
        bool done = nwork == 0;
        cudaMemsetAsync(&c.dc->mis_done, 0, sizeof(uint32_t), c.s);
        for (int batch = 1; !done; batch = std::min(batch * 2, 16)) {
            for (int b = 0; b < batch; b++, r++) {
                cudaMemsetAsync(&c.dc->nwin, 0, sizeof(uint32_t), c.s);
                if (r == 0 && ensure_tmp_u32(c, c.ncls + 1)) {   // first round: every candidate undecided
                    PFG_LAUNCH(K_MIS_WIN, clause_min_k, grid_for(c.ncls, 256), 256, 0, c.s, c.hdr, c.lits, c.ncls,
                               c.rank, c.tmp_u32);
                    // flag8 (the candidate flags, consumed above) holds the outcomes by rank
                    PFG_LAUNCH(K_MIS_WIN, mis_win_min_k, grid_for(V, mt), mt, 0, c.s, V, c.ot_off, c.ot_size,
                               c.ot_ids, c.tmp_u32, c.rank, c.mstate, c.winv, c.flag8, &c.dc->nwin);
                    PFG_LAUNCH(K_MIS_APPLY, mis_apply_min_k, grid_for(c.ncls, 256), 256, 0, c.s, c.hdr, c.lits,
                               c.ncls, c.tmp_u32, c.work, c.flag8, c.frozen, c.mstate, c.rank);
                    PFG_LAUNCH(K_MIS_APPLY, mis_elect_k, grid_for(V, 256), 256, 0, c.s, V, c.winv, r, mround, c.mstate,
                               c.rank, &c.dc->nwin);
                    continue;
                }
                PFG_LAUNCH(K_MIS_WIN, mis_win3_k, grid_for(V, mt), mt, 0, c.s, V, c.hdr, c.lits, c.ot_off,
                           c.ot_size, c.ot_ids, c.rank, c.mstate, c.winv, &c.dc->nwin, &c.dc->mis_done);
                PFG_LAUNCH(K_MIS_APPLY, mis_apply3_k, grid_for(V, mt), mt, 0, c.s, V, c.winv, r, mround, c.hdr,
                           c.lits, c.ot_off, c.ot_size, c.ot_ids, c.frozen, c.mstate, c.rank, &c.dc->nwin,
                           &c.dc->mis_done);
            }
            sync_counters(c);
            if (!c.err.empty()) return false;
            if (c.hc->nwin == 0) done = true;          // the last round found nothing undecided
            else if (r > (c.lim_mis_rounds ? (uint64_t)c.lim_mis_rounds : (uint64_t)nwork + 2)) {
                c.err = "MIS did not converge"; c.simpstate = PFG_TIMEOUT; return false;
            }
        }
        c.mis_rounds = r;
        // elected in (instance, round, rank) order: select in rank order, then a
        // stable sort by (instance, round)
        PFG_LAUNCH(K_LCVE, elected_flags_k, grid_for(nwork, 256), 256, 0, c.s, c.work, nwork, c.mstate, c.flag8);
        select_flagged(c.work, c.flag8, c.elected, nwork, &c.dc->nelected, c.vscan, c.tmp, c.s);
        sync_counters(c);
        c.nelected = c.hc->nelected;
        if (c.nelected > 1) {
            int rbits = 0;
            while (rbits < 32 && (r >> rbits)) rbits += 8;
            if (!ensure_tmp(c, radix_temp_bytes(c.nelected))) return false;
            const bool fused = ninst > 1 && rbits + ibits <= 32;
            if (fused)
                PFG_LAUNCH(K_LCVE, inst_keys_k, grid_for(c.nelected, 256), 256, 0, c.s, c.elected, c.nelected, c.vinst,
                           mround, rbits, c.keys_a);
            else
                PFG_LAUNCH(K_LCVE, round_keys_k, grid_for(c.nelected, 256), 256, 0, c.s, c.elected, c.nelected, mround,
                           c.keys_a);
            int which = radix_sort_pairs(c.keys_a, c.elected, c.keys_b, c.work_b, c.nelected, 0,
                                         fused ? rbits + ibits : rbits, c.tmp, c.s);
            if (which) cudaMemcpyAsync(c.elected, c.work_b, c.nelected * sizeof(uint32_t), cudaMemcpyDeviceToDevice, c.s);
            if (ninst > 1 && !fused) {
                PFG_LAUNCH(K_LCVE, inst_keys_k, grid_for(c.nelected, 256), 256, 0, c.s, c.elected, c.nelected, c.vinst,
                           (const uint32_t*)nullptr, 0, c.keys_a);
                which = radix_sort_pairs(c.keys_a, c.elected, c.keys_b, c.work_b, c.nelected, 0, ibits, c.tmp, c.s);
                if (which) cudaMemcpyAsync(c.elected, c.work_b, c.nelected * sizeof(uint32_t), cudaMemcpyDeviceToDevice, c.s);
            }
        }
        if (ninst > 1) {
            if (c.nelected)
                PFG_LAUNCH(K_LCVE, inst_count_k, grid_for(c.nelected, 256), 256, 0, c.s, c.elected, c.nelected, c.vinst,
                           c.dout.nelect);
        } else {
            cudaMemcpyAsync(c.dout.nelect, &c.dc->nelected, sizeof(uint32_t), cudaMemcpyDeviceToDevice, c.s);
        }
        if (any_vc) {
            PFG_LAUNCH(K_LCVE, frozen_u32_k, grid_for(V + 1, 256), 256, 0, c.s, c.frozen, V, c.vscan);
            exclusive_scan_u32(c.vscan, c.vscan, V + 1, 0u, c.vscan + V + 1, c.tmp, c.s);
            PFG_LAUNCH(K_LCVE, frozen_base_k, grid_for(ninst + 1, 256), 256, 0, c.s, c.vscan, c.di.voff, ninst,
                       c.dout.fbase);
            PFG_LAUNCH(K_LCVE, varcore_k, grid_for(V, 256), 256, 0, c.s, c.frozen, V, c.vscan, c.vinst, c.dout.fbase,
                       c.varcore);
        }
    } else {
        // every variable in (score, var) order
        sync_counters(c);
        const uint32_t maxscore = c.hc->nfrozen;   // nfrozen reused as the largest score
        int bits = 0;
        while (bits < 32 && (maxscore >> bits)) bits += 8;
        if (bits) {
            const int which = radix_sort_pairs(c.keys_a, c.eligible, c.keys_b, c.eligible_b, V, 0, bits, c.tmp, c.s);
            if (which) cudaMemcpyAsync(c.eligible, c.eligible_b, V * sizeof(uint32_t), cudaMemcpyDeviceToDevice, c.s);
        }
        // eligible grouped by instance (stable), so instance i owns positions [voff[i], voff[i+1])
        if (ninst > 1) {
            PFG_LAUNCH(K_LCVE, inst_keys_k, grid_for(V, 256), 256, 0, c.s, c.eligible, V, c.vinst,
                       (const uint32_t*)nullptr, 0, c.keys_a);
            const int which = radix_sort_pairs(c.keys_a, c.eligible, c.keys_b, c.eligible_b, V, 0, ibits, c.tmp, c.s);
            if (which) cudaMemcpyAsync(c.eligible, c.eligible_b, V * sizeof(uint32_t), cudaMemcpyDeviceToDevice, c.s);
        }
        // per-instance frozen lists in keys_b at the instance's offset
        cudaMemsetAsync(c.flag8, 0, V + 1, c.s);
        PFG_LAUNCH(K_LCVE, lcve_seq_k, grid_for(ninst, 32), 32, 0, c.s, c.eligible, c.di.voff, c.di.active, ninst,
                   c.flag8, c.keys_b, c.frozen, c.vstate, c.assumed, c.hist, c.hdr, c.lits, c.ot_off, c.ot_size,
                   c.ot_ids, pmax, nmax, maxoccurs, maxcsize, c.dout.nelect, c.dout.nfrozen);
        select_flagged(c.eligible, c.flag8, c.elected, V, &c.dc->nelected, c.vscan, c.tmp, c.s);
        if (any_vc)
            PFG_LAUNCH(K_LCVE, mapfrozen_k, grid_for(V, 256), 256, 0, c.s, c.keys_b, V, c.di.voff, c.vinst,
                       c.dout.nfrozen, c.varcore);
    }
    if (any_vc) {
        cudaMemsetAsync(c.fcut, 0, ninst * sizeof(uint32_t), c.s);
        PFG_LAUNCH(K_LCVE, fcut_k, grid_for(V, 256), 256, 0, c.s, c.frozen, c.varcore, V, c.vinst, c.fcut);
    }
    pull_inst_out(c);
    if (!c.err.empty()) return false;
    c.nelected = c.hc->nelected;
    for (uint32_t i = 0; i < ninst; i++) {
        InstHost& h = c.ih[i];
        if (!h.active) continue;
        h.nelected = c.hout.nelect[i];
        const uint32_t nf = c.o.lcve_fast ? (any_vc ? c.hout.fbase[i + 1] - c.hout.fbase[i] : 0u) : c.hout.nfrozen[i];
        if (h.varcore_on && !nf) h.varcore_on = false;   // vars->varcore = NULL (lcve.cu:403)
    }
    return cuda_ok(c, cudaGetLastError(), "lcve");
}

}  // namespace pfg
