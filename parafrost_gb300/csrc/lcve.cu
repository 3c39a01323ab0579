// Least-constrained variable elections (LCVE).
//
// Replaces Solver::varReorder + Solver::LCVE (src/gpu/lcve.cu:221-417):
//   - scores ps*ns (uint32, assign_scores :221) sorted by (score, var) with the
//     engine's stable radix sort instead of thrust::sort with GPU_LCV_CMP;
//   - the Luby-style MIS (mis_init_k/mis_round_k/mis_freeze_k :143-209) runs on
//     a shrinking worklist kept in rank order, so winners are appended in
//     (round, rank) order -- one legal order of the reference's atomic appends;
//   - frozen variables get their function-table index from a scan in
//     ascending variable order (mis_collect_k + mapfrozen_k :211-260).
// The sequential lcve_k (:63-98, option lcvefast=0) runs on one thread, as in
// the reference, over occurrence lists sorted by clause id.
#include "engine.cuh"

namespace pfg {
namespace {

constexpr uint8_t MIS_NONE = 0, MIS_UNDECIDED = 1, MIS_ELECTED = 2, MIS_FROZEN = 3;

__global__ void scores_k(const uint32_t* hist, uint32_t V, uint32_t* scores, uint32_t* keys, uint32_t* vals,
                         DevCounters* dc) {
    uint32_t mx = 0;
    for (uint32_t v = 1 + blockIdx.x * blockDim.x + threadIdx.x; v <= V; v += gridDim.x * blockDim.x) {
        const uint32_t s = hist[2 * v] * hist[2 * v + 1];   // uint32 product, as assign_scores
        scores[v] = s;
        keys[v - 1] = s;
        vals[v - 1] = v;
        mx = max(mx, s);
    }
    for (int d = 16; d > 0; d >>= 1) mx = max(mx, __shfl_down_sync(0xFFFFFFFFu, mx, d));
    if ((threadIdx.x & 31u) == 0 && mx) atomicMax(&dc->nfrozen, mx);   // nfrozen reused as max score here
}

PFG_D bool oversize(const ClsHdr* hdr, const uint32_t* ot_off, const uint32_t* ot_size, const uint32_t* ot_ids,
                    uint32_t lit, int maxcsize) {
    const uint32_t o = ot_off[lit], n = ot_size[lit];
    for (uint32_t i = 0; i < n; i++) {
        const ClsHdr h = hdr[ot_ids[o + i]];
        if (!m_deleted(h.meta) && (int)h.size > maxcsize) return true;
    }
    return false;
}

__global__ void mis_init_k(const uint32_t* eligible, uint32_t V, uint32_t* rank, uint8_t* mstate,
                           const uint8_t* vstate, const uint8_t* assumed, const uint32_t* hist,
                           const ClsHdr* hdr, const uint32_t* ot_off, const uint32_t* ot_size, const uint32_t* ot_ids,
                           uint32_t pmax, uint32_t nmax, uint32_t maxoccurs, int maxcsize, uint8_t* cand) {
    for (uint32_t ei = blockIdx.x * blockDim.x + threadIdx.x; ei < V; ei += gridDim.x * blockDim.x) {
        const uint32_t v = eligible[ei];
        rank[v] = ei;
        uint8_t st = MIS_NONE;
        if (!vstate[v] && !(assumed && assumed[v])) {
            const uint32_t p = 2 * v, n = p | 1;
            const uint32_t ps = hist[p], ns = hist[n];
            if ((ps || ns) && ps <= maxoccurs && ns <= maxoccurs && !(ps >= pmax && ns >= nmax) &&
                !oversize(hdr, ot_off, ot_size, ot_ids, p, maxcsize) &&
                !oversize(hdr, ot_off, ot_size, ot_ids, n, maxcsize))
                st = MIS_UNDECIDED;
        }
        mstate[v] = st;
        cand[ei] = st == MIS_UNDECIDED;
    }
}

PFG_D bool blocked(const ClsHdr* hdr, const uint32_t* lits, const uint32_t* ot_off, const uint32_t* ot_size,
                   const uint32_t* ot_ids, uint32_t lit, uint32_t cand, uint32_t r, const uint32_t* rank,
                   const uint8_t* mstate) {
    const uint32_t o = ot_off[lit], n = ot_size[lit];
    for (uint32_t i = 0; i < n; i++) {
        const ClsHdr h = hdr[ot_ids[o + i]];
        if (m_deleted(h.meta)) continue;
        for (uint32_t k = 0; k < h.size; k++) {
            const uint32_t u = ABSV(lits[h.off + k]);
            if (u != cand && mstate[u] == MIS_UNDECIDED && rank[u] < r) return true;
        }
    }
    return false;
}

PFG_D void freeze_list(const ClsHdr* hdr, const uint32_t* lits, const uint32_t* ot_off, const uint32_t* ot_size,
                       const uint32_t* ot_ids, uint32_t lit, uint32_t cand, uint8_t* frozen, uint8_t* mstate) {
    const uint32_t o = ot_off[lit], n = ot_size[lit];
    for (uint32_t i = 0; i < n; i++) {
        const ClsHdr h = hdr[ot_ids[o + i]];
        if (m_deleted(h.meta)) continue;
        for (uint32_t k = 0; k < h.size; k++) {
            const uint32_t u = ABSV(lits[h.off + k]);
            if (u != cand) {
                frozen[u] = 1;
                if (mstate[u] == MIS_UNDECIDED) mstate[u] = MIS_FROZEN;
            }
        }
    }
}

// var-order round kernels: every variable checks its own state (coalesced)
__global__ void mis_win3_k(uint32_t V, const ClsHdr* hdr, const uint32_t* lits, const uint32_t* ot_off,
                           const uint32_t* ot_size, const uint32_t* ot_ids, const uint32_t* rank,
                           const uint8_t* mstate, uint8_t* winv, uint32_t* undecided) {
    uint32_t cnt = 0;
    for (uint32_t v = 1 + blockIdx.x * blockDim.x + threadIdx.x; v <= V; v += gridDim.x * blockDim.x) {
        if (mstate[v] != MIS_UNDECIDED) continue;
        cnt++;
        const uint32_t r = rank[v];
        winv[v] = !(blocked(hdr, lits, ot_off, ot_size, ot_ids, 2 * v, v, r, rank, mstate) ||
                    blocked(hdr, lits, ot_off, ot_size, ot_ids, 2 * v + 1, v, r, rank, mstate));
    }
    for (int d = 16; d > 0; d >>= 1) cnt += __shfl_down_sync(0xFFFFFFFFu, cnt, d);
    if ((threadIdx.x & 31u) == 0 && cnt) atomicAdd(undecided, cnt);
}

__global__ void mis_apply3_k(uint32_t V, const uint8_t* winv, uint32_t r, uint32_t* mround, const ClsHdr* hdr,
                             const uint32_t* lits, const uint32_t* ot_off, const uint32_t* ot_size,
                             const uint32_t* ot_ids, uint8_t* frozen, uint8_t* mstate) {
    for (uint32_t v = 1 + blockIdx.x * blockDim.x + threadIdx.x; v <= V; v += gridDim.x * blockDim.x) {
        if (mstate[v] != MIS_UNDECIDED || !winv[v]) continue;
        mstate[v] = MIS_ELECTED;
        mround[v] = r;
        freeze_list(hdr, lits, ot_off, ot_size, ot_ids, 2 * v, v, frozen, mstate);
        freeze_list(hdr, lits, ot_off, ot_size, ot_ids, 2 * v + 1, v, frozen, mstate);
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

__global__ void varcore_k(const uint8_t* frozen, uint32_t V, const uint32_t* pos, uint32_t* varcore) {
    for (uint32_t v = 1 + blockIdx.x * blockDim.x + threadIdx.x; v <= V; v += gridDim.x * blockDim.x)
        if (frozen[v]) varcore[v] = pos[v];
}

// sequential lcve_k (lcve.cu:63-98) on one thread
__global__ void lcve_seq_k(const uint32_t* eligible, uint32_t V, uint32_t* elected, uint32_t* flist,
                           uint8_t* frozen, const uint8_t* vstate, const uint8_t* assumed, const uint32_t* hist,
                           const ClsHdr* hdr, const uint32_t* lits, const uint32_t* ot_off, const uint32_t* ot_size,
                           const uint32_t* ot_ids, uint32_t pmax, uint32_t nmax, uint32_t maxoccurs, int maxcsize,
                           DevCounters* dc) {
    uint32_t tail = 0, ne = 0;
    for (uint32_t ei = 0; ei < V; ei++) {
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
        if (okp) elected[ne++] = cand;
    }
    dc->nelected = ne;
    dc->nfrozen = tail;
}

__global__ void mapfrozen_k(const uint32_t* flist, uint32_t n, uint32_t* varcore) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        varcore[flist[i]] = i;
}

}  // namespace

bool lcve(Ctx& c) {
    const uint32_t V = c.V;
    // scores and the (score, var) order
    cudaMemsetAsync(&c.dc->nfrozen, 0, sizeof(uint32_t), c.s);
    PFG_LAUNCH(K_LCVE, scores_k, grid_for(V, 256), 256, 0, c.s, c.hist, V, c.scores, c.keys_a, c.eligible, c.dc);
    sync_counters(c);
    const uint32_t maxscore = c.hc->nfrozen;
    int bits = 0;
    while (bits < 32 && (maxscore >> bits)) bits += 8;
    if (!ensure_tmp(c, radix_temp_bytes(V))) return false;
    if (bits) {
        const int which = radix_sort_pairs(c.keys_a, c.eligible, c.keys_b, c.eligible_b, V, 0, bits, c.tmp, c.s);
        if (which) cudaMemcpyAsync(c.eligible, c.eligible_b, V * sizeof(uint32_t), cudaMemcpyDeviceToDevice, c.s);
    }
    const uint32_t maxoccurs = c.o.lcve_max_occurs;
    const uint32_t pmax = c.o.mu_pos << c.multiplier;
    const uint32_t nmax = c.o.mu_neg << c.multiplier;
    const int maxcsize = c.o.lcve_clause_max;
    cudaMemsetAsync(c.frozen, 0, V + 1, c.s);
    c.nelected = 0;
    c.mis_rounds = 0;
    uint32_t nfrozen = 0;
    if (c.o.lcve_fast) {
        PFG_LAUNCH(K_LCVE, mis_init_k, grid_for(V, 256), 256, 0, c.s, c.eligible, V, c.rank, c.mstate, c.vstate, c.assumed, c.hist,
                                                      c.hdr, c.ot_off, c.ot_size, c.ot_ids, pmax, nmax, maxoccurs,
                                                      maxcsize, c.flag8);
        if (!ensure_tmp(c, scan_temp_bytes(V + 1))) return false;
        select_flagged(c.eligible, c.flag8, c.work, V, &c.dc->nwork, c.vscan, c.tmp, c.s);
        sync_counters(c);
        const uint32_t nwork = c.hc->nwork;
        // Rounds run without compaction; each winner records its round. The host
        // reads the undecided count only every 1, 2, 4 .. 16 rounds.
        uint32_t* mround = c.scores;     // scores are dead once the order is sorted
        uint32_t r = 0;
        bool done = nwork == 0;
        for (int batch = 1; !done; batch = std::min(batch * 2, 16)) {
            for (int b = 0; b < batch; b++, r++) {
                cudaMemsetAsync(&c.dc->nwin, 0, sizeof(uint32_t), c.s);
                PFG_LAUNCH(K_MIS_WIN, mis_win3_k, grid_for(V, 128), 128, 0, c.s, V, c.hdr, c.lits, c.ot_off,
                           c.ot_size, c.ot_ids, c.rank, c.mstate, c.winv, &c.dc->nwin);
                PFG_LAUNCH(K_MIS_APPLY, mis_apply3_k, grid_for(V, 128), 128, 0, c.s, V, c.winv, r, mround, c.hdr,
                           c.lits, c.ot_off, c.ot_size, c.ot_ids, c.frozen, c.mstate);
            }
            sync_counters(c);
            if (!c.err.empty()) return false;
            if (c.hc->nwin == 0) done = true;          // the last round found nothing undecided
            else if (r > nwork + 2) { c.err = "MIS did not converge"; c.simpstate = PFG_TIMEOUT; return false; }
        }
        c.mis_rounds = r;
        // elected in (round, rank) order: select in rank order, then stable sort by round
        PFG_LAUNCH(K_LCVE, elected_flags_k, grid_for(nwork, 256), 256, 0, c.s, c.work, nwork, c.mstate, c.flag8);
        select_flagged(c.work, c.flag8, c.elected, nwork, &c.dc->nelected, c.vscan, c.tmp, c.s);
        sync_counters(c);
        c.nelected = c.hc->nelected;
        if (c.nelected > 1) {
            int rbits = 0;
            while (rbits < 32 && (r >> rbits)) rbits += 8;
            PFG_LAUNCH(K_LCVE, round_keys_k, grid_for(c.nelected, 256), 256, 0, c.s, c.elected, c.nelected, mround,
                       c.keys_a);
            if (!ensure_tmp(c, radix_temp_bytes(c.nelected))) return false;
            const int which = radix_sort_pairs(c.keys_a, c.elected, c.keys_b, c.work_b, c.nelected, 0, rbits, c.tmp, c.s);
            if (which) cudaMemcpyAsync(c.elected, c.work_b, c.nelected * sizeof(uint32_t), cudaMemcpyDeviceToDevice, c.s);
        }

        if (c.varcore_on) {
            PFG_LAUNCH(K_LCVE, frozen_u32_k, grid_for(V + 1, 256), 256, 0, c.s, c.frozen, V, c.vscan);
            exclusive_scan_u32(c.vscan, c.vscan, V + 1, 0u, &c.dc->nfrozen, c.tmp, c.s);
            PFG_LAUNCH(K_LCVE, varcore_k, grid_for(V, 256), 256, 0, c.s, c.frozen, V, c.vscan, c.varcore);
            sync_counters(c);
            nfrozen = c.hc->nfrozen;
        }
    } else {
        // flist in keys_b
        PFG_LAUNCH(K_LCVE, lcve_seq_k, 1, 1, 0, c.s, c.eligible, V, c.elected, c.keys_b, c.frozen, c.vstate, c.assumed, c.hist,
                                     c.hdr, c.lits, c.ot_off, c.ot_size, c.ot_ids, pmax, nmax, maxoccurs, maxcsize,
                                     c.dc);
        sync_counters(c);
        c.nelected = c.hc->nelected;
        nfrozen = c.hc->nfrozen;
        if (c.varcore_on && nfrozen) {
            PFG_LAUNCH(K_LCVE, mapfrozen_k, grid_for(nfrozen, 256), 256, 0, c.s, c.keys_b, nfrozen, c.varcore);
        }
    }
    if (c.varcore_on && !nfrozen) c.varcore_on = false;   // vars->varcore = NULL (lcve.cu:403)
    if (!cuda_ok(c, cudaGetLastError(), "lcve")) return false;
    return true;
}

}  // namespace pfg
