// Warp-per-variable versions of SUB, BVE phase 1 and BVE phase 3.
//
// A warp stages its variable's two occurrence lists (clause ids, headers and
// literals) in shared memory with coalesced loads, then runs the reference's
// sequential decision logic warp-synchronously on the staged copy: every lane
// follows the same control flow, reads are shared-memory broadcasts, and the
// costly parts are split across lanes with the sequential semantics kept:
//   - resolvent counting: 32 (i, j) pairs per step in row-major order; the
//     first failing pair in that order ends the count exactly where the
//     reference's loop returns (ballot + prefix sums);
//   - searches of neighbouring lists (fast_equality_check, makeArity,
//     self-subsumption, subsumption): lanes test consecutive candidates and the
//     first hit in list order wins.
// Header changes (molten, status) stay in shared memory while the variable is
// processed and are written back once at the end; no other warp reads them in
// a way that matters (elected variables share no clause). Variables whose lists
// do not fit the stage are handled by the thread-per-variable kernels.
// Included inside elim.cu's anonymous namespace.

constexpr uint32_t WS_MAXC = 96;    // staged clauses per variable
constexpr uint32_t WS_MAXL = 448;   // staged literal words per variable
constexpr int WS_WARPS = 4;         // warps per block
constexpr unsigned FULL = 0xFFFFFFFFu;

struct WS {
    uint32_t np, nn, nlit, pad;
    uint32_t id[WS_MAXC];
    uint32_t meta[WS_MAXC];
    uint32_t meta0[WS_MAXC];    // meta as staged (only changed words are written back)
    uint32_t size[WS_MAXC];
    uint32_t sig[WS_MAXC];
    uint32_t off[WS_MAXC];
    uint32_t goff[WS_MAXC];
    uint8_t dirty[WS_MAXC];     // literals/size/sig changed
    uint32_t lits[WS_MAXL];
    uint32_t outs[WS_MAXC + 24];
};

struct Side {
    uint32_t b, n, lit;         // staged range [b, b+n) = occurrence list of `lit`
};

PFG_D uint32_t* WL(WS& w, uint32_t c) { return w.lits + w.off[c]; }

// The next variable of a warp: its list bounds are loaded when the current
// variable starts and its id lines are prefetched into L2 when it ends, so the
// first two steps of its staging (list bounds, ids) do not wait on DRAM.
struct NextLists {
    uint32_t po, ps, no, ns;
};

PFG_D NextLists ws_next_lists(const EK& k, const uint32_t* elected, uint32_t qn, uint32_t nelected) {
    NextLists nl{0, 0, 0, 0};
    if (qn < nelected) {
        const uint32_t xn = elected[qn];
        nl.po = k.ot_off[2 * xn];
        nl.ps = k.ot_size[2 * xn];
        nl.no = k.ot_off[2 * xn + 1];
        nl.ns = k.ot_size[2 * xn + 1];
    }
    return nl;
}

PFG_D void ws_prefetch_lists(const EK& k, const NextLists& nl, unsigned lane) {
    if (nl.ps + nl.ns > WS_MAXC) return;      // it goes to the thread kernel
    const uint32_t side = lane >> 4, line = lane & 15u;   // lanes 0-15: positives, 16-31: negatives
    const uint32_t o = side ? nl.no : nl.po, n = side ? nl.ns : nl.ps;
    if (line * 32u < n) {
        const uint32_t* a = k.ot_ids + o + line * 32u;
        asm volatile("prefetch.global.L2 [%0];" :: "l"(a));
    }
}

// Work stealing: the grid is as large as the GPU holds at once and every warp
// draws its next variable from one counter (lane 0 draws, the warp reads it by
// shuffle), so a warp whose variables have long lists does not leave the rest
// of its fixed share to the end of the launch.
PFG_D uint32_t ws_ticket(uint32_t* ctr, unsigned lane) {
    uint32_t t = 0;
    if (lane == 0) t = atomicAdd(ctr, 1u);
    return __shfl_sync(0xFFFFFFFFu, t, 0);
}

// Loads both lists of x into the stage; false if they do not fit.
PFG_D bool ws_stage(const EK& k, WS& w, uint32_t p, uint32_t n, unsigned lane) {
    const uint32_t np = OLs(k, p), nn = OLs(k, n), nc = np + nn;
    if (nc > WS_MAXC) return false;
    const uint32_t* pl = OLp(k, p);
    const uint32_t* nl = OLp(k, n);
    for (uint32_t i = lane; i < nc; i += 32) {
        const uint32_t id = i < np ? pl[i] : nl[i - np];
        const ClsHdr h = k.hdr[id];
        w.id[i] = id;
        w.meta[i] = h.meta;
        w.meta0[i] = h.meta;
        w.size[i] = h.size;
        w.sig[i] = h.sig;
        w.goff[i] = h.off;
        w.dirty[i] = 0;
    }
    __syncwarp();
    uint32_t base = 0;
    for (uint32_t c0 = 0; c0 < nc; c0 += 32) {
        const uint32_t i = c0 + lane;
        const uint32_t sz = i < nc ? w.size[i] : 0u;
        uint32_t incl = sz;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint32_t o = __shfl_up_sync(FULL, incl, d);
            if (lane >= (unsigned)d) incl += o;
        }
        if (i < nc) w.off[i] = base + incl - sz;
        base += __shfl_sync(FULL, incl, 31);
    }
    if (base > WS_MAXL) return false;
    if (lane == 0) { w.np = np; w.nn = nn; w.nlit = base; }
    __syncwarp();
    for (uint32_t g = lane; g < base; g += 32) {
        // clause of literal word g: last staged clause whose offset is <= g
        uint32_t lo = 0, hi = nc;
        while (hi - lo > 1) {
            const uint32_t mid = (lo + hi) >> 1;
            if (w.off[mid] <= g) lo = mid; else hi = mid;
        }
        w.lits[g] = k.lits[w.goff[lo] + (g - w.off[lo])];
    }
    __syncwarp();
    return true;
}

// Writes staged header changes (and changed literals) back to global memory.
PFG_D void ws_flush(const EK& k, WS& w, unsigned lane) {
    __syncwarp();
    const uint32_t nc = w.np + w.nn;
    for (uint32_t i = lane; i < nc; i += 32) {
        const uint32_t id = w.id[i];
        if (w.meta[i] != w.meta0[i]) {
            k.hdr[id].meta = w.meta[i];
            w.meta0[i] = w.meta[i];
        }
        if (w.dirty[i]) {
            k.hdr[id].size = w.size[i];
            k.hdr[id].sig = w.sig[i];
            uint32_t* dst = k.lits + w.goff[i];
            const uint32_t* src = WL(w, i);
            for (uint32_t t = 0; t < w.size[i]; t++) dst[t] = src[t];
        }
    }
    __syncwarp();
}

PFG_D void ws_set_meta(WS& w, uint32_t c, uint32_t m, unsigned lane) {
    __syncwarp();
    if (lane == 0) w.meta[c] = m;
    __syncwarp();
}
PFG_D void ws_melt(WS& w, uint32_t c, uint32_t f, unsigned lane) { ws_set_meta(w, c, m_set_molten(w.meta[c], f), lane); }

PFG_D uint32_t warp_excl_scan(uint32_t v, unsigned lane, uint32_t& total) {
    uint32_t incl = v;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const uint32_t o = __shfl_up_sync(FULL, incl, d);
        if (lane >= (unsigned)d) incl += o;
    }
    total = __shfl_sync(FULL, incl, 31);
    return incl - v;
}

// merge(x, c1, c2, unit) on staged clauses (elimination.cuh:242-270)
PFG_D int ws_merge_cnt(WS& w, uint32_t x, uint32_t c1, uint32_t c2, uint32_t& unit) {
    const uint32_t* a = WL(w, c1);
    const uint32_t* b = WL(w, c2);
    const int n1 = (int)w.size[c1], n2 = (int)w.size[c2];
    int i = 0, j = 0, len = n1 + n2 - 2;
    unit = 0;
    while (i < n1 && j < n2) {
        const uint32_t l1 = a[i], l2 = b[j], v1 = ABSV(l1), v2 = ABSV(l2);
        if (v1 == x) i++;
        else if (v2 == x) j++;
        else if ((l1 ^ l2) == 1u) return 0;
        else if (v1 < v2) i++;
        else if (v2 < v1) j++;
        else { i++; j++; len--; if (len == 1) unit = l1; }
    }
    return len;
}

// merge(x, c1, c2, out_c) on staged clauses, written to `out` (elimination.cuh:302-331)
PFG_D int ws_merge_out(WS& w, uint32_t x, uint32_t c1, uint32_t c2, uint32_t* out) {
    const uint32_t* a = WL(w, c1);
    const uint32_t* b = WL(w, c2);
    const int n1 = (int)w.size[c1], n2 = (int)w.size[c2];
    int i = 0, j = 0, len = 0;
    while (i < n1 && j < n2) {
        const uint32_t l1 = a[i], l2 = b[j], v1 = ABSV(l1), v2 = ABSV(l2);
        if (v1 == x) i++;
        else if (v2 == x) j++;
        else if ((l1 ^ l2) == 1u) return 0;
        else if (v1 < v2) { i++; out[len++] = l1; }
        else if (v2 < v1) { j++; out[len++] = l2; }
        else { i++; j++; out[len++] = l1; }
    }
    while (i < n1) { const uint32_t l1 = a[i++]; if (ABSV(l1) != x) out[len++] = l1; }
    while (j < n2) { const uint32_t l2 = b[j++]; if (ABSV(l2) != x) out[len++] = l2; }
    return len;
}

constexpr int CNT_RES_UNBOUNDED = 0, CNT_RES_BOUNDED = 1, CNT_SUBS = 2, CNT_CORE = 3;

// Pair filter of the four counting loops.
PFG_D bool ws_pair_ok(int kind, uint32_t mi, uint32_t mj) {
    if (m_learnt(mi)) return false;
    if (kind == CNT_RES_UNBOUNDED || kind == CNT_RES_BOUNDED) return !m_learnt(mj);
    if (kind == CNT_SUBS) return m_orig(mj) && (m_molten(mi) != m_molten(mj));
    return m_orig(mj) && (!m_molten(mi) || !m_molten(mj));
}

// The four resolvent-counting loops (resolve.cuh:28-198, elimination.cuh:409-484,
// function.cuh:196-273) with 32 pairs per step. Returns true when the loop
// finished ("can resolve"), false when it returned early; the guards after the
// loop are applied by the caller.
PFG_D bool ws_count_pairs(WS& w, int kind, uint32_t x, const Side& me, const Side& ot, uint32_t nClsBefore,
                          uint32_t rlimit, uint32_t& nE, uint32_t& nC, uint32_t& nL, unsigned lane) {
    const uint32_t total = me.n * ot.n;
    for (uint32_t q0 = 0; q0 < total; q0 += 32) {
        const uint32_t q = q0 + lane;
        int rsize = 0;
        bool valid = false;
        if (q < total) {
            const uint32_t ci = me.b + q / ot.n, cj = ot.b + q % ot.n;
            if (ws_pair_ok(kind, w.meta[ci], w.meta[cj])) {
                valid = true;
                uint32_t u;
                rsize = ws_merge_cnt(w, x, ci, cj, u);
            }
        }
        const bool iscl = valid && rsize > 1;
        const bool isun = valid && rsize == 1;
        uint32_t tcl;
        const uint32_t excl = warp_excl_scan(iscl ? 1u : 0u, lane, tcl);
        bool fail = false;
        if (iscl) {
            if (kind == CNT_RES_UNBOUNDED) fail = rlimit && (uint32_t)rsize > rlimit;
            else fail = (nC + excl + 1 > nClsBefore) || (rlimit && (uint32_t)rsize > rlimit);
        }
        const unsigned fb = __ballot_sync(FULL, fail);
        const unsigned ub = __ballot_sync(FULL, isun);
        if (fb) {
            const int f = __ffs(fb) - 1;
            const unsigned before = (1u << f) - 1u;
            nE += __popc(ub & before);
            // clause resolvents before f, then the ++ on f (except the unbounded loop)
            const uint32_t clb = __popc(__ballot_sync(FULL, iscl) & before);
            uint32_t lsum = (iscl && lane < (unsigned)f) ? (uint32_t)rsize : 0u;
#pragma unroll
            for (int d = 16; d > 0; d >>= 1) lsum += __shfl_down_sync(FULL, lsum, d);
            nL += __shfl_sync(FULL, lsum, 0);
            nC += clb + (kind == CNT_RES_UNBOUNDED ? 0u : 1u);
            return false;
        }
        uint32_t lsum = iscl ? (uint32_t)rsize : 0u;
#pragma unroll
        for (int d = 16; d > 0; d >>= 1) lsum += __shfl_down_sync(FULL, lsum, d);
        nL += __shfl_sync(FULL, lsum, 0);
        nC += tcl;
        nE += __popc(ub);
    }
    return true;
}

// mergeProof (elimination.cuh:162-213) on staged clauses: proof bytes of the
// resolvent, 0 for a tautology
PFG_D uint32_t ws_merge_bytes(const EK& k, WS& w, uint32_t x, uint32_t c1, uint32_t c2) {
    const uint32_t* a = WL(w, c1);
    const uint32_t* b = WL(w, c2);
    const int n1 = (int)w.size[c1], n2 = (int)w.size[c2];
    int i = 0, j = 0;
    uint32_t bytes = 2;
    while (i < n1 && j < n2) {
        const uint32_t l1 = a[i], l2 = b[j], v1 = ABSV(l1), v2 = ABSV(l2);
        if (v1 == x) i++;
        else if (v2 == x) j++;
        else if ((l1 ^ l2) == 1u) return 0;
        else if (v1 < v2) { i++; bytes += k.lbyte[l1]; }
        else if (v2 < v1) { j++; bytes += k.lbyte[l2]; }
        else { i++; j++; bytes += k.lbyte[l1]; }
    }
    while (i < n1) { const uint32_t l1 = a[i++]; if (ABSV(l1) != x) bytes += k.lbyte[l1]; }
    while (j < n2) { const uint32_t l2 = b[j++]; if (ABSV(l2) != x) bytes += k.lbyte[l2]; }
    return bytes;
}

// proof_guard on the stage, 32 pairs per step: true = ruled out
PFG_D bool ws_proof_guard(const EK& k, WS& w, int kind, uint32_t x, const Side& me, const Side& ot, uint32_t nE,
                          unsigned lane) {
    if (nE > ADDEDCLS_MAX) return true;
    const uint32_t total = me.n * ot.n;
    unsigned long long bytes = 0;
    for (uint32_t q0 = 0; q0 < total; q0 += 32) {
        const uint32_t q = q0 + lane;
        uint32_t b = 0;
        if (q < total) {
            const uint32_t ci = me.b + q / ot.n, cj = ot.b + q % ot.n;
            if (ws_pair_ok(kind, w.meta[ci], w.meta[cj])) b = ws_merge_bytes(k, w, x, ci, cj);
        }
#pragma unroll
        for (int d = 16; d > 0; d >>= 1) b += __shfl_xor_sync(FULL, b, d);
        bytes += b;
    }
    return bytes > ADDEDPROOF_MAX;
}

PFG_D uint32_t ws_lits_before(const WS& w, const Side& s) {
    uint32_t t = 0;
    for (uint32_t i = 0; i < s.n; i++) if (m_orig(w.meta[s.b + i])) t += w.size[s.b + i];
    return t;
}

// One resolvent count with the guards its loop has (resolve.cuh:28-198,
// elimination.cuh:409-484): true = the variable can be eliminated this way.
// The literal bound (velitsbound) applies to the bounded and substitution
// counts; the proof guard to all three.
PFG_D bool ws_count(const EK& k, WS& w, int kind, uint32_t x, const Side& me, const Side& ot, uint32_t nClsBefore,
                    uint32_t& nE, uint32_t& nC, uint32_t& nL, unsigned lane) {
    if (!ws_count_pairs(w, kind, x, me, ot, nClsBefore, k.ve_clause_max, nE, nC, nL, lane)) return false;
    if (nC > ADDEDCLS_MAX || nL > ADDEDLITS_MAX) return false;
    if (kind != CNT_RES_UNBOUNDED && k.ve_lbound_en && nL > ws_lits_before(w, me) + ws_lits_before(w, ot))
        return false;
    return !(k.proof && ws_proof_guard(k, w, kind, x, me, ot, nE, lane));
}

// ---- model stack from the stage ----
PFG_D void ws_save_side(const EK& k, WS& w, const Side& s, uint32_t witlit, uint32_t wit, unsigned lane) {
    // word offsets of the side's original clauses (size + 1 words each), then [w, 1]
    uint32_t base = 0;
    unsigned long long sbase = 0;
    uint32_t total = 2;
    for (uint32_t c0 = 0; c0 < s.n; c0 += 32) {
        const uint32_t i = c0 + lane;
        const bool org = i < s.n && m_orig(w.meta[s.b + i]);
        const uint32_t words = org ? w.size[s.b + i] + 1 : 0u;
        uint32_t t;
        warp_excl_scan(words, lane, t);
        total += t;
    }
    if (lane == 0) {
        sbase = stack_reserve(k, ABSV(wit), (unsigned long long)total);
    }
    sbase = __shfl_sync(FULL, sbase, 0);
    if (sbase == ~0ull) return;
    for (uint32_t c0 = 0; c0 < s.n; c0 += 32) {
        const uint32_t i = c0 + lane;
        const uint32_t c = s.b + i;
        const bool org = i < s.n && m_orig(w.meta[c]);
        const uint32_t words = org ? w.size[c] + 1 : 0u;
        uint32_t t;
        const uint32_t ex = warp_excl_scan(words, lane, t);
        if (org) {
            uint32_t* d = k.stack + sbase + base + ex;
            const uint32_t* l = WL(w, c);
            const uint32_t sz = w.size[c];
            uint32_t wpos = 0;
            for (uint32_t q = 0; q < sz; q++) {
                if (l[q] == witlit) wpos = q;
                d[q] = org_lit(k, l[q]);
            }
            if (wpos) { const uint32_t tmp = d[0]; d[0] = d[wpos]; d[wpos] = tmp; }
            d[sz] = sz;
        }
        base += t;
    }
    if (lane == 0) {
        k.stack[sbase + base] = org_lit(k, wit);
        k.stack[sbase + base + 1] = 1;
    }
    __syncwarp();
}

PFG_D void ws_save_resolved_orgs(const EK& k, WS& w, const Side& P, const Side& N, uint32_t pOrgs, uint32_t nOrgs,
                                 unsigned lane) {
    const Side& S = pOrgs > nOrgs ? N : P;     // one call site of ws_save_side
    ws_save_side(k, w, S, S.lit, S.lit ^ 1u, lane);
}

// delete every staged clause, empty both lists (toblivion, elimination.cuh:540-549)
PFG_D void ws_toblivion(const EK& k, WS& w, const Side& P, const Side& N, unsigned lane) {
    __syncwarp();
    const uint32_t nc = w.np + w.nn;
    for (uint32_t i = lane; i < nc; i += 32) w.meta[i] = m_set_st(w.meta[i], ST_DELETED);
    if (lane == 0) { k.ot_size[P.lit] = 0; k.ot_size[N.lit] = 0; }
    __syncwarp();
}

// ---- gates on the stage ----
PFG_D void ws_freeze_binaries(WS& w, const Side& s, unsigned lane) {
    __syncwarp();
    if (lane == 0)
        for (uint32_t i = 0; i < s.n; i++) {
            const uint32_t c = s.b + i;
            if (m_orig(w.meta[c]) && w.size[c] == 2) w.meta[c] = m_set_molten(w.meta[c], 0);
        }
    __syncwarp();
}

PFG_D bool ws_is_equal(WS& w, uint32_t c, const uint32_t* d, uint32_t n) {
    const uint32_t* l = WL(w, c);
    for (uint32_t i = 0; i < n; i++) if (l[i] != d[i]) return false;
    return true;
}

// find_ao_gate (and.cuh:27-113)
// Clauses a found gate melted, for the undo when its substitution is too large.
struct GateUndo {
    uint32_t a, b, c, d;
};

// find_ao_gate (and.cuh:46-105) up to the substitution count: the gate's
// clauses are left molten and the count is made by the caller
PFG_D bool ws_find_ao_gate(const EK& k, WS& w, const Side& D, const Side& F, GateUndo& undo, unsigned lane) {
    if (w.size[D.b] > 2 || w.size[F.b + F.n - 1] < 3) return false;
    const uint32_t dx = D.lit, fx = F.lit;
    uint32_t sig = 0;
    int nImps = 0;
    __syncwarp();
    for (uint32_t i = 0; i < D.n; i++) {
        const uint32_t c = D.b + i;
        if (m_orig(w.meta[c]) && w.size[c] == 2) {
            const uint32_t* l = WL(w, c);
            const uint32_t imp = FLIPL(l[0] ^ l[1] ^ dx);
            if (lane == 0) { w.outs[nImps] = imp; w.meta[c] = m_set_molten(w.meta[c], 1); }
            nImps++;
            sig |= MAPHASH(imp);
        }
    }
    __syncwarp();
    if (nImps > 1) {
        if (lane == 0) { w.outs[nImps] = fx; sort_small(w.outs, (uint32_t)nImps + 1); }
        nImps++;
        sig |= MAPHASH(fx);
        __syncwarp();
        for (uint32_t i = 0; i < F.n; i++) {
            const uint32_t c = F.b + i;
            if (m_orig(w.meta[c]) && w.size[c] == (uint32_t)nImps && SUBSIG(w.sig[c], sig) &&
                ws_is_equal(w, c, w.outs, (uint32_t)nImps)) {
                ws_melt(w, c, 1, lane);
                undo.a = c;
                return true;
            }
        }
    }
    ws_freeze_binaries(w, D, lane);
    return false;
}

// First staged clause of side S equal to the sorted literals t[0..n) that is
// original (and not molten when `unmelted`), or NOREF. The reference searches
// the shortest occurrence list of t's literals (fast_equality_check,
// ifthenelse.cuh:27-48; makeArity, xor.cuh:69-100). Every clause equal to t
// holds the eliminated variable's literal, so it is in S as well; equal
// clauses share their sort key, so the first one in any of those sorted lists
// is the one with the smallest id -- the first one in S.
PFG_D uint32_t ws_match(const WS& w, const Side& S, const uint32_t* t, uint32_t n, bool unmelted, unsigned lane) {
    for (uint32_t i0 = 0; i0 < S.n; i0 += 32) {
        const uint32_t i = i0 + lane;
        bool hit = false;
        if (i < S.n) {
            const uint32_t c = S.b + i;
            const uint32_t m = w.meta[c];
            if (w.size[c] == n && m_orig(m) && !(unmelted && m_molten(m))) {
                const uint32_t* l = w.lits + w.off[c];
                hit = true;
                for (uint32_t q = 0; q < n; q++)
                    if (l[q] != t[q]) { hit = false; break; }
            }
        }
        const unsigned b = __ballot_sync(FULL, hit);
        if (b) return S.b + i0 + __ffs(b) - 1;
    }
    return NOREF;
}

// fast_equality_check (ifthenelse.cuh:27-48) for the clause (fx, y, z):
// staged index in F, or NOREF
PFG_D uint32_t ws_fast_eq(const WS& w, const Side& F, uint32_t y, uint32_t z, unsigned lane) {
    uint32_t x = F.lit, t;
    if (z < y) { t = y; y = z; z = t; }
    if (z < x) { t = x; x = z; z = t; }
    if (y < x) { t = x; x = y; y = t; }
    const uint32_t c[3] = {x, y, z};
    return ws_match(w, F, c, 3, true, lane);
}

// find_ite_gate (ifthenelse.cuh:50-123) up to the substitution count
PFG_D bool ws_find_ite_gate(const EK& k, WS& w, const Side& D, const Side& F, GateUndo& undo, unsigned lane) {
    if (w.size[D.b + D.n - 1] == 2) return false;
    const uint32_t dx = D.lit, fx = F.lit;
    for (uint32_t i = 0; i < D.n; i++) {
        const uint32_t ci = D.b + i;
        if (!(m_orig(w.meta[ci]) && w.size[ci] == 3)) continue;
        const uint32_t* li = WL(w, ci);
        uint32_t xi = li[0], yi = li[1], zi = li[2], t;
        if (yi == dx) { t = xi; xi = yi; yi = t; }
        if (zi == dx) { t = xi; xi = zi; zi = t; }
        for (uint32_t j = i + 1; j < D.n; j++) {
            const uint32_t cj = D.b + j;
            if (!(m_orig(w.meta[cj]) && w.size[cj] == 3)) continue;
            const uint32_t* lj = WL(w, cj);
            uint32_t xj = lj[0], yj = lj[1], zj = lj[2];
            if (yj == dx) { t = xj; xj = yj; yj = t; }
            if (zj == dx) { t = xj; xj = zj; zj = t; }
            if (ABSV(yi) == ABSV(zj)) { t = yj; yj = zj; zj = t; }
            if (ABSV(zi) == ABSV(zj)) continue;
            if (yi != FLIPL(yj)) continue;
            const uint32_t s1 = ws_fast_eq(w, F, yi, FLIPL(zi), lane);
            if (s1 == NOREF) continue;
            const uint32_t s2 = ws_fast_eq(w, F, yj, FLIPL(zj), lane);
            if (s2 == NOREF) continue;
            ws_melt(w, ci, 1, lane);
            ws_melt(w, cj, 1, lane);
            if (s1 != NOREF) ws_melt(w, s1, 1, lane);
            if (s2 != NOREF) ws_melt(w, s2, 1, lane);
            undo = GateUndo{ci, cj, s1, s2};
            return true;
        }
    }
    return false;
}

PFG_D void ws_freeze_arities(WS& w, unsigned lane) {
    __syncwarp();
    const uint32_t nc = w.np + w.nn;
    for (uint32_t i = lane; i < nc; i += 32)
        if (w.size[i] > 2 && m_molten(w.meta[i])) w.meta[i] = m_set_molten(w.meta[i], 0);
    __syncwarp();
}

// makeArity (xor.cuh:69-100); `lits` is warp-shared. The flipped clause
// holds the literal of D or of F, and is looked up on that side of the stage.
PFG_D bool ws_make_arity(WS& w, const Side& D, const Side& F, uint32_t& parity, uint32_t* lits, uint32_t size,
                         unsigned lane) {
    const uint32_t old = parity;
    do { parity++; } while (__popc(parity) & 1);
    __syncwarp();
    if (lane == 0)
        for (uint32_t q = 0; q < size; q++) {
            const uint32_t bit = 1u << q;
            if ((parity & bit) != (old & bit)) lits[q] = FLIPL(lits[q]);
        }
    __syncwarp();
    bool has_d = false;
    for (uint32_t q = 0; q < size; q++) has_d |= lits[q] == D.lit;
    const uint32_t s = ws_match(w, has_d ? D : F, lits, size, false, lane);
    if (s == NOREF) return false;
    ws_melt(w, s, 1, lane);
    return true;
}

// Original staged clauses other than ci over exactly ci's variables. An XOR
// gate of arity a on ci needs 2^a - 1 of them (one per other parity), so with
// fewer the search of makeArity fails on its first target or a later one.
PFG_D uint32_t ws_xor_partners(const WS& w, uint32_t ci, unsigned lane) {
    const uint32_t nc = w.np + w.nn, size = w.size[ci];
    const uint32_t* a = w.lits + w.off[ci];
    uint32_t cnt = 0;
    for (uint32_t c0 = 0; c0 < nc; c0 += 32) {
        const uint32_t c = c0 + lane;
        bool same = false;
        if (c < nc && c != ci && w.size[c] == size && m_orig(w.meta[c])) {
            const uint32_t* b = w.lits + w.off[c];
            same = true;
            for (uint32_t q = 0; q < size; q++)
                if ((a[q] >> 1) != (b[q] >> 1)) { same = false; break; }
        }
        cnt += __popc(__ballot_sync(FULL, same));
    }
    return cnt;
}

// find_xor_gate (xor.cuh:102-178) up to the substitution count. A clause of D
// without the 2^a - 1 partners its gate needs is passed over without the
// searches: they would fail before melting anything, and the freeze that
// follows a failure (freezeArities) only changes state the first time, since
// every later failure starts from a stage without molten clauses above size 2.
PFG_D bool ws_find_xor_gate(const EK& k, WS& w, const Side& D, const Side& F, unsigned lane) {
    if (w.size[D.b + D.n - 1] == 2 || w.size[F.b + F.n - 1] == 2) return false;
    const int maxarity = (int)k.xor_max_arity;
    if ((int)w.size[D.b] - 1 > maxarity) return false;
    uint32_t* out = w.outs;
    bool frozen = false;
    for (uint32_t i = 0; i < D.n; i++) {
        const uint32_t ci = D.b + i;
        if (!m_orig(w.meta[ci])) continue;
        const int size = (int)w.size[ci], arity = size - 1;
        if (size < 3 || arity > maxarity) continue;
        if (ws_xor_partners(w, ci, lane) < (1u << arity) - 1u) {
            if (!frozen) { ws_freeze_arities(w, lane); frozen = true; }
            continue;
        }
        __syncwarp();
        if (lane == 0) { const uint32_t* l = WL(w, ci); for (int q = 0; q < size; q++) out[q] = l[q]; }
        __syncwarp();
        uint32_t parity = 0;
        int itargets = 1 << arity;
        while (--itargets && ws_make_arity(w, D, F, parity, out, (uint32_t)size, lane)) {}
        if (itargets) { ws_freeze_arities(w, lane); frozen = true; }
        else {
            ws_melt(w, ci, 1, lane);
            return true;
        }
    }
    return false;
}

// ---- equivalence (equivalence.cuh) ----
PFG_D uint32_t ws_find_equ_gate(WS& w, const Side& P, const Side& N, unsigned lane) {
    if (w.size[P.b] > 2 || w.size[N.b] > 2) return 0;
    // find_sfanin over P (equivalence.cuh:106-122)
    uint32_t first = 0;
    int nImps = 0;
    bool multi = false;
    __syncwarp();
    for (uint32_t i = 0; i < P.n; i++) {
        const uint32_t c = P.b + i;
        if (m_orig(w.meta[c]) && w.size[c] == 2) {
            const uint32_t* l = WL(w, c);
            first = FLIPL(l[0] ^ l[1] ^ P.lit);
            if (lane == 0) w.meta[c] = m_set_molten(w.meta[c], 1);
            nImps++;
        }
        if (nImps > 1) { multi = true; break; }
    }
    __syncwarp();
    if (multi) first = 0;
    if (first) {
        uint32_t second = N.lit, def = first;
        if (second < def) { first = second; second = def; }
        for (uint32_t i = 0; i < N.n; i++) {
            const uint32_t c = N.b + i;
            const uint32_t* l = WL(w, c);
            if (m_orig(w.meta[c]) && w.size[c] == 2 && l[0] == first && l[1] == second) {
                ws_melt(w, c, 1, lane);
                return def;
            }
        }
    }
    ws_freeze_binaries(w, P, lane);
    return 0;
}

// substitute_single (equivalence.cuh:27-104) on the stage (lane 0; rare)
PFG_D void ws_substitute_single(const EK& k, WS& w, const Side& P, const Side& N, uint32_t def, unsigned lane) {
    __syncwarp();
    if (lane == 0) {
        const uint32_t def_f = FLIPL(def);
        uint32_t nNeg = 0, nPos = 0;
        for (int side = 0; side < 2; side++) {
            const Side& S = side ? P : N;
            const uint32_t dx = S.lit, dd = side ? def : def_f, forbid = side ? def_f : def;
            uint32_t& cnt = side ? nPos : nNeg;
            for (uint32_t i = 0; i < S.n; i++) {
                const uint32_t c = S.b + i;
                uint32_t* l = WL(w, c);
                bool has = false;
                for (uint32_t q = 0; q < w.size[c]; q++) if (l[q] == forbid) { has = true; break; }
                if (m_learnt(w.meta[c]) || m_molten(w.meta[c]) || has) { w.meta[c] = m_set_st(w.meta[c], ST_DELETED); continue; }
                uint32_t j = 0;
                for (uint32_t q = 0; q < w.size[c]; q++) {
                    const uint32_t lit = l[q];
                    if (lit == dx) l[j++] = dd;
                    else if (lit != dd) l[j++] = lit;
                }
                w.size[c] = j;
                w.dirty[c] = 1;
                k.cnew[w.id[c]] = 1;
                if (j == 1) cnt++;
                else {
                    sort_small(l, j);
                    uint32_t sg = 0;
                    for (uint32_t q = 0; q < j; q++) sg |= MAPHASH(l[q]);
                    w.sig[c] = sg;
                }
            }
        }
        if (nPos || nNeg) {
            if (nNeg) for (uint32_t i = 0; i < N.n; i++) if (w.size[N.b + i] == 1) push_unit(k, WL(w, N.b + i)[0]);
            if (nPos) for (uint32_t i = 0; i < P.n; i++) if (w.size[P.b + i] == 1) push_unit(k, WL(w, P.b + i)[0]);
        }
        if (k.proof) {   // addProof over negs, then poss (equivalence.cuh:100-111)
            uint32_t words = 0;
            for (int side = 0; side < 2; side++) {
                const Side& S = side ? P : N;
                for (uint32_t i = 0; i < S.n; i++) if (m_orig(w.meta[S.b + i])) words += w.size[S.b + i] + 1;
            }
            uint32_t* d = words ? pf_reserve(k, ABSV(P.lit), 0, words) : nullptr;
            if (d)
                for (int side = 0; side < 2; side++) {
                    const Side& S = side ? P : N;
                    for (uint32_t i = 0; i < S.n; i++)
                        if (m_orig(w.meta[S.b + i])) d += pf_put(k, d, false, WL(w, S.b + i), w.size[S.b + i]);
                }
        }
    }
    __syncwarp();
}

PFG_D void ws_store_info(uint32_t tid, uint32_t elimType, uint32_t nE, uint32_t nC, uint32_t nL, uint32_t* type,
                         uint32_t* ucnt, unsigned long long* rpos, unsigned long long* rref, unsigned lane) {
    if (lane == 0) store_elim_info(tid, elimType, nE, nC, nL, type, ucnt, rpos, rref);
}

// find_fun_gate maps the neighbours of x through varcore (their place in the
// instance's frozen list) and builds truth tables over the first MAXFUNVAR
// only: with one neighbour further down the list (in a clause that is not
// learnt) it returns false before it changes anything (function.cuh:283-290),
// and the variable goes straight on to n-by-m resolution.
// Every neighbour is frozen, and a frozen variable above the instance's cut
// (fcut) has varcore >= MAXFUNVAR, so most variables are decided without
// reading varcore.
PFG_D bool ws_fun_possible(const EK& k, WS& w, uint32_t x, unsigned lane) {
    const uint32_t nc = w.np + w.nn;
    const uint32_t cut = k.fcut[k.vinst[x]];
    bool far = false;
    for (uint32_t i = lane; i < nc && !far; i += 32) {
        if (m_learnt(w.meta[i])) continue;
        const uint32_t* l = WL(w, i);
        for (uint32_t t = 0; t < w.size[i]; t++) {
            const uint32_t v = ABSV(l[t]);
            if (v != x && v > cut) { far = true; break; }
        }
    }
    if (__any_sync(FULL, far)) return false;
    for (uint32_t i = lane; i < nc && !far; i += 32) {
        if (m_learnt(w.meta[i])) continue;
        const uint32_t* l = WL(w, i);
        for (uint32_t t = 0; t < w.size[i]; t++) {
            const uint32_t v = ABSV(l[t]);
            if (v != x && k.varcore[v] >= MAXFUNVAR) { far = true; break; }
        }
    }
    return !__any_sync(FULL, far);
}

// BVE phase 1 for one staged variable (bounded.cuh:282-394)
PFG_D void ws_ve1(const EK& k, WS& w, uint32_t tid, uint32_t x, uint32_t* type, uint32_t* ucnt,
                  unsigned long long* rpos, unsigned long long* rref, uint32_t* dlist, uint32_t* dcount,
                  unsigned lane) {
    const uint32_t p = 2 * x, n = p | 1;
    const Side P{0, w.np, p}, N{w.np, w.nn, n};
    uint32_t pOrgs = P.n, nOrgs = N.n;
    if (k.ve_inprocess) {
        pOrgs = 0; nOrgs = 0;
        for (uint32_t i = 0; i < P.n; i++) pOrgs += m_orig(w.meta[P.b + i]);
        for (uint32_t i = 0; i < N.n; i++) nOrgs += m_orig(w.meta[N.b + i]);
    }
    if (lane == 0) { type[tid] = 0; ucnt[tid] = 0; rpos[tid] = 0; rref[tid] = 0; }
    uint32_t elimType = 0, nE = 0, nC = 0, nL = 0, def = 0;
    // a pure literal goes straight to the common end: no resolvents
    if (pOrgs && nOrgs) {
        def = ws_find_equ_gate(w, P, N, lane);
        if (!def) {
            const uint32_t nClsBefore = pOrgs + nOrgs;
            // Every resolvent count goes through the one call of ws_count below (the
            // three loops inlined at three places made the kernel fetch-bound):
            //   g = -1: single-occurrence resolution (resolve.cuh:28-109), tried first
            //           when one side has one original clause;
            //   g = 0..5: AND/OR gates for both definitions, then ITE and XOR gates for
            //           both (bounded.cuh:336-356), each found gate's substitution
            //           counted; a second definition is tried only while no
            //           substitution was counted;
            //   g = 6: the function-table gate is deferred to ve1b_k, else n-by-m
            //           resolution (resolve.cuh:111-198) when nothing was counted.
#pragma unroll 1
            for (int g = (pOrgs == 1 || nOrgs == 1) ? -1 : 0; g <= 6; g++) {
                int kind;
                uint32_t ncb = nClsBefore;
                const int o = g & 1;
                // AND/OR: (N, P) then (P, N); ITE and XOR: (P, N) then (N, P)
                const bool pfirst = g < 0 || g >= 6 ? true : (g < 2 ? o != 0 : o == 0);
                const Side& D = pfirst ? P : N;
                const Side& F = pfirst ? N : P;
                GateUndo undo{NOREF, NOREF, NOREF, NOREF};
                if (g < 0) {
                    kind = CNT_RES_UNBOUNDED;
                    ncb = 0;
                } else if (g < 6) {
                    if (g < 2 ? nClsBefore <= 2 : nClsBefore <= 3) continue;
                    if (o && nC) continue;
                    bool found;
                    if (g < 2) found = (pfirst ? pOrgs : nOrgs) < SH_MAX_BVE_OUT1 && ws_find_ao_gate(k, w, D, F, undo, lane);
                    else if (g < 4) found = ws_find_ite_gate(k, w, D, F, undo, lane);
                    else found = ws_find_xor_gate(k, w, D, F, lane);
                    if (!found) continue;
                    nE = 0; nC = 0; nL = 0;
                    kind = CNT_SUBS;
                } else {
                    if (vc_on(k, x) && nClsBefore > 2 && ws_fun_possible(k, w, x, lane)) {
                        ws_flush(k, w, lane);
                        if (lane == 0) {
                            dlist[atomicAdd(dcount, 1u)] = tid;
                            ucnt[tid] = nC;
                            rpos[tid] = (unsigned long long)pOrgs | ((unsigned long long)nOrgs << 32);
                        }
                        return;
                    }
                    if (nC) break;
                    nE = 0; nC = 0; nL = 0;
                    kind = CNT_RES_BOUNDED;
                }
                const bool ok = ws_count(k, w, kind, x, D, F, ncb, nE, nC, nL, lane);
                if (g < 0) {
                    if (ok) { elimType = RES_MASK; break; }   // resolvents (nC > 0) or none: the common end
                    nE = 0; nC = 0; nL = 0;
                    continue;
                }
                if (g >= 6) {
                    if (ok) elimType = RES_MASK;
                    break;
                }
                if (ok) { elimType = AOIX_MASK; break; }
                // too many resolvents: undo what the detector melted
                if (g < 2) {
                    ws_melt(w, undo.a, 0, lane);
                    ws_freeze_binaries(w, D, lane);
                } else if (g < 4) {
                    ws_melt(w, undo.a, 0, lane);
                    ws_melt(w, undo.b, 0, lane);
                    if (undo.c != NOREF) ws_melt(w, undo.c, 0, lane);
                    if (undo.d != NOREF) ws_melt(w, undo.d, 0, lane);
                } else {
                    ws_freeze_arities(w, lane);
                }
            }
        }
    }
    // common end: eliminated without resolvents (pure literal, no clause
    // resolvent, or substituted by an equivalence: the side with fewer original
    // clauses saved, then the clauses deleted or rewritten), or the counts
    // stored for emission (elimType set), or kept
    if (!nC) {
        ws_save_resolved_orgs(k, w, P, N, pOrgs, nOrgs, lane);
        if (def) ws_substitute_single(k, w, P, N, def, lane);
        else ws_toblivion(k, w, P, N, lane);
        ws_flush(k, w, lane);
        if (lane == 0) k.elim[x] |= MELTING_MASK;
    }
    else {
        ws_flush(k, w, lane);
        if (elimType) ws_store_info(tid, elimType, nE, nC, nL, type, ucnt, rpos, rref, lane);
    }
}

__global__ void __launch_bounds__(WS_WARPS * 32) ve1w_k(EK k, const uint32_t* elected, uint32_t nelected,
                                                        uint32_t* type, uint32_t* ucnt, unsigned long long* rpos,
                                                        unsigned long long* rref, uint32_t* dlist, uint32_t* dcount,
                                                        uint32_t* big, uint32_t* nbig, uint32_t* steal) {
    __shared__ WS stage[WS_WARPS];
    const unsigned lane = threadIdx.x & 31u;
    WS& w = stage[threadIdx.x >> 5];
    uint32_t qn;
    for (uint32_t q = ws_ticket(steal, lane); q < nelected; q = qn) {
        qn = ws_ticket(steal, lane);     // drawn ahead: its lists are prefetched while this one runs
        const uint32_t tid = q;
        const uint32_t x = elected[tid];
        const NextLists nl = ws_next_lists(k, elected, qn, nelected);
        if (!ws_stage(k, w, 2 * x, 2 * x + 1, lane)) {
            if (lane == 0) big[atomicAdd(nbig, 1u)] = tid;
            continue;
        }
        ws_ve1(k, w, tid, x, type, ucnt, rpos, rref, dlist, dcount, lane);
        ws_prefetch_lists(k, nl, lane);
        __syncwarp();
    }
}

// ---- BVE phase 3 on the stage (bounded.cuh:69-258, 488-544) ----
__global__ void __launch_bounds__(WS_WARPS * 32) ve3w_k(EK k, const uint32_t* elected, uint32_t nelected,
                                                        const uint32_t* type, const uint32_t* ucnt,
                                                        const unsigned long long* rslot,
                                                        const unsigned long long* rlit, const uint8_t* fits,
                                                        uint32_t* big, uint32_t* nbig, uint32_t* steal,
                                                        uint32_t ticket) {
    __shared__ WS stage[WS_WARPS];
    const unsigned lane = threadIdx.x & 31u;
    WS& w = stage[threadIdx.x >> 5];
    // tickets of `ticket` variables (>= 1): most elected variables emit nothing
    // and are passed over at once, so one draw per variable would queue on the counter
    const uint32_t nchunks = (nelected + ticket - 1) / ticket;
    for (uint32_t t = ws_ticket(steal, lane); t < nchunks; t = ws_ticket(steal, lane))
    for (uint32_t q = t * ticket, qe = min(q + ticket, nelected); q < qe; q++) {
        const uint32_t tid = q;
        const uint32_t x = elected[tid];
        const uint32_t xinfo = type[tid];
        const uint32_t et = xinfo & 3u;
        if (!et) continue;
        const uint32_t p = 2 * x, n = p | 1;
        if (!ws_stage(k, w, p, n, lane)) {
            if (lane == 0) big[atomicAdd(nbig, 1u)] = tid;
            continue;
        }
        const Side P{0, w.np, p}, N{w.np, w.nn, n};
        const uint32_t nAddedCls = (xinfo & 0xFFFCu) >> 2;
        if (fits[tid]) {
            // saveResolved by list sizes (elimination.cuh:551-594)
            if (P.n > N.n) ws_save_side(k, w, N, N.lit, P.lit, lane);
            else ws_save_side(k, w, P, P.lit, N.lit, lane);
            const int kind = et == RES_MASK ? CNT_RES_BOUNDED : (et == CORE_MASK ? CNT_CORE : CNT_SUBS);
            unsigned long long slot = rslot[tid];
            unsigned long long woff = rlit[tid];
            uint32_t added = 0;
            const uint32_t total = P.n * N.n;
            // proof: the resolvent lines in pair order into one block, the rest padding
            const uint32_t pwords = k.proof ? pf_res_words(xinfo, ucnt[tid]) : 0u;
            uint32_t* pd = nullptr;
            if (pwords && lane == 0) pd = pf_reserve(k, x, 0, pwords);
            pd = (uint32_t*)__shfl_sync(FULL, (unsigned long long)pd, 0);
            uint32_t pused = 0;
            for (uint32_t q0 = 0; q0 < total && added < nAddedCls; q0 += 32) {
                const uint32_t q = q0 + lane;
                int rsize = 0;
                uint32_t unit = 0, ci = 0, cj = 0;
                if (q < total) {
                    ci = P.b + q / N.n;
                    cj = N.b + q % N.n;
                    const uint32_t mi = w.meta[ci], mj = w.meta[cj];
                    bool ok = !m_learnt(mi) && !m_learnt(mj);
                    if (ok && kind == CNT_SUBS) ok = m_molten(mi) != m_molten(mj);
                    if (ok && kind == CNT_CORE) ok = !(m_molten(mi) && m_molten(mj));
                    if (ok) rsize = ws_merge_cnt(w, x, ci, cj, unit);
                }
                const bool iscl = rsize > 1, isun = rsize == 1;
                uint32_t tcl;
                const uint32_t excl = warp_excl_scan(iscl ? 1u : 0u, lane, tcl);
                // a pair is visited while fewer than nAddedCls clauses were added before it
                const bool visited = q < total && (added + excl) < nAddedCls;
                if (visited && isun) push_unit(k, unit);
                const bool emit = visited && iscl;
                uint32_t ltot;
                const uint32_t lex = warp_excl_scan(emit ? (uint32_t)rsize : 0u, lane, ltot);
                const uint32_t ncl = __popc(__ballot_sync(FULL, emit));
                uint32_t* pl = nullptr;
                if (pd) {
                    const uint32_t pw = (visited && rsize) ? (uint32_t)rsize + 1 : 0u;
                    uint32_t ptot;
                    const uint32_t pex = warp_excl_scan(pw, lane, ptot);
                    if (pused + pex + pw <= pwords) pl = pd + pused + pex;
                    else if (pw) atomicOr(&k.dc->err, ERR_PROOF_OVERFLOW);
                    pused += ptot;
                    if (visited && isun && pl) pf_put(k, pl, false, &unit, 1);
                }
                if (emit) {
                    const unsigned long long o = woff + lex;
                    uint32_t* out = k.lits + o;
                    ws_merge_out(w, x, ci, cj, out);
                    if (pl) pf_put(k, pl, false, out, (uint32_t)rsize);
                    uint32_t sig = 0;
                    for (int t = 0; t < rsize; t++) sig |= MAPHASH(out[t]);
                    ClsHdr h;
                    h.off = (uint32_t)o;
                    h.size = (uint32_t)rsize;
                    h.sig = sig;
                    h.meta = m_make(ST_ORIGINAL, 0, 1, 0, 0);
                    k.hdr[slot + excl] = h;
                    k.cnew[slot + excl] = 1;
                }
                added += ncl;
                slot += ncl;
                woff += ltot;
            }
            if (added != nAddedCls && lane == 0) atomicOr(&k.dc->err, ERR_SLOT_MISMATCH);
            if (pd) for (uint32_t t = pused + lane; t < pwords; t += 32) pd[t] = 0u;
            ws_toblivion(k, w, P, N, lane);
            ws_flush(k, w, lane);
            if (lane == 0) k.elim[x] |= MELTING_MASK | ADDING_MASK;
        } else if (et != RES_MASK) {
            __syncwarp();
            const uint32_t nc = w.np + w.nn;
            for (uint32_t i = lane; i < nc; i += 32)
                if (m_orig(w.meta[i]) && m_molten(w.meta[i])) w.meta[i] = m_set_molten(w.meta[i], 0);
            ws_flush(k, w, lane);
        }
        __syncwarp();
    }
}

// ---- SUB on the stage (subsume.cuh:293-484) ----
PFG_D bool ws_sub(WS& w, uint32_t s, uint32_t t) {
    const uint32_t* d1 = WL(w, s);
    const uint32_t* d2 = WL(w, t);
    const uint32_t n1 = w.size[s], n2 = w.size[t];
    uint32_t i = 0, j = 0, sub = 0;
    while (i < n1 && j < n2) {
        if (d1[i] < d2[j]) i++;
        else if (d2[j] < d1[i]) j++;
        else { sub++; i++; j++; }
    }
    return sub == n1;
}

PFG_D bool ws_selfsub(WS& w, uint32_t x, uint32_t fx, uint32_t s, uint32_t t) {
    const uint32_t* d1 = WL(w, s);
    const uint32_t* d2 = WL(w, t);
    const uint32_t n1 = w.size[s], n2 = w.size[t];
    uint32_t i = 0, j = 0, sub = 0;
    bool self = false;
    while (i < n1 && j < n2) {
        const uint32_t l1 = d1[i], l2 = d2[j];
        if (l1 == fx) i++;
        else if (l2 == x) { self = true; j++; }
        else if (l1 < l2) i++;
        else if (l2 < l1) j++;
        else { sub++; i++; j++; }
    }
    if (sub + 1 == n1) {
        if (self) return true;
        while (j < n2) { if (d2[j] == x) return true; j++; }
    }
    return false;
}

// self-subsumption of cand by the first fitting clause of `L` (subsume.cuh:344-399)
PFG_D void ws_selfsubsume(WS& w, uint32_t x, uint32_t fx, const Side& L, uint32_t cand, uint32_t& nUnits,
                          unsigned lane) {
    const uint32_t candsz = w.size[cand], candsig = w.sig[cand];
    for (uint32_t j0 = 0; j0 < L.n; j0 += 32) {
        const uint32_t j = j0 + lane;
        int ev = 0;   // 1 = break (size), 2 = strengthen
        if (j < L.n) {
            const uint32_t s = L.b + j;
            const uint32_t subsize = w.size[s];
            if (subsize > candsz) ev = 1;
            else if (!m_deleted(w.meta[s]) && !m_molten(w.meta[s]) && subsize > 1 && selfsub_sig(w.sig[s], candsig) &&
                     ws_selfsub(w, x, fx, s, cand))
                ev = 2;
        }
        const unsigned b = __ballot_sync(FULL, ev != 0);
        if (!b) continue;
        const int first = __shfl_sync(FULL, ev, __ffs(b) - 1);
        if (first == 2) {
            __syncwarp();
            if (lane == 0) {
                // strengthen (subsume.cuh:233-291), then melt
                uint32_t* l = WL(w, cand);
                uint32_t jj = 0;
                for (uint32_t i = 0; i < w.size[cand]; i++) if (l[i] != x) l[jj++] = l[i];
                w.size[cand]--;
                w.dirty[cand] = 1;
                const uint32_t sz = w.size[cand];
                if (sz > 1) {
                    uint32_t sg = 0;
                    for (uint32_t i = 0; i < sz; i++) sg |= MAPHASH(l[i]);
                    w.sig[cand] = sg;
                    const uint32_t m = w.meta[cand];
                    if (m_learnt(m)) {
                        const int old_lbd = (int)m_lbd(m);
                        if (old_lbd > (int)LBD_TIER1) {
                            const int sz1 = (int)sz - 1;
                            const int new_lbd = sz1 < old_lbd ? sz1 : old_lbd;
                            if (new_lbd < old_lbd) w.meta[cand] = (m & 0xFu) | (USAGET3 << 4) | ((uint32_t)new_lbd << 6);
                        }
                    }
                }
                w.meta[cand] = m_set_molten(w.meta[cand], 1);
            }
            __syncwarp();
            if (w.size[cand] == 1) nUnits++;
        }
        return;
    }
}

// forward subsumption of cand by an earlier clause of `L` (subsume.cuh:305-342)
PFG_D void ws_subsume(WS& w, const Side& L, uint32_t end, uint32_t cand, unsigned lane) {
    const uint32_t candsz = w.size[cand], candsig = w.sig[cand];
    const bool candm = m_molten(w.meta[cand]);
    for (uint32_t j0 = 0; j0 < end; j0 += 32) {
        const uint32_t j = j0 + lane;
        bool hit = false;
        if (j < end) {
            const uint32_t s = L.b + j;
            const uint32_t ms = w.meta[s];
            if (!m_deleted(ms) && !(candm && w.size[s] > candsz) && w.size[s] > 1 && SUBSIG(w.sig[s], candsig) &&
                ws_sub(w, s, cand))
                hit = true;
        }
        const unsigned b = __ballot_sync(FULL, hit);
        if (!b) continue;
        const uint32_t s = L.b + j0 + __ffs(b) - 1;
        __syncwarp();
        if (lane == 0) {
            if (m_learnt(w.meta[s]) && m_orig(w.meta[cand])) w.meta[s] = m_set_st(w.meta[s], ST_ORIGINAL);
            w.meta[cand] = m_set_st(w.meta[cand], ST_DELETED);
        }
        __syncwarp();
        return;
    }
}

// saveProof over poss then negs (subsume.cuh:464-474): the stage holds poss
// then negs in list order; strengthened clauses are added, subsumed ones deleted
PFG_D void ws_proof_sub(const EK& k, WS& w, uint32_t x, unsigned lane) {
    __syncwarp();
    const uint32_t nc = w.np + w.nn;
    uint32_t total = 0;
    for (uint32_t c0 = 0; c0 < nc; c0 += 32) {
        const uint32_t i = c0 + lane;
        uint32_t words = 0;
        if (i < nc) words = (m_molten(w.meta[i]) ? w.size[i] + 1 : 0u) + (m_deleted(w.meta[i]) ? w.size[i] + 1 : 0u);
#pragma unroll
        for (int d = 16; d > 0; d >>= 1) words += __shfl_xor_sync(FULL, words, d);
        total += words;
    }
    if (!total) return;
    uint32_t* d = nullptr;
    if (lane == 0) d = pf_reserve(k, x, 0, total);
    d = (uint32_t*)__shfl_sync(FULL, (unsigned long long)d, 0);
    if (!d) return;
    uint32_t used = 0;
    for (uint32_t c0 = 0; c0 < nc; c0 += 32) {
        const uint32_t i = c0 + lane;
        const bool m = i < nc && m_molten(w.meta[i]), del = i < nc && m_deleted(w.meta[i]);
        const uint32_t words = (m ? w.size[i] + 1 : 0u) + (del ? w.size[i] + 1 : 0u);
        uint32_t t;
        const uint32_t ex = warp_excl_scan(words, lane, t);
        uint32_t* o = d + used + ex;
        if (m) o += pf_put(k, o, false, WL(w, i), w.size[i]);
        if (del) pf_put(k, o, true, WL(w, i), w.size[i]);
        used += t;
    }
    __syncwarp();
}

// updateOL (subsume.cuh:293-303) on the global list, order kept
PFG_D void ws_update_ol(const EK& k, WS& w, const Side& L, unsigned lane) {
    __syncwarp();
    // a list without a deleted or strengthened (molten) clause keeps every
    // entry in the order it was staged in: nothing to write back
    bool touched = false;
    for (uint32_t j = lane; j < L.n; j += 32) {
        const uint32_t m = w.meta[L.b + j];
        touched |= m_molten(m) || m_deleted(m);
    }
    if (!__any_sync(FULL, touched)) return;
    uint32_t* ol = OLp(k, L.lit);
    uint32_t kept = 0;
    for (uint32_t j0 = 0; j0 < L.n; j0 += 32) {
        const uint32_t j = j0 + lane;
        bool keepit = false;
        uint32_t c = 0;
        if (j < L.n) {
            c = L.b + j;
            const uint32_t m = w.meta[c];
            if (m_molten(m)) w.meta[c] = m_set_molten(m, 0);
            else keepit = !m_deleted(m);
        }
        uint32_t t;
        const uint32_t ex = warp_excl_scan(keepit ? 1u : 0u, lane, t);
        if (keepit) ol[kept + ex] = w.id[c];
        kept += t;
    }
    if (lane == 0) k.ot_size[L.lit] = kept;
    __syncwarp();
}

// Screen of SUB on the stage, into w.outs: clause i can only be subsumed by an
// earlier clause of its own list or strengthened by a clause of the other list
// whose signature fits. Strengthening removes x's own literals only, so a
// partner's signature without their bits (M) is contained in what it will be
// when clause i's turn comes, and clause i's own signature does not change
// before its turn; a clause with no fitting partner is left alone by both
// searches, which are skipped for it.
PFG_D void ws_sub_screen(WS& w, const Side& P, const Side& N, unsigned lane) {
    const uint32_t M = MAPHASH(P.lit) | MAPHASH(N.lit);
    const uint32_t nc = w.np + w.nn;
    for (uint32_t i = lane; i < nc; i += 32) {
        const bool inP = i < w.np;
        const uint32_t sb = inP ? P.b : N.b;
        const uint32_t ob = inP ? N.b : P.b, oe = ob + (inP ? N.n : P.n);
        const uint32_t cs = w.sig[i];
        bool maybe = false;
        for (uint32_t j = sb; j < i && !maybe; j++)
            maybe = w.size[j] > 1 && SUBSIG(w.sig[j] & ~M, cs);
        for (uint32_t j = ob; j < oe && !maybe; j++)
            maybe = w.size[j] > 1 && selfsub_sig(w.sig[j] & ~M, cs);
        w.outs[i] = maybe ? 1u : 0u;
    }
    __syncwarp();
}

// The candidates of one side in list order (subsume.cuh:424-455): up to the
// first clause above SUB_MAX_CL_SIZE (the list is sorted by size), those not
// deleted that passed the screen. Processing a candidate changes only that
// clause (strengthened or deleted) and earlier ones (a subsuming learnt clause
// turned original), so the candidates are known before the first one runs and
// are taken from one ballot per 32 clauses.
PFG_D void ws_sub_side(WS& w, const Side& L, const Side& O, uint32_t x, uint32_t fx, uint32_t& nUnits,
                       unsigned lane) {
    for (uint32_t i0 = 0; i0 < L.n; i0 += 32) {
        const uint32_t i = i0 + lane;
        bool big = false, cand = false;
        if (i < L.n) {
            const uint32_t c = L.b + i;
            big = w.size[c] > SUB_MAX_CL_SIZE;
            cand = !big && !m_deleted(w.meta[c]) && w.outs[c];
        }
        const unsigned bigm = __ballot_sync(FULL, big);
        unsigned cm = __ballot_sync(FULL, cand);
        if (bigm) cm &= (1u << (__ffs(bigm) - 1)) - 1u;
        for (; cm; cm &= cm - 1) {
            const uint32_t j = i0 + (uint32_t)__ffs(cm) - 1;
            ws_selfsubsume(w, x, fx, O, L.b + j, nUnits, lane);
            ws_subsume(w, L, j, L.b + j, lane);
        }
        if (bigm) break;
    }
}

__global__ void __launch_bounds__(WS_WARPS * 32) subw_k(EK k, const uint32_t* elected, uint32_t nelected,
                                                        uint32_t* big, uint32_t* nbig, uint32_t* steal) {
    __shared__ WS stage[WS_WARPS];
    const unsigned lane = threadIdx.x & 31u;
    WS& w = stage[threadIdx.x >> 5];
    for (uint32_t q = ws_ticket(steal, lane); q < nelected; q = ws_ticket(steal, lane)) {
        const uint32_t e = q;
        const uint32_t x = elected[e];
        const uint32_t p = 2 * x, n = p | 1;
        if (OLs(k, p) > k.sub_max_occurs || OLs(k, n) > k.sub_max_occurs) continue;
        if (!ws_stage(k, w, p, n, lane)) {
            if (lane == 0) big[atomicAdd(nbig, 1u)] = e;
            continue;
        }
        const Side P{0, w.np, p}, N{w.np, w.nn, n};
        ws_sub_screen(w, P, N, lane);
        uint32_t nPos = 0, nNeg = 0;
        ws_sub_side(w, P, N, p, n, nPos, lane);
        ws_sub_side(w, N, P, n, p, nNeg, lane);
        __syncwarp();
        if ((nPos || nNeg) && lane == 0) {
            if (nPos) for (uint32_t i = 0; i < P.n; i++) if (w.size[P.b + i] == 1) push_unit(k, WL(w, P.b + i)[0]);
            if (nNeg) for (uint32_t i = 0; i < N.n; i++) if (w.size[N.b + i] == 1) push_unit(k, WL(w, N.b + i)[0]);
        }
        if (k.proof) ws_proof_sub(k, w, x, lane);
        ws_update_ol(k, w, P, lane);
        ws_update_ol(k, w, N, lane);
        ws_flush(k, w, lane);
    }
}
