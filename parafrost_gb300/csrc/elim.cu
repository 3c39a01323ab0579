// Per-variable elimination passes: SUB (+ self-subsuming strengthening),
// BVE phase 1 (gate detection + resolvent counting), BVE phase 3 (resolvent
// emission into prefix-summed slots) and ERE.
//
// Elected variables share no clause (LCVE freezes every neighbour), so each
// thread owns the clauses of its variable; reads of neighbouring occurrence
// lists never match a clause that another thread is changing. The
// per-variable semantics follow the reference kernels:
//   sub_k        src/gpu/subsume.cuh:402-484
//   ve_k_1       src/gpu/bounded.cuh:282-473 (+ and/xor/ifthenelse/function/equivalence.cuh)
//   ve_k_2       src/gpu/bounded.cuh:69-258, 488-544
//   ere_k        src/gpu/redundancy.cuh:27-175
#include "engine.cuh"

namespace pfg {
namespace {

struct EK {
    ClsHdr* hdr;
    uint32_t* lits;
    const uint32_t* ot_off;
    uint32_t* ot_size;
    uint32_t* ot_ids;
    uint8_t* elim;
    const uint32_t* varcore;
    const uint32_t* fcut;                // per instance: largest variable that varcore maps below MAXFUNVAR
    const uint32_t* vorg;
    const uint32_t* vinst;               // instance of a variable
    const uint8_t* vc_on;                // per instance: function-table gates on
    uint32_t* units;                     // per-instance unit regions
    const unsigned long long* ubase;
    const uint32_t* ucap;
    uint32_t* ucount;
    uint32_t* stack;                     // per-instance model-stack regions
    const unsigned long long* sbase;
    const unsigned long long* scap;
    unsigned long long* scount;
    DevCounters* dc;
    uint32_t ve_clause_max, xor_max_arity, sub_max_occurs, ere_max_occurs, ere_clause_max;
    int ve_lbound_en, ve_inprocess;
    int proof;                           // DRAT lines are written (proof_en)
    uint32_t* pf_w;                      // proof line words of the running pass
    unsigned long long pf_wcap;
    ulonglong2* pf_b;                    // proof blocks {variable << 32 | sequence, first word}
    uint32_t pf_bcap;
    const uint8_t* lbyte;                // proof bytes per literal
    uint8_t* cnew;                       // clauses added or rewritten in place (occurrence-table update)
};

PFG_D uint32_t* OLp(const EK& k, uint32_t lit) { return k.ot_ids + k.ot_off[lit]; }
PFG_D uint32_t OLs(const EK& k, uint32_t lit) { return k.ot_size[lit]; }
PFG_D uint32_t* CLp(const EK& k, uint32_t c) { return k.lits + k.hdr[c].off; }
PFG_D uint32_t META(const EK& k, uint32_t c) { return k.hdr[c].meta; }
PFG_D uint32_t SIZE(const EK& k, uint32_t c) { return k.hdr[c].size; }
PFG_D void SET_MOLTEN(const EK& k, uint32_t c, uint32_t f) { k.hdr[c].meta = m_set_molten(k.hdr[c].meta, f); }
PFG_D void SET_DELETED(const EK& k, uint32_t c) { k.hdr[c].meta = m_set_st(k.hdr[c].meta, ST_DELETED); }

PFG_D void push_unit(const EK& k, uint32_t lit) {
    const uint32_t inst = k.vinst[ABSV(lit)];
    const uint32_t i = atomicAdd(&k.ucount[inst], 1u);
    if (i < k.ucap[inst]) k.units[k.ubase[inst] + i] = lit;
    else atomicOr(&k.dc->err, ERR_UNITS_OVERFLOW);
}

// reserve `words` of the model stack of variable v's instance; ~0 on overflow
PFG_D unsigned long long stack_reserve(const EK& k, uint32_t v, unsigned long long words) {
    const uint32_t inst = k.vinst[v];
    const unsigned long long base = atomicAdd(&k.scount[inst], words);
    if (base + words > k.scap[inst]) { atomicOr(&k.dc->err, ERR_STACK_OVERFLOW); return ~0ull; }
    return k.sbase[inst] + base;
}

PFG_D bool vc_on(const EK& k, uint32_t x) { return k.vc_on[k.vinst[x]] != 0; }

PFG_D void sort_small(uint32_t* d, uint32_t n) {
    for (uint32_t i = 1; i < n; i++) {
        const uint32_t t = d[i];
        uint32_t j = i;
        while (j > 0 && t < d[j - 1]) { d[j] = d[j - 1]; j--; }
        d[j] = t;
    }
}

PFG_D void calc_sig(const EK& k, uint32_t c) {   // calcSig(SCLAUSE&): only for size > 1
    const uint32_t sz = SIZE(k, c);
    if (sz <= 1) return;
    const uint32_t* l = CLp(k, c);
    uint32_t s = 0;
    for (uint32_t i = 0; i < sz; i++) s |= MAPHASH(l[i]);
    k.hdr[c].sig = s;
}

PFG_D bool selfsub_sig(uint32_t A, uint32_t B) {
    const uint32_t Bt = B | ((B & 0xAAAAAAAAu) >> 1) | ((B & 0x55555555u) << 1);
    return !(A & ~Bt);
}

PFG_D void freeze_binaries(const EK& k, uint32_t lit) {
    const uint32_t* ol = OLp(k, lit);
    const uint32_t n = OLs(k, lit);
    for (uint32_t i = 0; i < n; i++) {
        const uint32_t c = ol[i];
        const ClsHdr h = k.hdr[c];
        if (m_orig(h.meta) && h.size == 2) SET_MOLTEN(k, c, 0);
    }
}

PFG_D void freeze_clauses(const EK& k, uint32_t p, uint32_t n) {
    for (int s = 0; s < 2; s++) {
        const uint32_t lit = s ? n : p;
        const uint32_t* ol = OLp(k, lit);
        const uint32_t sz = OLs(k, lit);
        for (uint32_t i = 0; i < sz; i++) {
            const uint32_t m = META(k, ol[i]);
            if (m_orig(m) && m_molten(m)) SET_MOLTEN(k, ol[i], 0);
        }
    }
}

PFG_D void append_units(const EK& k, uint32_t lit) {
    const uint32_t* ol = OLp(k, lit);
    const uint32_t n = OLs(k, lit);
    for (uint32_t i = 0; i < n; i++) {
        const ClsHdr h = k.hdr[ol[i]];
        if (h.size == 1) push_unit(k, k.lits[h.off]);
    }
}

PFG_D bool is_equal(const EK& k, uint32_t c, const uint32_t* d, uint32_t n) {
    const uint32_t* l = CLp(k, c);
    for (uint32_t i = 0; i < n; i++) if (l[i] != d[i]) return false;
    return true;
}

// merge(x, c1, c2, unit) counting version (elimination.cuh:242-270)
PFG_D int merge_cnt(const EK& k, uint32_t x, uint32_t c1, uint32_t c2, uint32_t& unit) {
    const ClsHdr h1 = k.hdr[c1], h2 = k.hdr[c2];
    const uint32_t* a = k.lits + h1.off;
    const uint32_t* b = k.lits + h2.off;
    const int n1 = (int)h1.size, n2 = (int)h2.size;
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

// merge(x, c1, c2, out_c) (elimination.cuh:302-331)
PFG_D int merge_out(const EK& k, uint32_t x, uint32_t c1, uint32_t c2, uint32_t* out) {
    const ClsHdr h1 = k.hdr[c1], h2 = k.hdr[c2];
    const uint32_t* a = k.lits + h1.off;
    const uint32_t* b = k.lits + h2.off;
    const int n1 = (int)h1.size, n2 = (int)h2.size;
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

PFG_D uint32_t count_lits_before(const EK& k, uint32_t lit) {
    const uint32_t* ol = OLp(k, lit);
    const uint32_t n = OLs(k, lit);
    uint32_t s = 0;
    for (uint32_t i = 0; i < n; i++) {
        const ClsHdr h = k.hdr[ol[i]];
        if (m_orig(h.meta)) s += h.size;
    }
    return s;
}

constexpr int PAIR_RES = 0, PAIR_SUBS = 1, PAIR_CORE = 2;

PFG_D bool pair_ok(int kind, uint32_t mi, uint32_t mj) {
    if (kind == PAIR_RES) return !m_learnt(mj);
    if (kind == PAIR_SUBS) return m_orig(mj) && (m_molten(mi) != m_molten(mj));
    return m_orig(mj) && (!m_molten(mi) || !m_molten(mj));
}

// mergeProof (elimination.cuh:162-213): proof bytes of the resolvent of c1 and
// c2 on x, 0 for a tautology
PFG_D uint32_t merge_bytes(const EK& k, uint32_t x, uint32_t c1, uint32_t c2) {
    const ClsHdr h1 = k.hdr[c1], h2 = k.hdr[c2];
    const uint32_t* a = k.lits + h1.off;
    const uint32_t* b = k.lits + h2.off;
    const int n1 = (int)h1.size, n2 = (int)h2.size;
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

// The guard the counting loops add when proofs are on (resolve.cuh:66-70,
// elimination.cuh:445-447, function.cuh:233): more than ADDEDCLS_MAX unit
// resolvents or more than ADDEDPROOF_MAX proof bytes rule x out. true = ruled out.
PFG_D bool proof_guard(const EK& k, int kind, uint32_t x, uint32_t me, uint32_t other, uint32_t nE) {
    if (nE > ADDEDCLS_MAX) return true;
    const uint32_t* ml = OLp(k, me);
    const uint32_t* ot = OLp(k, other);
    const uint32_t ms = OLs(k, me), os = OLs(k, other);
    unsigned long long bytes = 0;
    for (uint32_t i = 0; i < ms; i++) {
        const uint32_t ci = ml[i];
        const uint32_t mi = META(k, ci);
        if (m_learnt(mi)) continue;
        for (uint32_t j = 0; j < os; j++) {
            const uint32_t cj = ot[j];
            if (!pair_ok(kind, mi, META(k, cj))) continue;
            bytes += merge_bytes(k, x, ci, cj);
        }
    }
    return bytes > ADDEDPROOF_MAX;
}

// countSubstituted / countCoreSubstituted: true = cannot substitute
PFG_D bool count_subst(const EK& k, int kind, uint32_t x, uint32_t nClsBefore, uint32_t me, uint32_t other,
                       uint32_t& nE, uint32_t& nC, uint32_t& nL) {
    const int rlimit = (int)k.ve_clause_max;
    const uint32_t* ml = OLp(k, me);
    const uint32_t* ot = OLp(k, other);
    const uint32_t ms = OLs(k, me), os = OLs(k, other);
    for (uint32_t i = 0; i < ms; i++) {
        const uint32_t ci = ml[i];
        const uint32_t mi = META(k, ci);
        if (m_learnt(mi)) continue;
        for (uint32_t j = 0; j < os; j++) {
            const uint32_t cj = ot[j];
            if (!pair_ok(kind, mi, META(k, cj))) continue;
            uint32_t u;
            const int rsize = merge_cnt(k, x, ci, cj, u);
            if (rsize == 1) nE++;
            else if (rsize) {
                if (++nC > nClsBefore || (rlimit && rsize > rlimit)) return true;
                nL += (uint32_t)rsize;
            }
        }
    }
    if (nC > ADDEDCLS_MAX || nL > ADDEDLITS_MAX) return true;
    if (k.ve_lbound_en) {
        const uint32_t before = count_lits_before(k, me) + count_lits_before(k, other);
        if (nL > before) return true;
    }
    if (k.proof && proof_guard(k, kind, x, me, other, nE)) return true;
    return false;
}

// countResolvents, unbounded (resolve.cuh:28-109): true = can resolve
PFG_D bool count_res_unbounded(const EK& k, uint32_t x, uint32_t me, uint32_t other, uint32_t& nE, uint32_t& nC,
                               uint32_t& nL) {
    const int rlimit = (int)k.ve_clause_max;
    const uint32_t* ml = OLp(k, me);
    const uint32_t* ot = OLp(k, other);
    const uint32_t ms = OLs(k, me), os = OLs(k, other);
    for (uint32_t i = 0; i < ms; i++) {
        const uint32_t ci = ml[i];
        if (m_learnt(META(k, ci))) continue;
        for (uint32_t j = 0; j < os; j++) {
            const uint32_t cj = ot[j];
            if (m_learnt(META(k, cj))) continue;
            uint32_t u;
            const int rsize = merge_cnt(k, x, ci, cj, u);
            if (rsize == 1) nE++;
            else if (rsize) {
                if (rlimit && rsize > rlimit) return false;
                ++nC;
                nL += (uint32_t)rsize;
            }
        }
    }
    if (nC > ADDEDCLS_MAX || nL > ADDEDLITS_MAX) return false;
    if (k.proof && proof_guard(k, PAIR_RES, x, me, other, nE)) return false;
    return true;
}

// countResolvents, bounded (resolve.cuh:111-198): true = can resolve
PFG_D bool count_res_bounded(const EK& k, uint32_t x, uint32_t nClsBefore, uint32_t me, uint32_t other,
                             uint32_t& nE, uint32_t& nC, uint32_t& nL) {
    nE = 0; nC = 0; nL = 0;
    const int rlimit = (int)k.ve_clause_max;
    const uint32_t* ml = OLp(k, me);
    const uint32_t* ot = OLp(k, other);
    const uint32_t ms = OLs(k, me), os = OLs(k, other);
    for (uint32_t i = 0; i < ms; i++) {
        const uint32_t ci = ml[i];
        if (m_learnt(META(k, ci))) continue;
        for (uint32_t j = 0; j < os; j++) {
            const uint32_t cj = ot[j];
            if (m_learnt(META(k, cj))) continue;
            uint32_t u;
            const int rsize = merge_cnt(k, x, ci, cj, u);
            if (rsize == 1) nE++;
            else if (rsize) {
                if (++nC > nClsBefore || (rlimit && rsize > rlimit)) return false;
                nL += (uint32_t)rsize;
            }
        }
    }
    if (nC > ADDEDCLS_MAX || nL > ADDEDLITS_MAX) return false;
    if (k.ve_lbound_en) {
        const uint32_t before = count_lits_before(k, me) + count_lits_before(k, other);
        if (nL > before) return false;
    }
    if (k.proof && proof_guard(k, PAIR_RES, x, me, other, nE)) return false;
    return true;
}

// ---- model stack (model.cuh:29-49) ----
PFG_D uint32_t org_lit(const EK& k, uint32_t lit) { return (k.vorg[ABSV(lit)] << 1) | SIGNL(lit); }

// ---- DRAT proof lines (proofutils.cuh:30-200) ----
// Reserves `words` line words in one block keyed (x, seq); nullptr on overflow.
PFG_D uint32_t* pf_reserve(const EK& k, uint32_t x, uint32_t seq, uint32_t words) {
    const unsigned long long s = atomicAdd(&k.dc->pf_words, (unsigned long long)words);
    const uint32_t b = atomicAdd(&k.dc->pf_blocks, 1u);
    if (s + words > k.pf_wcap || b >= k.pf_bcap) { atomicOr(&k.dc->err, ERR_PROOF_OVERFLOW); return nullptr; }
    k.pf_b[b] = make_ulonglong2(((unsigned long long)x << 32) | seq, s);
    return k.pf_w + s;
}

// one line: header (bit 31 = deletion, low bits = length), then the literals in
// original numbering (ORIGINIZELIT); returns the words written
PFG_D uint32_t pf_put(const EK& k, uint32_t* dst, bool del, const uint32_t* l, uint32_t n) {
    dst[0] = (del ? 0x80000000u : 0u) | n;
    for (uint32_t i = 0; i < n; i++) dst[1 + i] = org_lit(k, l[i]);
    return n + 1;
}

// saveProof over poss then negs after SUB of x (subsume.cuh:464-474,
// proofutils.cuh:180-200): strengthened clauses are added, subsumed ones deleted
PFG_D void proof_sub(const EK& k, uint32_t x, uint32_t p, uint32_t n) {
    uint32_t words = 0;
    for (int side = 0; side < 2; side++) {
        const uint32_t lit = side ? n : p;
        const uint32_t* ol = OLp(k, lit);
        for (uint32_t i = 0; i < OLs(k, lit); i++) {
            const ClsHdr h = k.hdr[ol[i]];
            words += (m_molten(h.meta) ? h.size + 1 : 0u) + (m_deleted(h.meta) ? h.size + 1 : 0u);
        }
    }
    if (!words) return;
    uint32_t* d = pf_reserve(k, x, 0, words);
    if (!d) return;
    for (int side = 0; side < 2; side++) {
        const uint32_t lit = side ? n : p;
        const uint32_t* ol = OLp(k, lit);
        for (uint32_t i = 0; i < OLs(k, lit); i++) {
            const ClsHdr h = k.hdr[ol[i]];
            if (m_molten(h.meta)) d += pf_put(k, d, false, k.lits + h.off, h.size);
            if (m_deleted(h.meta)) d += pf_put(k, d, true, k.lits + h.off, h.size);
        }
    }
}

// original clauses of `side` (witness literal first) followed by [w, 1]
PFG_D void save_side(const EK& k, uint32_t side, uint32_t witlit, uint32_t w) {
    const uint32_t* ol = OLp(k, side);
    const uint32_t n = OLs(k, side);
    unsigned long long words = 2;
    for (uint32_t i = 0; i < n; i++) {
        const ClsHdr h = k.hdr[ol[i]];
        if (m_orig(h.meta)) words += h.size + 1ull;
    }
    const unsigned long long base = stack_reserve(k, ABSV(w), words);
    if (base == ~0ull) return;
    uint32_t* s = k.stack + base;
    for (uint32_t i = 0; i < n; i++) {
        const ClsHdr h = k.hdr[ol[i]];
        if (!m_orig(h.meta)) continue;
        const uint32_t* l = k.lits + h.off;
        uint32_t wpos = 0;
        for (uint32_t t = 0; t < h.size; t++) {
            if (l[t] == witlit) wpos = t;
            s[t] = org_lit(k, l[t]);
        }
        if (wpos) { const uint32_t tmp = s[0]; s[0] = s[wpos]; s[wpos] = tmp; }
        s[h.size] = h.size;
        s += h.size + 1;
    }
    s[0] = org_lit(k, w);
    s[1] = 1;
}

PFG_D void save_resolved_orgs(const EK& k, uint32_t p, uint32_t n, uint32_t pOrgs, uint32_t nOrgs) {
    if (pOrgs > nOrgs) save_side(k, n, n, p);
    else save_side(k, p, p, n);
}

PFG_D void save_resolved_lists(const EK& k, uint32_t p, uint32_t n) {
    if (OLs(k, p) > OLs(k, n)) save_side(k, n, n, p);
    else save_side(k, p, p, n);
}

PFG_D void delete_list(const EK& k, uint32_t lit) {
    const uint32_t* ol = OLp(k, lit);
    const uint32_t n = OLs(k, lit);
    for (uint32_t i = 0; i < n; i++) SET_DELETED(k, ol[i]);
}

PFG_D void toblivion(const EK& k, uint32_t p, uint32_t n) {
    delete_list(k, p);
    delete_list(k, n);
    k.ot_size[p] = 0;
    k.ot_size[n] = 0;
}

// ---- gates ----
PFG_D int find_fanin(const EK& k, uint32_t gate_out, uint32_t* out, uint32_t& sig) {
    sig = 0;
    int nImps = 0;
    const uint32_t* ol = OLp(k, gate_out);
    const uint32_t n = OLs(k, gate_out);
    for (uint32_t i = 0; i < n; i++) {
        const uint32_t c = ol[i];
        const ClsHdr h = k.hdr[c];
        if (m_orig(h.meta) && h.size == 2) {
            const uint32_t* l = k.lits + h.off;
            const uint32_t imp = FLIPL(l[0] ^ l[1] ^ gate_out);
            out[nImps++] = imp;
            sig |= MAPHASH(imp);
            SET_MOLTEN(k, c, 1);
        }
    }
    return nImps;
}

// find_ao_gate (and.cuh:46-113)
PFG_D bool find_ao_gate(const EK& k, uint32_t dx, uint32_t fx, uint32_t nOrgCls, uint32_t* out, uint32_t& nE,
                        uint32_t& nC, uint32_t& nL) {
    const uint32_t* dl = OLp(k, dx);
    const uint32_t* fl = OLp(k, fx);
    const uint32_t fsz = OLs(k, fx);
    if (SIZE(k, dl[0]) > 2 || SIZE(k, fl[fsz - 1]) < 3) return false;
    uint32_t sig;
    int nImps = find_fanin(k, dx, out, sig);
    if (nImps > 1) {
        const uint32_t x = ABSV(dx);
        out[nImps++] = fx;
        sig |= MAPHASH(fx);
        sort_small(out, (uint32_t)nImps);
        for (uint32_t i = 0; i < fsz; i++) {
            const uint32_t c = fl[i];
            const ClsHdr h = k.hdr[c];
            if (m_orig(h.meta) && h.size == (uint32_t)nImps && SUBSIG(h.sig, sig) && is_equal(k, c, out, (uint32_t)nImps)) {
                SET_MOLTEN(k, c, 1);
                nE = 0; nC = 0; nL = 0;
                if (count_subst(k, PAIR_SUBS, x, nOrgCls, dx, fx, nE, nC, nL)) { SET_MOLTEN(k, c, 0); break; }
                return true;
            }
        }
    }
    freeze_binaries(k, dx);
    return false;
}

// fast_equality_check (ifthenelse.cuh:27-48). The reference searches the
// shortest of the three lists; every clause (x, y, z) holds x, the eliminated
// variable's literal, and equal clauses share their sort key, so the first
// match in x's own list is the same clause.
PFG_D uint32_t fast_equality_check(const EK& k, uint32_t x, uint32_t y, uint32_t z) {
    uint32_t t;
    const uint32_t lst = x;
    if (z < y) { t = y; y = z; z = t; }
    if (z < x) { t = x; x = z; z = t; }
    if (y < x) { t = x; x = y; y = t; }
    const uint32_t* ol = OLp(k, lst);
    const uint32_t n = OLs(k, lst);
    for (uint32_t i = 0; i < n; i++) {
        const ClsHdr h = k.hdr[ol[i]];
        if (m_molten(h.meta)) continue;
        if (m_orig(h.meta) && h.size == 3) {
            const uint32_t* l = k.lits + h.off;
            if (l[0] == x && l[1] == y && l[2] == z) return ol[i];
        }
    }
    return NOREF;
}

// find_ite_gate (ifthenelse.cuh:50-123)
PFG_D bool find_ite_gate(const EK& k, uint32_t dx, uint32_t fx, uint32_t nOrgCls, uint32_t& nE, uint32_t& nC,
                         uint32_t& nL) {
    const uint32_t* dl = OLp(k, dx);
    const uint32_t dsz = OLs(k, dx);
    if (SIZE(k, dl[dsz - 1]) == 2) return false;
    const uint32_t v = ABSV(dx);
    for (uint32_t i = 0; i < dsz; i++) {
        const uint32_t ci = dl[i];
        const ClsHdr hi = k.hdr[ci];
        if (!(m_orig(hi.meta) && hi.size == 3)) continue;
        const uint32_t* li = k.lits + hi.off;
        uint32_t xi = li[0], yi = li[1], zi = li[2], t;
        if (yi == dx) { t = xi; xi = yi; yi = t; }
        if (zi == dx) { t = xi; xi = zi; zi = t; }
        for (uint32_t j = i + 1; j < dsz; j++) {
            const uint32_t cj = dl[j];
            const ClsHdr hj = k.hdr[cj];
            if (!(m_orig(hj.meta) && hj.size == 3)) continue;
            const uint32_t* lj = k.lits + hj.off;
            uint32_t xj = lj[0], yj = lj[1], zj = lj[2];
            if (yj == dx) { t = xj; xj = yj; yj = t; }
            if (zj == dx) { t = xj; xj = zj; zj = t; }
            if (ABSV(yi) == ABSV(zj)) { t = yj; yj = zj; zj = t; }
            if (ABSV(zi) == ABSV(zj)) continue;
            if (yi != FLIPL(yj)) continue;
            const uint32_t r1 = fast_equality_check(k, fx, yi, FLIPL(zi));
            if (r1 == NOREF) continue;
            const uint32_t r2 = fast_equality_check(k, fx, yj, FLIPL(zj));
            if (r2 == NOREF) continue;
            SET_MOLTEN(k, ci, 1); SET_MOLTEN(k, cj, 1);
            SET_MOLTEN(k, r1, 1); SET_MOLTEN(k, r2, 1);
            nE = 0; nC = 0; nL = 0;
            if (count_subst(k, PAIR_SUBS, v, nOrgCls, dx, fx, nE, nC, nL)) {
                SET_MOLTEN(k, ci, 0); SET_MOLTEN(k, cj, 0);
                SET_MOLTEN(k, r1, 0); SET_MOLTEN(k, r2, 0);
                return false;
            }
            return true;
        }
    }
    return false;
}

PFG_D void freeze_arities(const EK& k, uint32_t me, uint32_t other) {
    for (int s = 0; s < 2; s++) {
        const uint32_t lit = s ? other : me;
        const uint32_t* ol = OLp(k, lit);
        const uint32_t n = OLs(k, lit);
        for (uint32_t i = 0; i < n; i++) {
            const ClsHdr h = k.hdr[ol[i]];
            if (h.size > 2 && m_molten(h.meta)) SET_MOLTEN(k, ol[i], 0);
        }
    }
}

PFG_D bool check_arity(const EK& k, const ClsHdr& h, const uint32_t* lits, uint32_t size) {
    const uint32_t* l = k.lits + h.off;
    for (uint32_t i = 0; i < h.size; i++) {
        uint32_t j;
        for (j = 0; j < size; j++) if (l[i] == lits[j]) break;
        if (j == size) return false;
    }
    return true;
}

// makeArity (xor.cuh:69-100). The flipped clause holds a literal of the
// eliminated variable v; it is looked up in that literal's own list (the
// reference takes the shortest list of the clause; the first match is the same).
PFG_D bool make_arity(const EK& k, uint32_t v, uint32_t& parity, uint32_t* lits, uint32_t size) {
    const uint32_t old = parity;
    do { parity++; } while (__popc(parity) & 1);
    for (uint32_t q = 0; q < size; q++) {
        const uint32_t bit = 1u << q;
        if ((parity & bit) != (old & bit)) lits[q] = FLIPL(lits[q]);
    }
    uint32_t best = lits[0];
    for (uint32_t q = 0; q < size; q++)
        if (ABSV(lits[q]) == v) best = lits[q];
    const uint32_t* ol = OLp(k, best);
    const uint32_t n = OLs(k, best);
    for (uint32_t i = 0; i < n; i++) {
        const ClsHdr h = k.hdr[ol[i]];
        if (m_orig(h.meta) && h.size == size && check_arity(k, h, lits, size)) { SET_MOLTEN(k, ol[i], 1); return true; }
    }
    return false;
}

// find_xor_gate (xor.cuh:102-178)
PFG_D bool find_xor_gate(const EK& k, uint32_t dx, uint32_t fx, uint32_t nOrgCls, uint32_t* out, uint32_t& nE,
                         uint32_t& nC, uint32_t& nL) {
    const uint32_t* dl = OLp(k, dx);
    const uint32_t* fl = OLp(k, fx);
    const uint32_t dsz = OLs(k, dx), fsz = OLs(k, fx);
    if (SIZE(k, dl[dsz - 1]) == 2 || SIZE(k, fl[fsz - 1]) == 2) return false;
    const int maxarity = (int)k.xor_max_arity;
    const int arity0 = (int)SIZE(k, dl[0]) - 1;
    if (arity0 > maxarity) return false;
    const uint32_t v = ABSV(dx);
    for (uint32_t i = 0; i < dsz; i++) {
        const uint32_t ci = dl[i];
        const ClsHdr h = k.hdr[ci];
        if (!m_orig(h.meta)) continue;
        const int size = (int)h.size, arity = size - 1;
        if (size < 3 || arity > maxarity) continue;
        const uint32_t* l = k.lits + h.off;
        for (int q = 0; q < size; q++) out[q] = l[q];
        uint32_t parity = 0;
        int itargets = 1 << arity;
        while (--itargets && make_arity(k, v, parity, out, (uint32_t)size)) {}
        if (itargets) freeze_arities(k, dx, fx);
        else {
            SET_MOLTEN(k, ci, 1);
            nE = 0; nC = 0; nL = 0;
            if (count_subst(k, PAIR_SUBS, v, nOrgCls, dx, fx, nE, nC, nL)) {
                freeze_arities(k, dx, fx);
                break;
            }
            return true;
        }
    }
    return false;
}

// ---- function tables (function.cuh) ----
constexpr int FUNTABLEN = 64;
constexpr uint32_t MAXFUNVAR = 12;
__constant__ uint64_t MAGIC[6] = {
    0xaaaaaaaaaaaaaaaaULL, 0xccccccccccccccccULL, 0xf0f0f0f0f0f0f0f0ULL,
    0xff00ff00ff00ff00ULL, 0xffff0000ffff0000ULL, 0xffffffff00000000ULL,
};

// ---- equivalences (equivalence.cuh) ----
PFG_D bool has_lit(const EK& k, uint32_t c, uint32_t lit) {
    const ClsHdr h = k.hdr[c];
    const uint32_t* l = k.lits + h.off;
    for (uint32_t i = 0; i < h.size; i++) if (l[i] == lit) return true;
    return false;
}

PFG_D void substitute_one(const EK& k, uint32_t dx, uint32_t def, uint32_t c, uint32_t& nUnits) {
    k.cnew[c] = 1;
    const ClsHdr h = k.hdr[c];
    uint32_t* l = k.lits + h.off;
    uint32_t j = 0;
    for (uint32_t i = 0; i < h.size; i++) {
        const uint32_t lit = l[i];
        if (lit == dx) l[j++] = def;
        else if (lit != def) l[j++] = lit;
    }
    k.hdr[c].size = j;
    if (j == 1) nUnits++;
    else { sort_small(l, j); calc_sig(k, c); }
}

PFG_D void substitute_single(const EK& k, uint32_t p, uint32_t n, uint32_t def) {
    const uint32_t def_f = FLIPL(def);
    uint32_t nNeg = 0, nPos = 0;
    const uint32_t* nl = OLp(k, n);
    const uint32_t ns = OLs(k, n);
    for (uint32_t i = 0; i < ns; i++) {
        const uint32_t c = nl[i];
        const uint32_t m = META(k, c);
        if (m_learnt(m) || m_molten(m) || has_lit(k, c, def)) SET_DELETED(k, c);
        else substitute_one(k, n, def_f, c, nNeg);
    }
    const uint32_t* pl = OLp(k, p);
    const uint32_t ps = OLs(k, p);
    for (uint32_t i = 0; i < ps; i++) {
        const uint32_t c = pl[i];
        const uint32_t m = META(k, c);
        if (m_learnt(m) || m_molten(m) || has_lit(k, c, def_f)) SET_DELETED(k, c);
        else substitute_one(k, p, def, c, nPos);
    }
    if (nPos || nNeg) {
        if (nNeg) append_units(k, n);
        if (nPos) append_units(k, p);
    }
    if (k.proof) {   // addProof over negs, then poss (equivalence.cuh:100-111)
        uint32_t words = 0;
        for (int side = 0; side < 2; side++) {
            const uint32_t lit = side ? p : n;
            const uint32_t* ol = OLp(k, lit);
            for (uint32_t i = 0; i < OLs(k, lit); i++) {
                const ClsHdr h = k.hdr[ol[i]];
                if (m_orig(h.meta)) words += h.size + 1;
            }
        }
        uint32_t* d = words ? pf_reserve(k, ABSV(p), 0, words) : nullptr;
        if (d) {
            for (int side = 0; side < 2; side++) {
                const uint32_t lit = side ? p : n;
                const uint32_t* ol = OLp(k, lit);
                for (uint32_t i = 0; i < OLs(k, lit); i++) {
                    const ClsHdr h = k.hdr[ol[i]];
                    if (m_orig(h.meta)) d += pf_put(k, d, false, k.lits + h.off, h.size);
                }
            }
        }
    }
}

PFG_D uint32_t find_sfanin(const EK& k, uint32_t gate_out) {
    uint32_t imp = 0;
    int nImps = 0;
    const uint32_t* ol = OLp(k, gate_out);
    const uint32_t n = OLs(k, gate_out);
    for (uint32_t i = 0; i < n; i++) {
        const uint32_t c = ol[i];
        const ClsHdr h = k.hdr[c];
        if (m_orig(h.meta) && h.size == 2) {
            const uint32_t* l = k.lits + h.off;
            imp = FLIPL(l[0] ^ l[1] ^ gate_out);
            SET_MOLTEN(k, c, 1);
            nImps++;
        }
        if (nImps > 1) return 0;
    }
    return imp;
}

PFG_D uint32_t find_equ_gate(const EK& k, uint32_t p, uint32_t n) {
    const uint32_t* pl = OLp(k, p);
    const uint32_t* nl = OLp(k, n);
    if (SIZE(k, pl[0]) > 2 || SIZE(k, nl[0]) > 2) return 0;
    uint32_t first = find_sfanin(k, p);
    if (first) {
        uint32_t second = n, def = first;
        if (second < def) { first = second; second = def; }
        const uint32_t ns = OLs(k, n);
        for (uint32_t i = 0; i < ns; i++) {
            const uint32_t c = nl[i];
            const ClsHdr h = k.hdr[c];
            const uint32_t* l = k.lits + h.off;
            if (m_orig(h.meta) && h.size == 2 && l[0] == first && l[1] == second) {
                SET_MOLTEN(k, c, 1);
                return def;
            }
        }
    }
    freeze_binaries(k, p);
    return 0;
}

// ---- SUB (subsume.cuh) ----
PFG_D bool sub_c(const EK& k, const ClsHdr& s, const ClsHdr& t) {
    const uint32_t* d1 = k.lits + s.off;
    const uint32_t* d2 = k.lits + t.off;
    uint32_t i = 0, j = 0, sub = 0;
    while (i < s.size && j < t.size) {
        if (d1[i] < d2[j]) i++;
        else if (d2[j] < d1[i]) j++;
        else { sub++; i++; j++; }
    }
    return sub == s.size;
}

PFG_D bool selfsub_c(const EK& k, uint32_t x, uint32_t fx, const ClsHdr& s, const ClsHdr& t) {
    const uint32_t* d1 = k.lits + s.off;
    const uint32_t* d2 = k.lits + t.off;
    uint32_t i = 0, j = 0, sub = 0;
    bool self = false;
    while (i < s.size && j < t.size) {
        const uint32_t l1 = d1[i], l2 = d2[j];
        if (l1 == fx) i++;
        else if (l2 == x) { self = true; j++; }
        else if (l1 < l2) i++;
        else if (l2 < l1) j++;
        else { sub++; i++; j++; }
    }
    if (sub + 1 == s.size) {
        if (self) return true;
        while (j < t.size) { if (d2[j] == x) return true; j++; }
    }
    return false;
}

PFG_D void strengthen(const EK& k, uint32_t c, uint32_t self) {
    ClsHdr h = k.hdr[c];
    uint32_t* l = k.lits + h.off;
    uint32_t j = 0;
    for (uint32_t i = 0; i < h.size; i++) if (l[i] != self) l[j++] = l[i];
    h.size--;
    k.hdr[c].size = h.size;
    if (h.size > 1) {
        calc_sig(k, c);
        if (m_learnt(h.meta)) {   // bumpShrunken (subsume.cuh:216-231)
            const int old_lbd = (int)m_lbd(h.meta);
            if (old_lbd > (int)LBD_TIER1) {
                const int sz1 = (int)h.size - 1;
                const int new_lbd = sz1 < old_lbd ? sz1 : old_lbd;
                if (new_lbd < old_lbd) {
                    const uint32_t m = k.hdr[c].meta;
                    k.hdr[c].meta = (m & 0xFu) | (USAGET3 << 4) | ((uint32_t)new_lbd << 6);
                }
            }
        }
    }
}

PFG_D void update_ol(const EK& k, uint32_t lit) {
    uint32_t* ol = OLp(k, lit);
    const uint32_t n = OLs(k, lit);
    uint32_t j = 0;
    for (uint32_t i = 0; i < n; i++) {
        const uint32_t c = ol[i];
        const uint32_t m = META(k, c);
        if (m_molten(m)) SET_MOLTEN(k, c, 0);
        else if (!m_deleted(m)) ol[j++] = c;
    }
    k.ot_size[lit] = j;
}

PFG_D void subsume_cand(const EK& k, uint32_t lit, uint32_t end, uint32_t cand) {
    const ClsHdr ch = k.hdr[cand];
    const uint32_t* ol = OLp(k, lit);
    for (uint32_t j = 0; j < end; j++) {
        const uint32_t sc = ol[j];
        const ClsHdr s = k.hdr[sc];
        if (m_deleted(s.meta)) continue;
        if (m_molten(ch.meta) && s.size > ch.size) continue;
        if (s.size > 1 && SUBSIG(s.sig, ch.sig) && sub_c(k, s, ch)) {
            if (m_learnt(s.meta) && m_orig(ch.meta)) k.hdr[sc].meta = m_set_st(s.meta, ST_ORIGINAL);
            SET_DELETED(k, cand);
            break;
        }
    }
}

PFG_D void self_subsume(const EK& k, uint32_t x, uint32_t fx, uint32_t lit, uint32_t cand, uint32_t& nUnits) {
    const ClsHdr ch = k.hdr[cand];
    const uint32_t* ol = OLp(k, lit);
    const uint32_t n = OLs(k, lit);
    for (uint32_t j = 0; j < n; j++) {
        const ClsHdr s = k.hdr[ol[j]];
        if (s.size > ch.size) break;
        if (m_deleted(s.meta) || m_molten(s.meta)) continue;
        if (s.size > 1 && selfsub_sig(s.sig, ch.sig) && selfsub_c(k, x, fx, s, ch)) {
            strengthen(k, cand, x);
            SET_MOLTEN(k, cand, 1);
            if (SIZE(k, cand) == 1) nUnits++;
            break;
        }
    }
}

// Thread-per-variable kernels below take an optional device-side index list
// (the variables the warp kernels could not stage); nelected bounds the grid.
PFG_D uint32_t list_count(const uint32_t* list, const uint32_t* count, uint32_t n) { return list ? *count : n; }

__global__ void sub_k(EK k, const uint32_t* elected, uint32_t nelected, const uint32_t* list, const uint32_t* count) {
    const uint32_t nn = list_count(list, count, nelected);
    for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < nn; q += gridDim.x * blockDim.x) {
        const uint32_t e = list ? list[q] : q;
        const uint32_t x = elected[e];
        const uint32_t p = 2 * x, n = p | 1;
        if (OLs(k, p) > k.sub_max_occurs || OLs(k, n) > k.sub_max_occurs) continue;
        uint32_t nPos = 0, nNeg = 0;
        const uint32_t* pl = OLp(k, p);
        const uint32_t ps = OLs(k, p);
        for (uint32_t i = 0; i < ps; i++) {
            const uint32_t c = pl[i];
            const ClsHdr h = k.hdr[c];
            if (h.size > SUB_MAX_CL_SIZE) break;
            if (m_deleted(h.meta)) continue;
            self_subsume(k, p, n, n, c, nPos);
            subsume_cand(k, p, i, c);
        }
        const uint32_t* nl = OLp(k, n);
        const uint32_t ns = OLs(k, n);
        for (uint32_t i = 0; i < ns; i++) {
            const uint32_t c = nl[i];
            const ClsHdr h = k.hdr[c];
            if (h.size > SUB_MAX_CL_SIZE) break;
            if (m_deleted(h.meta)) continue;
            self_subsume(k, n, p, p, c, nNeg);
            subsume_cand(k, n, i, c);
        }
        if (nPos || nNeg) {
            if (nPos) append_units(k, p);
            if (nNeg) append_units(k, n);
        }
        if (k.proof) proof_sub(k, x, p, n);
        update_ol(k, p);
        update_ol(k, n);
    }
}

// ---- BVE phase 1 ----
// Phase 1 runs in two kernels so that the rarely reached function-table gate
// (64-word truth tables) does not set the register budget of the common path:
// ve1a_k takes every decision up to that gate; variables that reach it are
// flagged and finished by ve1b_k with the same state (pOrgs, nOrgs, nC).

PFG_D void elim_no_resolvents(const EK& k, uint32_t x, uint32_t p, uint32_t n, uint32_t pOrgs, uint32_t nOrgs) {
    save_resolved_orgs(k, p, n, pOrgs, nOrgs);
    toblivion(k, p, n);
    k.elim[x] |= MELTING_MASK;
}

PFG_D void store_elim_info(uint32_t tid, uint32_t elimType, uint32_t nE, uint32_t nC, uint32_t nL, uint32_t* type,
                           uint32_t* ucnt, unsigned long long* rpos, unsigned long long* rref) {
    type[tid] = elimType | (nC << 2) | (nL << 16);
    ucnt[tid] = nE;
    rpos[tid] = nC;
    rref[tid] = nL + (unsigned long long)NBUCKETS * nC;
}

__global__ void __launch_bounds__(128) ve1a_k(EK k, const uint32_t* elected, uint32_t nelected, uint32_t* type,
                                              uint32_t* ucnt, unsigned long long* rpos, unsigned long long* rref,
                                              uint32_t* dlist, uint32_t* dcount, const uint32_t* list,
                                              const uint32_t* count) {
    uint32_t outs[SH_MAX_BVE_OUT1 + 2];
    const uint32_t nn = list_count(list, count, nelected);
    for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < nn; q += gridDim.x * blockDim.x) {
        const uint32_t tid = list ? list[q] : q;
        const uint32_t x = elected[tid];
        const uint32_t p = 2 * x, n = p | 1;
        uint32_t pOrgs = 0, nOrgs = 0;
        if (k.ve_inprocess) {
            const uint32_t* pl = OLp(k, p);
            const uint32_t* nl = OLp(k, n);
            for (uint32_t i = 0; i < OLs(k, p); i++) if (m_orig(META(k, pl[i]))) pOrgs++;
            for (uint32_t i = 0; i < OLs(k, n); i++) if (m_orig(META(k, nl[i]))) nOrgs++;
        } else {
            pOrgs = OLs(k, p);
            nOrgs = OLs(k, n);
        }
        uint32_t elimType = 0, nE = 0, nC = 0, nL = 0;
        type[tid] = 0; ucnt[tid] = 0; rpos[tid] = 0; rref[tid] = 0;
        if (!pOrgs || !nOrgs) { elim_no_resolvents(k, x, p, n, pOrgs, nOrgs); continue; }
        const uint32_t def = find_equ_gate(k, p, n);
        if (def) {
            save_resolved_orgs(k, p, n, pOrgs, nOrgs);
            substitute_single(k, p, n, def);
            k.elim[x] |= MELTING_MASK;
            continue;
        }
        if ((pOrgs == 1 || nOrgs == 1) && count_res_unbounded(k, x, p, n, nE, nC, nL)) {
            if (nC) store_elim_info(tid, RES_MASK, nE, nC, nL, type, ucnt, rpos, rref);
            else elim_no_resolvents(k, x, p, n, pOrgs, nOrgs);
            continue;
        }
        const uint32_t nClsBefore = pOrgs + nOrgs;
        elimType = 0; nE = 0; nC = 0; nL = 0;
        if (nClsBefore > 2) {
            if (nOrgs < SH_MAX_BVE_OUT1 && find_ao_gate(k, n, p, nClsBefore, outs, nE, nC, nL)) elimType = AOIX_MASK;
            else if (!nC && pOrgs < SH_MAX_BVE_OUT1 && find_ao_gate(k, p, n, nClsBefore, outs, nE, nC, nL)) elimType = AOIX_MASK;
        }
        if (!elimType && nClsBefore > 3) {
            if (find_ite_gate(k, p, n, nClsBefore, nE, nC, nL)) elimType = AOIX_MASK;
            else if (!nC && find_ite_gate(k, n, p, nClsBefore, nE, nC, nL)) elimType = AOIX_MASK;
            else if (find_xor_gate(k, p, n, nClsBefore, outs, nE, nC, nL)) elimType = AOIX_MASK;
            else if (!nC && find_xor_gate(k, n, p, nClsBefore, outs, nE, nC, nL)) elimType = AOIX_MASK;
        }
        if (vc_on(k, x) && !elimType && nClsBefore > 2) {
            // function-table stage (and what follows it) is finished by ve1b_k
            dlist[atomicAdd(dcount, 1u)] = tid;
            ucnt[tid] = nC;
            rpos[tid] = (unsigned long long)pOrgs | ((unsigned long long)nOrgs << 32);
            continue;
        }
        if (!elimType && !nC && count_res_bounded(k, x, nClsBefore, p, n, nE, nC, nL)) elimType = RES_MASK;
        if (!nC) elim_no_resolvents(k, x, p, n, pOrgs, nOrgs);
        else if (elimType) store_elim_info(tid, elimType, nE, nC, nL, type, ucnt, rpos, rref);
    }
}

// ---- function-table stage, one warp per deferred variable ----
// Lane l owns words 2l and 2l+1 of each 64-word truth table (function.cuh:27-115);
// list walks run redundantly on all lanes (broadcast loads), writes by lane 0.

struct WFun { uint64_t w0, w1; };

PFG_D void wf_set(WFun& f, uint64_t v) { f.w0 = v; f.w1 = v; }

// clause2fun for the lane's two words (function.cuh:91-114): variable v < 6 uses
// the magic constant; v >= 6 alternates all-ones/zero every 2^(v-6) words.
PFG_D void wf_clause2fun(uint32_t v, uint32_t sign, WFun& f, unsigned lane) {
    if (v < 6) {
        uint64_t val = MAGIC[v];
        if (sign) val = ~val;
        f.w0 |= val;
        f.w1 |= val;
    } else {
        const uint64_t base = sign ? ~0ULL : 0ULL;
        const uint32_t sh = v - 6;
        const uint32_t i0 = 2 * lane, i1 = 2 * lane + 1;
        f.w0 |= ((i0 >> sh) & 1u) ? ~base : base;
        f.w1 |= ((i1 >> sh) & 1u) ? ~base : base;
    }
}

PFG_D bool wf_build(const EK& k, uint32_t lit, WFun& f, unsigned lane) {
    wf_set(f, ~0ULL);
    const uint32_t* ol = OLp(k, lit);
    const uint32_t n = OLs(k, lit);
    for (uint32_t i = 0; i < n; i++) {
        const ClsHdr h = k.hdr[ol[i]];
        if (m_learnt(h.meta)) continue;
        WFun cls{0, 0};
        const uint32_t* l = k.lits + h.off;
        for (uint32_t t = 0; t < h.size; t++) {
            const uint32_t other = l[t];
            if (other == lit) continue;
            const uint32_t mvar = k.varcore[ABSV(other)];
            if (mvar >= MAXFUNVAR) return false;
            wf_clause2fun(mvar, SIGNL(other), cls, lane);
        }
        f.w0 &= cls.w0;
        f.w1 &= cls.w1;
    }
    return true;
}

// The core test of find_fun_gate for every original clause i of lit's list:
// `base` AND the functions of the non-learnt clauses before i; when that is
// all-false, clause i is not part of the gate and is melted. The reference
// rebuilds the prefix for every i; one running AND in list order gives the
// same prefixes (melting changes no clause's status).
PFG_D void wf_cores(const EK& k, uint32_t lit, const WFun& base, bool& core, unsigned lane) {
    const uint32_t* ol = OLp(k, lit);
    const uint32_t n = OLs(k, lit);
    WFun run;
    wf_set(run, ~0ULL);
    for (uint32_t i = 0; i < n; i++) {
        const ClsHdr h = k.hdr[ol[i]];
        if (m_orig(h.meta)) {
            const uint64_t w0 = base.w0 & run.w0, w1 = base.w1 & run.w1;
            const bool isfalse = __all_sync(0xFFFFFFFFu, (w0 | w1) == 0);
            if (isfalse) {
                if (lane == 0) SET_MOLTEN(k, ol[i], 1);   // non-gate clause
                core = true;
            }
        }
        if (!m_learnt(h.meta)) {
            WFun cls{0, 0};
            const uint32_t* l = k.lits + h.off;
            for (uint32_t t = 0; t < h.size; t++) {
                const uint32_t other = l[t];
                if (other == lit) continue;
                wf_clause2fun(k.varcore[ABSV(other)], SIGNL(other), cls, lane);
            }
            run.w0 &= cls.w0;
            run.w1 &= cls.w1;
        }
    }
    __syncwarp();
}

// find_fun_gate (function.cuh:275-325) for one warp
PFG_D bool wf_find_fun_gate(const EK& k, uint32_t p, uint32_t n, uint32_t nOrgCls, uint32_t& nE, uint32_t& nC,
                            uint32_t& nL, unsigned lane) {
    WFun pos, neg;
    if (!wf_build(k, p, pos, lane) || !wf_build(k, n, neg, lane)) return false;
    const bool nonzero = __any_sync(0xFFFFFFFFu, ((pos.w0 & neg.w0) | (pos.w1 & neg.w1)) != 0);
    if (nonzero) return false;
    bool core = false;
    wf_cores(k, p, neg, core, lane);
    WFun ones;
    wf_set(ones, ~0ULL);
    wf_cores(k, n, ones, core, lane);
    nE = 0; nC = 0; nL = 0;
    if (count_subst(k, PAIR_CORE, ABSV(p), nOrgCls, p, n, nE, nC, nL)) {
        __syncwarp();
        if (core && lane == 0) freeze_clauses(k, p, n);
        __syncwarp();
        return false;
    }
    return true;
}

__global__ void __launch_bounds__(128) ve1b_k(EK k, const uint32_t* elected, const uint32_t* dlist,
                                              const uint32_t* dcount, uint32_t* type, uint32_t* ucnt,
                                              unsigned long long* rpos, unsigned long long* rref) {
    const unsigned lane = threadIdx.x & 31u;
    const uint32_t nd = *dcount;
    for (uint32_t w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < nd; w += (gridDim.x * blockDim.x) >> 5) {
        const uint32_t tid = dlist[w];
        const uint32_t x = elected[tid];
        const uint32_t p = 2 * x, n = p | 1;
        uint32_t nC = ucnt[tid];
        const unsigned long long po = rpos[tid];
        const uint32_t pOrgs = (uint32_t)po, nOrgs = (uint32_t)(po >> 32);
        const uint32_t nClsBefore = pOrgs + nOrgs;
        uint32_t elimType = 0, nE = 0, nL = 0;
        if (wf_find_fun_gate(k, p, n, nClsBefore, nE, nC, nL, lane)) elimType = CORE_MASK;
        else if (!nC && count_res_bounded(k, x, nClsBefore, p, n, nE, nC, nL)) elimType = RES_MASK;
        __syncwarp();
        if (lane == 0) {
            ucnt[tid] = 0;
            rpos[tid] = 0;
            if (!nC) elim_no_resolvents(k, x, p, n, pOrgs, nOrgs);
            else if (elimType) store_elim_info(tid, elimType, nE, nC, nL, type, ucnt, rpos, rref);
        }
        __syncwarp();
    }
}

// ---- BVE phase 3 ----
// proof words of x's resolvent lines: one line per clause resolvent and per
// unit resolvent (emission may stop before the last units; the rest is padding)
PFG_D uint32_t pf_res_words(uint32_t xinfo, uint32_t units) {
    const uint32_t nC = (xinfo & 0xFFFCu) >> 2, nL = xinfo >> 16;
    return nL + nC + 2 * units;
}

__global__ void __launch_bounds__(128) ve3_k(EK k, const uint32_t* elected, uint32_t nelected, const uint32_t* type,
                                             const uint32_t* ucnt, const unsigned long long* rslot,
                                             const unsigned long long* rlit, const uint8_t* fits,
                                             const uint32_t* list, const uint32_t* count) {
    const uint32_t nn = list_count(list, count, nelected);
    for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < nn; q += gridDim.x * blockDim.x) {
        const uint32_t tid = list ? list[q] : q;
        const uint32_t x = elected[tid];
        const uint32_t xinfo = type[tid];
        const uint32_t et = xinfo & 3u;
        if (et) {
            const uint32_t p = 2 * x, n = p | 1;
            const uint32_t nAddedCls = (xinfo & 0xFFFCu) >> 2, nAddedLits = xinfo >> 16;
            (void)nAddedLits;
            if (fits[tid]) {
                save_resolved_lists(k, p, n);
                const int kind = et == RES_MASK ? PAIR_RES : (et == CORE_MASK ? PAIR_CORE : PAIR_SUBS);
                // resolvents go to physical slots rslot.. with literals packed from rlit
                unsigned long long slot = rslot[tid];
                unsigned long long woff = rlit[tid];
                const unsigned long long checksum = slot + nAddedCls;
                const uint32_t* ml = OLp(k, p);
                const uint32_t* ol = OLp(k, n);
                const uint32_t ms = OLs(k, p), os = OLs(k, n);
                const uint32_t pwords = k.proof ? pf_res_words(xinfo, ucnt[tid]) : 0u;
                uint32_t* pd = pwords ? pf_reserve(k, x, 0, pwords) : nullptr;
                uint32_t* const pend = pd ? pd + pwords : nullptr;
                for (uint32_t i = 0; i < ms && slot < checksum; i++) {
                    const uint32_t ci = ml[i];
                    const uint32_t mi = META(k, ci);
                    if (m_learnt(mi)) continue;
                    for (uint32_t j = 0; j < os && slot < checksum; j++) {
                        const uint32_t cj = ol[j];
                        const uint32_t mj = META(k, cj);
                        if (m_learnt(mj)) continue;
                        if (kind == PAIR_SUBS && m_molten(mi) == m_molten(mj)) continue;
                        if (kind == PAIR_CORE && m_molten(mi) && m_molten(mj)) continue;
                        uint32_t unit;
                        const int rsize = merge_cnt(k, x, ci, cj, unit);
                        if (!rsize) continue;
                        if (pd && pd + rsize + 1 > pend) { atomicOr(&k.dc->err, ERR_PROOF_OVERFLOW); pd = nullptr; }
                        if (rsize == 1) {
                            push_unit(k, unit);
                            if (pd) pd += pf_put(k, pd, false, &unit, 1);
                            continue;
                        }
                        uint32_t* out = k.lits + woff;
                        merge_out(k, x, ci, cj, out);
                        if (pd) pd += pf_put(k, pd, false, out, (uint32_t)rsize);
                        uint32_t sig = 0;
                        for (int q = 0; q < rsize; q++) sig |= MAPHASH(out[q]);
                        ClsHdr h;
                        h.off = (uint32_t)woff;
                        h.size = (uint32_t)rsize;
                        h.sig = sig;
                        h.meta = m_make(ST_ORIGINAL, 0, 1, 0, 0);
                        k.hdr[slot] = h;
                        k.cnew[slot] = 1;
                        slot++;
                        woff += (unsigned long long)rsize;
                    }
                }
                if (slot != checksum) atomicOr(&k.dc->err, ERR_SLOT_MISMATCH);
                if (pd) while (pd < pend) *pd++ = 0u;
                toblivion(k, p, n);
                k.elim[x] |= MELTING_MASK | ADDING_MASK;
            } else if (et != RES_MASK) {
                freeze_clauses(k, p, n);
            }
        }
    }
}

// ---- ERE (redundancy.cuh:27-175) ----
// The reference searches, for every resolvent r, the sorted occurrence list of
// r's rarest literal with 32 strided lanes, and every lane deletes the first
// clause on its positions that equals r and has a matching type. The clauses
// equal to r form one block of that list, ordered by id (they share the sort
// key), so lane j's first hit is the first matching clause at a block offset
// congruent to j modulo 32, wherever the block starts. The block is found
// through a hash table of the live clauses (by literal set) instead of a list
// scan, so the lists of other variables need no sorting.
constexpr uint32_t ERE_EMPTY = 0xFFFFFFFFu;

// A running combination of the literals, then the length, then MurmurHash3's
// 32-bit finalizer; computable while a resolvent is being merged.
PFG_D uint32_t hash_step(uint32_t h, uint32_t lit) { return h ^ (lit + 0x9E3779B9u + (h << 6) + (h >> 2)); }

PFG_D uint32_t hash_final(uint32_t h, uint32_t n) {
    h ^= n * 0x9E3779B9u;
    h ^= h >> 16;
    h *= 0x85EBCA6Bu;
    h ^= h >> 13;
    h *= 0xC2B2AE35u;
    h ^= h >> 16;
    return h;
}

PFG_D uint32_t cls_hash(const uint32_t* l, uint32_t n) {
    uint32_t h = 0;
    for (uint32_t i = 0; i < n; i++) h = hash_step(h, l[i]);
    return hash_final(h, n);
}

// length and hash of the resolvent of two clauses on x without writing it;
// 0 for a tautology (the merge order of merge_out, elimination.cuh:216-240)
PFG_D int merge_hash(const EK& k, uint32_t x, const ClsHdr& h1, const ClsHdr& h2, uint32_t& hash) {
    const uint32_t* a = k.lits + h1.off;
    const uint32_t* b = k.lits + h2.off;
    const int n1 = (int)h1.size, n2 = (int)h2.size;
    int i = 0, j = 0, len = 0;
    uint32_t h = 0;
    while (i < n1 && j < n2) {
        const uint32_t l1 = a[i], l2 = b[j], v1 = ABSV(l1), v2 = ABSV(l2);
        if (v1 == x) i++;
        else if (v2 == x) j++;
        else if ((l1 ^ l2) == 1u) return 0;
        else if (v1 < v2) { i++; h = hash_step(h, l1); len++; }
        else if (v2 < v1) { j++; h = hash_step(h, l2); len++; }
        else { i++; j++; h = hash_step(h, l1); len++; }
    }
    for (; i < n1; i++) if (ABSV(a[i]) != x) { h = hash_step(h, a[i]); len++; }
    for (; j < n2; j++) if (ABSV(b[j]) != x) { h = hash_step(h, b[j]); len++; }
    hash = hash_final(h, (uint32_t)len);
    return len;
}

// does clause c equal the resolvent of h1 and h2 on x (of length len)?
PFG_D bool merge_equals(const EK& k, uint32_t x, const ClsHdr& h1, const ClsHdr& h2, uint32_t c) {
    const uint32_t* a = k.lits + h1.off;
    const uint32_t* b = k.lits + h2.off;
    const uint32_t* d = CLp(k, c);
    const int n1 = (int)h1.size, n2 = (int)h2.size;
    int i = 0, j = 0, q = 0;
    while (i < n1 || j < n2) {
        uint32_t lit;
        if (i < n1 && ABSV(a[i]) == x) { i++; continue; }
        if (j < n2 && ABSV(b[j]) == x) { j++; continue; }
        if (i < n1 && j < n2) {
            const uint32_t l1 = a[i], l2 = b[j];
            if (ABSV(l1) < ABSV(l2)) { lit = l1; i++; }
            else if (ABSV(l2) < ABSV(l1)) { lit = l2; j++; }
            else { lit = l1; i++; j++; }
        } else if (i < n1) {
            lit = a[i++];
        } else {
            lit = b[j++];
        }
        if (d[q++] != lit) return false;
    }
    return true;
}

// A resolvent of an instance's variable can only equal a clause of that
// instance, so only the clauses of the instances running ERE this round
// (mode 2) go into the table.
__global__ void ere_table_k(const ClsHdr* __restrict__ hdr, const uint32_t* __restrict__ lits, uint64_t ncls,
                            const uint32_t* __restrict__ vinst, const uint8_t* __restrict__ mode, uint32_t* table,
                            uint32_t mask) {
    for (uint64_t c = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; c < ncls; c += (uint64_t)gridDim.x * blockDim.x) {
        const ClsHdr h = hdr[c];
        if (m_deleted(h.meta) || h.size < 2) continue;
        if (mode[vinst[ABSV(lits[h.off])]] != 2) continue;
        uint32_t s = cls_hash(lits + h.off, h.size) & mask;
        for (uint32_t q = 0; q <= mask; q++) {   // the table has room for every clause twice over
            if (atomicCAS(&table[s], ERE_EMPTY, (uint32_t)c) == ERE_EMPTY) break;
            s = (s + 1) & mask;
        }
    }
}

// smallest id above `after` (or any id when after < 0) of a clause equal to d[0..n)
PFG_D uint32_t ere_next_equal(const EK& k, const uint32_t* table, uint32_t mask, uint32_t s0, const uint32_t* d,
                              uint32_t n, int64_t after) {
    uint32_t best = ERE_EMPTY;
    uint32_t s = s0;
    for (uint32_t q = 0; q <= mask; q++) {
        const uint32_t id = table[s];
        if (id == ERE_EMPTY) break;
        if ((int64_t)id > after && id < best && SIZE(k, id) == n && is_equal(k, id, d, n)) best = id;
        s = (s + 1) & mask;
    }
    return best;
}

// one warp per elected variable. The lanes test 32 resolvents at a time for an
// equal clause in the table; lane 0 then walks, in pair order, the resolvents
// that have one, and for each the block of equal clauses in id order. (No
// clause of the variable equals one of its resolvents, and another elected
// variable's resolvents never contain it, so the pair tests cannot be changed
// by the deletions.)
__global__ void __launch_bounds__(128) ere_k(EK k, const uint32_t* elected, uint32_t nelected, const uint32_t* table,
                                             uint32_t mask) {
    __shared__ uint32_t bufs[4][SH_MAX_ERE_OUT + 8];
    const uint32_t wib = threadIdx.x >> 5;
    const unsigned lane = threadIdx.x & 31u;
    uint32_t* buf = bufs[wib];
    const uint32_t cmax = k.ere_clause_max;
    for (uint32_t q = blockIdx.x * 4 + wib; q < nelected; q += gridDim.x * 4) {
        const uint32_t v = elected[q], p = 2 * v, n = p | 1;
        uint32_t pseq = 0;   // proof lines of v, in deletion order
        const uint32_t ds = OLs(k, p), fs = OLs(k, n);
        if (!(ds && fs && ds <= k.ere_max_occurs && fs <= k.ere_max_occurs)) continue;
        const uint32_t* pl = OLp(k, p);
        const uint32_t* nl = OLp(k, n);
        if (!(SIZE(k, pl[0]) <= cmax && SIZE(k, nl[0]) <= cmax)) continue;
        const uint32_t total = ds * fs;
        for (uint32_t b0 = 0; b0 < total; b0 += 32) {
            const uint32_t pr = b0 + lane;
            bool hit = false;
            if (pr < total) {
                const uint32_t pc = pl[pr / fs], nc = nl[pr % fs];
                const ClsHdr ph = k.hdr[pc], nh = k.hdr[nc];
                if (!m_deleted(ph.meta) && !m_deleted(nh.meta) && ph.size + nh.size - 2 <= cmax) {
                    uint32_t hs;
                    const int mlen = merge_hash(k, v, ph, nh, hs);
                    if (mlen > 1) {
                        uint32_t s = hs & mask;
                        for (uint32_t t = 0; t <= mask && !hit; t++) {
                            const uint32_t id = table[s];
                            if (id == ERE_EMPTY) break;
                            hit = SIZE(k, id) == (uint32_t)mlen && merge_equals(k, v, ph, nh, id);
                            s = (s + 1) & mask;
                        }
                    }
                }
            }
            unsigned todo = __ballot_sync(0xFFFFFFFFu, hit);
            if (lane == 0) {
                for (; todo; todo &= todo - 1) {
                    const uint32_t r = b0 + (uint32_t)(__ffs(todo) - 1);
                    const uint32_t pc = pl[r / fs], nc = nl[r % fs];
                    const ClsHdr ph = k.hdr[pc], nh = k.hdr[nc];
                    const int mlen = merge_out(k, v, pc, nc, buf);
                    const uint32_t type = (m_learnt(ph.meta) || m_learnt(nh.meta)) ? ST_LEARNT : ST_ORIGINAL;
                    const uint32_t s0 = cls_hash(buf, (uint32_t)mlen) & mask;
                    uint32_t done = 0;        // strided lanes that already deleted a clause
                    int64_t after = -1;
                    for (uint32_t t = 0; done != 0xFFFFFFFFu; t++) {
                        const uint32_t c = ere_next_equal(k, table, mask, s0, buf, (uint32_t)mlen, after);
                        if (c == ERE_EMPTY) break;
                        after = c;
                        const uint32_t bit = 1u << (t & 31u);
                        if (done & bit) continue;
                        unsigned int* mp = (unsigned int*)&k.hdr[c].meta;
                        unsigned int old = *((volatile unsigned int*)mp);
                        if (!(m_learnt(old) || m_st(old) == type)) continue;
                        for (int it = 0; it < 8; it++) {
                            if (m_deleted(old)) break;
                            const unsigned int prev = atomicCAS(mp, old, m_set_st(old, ST_DELETED));
                            if (prev == old) {
                                done |= bit;
                                if (k.proof) {   // redundancy.cuh:122-128
                                    uint32_t* d = pf_reserve(k, v, pseq++, (uint32_t)mlen + 1);
                                    if (d) pf_put(k, d, true, buf, (uint32_t)mlen);
                                }
                                break;
                            }
                            old = prev;
                        }
                    }
                }
            }
            __syncwarp();
        }
    }
}

#include "elimw.cuh"

// ---- BCE (blocked.cuh:26-100): warp per surviving elected variable ----
// isTautology (elimination.cuh:119-138)
PFG_D bool clash_except(const EK& k, uint32_t x, const ClsHdr& h1, const ClsHdr& h2) {
    const uint32_t* a = k.lits + h1.off;
    const uint32_t* b = k.lits + h2.off;
    const int n1 = (int)h1.size, n2 = (int)h2.size;
    int i = 0, j = 0;
    while (i < n1 && j < n2) {
        const uint32_t l1 = a[i], l2 = b[j], v1 = ABSV(l1), v2 = ABSV(l2);
        if (v1 == x) i++;
        else if (v2 == x) j++;
        else if ((l1 ^ l2) == 1u) return true;
        else if (v1 < v2) i++;
        else if (v2 < v1) j++;
        else { i++; j++; }
    }
    return false;
}

// A lane per clause of -x (32 at a time): blocked when every non-learnt clause
// of x clashes with it on another variable. Blocked clauses are saved with
// witness -x in list order (one stack reservation per chunk) and deleted.
__global__ void __launch_bounds__(128) bce_k(EK k, const uint32_t* elected, uint32_t nelected, uint32_t maxoccurs) {
    const unsigned lane = threadIdx.x & 31u;
    for (uint32_t q = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; q < nelected; q += (gridDim.x * blockDim.x) >> 5) {
        const uint32_t x = elected[q];
        if (k.elim[x]) continue;                          // eliminated by BVE this round
        const uint32_t p = 2 * x, n = p | 1;
        const uint32_t ps = OLs(k, p), ns = OLs(k, n);
        if (ps > maxoccurs || ns > maxoccurs) continue;
        const uint32_t* pl = OLp(k, p);
        const uint32_t* nl = OLp(k, n);
        for (uint32_t b = 0; b < ns; b += 32) {
            const uint32_t i = b + lane;
            bool blocked = false;
            uint32_t ci = 0;
            ClsHdr hi{0, 0, 0, 0};
            if (i < ns) {
                ci = nl[i];
                hi = k.hdr[ci];
                if (!m_deleted(hi.meta) && !m_learnt(hi.meta)) {
                    blocked = true;
                    for (uint32_t j = 0; j < ps && blocked; j++) {
                        const ClsHdr hj = k.hdr[pl[j]];
                        if (m_deleted(hj.meta) || m_learnt(hj.meta)) continue;
                        if (!clash_except(k, x, hi, hj)) blocked = false;
                    }
                }
            }
            const uint32_t words = blocked ? hi.size + 1 : 0u;
            uint32_t total;
            const uint32_t ex = warp_excl_scan(words, lane, total);
            if (!total) continue;
            unsigned long long base = 0;
            uint32_t* pd = nullptr;
            if (lane == 0) {
                base = stack_reserve(k, x, total);
                if (k.proof) pd = pf_reserve(k, x, b, total);   // one 'd' line per blocked clause (blocked.cuh:67-72)
            }
            base = __shfl_sync(0xFFFFFFFFu, base, 0);
            pd = (uint32_t*)__shfl_sync(0xFFFFFFFFu, (unsigned long long)pd, 0);
            if (blocked && pd) pf_put(k, pd + ex, true, k.lits + hi.off, hi.size);
            if (blocked && base != ~0ull) {
                uint32_t* s = k.stack + base + ex;
                const uint32_t* l = k.lits + hi.off;
                uint32_t wpos = 0;
                for (uint32_t t = 0; t < hi.size; t++) {
                    if (l[t] == n) wpos = t;
                    s[t] = org_lit(k, l[t]);
                }
                if (wpos) { const uint32_t tmp = s[0]; s[0] = s[wpos]; s[wpos] = tmp; }
                s[hi.size] = hi.size;
                k.hdr[ci].meta = m_set_st(hi.meta, ST_DELETED);
            }
        }
    }
}


EK make_ek(Ctx& c) {
    EK k;
    k.hdr = c.hdr;
    k.lits = c.lits;
    k.ot_off = c.ot_off;
    k.ot_size = c.ot_size;
    k.ot_ids = c.ot_ids;
    k.elim = c.elim;
    k.varcore = c.varcore;
    k.fcut = c.fcut;
    k.vorg = c.vorg;
    k.vinst = c.vinst;
    k.vc_on = c.di.vc_on;
    k.units = c.units;
    k.ubase = c.di.ubase;
    k.ucap = c.di.ucap;
    k.ucount = c.dout.ucount;
    k.stack = c.stack;
    k.sbase = c.di.sbase;
    k.scap = c.di.scap;
    k.scount = c.dout.scount;
    k.dc = c.dc;
    k.ve_clause_max = c.o.ve_clause_max;
    k.xor_max_arity = c.o.xor_max_arity;
    k.sub_max_occurs = c.o.sub_max_occurs;
    k.ere_max_occurs = c.o.ere_max_occurs;
    k.ere_clause_max = c.o.ere_clause_max;
    k.ve_lbound_en = c.o.ve_lbound_en;
    k.ve_inprocess = c.o.ve_inprocess;
    k.proof = c.o.proof_en ? 1 : 0;
    k.pf_w = c.pf_w;
    k.pf_wcap = c.pf_wcap;
    k.pf_b = c.pf_b;
    k.pf_bcap = c.pf_bcap;
    k.lbyte = c.lbyte;
    k.cnew = c.cnew;
    return k;
}

// proof words BVE emission needs: the resolvent lines of every variable whose slots fit
__global__ void pf_need_k(const uint32_t* type, const uint32_t* ucnt, const uint8_t* fits, uint32_t E,
                          unsigned long long* need) {
    unsigned long long t = 0;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < E; i += gridDim.x * blockDim.x)
        if ((type[i] & 3u) && fits[i]) t += pf_res_words(type[i], ucnt[i]);
    for (int d = 16; d > 0; d >>= 1) t += __shfl_down_sync(0xFFFFFFFFu, t, d);
    if ((threadIdx.x & 31u) == 0 && t) atomicAdd(need, t);
}

// MEMORY_SAFE (bounded.cuh:279) per instance: gpos / gref are the exclusive
// scans of added clauses / buckets over the whole BVE set; an instance's own
// scan is the difference to its first entry, offset by its reference clause
// count and data size. Slots that fit get their physical size counted in
// cslot / clit (scanned next); the rest stay out of the store.
__global__ void ve_place_k(const uint32_t* veset, uint32_t E, const uint32_t* type,
                           const unsigned long long* gpos, const unsigned long long* gref, const uint32_t* vinst,
                           const uint32_t* seg, const unsigned long long* acc, uint8_t* fits,
                           unsigned long long* cslot, unsigned long long* clit) {
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < E; t += gridDim.x * blockDim.x) {
        const uint32_t xinfo = type[t];
        const uint32_t et = xinfo & 3u;
        const unsigned long long nC = (xinfo & 0xFFFCu) >> 2, nL = xinfo >> 16;
        bool ok = false;
        if (et) {
            const uint32_t i = vinst[veset[t]];
            const uint32_t s0 = seg[i];
            const unsigned long long* a = acc + 4 * (uint64_t)i;
            const unsigned long long vpos = a[0] + gpos[t] - gpos[s0];
            const unsigned long long vref = a[1] + gref[t] - gref[s0];
            ok = vpos + nC <= a[2] && vref + nL + (unsigned long long)NBUCKETS * nC <= a[3];
        }
        fits[t] = ok ? 1 : 0;
        cslot[t] = ok ? nC : 0ull;
        clit[t] = ok ? nL : 0ull;
    }
}

// clauses / literal words each instance added (differences of the physical scans)
__global__ void inst_add_k(const unsigned long long* cslot, const unsigned long long* clit, const uint32_t* seg,
                           uint32_t ninst, unsigned long long* add) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < ninst; i += gridDim.x * blockDim.x) {
        const uint32_t b = seg[i], e = seg[i + 1];
        add[2 * i] = e > b ? cslot[e] - cslot[b] : 0ull;
        add[2 * i + 1] = e > b ? clit[e] - clit[b] : 0ull;
    }
}

}  // namespace

// A persistent grid for a warp kernel: the blocks per SM the kernel's
// occupancy allows (or fewer, as the tuning asks) on every SM, no more blocks
// than the variables need.
template <typename Kern>
static unsigned blocks_per_sm(Kern kern, unsigned threads) {
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kern, (int)threads, 0) != cudaSuccess) {
        cudaGetLastError();
        nb = 1;
    }
    return (unsigned)std::max(1, nb);
}

static unsigned warp_grid(unsigned occ, uint32_t want, uint32_t nvars) {
    const uint64_t per_sm = want ? std::min<unsigned>(want, occ) : occ;
    const uint64_t need = ((uint64_t)nvars + WS_WARPS - 1) / WS_WARPS;
    return (unsigned)std::max<uint64_t>(1, std::min<uint64_t>(need, per_sm * sm_count()));
}

bool sub_pass(Ctx& c) {
    const uint32_t E = c.nve;
    if (!E) return true;
    if (c.o.proof_en && !proof_prepare(c, 2 * (c.lits_used + c.ncls))) return false;
    const EK k = make_ek(c);
    cudaMemsetAsync(&c.dc->nbig_sub, 0, sizeof(uint32_t), c.s);
    // warp per variable on the shared-memory stage; larger variables by one thread each
    static const unsigned sub_occ = blocks_per_sm(subw_k, WS_WARPS * 32);
    cudaMemsetAsync(&c.dc->steal[0], 0, sizeof(uint32_t), c.s);
    PFG_LAUNCH(K_SUB, subw_k, warp_grid(sub_occ, c.tune.sub_blocks_per_sm, E), WS_WARPS * 32, 0, c.s, k, c.veset, E, c.work_b, &c.dc->nbig_sub,
               &c.dc->steal[0]);
    PFG_LAUNCH(K_BIGVAR, sub_k, grid_for(E, 64, 8), 64, 0, c.s, k, c.veset, E, c.work_b, &c.dc->nbig_sub);
    return !c.o.proof_en || proof_collect(c);
}

bool ve_pass(Ctx& c) {
    const uint32_t E = c.nve;
    if (!E) return true;
    if (c.o.proof_en && !proof_prepare(c, 2 * (c.lits_used + c.ncls))) return false;
    const EK k = make_ek(c);
    bool any_vc = false;
    for (uint32_t i = 0; i < c.ninst; i++) any_vc |= c.ih[i].mode == 1 && c.ih[i].varcore_on;
    cudaMemsetAsync(&c.dc->nwork, 0, sizeof(uint32_t), c.s);
    cudaMemsetAsync(&c.dc->nbig_ve1, 0, 2 * sizeof(uint32_t), c.s);
    static const unsigned ve1_occ = blocks_per_sm(ve1w_k, WS_WARPS * 32);
    cudaMemsetAsync(&c.dc->steal[1], 0, sizeof(uint32_t), c.s);
    PFG_LAUNCH(K_VE1, ve1w_k, warp_grid(ve1_occ, c.tune.ve1_blocks_per_sm, E), WS_WARPS * 32, 0, c.s, k, c.veset, E, c.type, c.ucnt, c.rpos,
               c.rref, c.work, &c.dc->nwork, c.work_b, &c.dc->nbig_ve1, &c.dc->steal[1]);
    PFG_LAUNCH(K_BIGVAR, ve1a_k, grid_for(E, 128, 8), 128, 0, c.s, k, c.veset, E, c.type, c.ucnt, c.rpos, c.rref, c.work,
               &c.dc->nwork, c.work_b, &c.dc->nbig_ve1);
    if (any_vc)   // one warp per deferred variable; the grid walks the device-side count
        PFG_LAUNCH(K_VE1B, ve1b_k, grid_for((uint64_t)E * 32, 128, 16), 128, 0, c.s, k, c.veset, c.work,
                   &c.dc->nwork, c.type, c.ucnt, c.rpos, c.rref);
    if (c.o.proof_en && !proof_collect(c)) return false;   // substitution lines (ve_k_1)
    if (!ensure_tmp(c, scan_temp_bytes(E))) return false;
    // vePhase2 (elimination.cu:74-100) per instance, then physical placement
    exclusive_scan_u64(c.rpos, c.rpos, E, 0ull, nullptr, c.tmp, c.s);
    exclusive_scan_u64(c.rref, c.rref, E, 0ull, nullptr, c.tmp, c.s);
    PFG_LAUNCH(K_SCAN, ve_place_k, grid_for(E, 256), 256, 0, c.s, c.veset, E, c.type, c.rpos, c.rref, c.vinst,
               c.di.seg, c.di.acc, c.winv, c.rslot, c.rlit);
    exclusive_scan_u64(c.rslot, c.rslot, E, (unsigned long long)c.ncls, c.rslot + E, c.tmp, c.s);
    exclusive_scan_u64(c.rlit, c.rlit, E, (unsigned long long)c.lits_used, c.rlit + E, c.tmp, c.s);
    PFG_LAUNCH(K_SCAN, inst_add_k, grid_for(c.ninst, 256), 256, 0, c.s, c.rslot, c.rlit, c.di.seg, c.ninst,
               c.dout.add);
    cudaMemcpyAsync(&c.dc->ve_cls, c.rslot + E, sizeof(unsigned long long), cudaMemcpyDeviceToDevice, c.s);
    cudaMemcpyAsync(&c.dc->ve_lits, c.rlit + E, sizeof(unsigned long long), cudaMemcpyDeviceToDevice, c.s);
    EK k3 = k;
    if (c.o.proof_en) {   // room for the resolvent lines
        cudaMemsetAsync(&c.dc->pf_need, 0, sizeof(unsigned long long), c.s);
        PFG_LAUNCH(K_SCAN, pf_need_k, grid_for(E, 256), 256, 0, c.s, c.type, c.ucnt, c.winv, E, &c.dc->pf_need);
        sync_counters(c);
        if (!proof_prepare(c, c.hc->pf_need)) return false;
        k3 = make_ek(c);
    }
    static const unsigned ve3_occ = blocks_per_sm(ve3w_k, WS_WARPS * 32);
    cudaMemsetAsync(&c.dc->steal[2], 0, sizeof(uint32_t), c.s);
    PFG_LAUNCH(K_VE3, ve3w_k, warp_grid(ve3_occ, c.tune.ve3_blocks_per_sm, E), WS_WARPS * 32, 0, c.s, k3, c.veset, E,
               c.type, c.ucnt, c.rslot, c.rlit, c.winv, c.eligible_b, &c.dc->nbig_ve3, &c.dc->steal[2],
               c.tune.ve3_ticket ? c.tune.ve3_ticket : VE3_TICKET);
    PFG_LAUNCH(K_BIGVAR, ve3_k, grid_for(E, 128, 8), 128, 0, c.s, k3, c.veset, E, c.type, c.ucnt, c.rslot, c.rlit,
               c.winv, c.eligible_b, &c.dc->nbig_ve3);
    if (c.o.proof_en && !proof_collect(c)) return false;
    // resizeCNF_k (cnf.cu:55-80): the store ends after the last slot that fit
    pull_inst_out(c);
    if (!c.err.empty()) return false;
    c.ncls = c.hc->ve_cls;
    c.lits_used = c.hc->ve_lits;
    for (uint32_t i = 0; i < c.ninst; i++) {
        const unsigned long long ac = c.hout.add[2 * i], al = c.hout.add[2 * i + 1];
        unsigned long long* acc = c.hi.acc + 4 * i;
        acc[0] += ac;
        acc[1] += al + (unsigned long long)NBUCKETS * ac;
        c.ih[i].resolvents += ac;
    }
    push_inst_in(c);
    return cuda_ok(c, cudaGetLastError(), "ve");
}

bool bce_pass(Ctx& c) {
    if (!c.nve) return true;
    if (c.o.proof_en && !proof_prepare(c, 2 * (c.lits_used + c.ncls))) return false;
    PFG_LAUNCH(K_BCE, bce_k, grid_for((uint64_t)c.nve * 32, 128), 128, 0, c.s, make_ek(c), c.veset, c.nve,
               c.o.bce_max_occurs);
    return !c.o.proof_en || proof_collect(c);
}

bool ere_pass(Ctx& c) {
    if (!c.nere) return true;
    // hash table of the live clauses of the instances running ERE, at least
    // twice their number of slots
    uint64_t ncl = 0;
    for (uint32_t i = 0; i < c.ninst; i++)
        if (c.ih[i].mode == 2) ncl += c.ih[i].numClauses;
    uint64_t cap = 1024;
    while (cap < 2 * ncl + 2) cap <<= 1;
    if (cap > (1ull << 32)) { c.err = "ERE table exceeds 2^32 slots"; c.simpstate = PFG_OTALLOC_FAIL; return false; }
    uint32_t* table = nullptr;
    if (!dalloc_t(c, &table, cap)) { c.simpstate = PFG_OTALLOC_FAIL; return false; }
    const uint32_t mask = (uint32_t)(cap - 1);
    if (c.o.proof_en && !proof_prepare(c, 2 * (c.lits_used + c.ncls))) { dfree(c, table); return false; }
    cudaMemsetAsync(table, 0xFF, cap * sizeof(uint32_t), c.s);
    PFG_LAUNCH(K_ERE, ere_table_k, grid_for(c.ncls, 256), 256, 0, c.s, c.hdr, c.lits, c.ncls, c.vinst, c.di.mode,
               table, mask);
    PFG_LAUNCH(K_ERE, ere_k, grid_for((uint64_t)c.nere * 32, 128), 128, 0, c.s, make_ek(c), c.ereset, c.nere, table,
               mask);
    dfree(c, table);
    if (c.o.proof_en && !proof_collect(c)) return false;
    return cuda_ok(c, cudaGetLastError(), "ere");
}

}  // namespace pfg
