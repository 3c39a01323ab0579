/*
 * pfo.c - oracle for the GPU simplify path (TEST INFRASTRUCTURE ONLY).
 *
 * Sequential CPU restatement of one `Solver::simplify` call of ParaFROST's
 * GPU simplifier (src/gpu/simplify.cu:136-241). Every function cites the
 * reference code it restates. Only the test-suite, the smoke check and the
 * benchmark's CPU-baseline leg use this file; the engine under
 * parafrost_gb300/ never links it.
 *
 * Parity unpinned: the reference GPU simplifier cannot run here and the
 * reference has no golden vectors for this path (see pfo.h).
 *
 * Legal schedule chosen where the reference appends through atomics:
 *   - the elected array is ordered by (MIS round, rank)   [lcve.cu:193-208]
 *   - the frozen list is in ascending variable order       [lcve.cu:211-219]
 *   - an unsorted occurrence list is in clause order       [occurrence.cu:50-62]
 *   - kernels run their threads in ascending index order.
 * Per-variable work of one pass is independent (elected variables share no
 * clause), so the sequential loop reproduces every such schedule except for
 * the order of atomic appends, which the canonical form removes.
 */
#include "pfo.h"

#include <stdio.h>
#include <stdlib.h>
#include <string.h>

/* ---- constants (src/gpu/constants.hpp:49-82, constants.cuh:26-88) ---- */
#define ST_ORIGINAL 0u
#define ST_LEARNT   1u
#define ST_DELETED  2u
#define MELTING_MASK 0x01u
#define ADDING_MASK  0x02u
#define FORCED_MASK  0x04u
#define RES_MASK  1u
#define AOIX_MASK 2u
#define CORE_MASK 3u
#define ADDEDCLS_MAX  0x3FFFu
#define ADDEDLITS_MAX 0xFFFFu
#define NBUCKETS 3u              /* sizeof(SCLAUSE) / sizeof(uint32), sclause.cuh:208 */
#define SH_MAX_BVE_OUT1 250u     /* EXTSHMEM build (install.sh:409-415 on cc >= 7)    */
#define SH_MAX_ERE_OUT  250u
#define SUB_MAX_CL_SIZE 1000u
#define LBD_TIER1 2u
#define USAGET3 1u
#define MAX_LBD_M 0x03FFFFFFu
#define NOREF32 0xFFFFFFFFu
#define ERE_LANES 32u            /* blockDim.x of ere_k = warpSize (elimination.cu:201) */
#define ADDEDPROOF_MAX 0x3FFFFu  /* proof bytes one variable may add (constants.cuh:46)  */
#define PROOF_ADDED   97u        /* 'a' (constants.hpp:45)                              */
#define PROOF_DELETED 100u       /* 'd' (constants.hpp:46)                              */

#define ABSV(l) ((l) >> 1)
#define SIGNL(l) ((l) & 1u)
#define FLIPL(l) ((l) ^ 1u)
#define MAPHASH(l) (1u << ((l) & 31u))
#define SUBSIG(A, B) (!((A) & ~(B)))

typedef struct {
    uint64_t off;     /* first literal in ctx->lits            */
    uint32_t size;    /* current size                          */
    uint32_t sig;
    uint32_t lbd;
    uint8_t  st;      /* ORIGINAL / LEARNT / DELETED           */
    uint8_t  molten;
    uint8_t  added;
    uint8_t  usage;
} Cls;

typedef struct { uint32_t* d; uint64_t n, cap; } Vec;

static void vpush(Vec* v, uint32_t x) {
    if (v->n == v->cap) {
        v->cap = v->cap ? v->cap * 2 : 64;
        v->d = (uint32_t*)realloc(v->d, v->cap * sizeof(uint32_t));
    }
    v->d[v->n++] = x;
}

typedef struct {
    pfg_options o;
    uint32_t V;
    uint32_t* vorg;
    uint8_t* vstate;
    uint8_t* assumed;
    /* clause store (in reference ref order) */
    uint32_t* lits; uint64_t nlits, lits_cap;
    Cls* cls; uint64_t ncls, cls_cap;
    /* reference arena accounting (buckets of 4 bytes, memory.cu:360-419) */
    uint64_t data_size, data_cap, cs_cap;
    uint64_t orig_lits_stat;
    uint64_t numClauses, numLiterals;
    /* occurrence table */
    uint32_t* hist;            /* 2V+2 */
    uint64_t* ot_off;          /* 2V+3 */
    uint32_t* ot_size;         /* 2V+2 */
    uint32_t* ot_pool;
    uint64_t ot_pool_cap;
    /* per-variable */
    uint8_t* eliminated;       /* V+1 */
    uint32_t* elected; uint32_t nelected;
    uint32_t* varcore; int varcore_on;
    uint32_t* eligible;        /* V   */
    uint32_t* scores;          /* V+1 */
    uint32_t* rank;            /* V+1 */
    uint32_t* mstate;          /* V+1 */
    uint32_t* mround;          /* V+1 */
    uint8_t* frozen;           /* V+1 */
    uint8_t* win;              /* V+1 */
    /* BVE scratch per elected index */
    uint32_t* type; uint32_t* ucnt; uint64_t* rpos; uint64_t* rref;
    /* vectors */
    Vec units;                 /* vars->units (device)            */
    uint64_t nUnits;           /* vars->nUnits                    */
    Vec trail;                 /* units enqueued on the host       */
    Vec resolved;              /* model stack                      */
    Vec round_ends_v;
    uint64_t* round_ends; uint64_t nround_ends, round_ends_cap;
    pfo_round* rstats; uint64_t nrstats, rstats_cap;
    uint32_t mis_rounds;
    int phase, multiplier, simpstate, status, ere_ran;
    uint32_t* mbuf; uint64_t mcap;   /* resolvent scratch, grown to the longest merge */
    /* DRAT proof (proofutils.cuh): lines of the running pass, in chunks keyed by
       (variable << 32 | sequence); the pass's chunks are appended to the stream
       in key order */
    uint8_t* pbuf; uint64_t pn, pcap;
    uint64_t* pch; uint64_t npch, pchcap;   /* triples: key, start, length */
    uint64_t pkey, pstart;
    uint8_t* proof; uint64_t nproof, proofcap;
} Ctx;

static inline uint32_t* CL(Ctx* c, const Cls* k) { return c->lits + k->off; }
static inline int is_orig(const Cls* k) { return k->st == ST_ORIGINAL; }
static inline int is_learnt(const Cls* k) { return (k->st & ST_LEARNT) != 0; }
static inline int is_deleted(const Cls* k) { return (k->st & ST_DELETED) != 0; }

/* occurrence list view */
static inline uint32_t* OL(Ctx* c, uint32_t lit) { return c->ot_pool + c->ot_off[lit]; }
#define OLSZ(c, lit) ((c)->ot_size[lit])

static void* xcalloc(size_t n, size_t s) {
    void* p = calloc(n ? n : 1, s);
    if (!p) { fprintf(stderr, "pfo: out of memory\n"); abort(); }
    return p;
}

/* ---- primitives (src/gpu/primitives.cuh:34-190) ---- */
static inline uint32_t orgLit(Ctx* c, uint32_t lit) {      /* ORIGINIZELIT, primitives.cuh:34 */
    return (c->vorg[ABSV(lit)] << 1) | SIGNL(lit);
}

/* ---- DRAT proof bytes (proofutils.cuh:30-200, proof.cu:30-44) ----
   A line is the byte 'a' or 'd', then every literal of the clause in original
   numbering as 7-bit groups (low group first, high bit = more groups follow),
   then a zero byte. */
static uint32_t varint_len(uint32_t x) {             /* COUNTBYTES / BLUT (proof.cu:30-44) */
    uint32_t n = 1;
    while (x >= 0x80u) { x >>= 7; n++; }
    return n;
}

static void pf_grow(Ctx* c, uint64_t more) {
    if (c->pn + more <= c->pcap) return;
    while (c->pn + more > c->pcap) c->pcap = c->pcap ? 2 * c->pcap : 4096;
    c->pbuf = (uint8_t*)realloc(c->pbuf, c->pcap);
    if (!c->pbuf) { fprintf(stderr, "pfo: out of memory\n"); abort(); }
}

static void pf_open(Ctx* c, uint32_t x, uint32_t seq) {
    c->pkey = ((uint64_t)x << 32) | seq;
    c->pstart = c->pn;
}

static void pf_close(Ctx* c) {
    if (c->pn == c->pstart) return;
    if (c->npch + 3 > c->pchcap) {
        c->pchcap = c->pchcap ? 2 * c->pchcap : 768;
        c->pch = (uint64_t*)realloc(c->pch, c->pchcap * sizeof(uint64_t));
        if (!c->pch) { fprintf(stderr, "pfo: out of memory\n"); abort(); }
    }
    c->pch[c->npch++] = c->pkey;
    c->pch[c->npch++] = c->pstart;
    c->pch[c->npch++] = c->pn - c->pstart;
}

/* saveProofClause / saveProofUnit (proofutils.cuh:113-170) */
static void pf_line(Ctx* c, uint32_t state, const uint32_t* l, uint32_t n) {
    pf_grow(c, 2 + 5ull * n);
    c->pbuf[c->pn++] = (uint8_t)state;
    for (uint32_t i = 0; i < n; i++) {
        uint32_t v = (c->vorg[l[i] >> 1] << 1) | (l[i] & 1u);        /* ORIGINIZELIT */
        while (v >= 0x80u) { c->pbuf[c->pn++] = (uint8_t)((v & 0x7Fu) | 0x80u); v >>= 7; }
        c->pbuf[c->pn++] = (uint8_t)v;
    }
    c->pbuf[c->pn++] = 0;
}

static int pch_cmp(const void* pa, const void* pb) {
    const uint64_t a = *(const uint64_t*)pa, b = *(const uint64_t*)pb;
    return a < b ? -1 : (a > b ? 1 : 0);
}

/* end of a pass: its chunks join the stream ordered by (variable, sequence) */
static void pf_flush(Ctx* c) {
    if (!c->o.proof_en || !c->npch) { c->pn = 0; c->npch = 0; return; }
    qsort(c->pch, c->npch / 3, 3 * sizeof(uint64_t), pch_cmp);
    for (uint64_t i = 0; i < c->npch; i += 3) {
        const uint64_t st = c->pch[i + 1], len = c->pch[i + 2];
        if (c->nproof + len > c->proofcap) {
            while (c->nproof + len > c->proofcap) c->proofcap = c->proofcap ? 2 * c->proofcap : 4096;
            c->proof = (uint8_t*)realloc(c->proof, c->proofcap);
            if (!c->proof) { fprintf(stderr, "pfo: out of memory\n"); abort(); }
        }
        memcpy(c->proof + c->nproof, c->pbuf + st, len);
        c->nproof += len;
    }
    c->pn = 0;
    c->npch = 0;
}

static void sort_u32(uint32_t* d, uint32_t n) {             /* devSort result: ascending */
    for (uint32_t i = 1; i < n; i++) {
        uint32_t t = d[i], j = i;
        while (j > 0 && t < d[j - 1]) { d[j] = d[j - 1]; j--; }
        d[j] = t;
    }
}

static inline void calcSig(Ctx* c, Cls* k) {                /* calcSig(SCLAUSE&), primitives.cuh:177 */
    if (k->size <= 1) return;
    uint32_t s = 0; const uint32_t* l = CL(c, k);
    for (uint32_t i = 0; i < k->size; i++) s |= MAPHASH(l[i]);
    k->sig = s;
}

/* ---- clause store ---- */
static uint64_t push_lits(Ctx* c, const uint32_t* src, uint32_t n) {
    if (c->nlits + n > c->lits_cap) {
        uint64_t nc = c->lits_cap ? c->lits_cap : 1024;
        while (nc < c->nlits + n) nc *= 2;
        c->lits = (uint32_t*)realloc(c->lits, nc * sizeof(uint32_t));
        c->lits_cap = nc;
    }
    uint64_t off = c->nlits;
    if (src) memcpy(c->lits + off, src, n * sizeof(uint32_t));
    c->nlits += n;
    return off;
}

static Cls* push_cls(Ctx* c) {
    if (c->ncls == c->cls_cap) {
        c->cls_cap = c->cls_cap ? c->cls_cap * 2 : 1024;
        c->cls = (Cls*)realloc(c->cls, c->cls_cap * sizeof(Cls));
    }
    Cls* k = &c->cls[c->ncls++];
    memset(k, 0, sizeof(*k));
    return k;
}

/* countAll (count.cu:83-131,171): live = not DELETED */
static void countAll(Ctx* c, uint64_t* ncl, uint64_t* nli) {
    uint64_t a = 0, b = 0;
    for (uint64_t i = 0; i < c->ncls; i++)
        if (!is_deleted(&c->cls[i])) { a++; b += c->cls[i].size; }
    *ncl = a; *nli = b;
}

/* cuMM::resizeCNF with compaction (memory.cu:360-419, recycle.cu:60-103),
   called by Solver::reallocCNF(true) (cnf.cu:129-144) */
static void compactCNF(Ctx* c) {
    const uint64_t addCls = c->o.ve_en ? c->numClauses : 0;
    const uint64_t addLits = c->o.ve_en ? (uint64_t)((double)c->orig_lits_stat * c->o.lits_mul) : 0;
    const uint64_t clsCap = c->numClauses + addCls, litsCap = c->numLiterals + addLits;
    uint32_t* nl = (uint32_t*)xcalloc(c->numLiterals + 1, sizeof(uint32_t));
    Cls* nc = (Cls*)xcalloc(c->numClauses + 1, sizeof(Cls));
    uint64_t j = 0, lo = 0;
    for (uint64_t i = 0; i < c->ncls; i++) {
        Cls* k = &c->cls[i];
        if (is_deleted(k)) continue;
        nc[j] = *k;
        nc[j].off = lo;
        memcpy(nl + lo, CL(c, k), k->size * sizeof(uint32_t));
        lo += k->size;
        j++;
    }
    free(c->lits); free(c->cls);
    c->lits = nl; c->lits_cap = c->numLiterals + 1; c->nlits = lo;
    c->cls = nc; c->cls_cap = c->numClauses + 1; c->ncls = j;
    c->cs_cap = clsCap;
    c->data_cap = clsCap * NBUCKETS + litsCap;
    c->data_size = c->numClauses * NBUCKETS + c->numLiterals;
}

/* ---- occurrence table: histSimp + resizeOTAsync + create_ot_k
        (histogram.cu:54-71, memory.cu:421-466, occurrence.cu:50-62) ---- */
static void createOT(Ctx* c) {
    const uint64_t nl = 2ull * c->V + 2;
    memset(c->hist, 0, nl * sizeof(uint32_t));
    uint64_t total = 0;
    for (uint64_t i = 0; i < c->ncls; i++) {
        Cls* k = &c->cls[i];
        if (is_deleted(k)) continue;
        const uint32_t* l = CL(c, k);
        for (uint32_t j = 0; j < k->size; j++) c->hist[l[j]]++;
        total += k->size;
    }
    if (total > c->ot_pool_cap) {
        free(c->ot_pool);
        c->ot_pool = (uint32_t*)xcalloc(total, sizeof(uint32_t));
        c->ot_pool_cap = total;
    }
    uint64_t s = 0;
    for (uint64_t l = 0; l < nl; l++) { c->ot_off[l] = s; s += c->hist[l]; c->ot_size[l] = 0; }
    c->ot_off[nl] = s;
    /* legal schedule: insertion in clause order */
    for (uint64_t i = 0; i < c->ncls; i++) {
        Cls* k = &c->cls[i];
        if (is_deleted(k)) continue;
        const uint32_t* l = CL(c, k);
        for (uint32_t j = 0; j < k->size; j++) {
            const uint32_t lit = l[j];
            OL(c, lit)[c->ot_size[lit]++] = (uint32_t)i;
        }
    }
}

/* OLIST_CMP (key.cuh:67-85): (size, first, last, sig, ref) */
static Ctx* g_sort_ctx;
static int olist_cmp(const void* pa, const void* pb) {
    Ctx* c = g_sort_ctx;
    const uint32_t a = *(const uint32_t*)pa, b = *(const uint32_t*)pb;
    const Cls* x = &c->cls[a]; const Cls* y = &c->cls[b];
    if (x->size != y->size) return x->size < y->size ? -1 : 1;
    uint32_t xd = CL(c, x)[0], yd = CL(c, y)[0];
    if (xd != yd) return xd < yd ? -1 : 1;
    xd = CL(c, x)[x->size - 1]; yd = CL(c, y)[y->size - 1];
    if (xd != yd) return xd < yd ? -1 : 1;
    if (x->sig != y->sig) return x->sig < y->sig ? -1 : 1;
    return a < b ? -1 : (a > b ? 1 : 0);
}

/* Solver::sortOT (segsort.cu:37-47) */
static void sortOT(Ctx* c) {
    g_sort_ctx = c;
    const uint64_t nl = 2ull * c->V + 2;
    for (uint64_t l = 2; l < nl; l++)
        if (c->ot_size[l] > 1) qsort(OL(c, (uint32_t)l), c->ot_size[l], sizeof(uint32_t), olist_cmp);
}

/* ---- device BCP (Solver::prop, elimbcp.cu:43-215) ---- */
static inline int litval(const uint8_t* st, uint32_t lit) {   /* bcp_lit_val, elimbcp.cu:33 */
    const uint8_t s = st[ABSV(lit)];
    if (!s) return 0;
    const int sat = SIGNL(lit) ? (s == 2) : (s == 1);
    return sat ? 1 : 2;
}

static int prop(Ctx* c) {
    if (!c->nUnits) return 1;
    uint8_t* st = (uint8_t*)xcalloc(c->V + 1, 1);
    uint32_t* queue = (uint32_t*)xcalloc(c->V + 1, sizeof(uint32_t));
    uint64_t qh = 0, qt = 0;
    int conflict = 0;
    for (uint64_t i = 0; i < c->nUnits && !conflict; i++) {          /* bcp_seed_k */
        const uint32_t u = c->units.d[i], v = ABSV(u);
        const uint8_t desired = SIGNL(u) ? 2 : 1;
        if (!st[v]) { st[v] = desired; c->eliminated[v] |= FORCED_MASK; queue[qt++] = FLIPL(u); vpush(&c->trail, u); }
        else if (st[v] != desired) conflict = 1;
    }
    while (qh < qt && !conflict) {                                  /* bcp_propagate_k to fixpoint */
        const uint32_t f = queue[qh++];
        const uint32_t* ol = OL(c, f);
        for (uint32_t j = 0; j < OLSZ(c, f) && !conflict; j++) {
            const Cls* k = &c->cls[ol[j]];
            if (is_deleted(k)) continue;
            uint32_t unit = 0; int nunset = 0, sat = 0;
            const uint32_t* l = CL(c, k);
            for (uint32_t t = 0; t < k->size; t++) {
                const int ve = litval(st, l[t]);
                if (ve == 1) { sat = 1; break; }
                if (ve == 0) { unit = l[t]; if (++nunset > 1) break; }
            }
            if (sat) continue;
            if (!nunset) { conflict = 1; break; }
            if (nunset == 1) {
                const uint32_t v = ABSV(unit);
                const uint8_t desired = SIGNL(unit) ? 2 : 1;
                if (!st[v]) { st[v] = desired; c->eliminated[v] |= FORCED_MASK; queue[qt++] = FLIPL(unit); vpush(&c->trail, unit); }
                else if (st[v] != desired) conflict = 1;
            }
        }
    }
    if (conflict) { free(st); free(queue); return 0; }
    for (uint64_t i = 0; i < c->ncls; i++) {                         /* bcp_apply_k */
        Cls* k = &c->cls[i];
        if (is_deleted(k)) continue;
        uint32_t* l = CL(c, k);
        uint32_t sig = 0, n = 0; int sat = 0;
        for (uint32_t t = 0; t < k->size; t++) {
            const int ve = litval(st, l[t]);
            if (ve == 1) { sat = 1; break; }
            if (ve == 2) continue;
            l[n++] = l[t]; sig |= MAPHASH(l[t]);
        }
        if (sat) k->st = ST_DELETED;
        else { k->sig = sig; k->size = n; }
    }
    free(st); free(queue);
    countAll(c, &c->numClauses, &c->numLiterals);
    createOT(c);
    c->units.n = 0;
    c->nUnits = 0;
    return 1;
}

/* ---- LCVE (lcve.cu:221-417) ---- */
static Ctx* g_lcv_ctx;
static int lcv_cmp(const void* pa, const void* pb) {          /* GPU_LCV_CMP, key.cuh:33-42 */
    const uint32_t a = *(const uint32_t*)pa, b = *(const uint32_t*)pb;
    const uint32_t x = g_lcv_ctx->scores[a], y = g_lcv_ctx->scores[b];
    if (x != y) return x < y ? -1 : 1;
    return a < b ? -1 : (a > b ? 1 : 0);
}

#define MIS_NONE 0u
#define MIS_UNDECIDED 1u
#define MIS_ELECTED 2u
#define MIS_FROZEN 3u

static int mis_oversize(Ctx* c, uint32_t lit, int maxcsize) {  /* lcve.cu:102-110 */
    const uint32_t* ol = OL(c, lit);
    for (uint32_t i = 0; i < OLSZ(c, lit); i++) {
        const Cls* k = &c->cls[ol[i]];
        if (!is_deleted(k) && (int)k->size > maxcsize) return 1;
    }
    return 0;
}

static int mis_blocked(Ctx* c, uint32_t lit, uint32_t cand, uint32_t r) {  /* lcve.cu:112-125 */
    const uint32_t* ol = OL(c, lit);
    for (uint32_t i = 0; i < OLSZ(c, lit); i++) {
        const Cls* k = &c->cls[ol[i]];
        if (is_deleted(k)) continue;
        const uint32_t* l = CL(c, k);
        for (uint32_t t = 0; t < k->size; t++) {
            const uint32_t u = ABSV(l[t]);
            if (u != cand && c->mstate[u] == MIS_UNDECIDED && c->rank[u] < r) return 1;
        }
    }
    return 0;
}

static void mis_freeze(Ctx* c, uint32_t lit, uint32_t cand) {   /* lcve.cu:127-141 */
    const uint32_t* ol = OL(c, lit);
    for (uint32_t i = 0; i < OLSZ(c, lit); i++) {
        const Cls* k = &c->cls[ol[i]];
        if (is_deleted(k)) continue;
        const uint32_t* l = CL(c, k);
        for (uint32_t t = 0; t < k->size; t++) {
            const uint32_t u = ABSV(l[t]);
            if (u != cand) {
                c->frozen[u] = 1;
                if (c->mstate[u] == MIS_UNDECIDED) c->mstate[u] = MIS_FROZEN;
            }
        }
    }
}

/* depFreeze_d (lcve.cu:32-61) */
static int depFreeze(Ctx* c, uint32_t lit, uint32_t* flist, uint32_t* ftail, uint32_t cand, int maxcsize) {
    const uint32_t saved = *ftail;
    const uint32_t* ol = OL(c, lit);
    for (uint32_t i = 0; i < OLSZ(c, lit); i++) {
        const Cls* k = &c->cls[ol[i]];
        if (is_deleted(k)) continue;
        if ((int)k->size > maxcsize) {
            for (uint32_t q = saved; q < *ftail; q++) c->frozen[flist[q]] = 0;
            *ftail = saved;
            return 0;
        }
        const uint32_t* l = CL(c, k);
        for (uint32_t t = 0; t < k->size; t++) {
            const uint32_t v = ABSV(l[t]);
            if (!c->frozen[v] && v != cand) { c->frozen[v] = 1; flist[(*ftail)++] = v; }
        }
    }
    return 1;
}

static int LCVE(Ctx* c) {
    const uint32_t V = c->V;
    /* varReorder: assign_scores + thrust::sort with GPU_LCV_CMP (lcve.cu:221-299) */
    for (uint32_t v = 1; v <= V; v++) {
        c->eligible[v - 1] = v;
        c->scores[v] = c->hist[2 * v] * c->hist[2 * v + 1];       /* uint32 product */
    }
    g_lcv_ctx = c;
    qsort(c->eligible, V, sizeof(uint32_t), lcv_cmp);
    const uint32_t maxoccurs = c->o.lcve_max_occurs;
    const uint32_t pmax = c->o.mu_pos << c->multiplier;
    const uint32_t nmax = c->o.mu_neg << c->multiplier;
    const int maxcsize = c->o.lcve_clause_max;
    memset(c->frozen, 0, V + 1);   /* host vstate carries no frozen bits (solver.hpp:298) */
    c->nelected = 0;
    c->mis_rounds = 0;
    uint32_t* flist = (uint32_t*)xcalloc(V + 1, sizeof(uint32_t));
    uint32_t nfrozen = 0;
    if (c->o.lcve_fast) {
        /* mis_init_k (lcve.cu:143-169) */
        for (uint32_t ei = 0; ei < V; ei++) {
            const uint32_t v = c->eligible[ei];
            c->rank[v] = ei;
            uint32_t stt = MIS_NONE;
            if (!(c->vstate && c->vstate[v]) && !(c->assumed && c->assumed[v])) {
                const uint32_t p = 2 * v, n = p | 1;
                const uint32_t ps = c->hist[p], ns = c->hist[n];
                if ((ps || ns) && ps <= maxoccurs && ns <= maxoccurs && !(ps >= pmax && ns >= nmax)
                    && !mis_oversize(c, p, maxcsize) && !mis_oversize(c, n, maxcsize))
                    stt = MIS_UNDECIDED;
            }
            c->mstate[v] = stt;
        }
        /* rounds of mis_round_k + mis_freeze_k until none undecided (lcve.cu:171-209,353-363) */
        for (;;) {
            int rem = 0;
            for (uint32_t ei = 0; ei < V; ei++) {
                const uint32_t v = c->eligible[ei];
                if (c->mstate[v] == MIS_UNDECIDED) {
                    rem = 1;
                    c->win[v] = !(mis_blocked(c, 2 * v, v, ei) || mis_blocked(c, 2 * v + 1, v, ei));
                }
            }
            for (uint32_t ei = 0; ei < V; ei++) {
                const uint32_t v = c->eligible[ei];
                if (c->mstate[v] == MIS_UNDECIDED && c->win[v]) {
                    c->mstate[v] = MIS_ELECTED;
                    c->elected[c->nelected++] = v;
                    mis_freeze(c, 2 * v, v);
                    mis_freeze(c, 2 * v + 1, v);
                }
            }
            c->mis_rounds++;
            if (!rem) break;
        }
        /* mis_collect_k (lcve.cu:211-219): ascending variable order */
        for (uint32_t v = 1; v <= V; v++) if (c->frozen[v]) flist[nfrozen++] = v;
    } else {
        /* lcve_k (lcve.cu:63-98): sequential greedy with break at the thresholds */
        for (uint32_t ei = 0; ei < V; ei++) {
            const uint32_t cand = c->eligible[ei];
            if (c->frozen[cand]) continue;
            if (c->vstate && c->vstate[cand]) continue;
            if (c->assumed && c->assumed[cand]) continue;
            const uint32_t p = 2 * cand, n = p | 1;
            const uint32_t ps = c->hist[p], ns = c->hist[n];
            if (!ps && !ns) continue;
            if (ps > maxoccurs || ns > maxoccurs) break;
            if (ps >= pmax && ns >= nmax) break;
            if (depFreeze(c, p, flist, &nfrozen, cand, maxcsize) &&
                depFreeze(c, n, flist, &nfrozen, cand, maxcsize))
                c->elected[c->nelected++] = cand;
        }
    }
    /* mapFrozen (lcve.cu:398-417) */
    if (c->varcore_on) {
        if (!nfrozen) c->varcore_on = 0;      /* vars->varcore = NULL */
        else for (uint32_t i = 0; i < nfrozen; i++) c->varcore[flist[i]] = i;
    }
    free(flist);
    return c->nelected >= c->o.lcve_min_vars;
}

/* ---- elimination helpers (elimination.cuh) ---- */
static int selfsub_sig(uint32_t A, uint32_t B) {                 /* elimination.cuh:67 */
    const uint32_t Bt = B | ((B & 0xAAAAAAAAu) >> 1) | ((B & 0x55555555u) << 1);
    return !(A & ~Bt);
}

static void freezeBinaries(Ctx* c, uint32_t lit) {               /* elimination.cuh:73 */
    const uint32_t* ol = OL(c, lit);
    for (uint32_t i = 0; i < OLSZ(c, lit); i++) {
        Cls* k = &c->cls[ol[i]];
        if (is_orig(k) && k->size == 2) k->molten = 0;
    }
}

static void freezeClauses(Ctx* c, uint32_t p, uint32_t n) {      /* elimination.cuh:81 */
    uint32_t lits2[2] = {p, n};
    for (int s = 0; s < 2; s++) {
        const uint32_t* ol = OL(c, lits2[s]);
        for (uint32_t i = 0; i < OLSZ(c, lits2[s]); i++) {
            Cls* k = &c->cls[ol[i]];
            if (is_orig(k) && k->molten) k->molten = 0;
        }
    }
}

static void appendUnits(Ctx* c, uint32_t lit) {                   /* elimination.cuh:95 */
    const uint32_t* ol = OL(c, lit);
    for (uint32_t i = 0; i < OLSZ(c, lit); i++) {
        Cls* k = &c->cls[ol[i]];
        if (k->size == 1) vpush(&c->units, CL(c, k)[0]);
    }
}

static int isEqual(Ctx* c, Cls* k, const uint32_t* d, uint32_t n) {   /* elimination.cuh:56 */
    const uint32_t* l = CL(c, k);
    for (uint32_t i = 0; i < n; i++) if (l[i] != d[i]) return 0;
    return 1;
}

/* merge(x, c1, c2) counting version (elimination.cuh:214-240) */
static int merge_cnt(Ctx* c, uint32_t x, Cls* c1, Cls* c2) {
    const uint32_t* a = CL(c, c1); const uint32_t* b = CL(c, c2);
    const int n1 = (int)c1->size, n2 = (int)c2->size;
    int i = 0, j = 0, len = n1 + n2 - 2;
    while (i < n1 && j < n2) {
        const uint32_t l1 = a[i], l2 = b[j], v1 = ABSV(l1), v2 = ABSV(l2);
        if (v1 == x) i++;
        else if (v2 == x) j++;
        else if ((l1 ^ l2) == 1u) return 0;
        else if (v1 < v2) i++;
        else if (v2 < v1) j++;
        else { i++; j++; len--; }
    }
    return len;
}

/* merge(x, c1, c2, out_c) buffer version (elimination.cuh:302-331) */
static int merge_out(Ctx* c, uint32_t x, Cls* c1, Cls* c2, uint32_t* out) {
    const uint32_t* a = CL(c, c1); const uint32_t* b = CL(c, c2);
    const int n1 = (int)c1->size, n2 = (int)c2->size;
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

/* mergeProof (elimination.cuh:162-213): proof bytes of the resolvent of c1 and
   c2 on x (prefix + literals + terminator), 0 for a tautology */
static uint32_t merge_bytes(Ctx* c, uint32_t x, Cls* c1, Cls* c2) {
    const uint32_t* a = CL(c, c1); const uint32_t* b = CL(c, c2);
    const int n1 = (int)c1->size, n2 = (int)c2->size;
    int i = 0, j = 0;
    uint32_t bytes = 2;
    while (i < n1 && j < n2) {
        const uint32_t l1 = a[i], l2 = b[j], v1 = ABSV(l1), v2 = ABSV(l2);
        if (v1 == x) i++;
        else if (v2 == x) j++;
        else if ((l1 ^ l2) == 1u) return 0;
        else if (v1 < v2) { i++; bytes += varint_len(orgLit(c, l1)); }
        else if (v2 < v1) { j++; bytes += varint_len(orgLit(c, l2)); }
        else { i++; j++; bytes += varint_len(orgLit(c, l1)); }
    }
    while (i < n1) { const uint32_t l1 = a[i++]; if (ABSV(l1) != x) bytes += varint_len(orgLit(c, l1)); }
    while (j < n2) { const uint32_t l2 = b[j++]; if (ABSV(l2) != x) bytes += varint_len(orgLit(c, l2)); }
    return bytes;
}

static inline int pair_ok(int kind, Cls* ci, Cls* cj);

/* the guard the counting loops add when proofs are on (resolve.cuh:66-70,
   elimination.cuh:445-447, function.cuh:233): more than ADDEDCLS_MAX unit
   resolvents or more than ADDEDPROOF_MAX proof bytes rule the variable out;
   true = ruled out */
static int proof_guard(Ctx* c, int kind, uint32_t x, uint32_t me, uint32_t other, uint32_t nUnits) {
    if (nUnits > ADDEDCLS_MAX) return 1;
    uint64_t bytes = 0;
    const uint32_t* ml = OL(c, me); const uint32_t* ot = OL(c, other);
    for (uint32_t i = 0; i < OLSZ(c, me); i++) {
        Cls* ci = &c->cls[ml[i]];
        if (is_learnt(ci)) continue;
        for (uint32_t j = 0; j < OLSZ(c, other); j++) {
            Cls* cj = &c->cls[ot[j]];
            if (!pair_ok(kind, ci, cj)) continue;
            bytes += merge_bytes(c, x, ci, cj);
        }
    }
    return bytes > ADDEDPROOF_MAX;
}

static uint32_t countLitsBefore(Ctx* c, uint32_t lit) {           /* elimination.cuh:365 */
    uint32_t s = 0; const uint32_t* ol = OL(c, lit);
    for (uint32_t i = 0; i < OLSZ(c, lit); i++) {
        Cls* k = &c->cls[ol[i]];
        if (is_orig(k)) s += k->size;
    }
    return s;
}

/* pair filters of the three counting/emitting loops */
#define PAIR_RES  0   /* resolve: both non-learnt            (resolve.cuh, bounded.cuh:146) */
#define PAIR_SUBS 1   /* substitute: molten differ           (elimination.cuh:409, bounded.cuh:184) */
#define PAIR_CORE 2   /* core: not both molten               (function.cuh:196, bounded.cuh:223) */

static inline int pair_ok(int kind, Cls* ci, Cls* cj) {
    if (kind == PAIR_RES) return !is_learnt(cj);
    if (kind == PAIR_SUBS) return is_orig(cj) && (ci->molten != cj->molten);
    return is_orig(cj) && (!ci->molten || !cj->molten);
}

/* countSubstituted / countCoreSubstituted (elimination.cuh:409-484,
   function.cuh:196-273); return 1 = cannot be substituted */
static int countSubst(Ctx* c, int kind, uint32_t x, uint32_t nClsBefore, uint32_t me, uint32_t other,
                      uint32_t* nE, uint32_t* nC, uint32_t* nL) {
    const int rlimit = (int)c->o.ve_clause_max;
    const uint32_t* ml = OL(c, me); const uint32_t* ot = OL(c, other);
    for (uint32_t i = 0; i < OLSZ(c, me); i++) {
        Cls* ci = &c->cls[ml[i]];
        if (is_learnt(ci)) continue;
        for (uint32_t j = 0; j < OLSZ(c, other); j++) {
            Cls* cj = &c->cls[ot[j]];
            if (!pair_ok(kind, ci, cj)) continue;
            const int rsize = merge_cnt(c, x, ci, cj);
            if (rsize == 1) (*nE)++;
            else if (rsize) {
                if (++(*nC) > nClsBefore || (rlimit && rsize > rlimit)) return 1;
                *nL += (uint32_t)rsize;
            }
        }
    }
    if (*nC > ADDEDCLS_MAX || *nL > ADDEDLITS_MAX) return 1;
    if (c->o.ve_lbound_en) {
        const uint32_t before = countLitsBefore(c, me) + countLitsBefore(c, other);
        if (*nL > before) return 1;
    }
    if (c->o.proof_en && proof_guard(c, kind, x, me, other, *nE)) return 1;
    return 0;
}

/* countResolvents unbounded (resolve.cuh:28-109); return 1 = can resolve */
static int countResolventsU(Ctx* c, uint32_t x, uint32_t me, uint32_t other,
                            uint32_t* nE, uint32_t* nC, uint32_t* nL) {
    const int rlimit = (int)c->o.ve_clause_max;
    const uint32_t* ml = OL(c, me); const uint32_t* ot = OL(c, other);
    for (uint32_t i = 0; i < OLSZ(c, me); i++) {
        Cls* ci = &c->cls[ml[i]];
        if (is_learnt(ci)) continue;
        for (uint32_t j = 0; j < OLSZ(c, other); j++) {
            Cls* cj = &c->cls[ot[j]];
            if (is_learnt(cj)) continue;
            const int rsize = merge_cnt(c, x, ci, cj);
            if (rsize == 1) (*nE)++;
            else if (rsize) {
                if (rlimit && rsize > rlimit) return 0;
                ++(*nC);
                *nL += (uint32_t)rsize;
            }
        }
    }
    if (*nC > ADDEDCLS_MAX || *nL > ADDEDLITS_MAX) return 0;
    if (c->o.proof_en && proof_guard(c, PAIR_RES, x, me, other, *nE)) return 0;
    return 1;
}

/* countResolvents bounded (resolve.cuh:111-198); return 1 = can resolve */
static int countResolventsB(Ctx* c, uint32_t x, uint32_t nClsBefore, uint32_t me, uint32_t other,
                            uint32_t* nE, uint32_t* nC, uint32_t* nL) {
    *nE = 0; *nC = 0; *nL = 0;
    const int rlimit = (int)c->o.ve_clause_max;
    const uint32_t* ml = OL(c, me); const uint32_t* ot = OL(c, other);
    for (uint32_t i = 0; i < OLSZ(c, me); i++) {
        Cls* ci = &c->cls[ml[i]];
        if (is_learnt(ci)) continue;
        for (uint32_t j = 0; j < OLSZ(c, other); j++) {
            Cls* cj = &c->cls[ot[j]];
            if (is_learnt(cj)) continue;
            const int rsize = merge_cnt(c, x, ci, cj);
            if (rsize == 1) (*nE)++;
            else if (rsize) {
                if (++(*nC) > nClsBefore || (rlimit && rsize > rlimit)) return 0;
                *nL += (uint32_t)rsize;
            }
        }
    }
    if (*nC > ADDEDCLS_MAX || *nL > ADDEDLITS_MAX) return 0;
    if (c->o.ve_lbound_en) {
        const uint32_t before = countLitsBefore(c, me) + countLitsBefore(c, other);
        if (*nL > before) return 0;
    }
    if (c->o.proof_en && proof_guard(c, PAIR_RES, x, me, other, *nE)) return 0;
    return 1;
}

/* ---- model stack (model.cuh:29-49, elimination.cuh:486-641) ---- */
static void saveClause(Ctx* c, Cls* k, uint32_t witlit) {
    const uint64_t first = c->resolved.n;
    uint64_t wpos = first;
    const uint32_t* l = CL(c, k);
    for (uint32_t i = 0; i < k->size; i++) {
        if (l[i] == witlit) wpos = c->resolved.n;
        vpush(&c->resolved, orgLit(c, l[i]));
    }
    if (wpos != first) {
        const uint32_t t = c->resolved.d[first];
        c->resolved.d[first] = c->resolved.d[wpos];
        c->resolved.d[wpos] = t;
    }
    vpush(&c->resolved, k->size);
}

static void saveWitness(Ctx* c, uint32_t w) {
    vpush(&c->resolved, orgLit(c, w));
    vpush(&c->resolved, 1);
}

/* saves the original clauses of `side` (containing `witlit`) then witness `w` */
static void saveSide(Ctx* c, uint32_t side, uint32_t witlit, uint32_t w) {
    const uint32_t* ol = OL(c, side);
    for (uint32_t i = 0; i < OLSZ(c, side); i++) {
        Cls* k = &c->cls[ol[i]];
        if (is_orig(k)) saveClause(c, k, witlit);
    }
    saveWitness(c, w);
}

/* saveResolved(p, n, pOrgs, nOrgs, ...) (elimination.cuh:596-641) */
static void saveResolvedOrgs(Ctx* c, uint32_t p, uint32_t n, uint32_t pOrgs, uint32_t nOrgs) {
    if (pOrgs > nOrgs) saveSide(c, n, n, p);
    else saveSide(c, p, p, n);
}

/* saveResolved(p, n, cnf, poss, negs) list-size version (elimination.cuh:551-594) */
static void saveResolvedLists(Ctx* c, uint32_t p, uint32_t n) {
    if (OLSZ(c, p) > OLSZ(c, n)) saveSide(c, n, n, p);
    else saveSide(c, p, p, n);
}

static void deleteList(Ctx* c, uint32_t lit) {
    const uint32_t* ol = OL(c, lit);
    for (uint32_t i = 0; i < OLSZ(c, lit); i++) c->cls[ol[i]].st = ST_DELETED;
}

/* toblivion with model saving (elimination.cuh:486-538) */
static void toblivionSave(Ctx* c, uint32_t p, uint32_t n, uint32_t pOrgs, uint32_t nOrgs) {
    saveResolvedOrgs(c, p, n, pOrgs, nOrgs);
    deleteList(c, p); deleteList(c, n);
    OLSZ(c, p) = 0; OLSZ(c, n) = 0;
}

/* toblivion(cnf, poss, negs) (elimination.cuh:540-549) */
static void toblivion(Ctx* c, uint32_t p, uint32_t n) {
    deleteList(c, p); deleteList(c, n);
    OLSZ(c, p) = 0; OLSZ(c, n) = 0;
}

/* ---- gate detection ---- */
/* find_fanin (and.cuh:27-44) */
static int find_fanin(Ctx* c, uint32_t gate_out, uint32_t lit, uint32_t* out, uint32_t* sig) {
    *sig = 0; int nImps = 0;
    const uint32_t* ol = OL(c, lit);
    for (uint32_t i = 0; i < OLSZ(c, lit); i++) {
        Cls* k = &c->cls[ol[i]];
        if (is_orig(k) && k->size == 2) {
            const uint32_t* l = CL(c, k);
            const uint32_t imp = FLIPL(l[0] ^ l[1] ^ gate_out);
            out[nImps++] = imp;
            *sig |= MAPHASH(imp);
            k->molten = 1;
        }
    }
    return nImps;
}

/* find_ao_gate (and.cuh:46-113) */
static int find_ao_gate(Ctx* c, uint32_t dx, uint32_t fx, uint32_t nOrgCls, uint32_t* out,
                        uint32_t* nE, uint32_t* nC, uint32_t* nL) {
    const uint32_t* dl = OL(c, dx); const uint32_t* fl = OL(c, fx);
    if (c->cls[dl[0]].size > 2 || c->cls[fl[OLSZ(c, fx) - 1]].size < 3) return 0;
    uint32_t sig;
    int nImps = find_fanin(c, dx, dx, out, &sig);
    if (nImps > 1) {
        const uint32_t x = ABSV(dx);
        out[nImps++] = fx;
        sig |= MAPHASH(fx);
        sort_u32(out, (uint32_t)nImps);
        for (uint32_t i = 0; i < OLSZ(c, fx); i++) {
            Cls* k = &c->cls[fl[i]];
            if (is_orig(k) && k->size == (uint32_t)nImps && SUBSIG(k->sig, sig) && isEqual(c, k, out, (uint32_t)nImps)) {
                k->molten = 1;
                *nE = 0; *nC = 0; *nL = 0;
                if (countSubst(c, PAIR_SUBS, x, nOrgCls, dx, fx, nE, nC, nL)) { k->molten = 0; break; }
                return 1;
            }
        }
    }
    freezeBinaries(c, dx);
    return 0;
}

/* fast_equality_check (ifthenelse.cuh:27-48) */
static uint32_t fast_equality_check(Ctx* c, uint32_t x, uint32_t y, uint32_t z) {
    uint32_t t;
    if (OLSZ(c, y) > OLSZ(c, z)) { t = y; y = z; z = t; }
    if (OLSZ(c, x) > OLSZ(c, y)) { t = x; x = y; y = t; }
    const uint32_t lst = x;
    /* sort3 (primitives.cuh:50-56) */
    if (z < y) { t = y; y = z; z = t; }
    if (z < x) { t = x; x = z; z = t; }
    if (y < x) { t = x; x = y; y = t; }
    const uint32_t* ol = OL(c, lst);
    for (uint32_t i = 0; i < OLSZ(c, lst); i++) {
        Cls* k = &c->cls[ol[i]];
        if (k->molten) continue;
        const uint32_t* l = CL(c, k);
        if (is_orig(k) && k->size == 3 && l[0] == x && l[1] == y && l[2] == z) return ol[i];
    }
    return NOREF32;
}

/* find_ite_gate (ifthenelse.cuh:50-123) */
static int find_ite_gate(Ctx* c, uint32_t dx, uint32_t fx, uint32_t nOrgCls,
                         uint32_t* nE, uint32_t* nC, uint32_t* nL) {
    const uint32_t* dl = OL(c, dx);
    const uint32_t dsz = OLSZ(c, dx);
    if (c->cls[dl[dsz - 1]].size == 2) return 0;
    const uint32_t v = ABSV(dx);
    for (uint32_t i = 0; i < dsz; i++) {
        Cls* ci = &c->cls[dl[i]];
        if (!(is_orig(ci) && ci->size == 3)) continue;
        const uint32_t* li = CL(c, ci);
        uint32_t xi = li[0], yi = li[1], zi = li[2], t;
        if (yi == dx) { t = xi; xi = yi; yi = t; }
        if (zi == dx) { t = xi; xi = zi; zi = t; }
        for (uint32_t j = i + 1; j < dsz; j++) {
            Cls* cj = &c->cls[dl[j]];
            if (!(is_orig(cj) && cj->size == 3)) continue;
            const uint32_t* lj = CL(c, cj);
            uint32_t xj = lj[0], yj = lj[1], zj = lj[2];
            if (yj == dx) { t = xj; xj = yj; yj = t; }
            if (zj == dx) { t = xj; xj = zj; zj = t; }
            if (ABSV(yi) == ABSV(zj)) { t = yj; yj = zj; zj = t; }
            if (ABSV(zi) == ABSV(zj)) continue;
            if (yi != FLIPL(yj)) continue;
            const uint32_t r1 = fast_equality_check(c, fx, yi, FLIPL(zi));
            if (r1 == NOREF32) continue;
            const uint32_t r2 = fast_equality_check(c, fx, yj, FLIPL(zj));
            if (r2 == NOREF32) continue;
            ci->molten = 1; cj->molten = 1;
            c->cls[r1].molten = 1; c->cls[r2].molten = 1;
            *nE = 0; *nC = 0; *nL = 0;
            if (countSubst(c, PAIR_SUBS, v, nOrgCls, dx, fx, nE, nC, nL)) {
                ci->molten = 0; cj->molten = 0;
                c->cls[r1].molten = 0; c->cls[r2].molten = 0;
                return 0;
            }
            return 1;
        }
    }
    return 0;
}

/* freeze_arities (xor.cuh:36-50) */
static void freeze_arities(Ctx* c, uint32_t me, uint32_t other) {
    uint32_t l2[2] = {me, other};
    for (int s = 0; s < 2; s++) {
        const uint32_t* ol = OL(c, l2[s]);
        for (uint32_t i = 0; i < OLSZ(c, l2[s]); i++) {
            Cls* k = &c->cls[ol[i]];
            if (k->size > 2 && k->molten) k->molten = 0;
        }
    }
}

/* checkArity (xor.cuh:52-67) */
static int checkArity(Ctx* c, Cls* k, const uint32_t* lits, uint32_t size) {
    const uint32_t* l = CL(c, k);
    for (uint32_t i = 0; i < k->size; i++) {
        uint32_t j;
        for (j = 0; j < size; j++) if (l[i] == lits[j]) break;
        if (j == size) return 0;
    }
    return 1;
}

/* makeArity (xor.cuh:69-100) */
static int makeArity(Ctx* c, uint32_t* parity, uint32_t* lits, uint32_t size) {
    const uint32_t old = *parity;
    do { (*parity)++; } while (__builtin_popcount(*parity) & 1);   /* COUNTFLIPS */
    for (uint32_t k = 0; k < size; k++) {
        const uint32_t bit = 1u << k;
        if ((*parity & bit) != (old & bit)) lits[k] = FLIPL(lits[k]);
    }
    uint32_t best = lits[0];
    uint32_t minsize = OLSZ(c, best);
    for (uint32_t k = 1; k < size; k++) {
        const uint32_t ls = OLSZ(c, lits[k]);
        if (ls < minsize) { minsize = ls; best = lits[k]; }
    }
    const uint32_t* ol = OL(c, best);
    for (uint32_t i = 0; i < OLSZ(c, best); i++) {
        Cls* k = &c->cls[ol[i]];
        if (is_orig(k) && k->size == size && checkArity(c, k, lits, size)) { k->molten = 1; return 1; }
    }
    return 0;
}

/* find_xor_gate (xor.cuh:102-178) */
static int find_xor_gate(Ctx* c, uint32_t dx, uint32_t fx, uint32_t nOrgCls, uint32_t* out,
                         uint32_t* nE, uint32_t* nC, uint32_t* nL) {
    const uint32_t* dl = OL(c, dx); const uint32_t* fl = OL(c, fx);
    const uint32_t dsz = OLSZ(c, dx), fsz = OLSZ(c, fx);
    if (c->cls[dl[dsz - 1]].size == 2 || c->cls[fl[fsz - 1]].size == 2) return 0;
    const int maxarity = (int)c->o.xor_max_arity;
    int arity0 = (int)c->cls[dl[0]].size - 1;
    if (arity0 > maxarity) return 0;
    const uint32_t v = ABSV(dx);
    for (uint32_t i = 0; i < dsz; i++) {
        Cls* ci = &c->cls[dl[i]];
        if (!is_orig(ci)) continue;
        const int size = (int)ci->size, arity = size - 1;
        if (size < 3 || arity > maxarity) continue;
        memcpy(out, CL(c, ci), (size_t)size * sizeof(uint32_t));
        uint32_t parity = 0;
        int itargets = 1 << arity;
        while (--itargets && makeArity(c, &parity, out, (uint32_t)size));
        if (itargets) freeze_arities(c, dx, fx);
        else {
            ci->molten = 1;
            *nE = 0; *nC = 0; *nL = 0;
            if (countSubst(c, PAIR_SUBS, v, nOrgCls, dx, fx, nE, nC, nL)) {
                freeze_arities(c, dx, fx);
                break;
            }
            return 1;
        }
    }
    return 0;
}

/* ---- function-table gates (function.cuh) ---- */
#define FUNTABLEN 64
#define MAXFUNVAR 12u
typedef uint64_t Fun[FUNTABLEN];
static const uint64_t MAGIC[6] = {
    0xaaaaaaaaaaaaaaaaULL, 0xccccccccccccccccULL, 0xf0f0f0f0f0f0f0f0ULL,
    0xff00ff00ff00ff00ULL, 0xffff0000ffff0000ULL, 0xffffffff00000000ULL,
};

static void clause2fun(uint32_t v, uint32_t sign, Fun f) {          /* function.cuh:91-114 */
    if (v < 6) {
        uint64_t val = MAGIC[v];
        if (sign) val = ~val;
        for (int i = 0; i < FUNTABLEN; i++) f[i] |= val;
    } else {
        uint64_t val = sign ? ~0ULL : 0ULL;
        int j = 0;
        const int sv = 1 << (v - 6);
        for (int i = 0; i < FUNTABLEN; i++) {
            f[i] |= val;
            if (++j >= sv) { val = ~val; j = 0; }
        }
    }
}

static int isfalsefun(const Fun f) { for (int i = 0; i < FUNTABLEN; i++) if (f[i]) return 0; return 1; }

/* buildfuntab (function.cuh:116-146); return 0 if a neighbour maps >= MAXFUNVAR */
static int buildfuntab(Ctx* c, uint32_t lit, Fun f) {
    for (int i = 0; i < FUNTABLEN; i++) f[i] = ~0ULL;
    const uint32_t* ol = OL(c, lit);
    Fun cls;
    for (uint32_t i = 0; i < OLSZ(c, lit); i++) {
        Cls* k = &c->cls[ol[i]];
        if (is_learnt(k)) continue;
        memset(cls, 0, sizeof(cls));
        const uint32_t* l = CL(c, k);
        for (uint32_t t = 0; t < k->size; t++) {
            const uint32_t other = l[t];
            if (other == lit) continue;
            const uint32_t mvar = c->varcore[ABSV(other)];
            if (mvar >= MAXFUNVAR) return 0;
            clause2fun(mvar, SIGNL(other), cls);
        }
        for (int q = 0; q < FUNTABLEN; q++) f[q] &= cls[q];
    }
    return 1;
}

/* buildfuntab core variant (function.cuh:148-176) */
static void buildfuntab_core(Ctx* c, uint32_t lit, uint32_t tail, Fun fun, int* core) {
    const uint32_t* ol = OL(c, lit);
    Fun cls;
    for (uint32_t j = 0; j < tail; j++) {
        Cls* k = &c->cls[ol[j]];
        if (is_learnt(k)) continue;
        memset(cls, 0, sizeof(cls));
        const uint32_t* l = CL(c, k);
        for (uint32_t t = 0; t < k->size; t++) {
            const uint32_t other = l[t];
            if (other == lit) continue;
            clause2fun(c->varcore[ABSV(other)], SIGNL(other), cls);
        }
        for (int q = 0; q < FUNTABLEN; q++) fun[q] &= cls[q];
    }
    if (isfalsefun(fun)) { c->cls[ol[tail]].molten = 1; *core = 1; }
}

/* find_fun_gate (function.cuh:275-325) */
static int find_fun_gate(Ctx* c, uint32_t p, uint32_t n, uint32_t nOrgCls,
                         uint32_t* nE, uint32_t* nC, uint32_t* nL) {
    Fun pos, neg;
    if (!buildfuntab(c, p, pos) || !buildfuntab(c, n, neg)) return 0;
    uint64_t allzero = 0;
    for (int i = 0; i < FUNTABLEN; i++) allzero |= pos[i] & neg[i];
    if (allzero) return 0;
    int core = 0;
    const uint32_t* pl = OL(c, p);
    for (int i = (int)OLSZ(c, p) - 1; i >= 0; i--) {
        memcpy(pos, neg, sizeof(Fun));
        if (is_orig(&c->cls[pl[i]])) buildfuntab_core(c, p, (uint32_t)i, pos, &core);
    }
    const uint32_t* nl = OL(c, n);
    for (int i = (int)OLSZ(c, n) - 1; i >= 0; i--) {
        for (int q = 0; q < FUNTABLEN; q++) pos[q] = ~0ULL;
        if (is_orig(&c->cls[nl[i]])) buildfuntab_core(c, n, (uint32_t)i, pos, &core);
    }
    *nE = 0; *nC = 0; *nL = 0;
    if (countSubst(c, PAIR_CORE, ABSV(p), nOrgCls, p, n, nE, nC, nL)) {
        if (core) freezeClauses(c, p, n);
        return 0;
    }
    return 1;
}

/* ---- equivalence gates (equivalence.cuh) ---- */
static int has_lit(Ctx* c, Cls* k, uint32_t lit) {   /* SCLAUSE::has on a sorted clause */
    const uint32_t* l = CL(c, k);
    for (uint32_t i = 0; i < k->size; i++) if (l[i] == lit) return 1;
    return 0;
}

/* substitute_single on one clause (equivalence.cuh:27-52) */
static void substitute_one(Ctx* c, uint32_t dx, uint32_t def, Cls* k, uint32_t* nUnits) {
    uint32_t* l = CL(c, k);
    uint32_t j = 0;
    for (uint32_t i = 0; i < k->size; i++) {
        const uint32_t lit = l[i];
        if (lit == dx) l[j++] = def;
        else if (lit != def) l[j++] = lit;
    }
    k->size = j;
    if (j == 1) (*nUnits)++;
    else { sort_u32(l, j); calcSig(c, k); }
}

/* substitute_single over both lists (equivalence.cuh:54-104) */
static void substitute_single(Ctx* c, uint32_t p, uint32_t n, uint32_t def) {
    const uint32_t def_f = FLIPL(def);
    uint32_t nNeg = 0, nPos = 0;
    const uint32_t* nl = OL(c, n);
    for (uint32_t i = 0; i < OLSZ(c, n); i++) {
        Cls* k = &c->cls[nl[i]];
        if (is_learnt(k) || k->molten || has_lit(c, k, def)) k->st = ST_DELETED;
        else substitute_one(c, n, def_f, k, &nNeg);
    }
    const uint32_t* pl = OL(c, p);
    for (uint32_t i = 0; i < OLSZ(c, p); i++) {
        Cls* k = &c->cls[pl[i]];
        if (is_learnt(k) || k->molten || has_lit(c, k, def_f)) k->st = ST_DELETED;
        else substitute_one(c, p, def, k, &nPos);
    }
    if (nPos || nNeg) {
        if (nNeg) appendUnits(c, n);
        if (nPos) appendUnits(c, p);
    }
    if (c->o.proof_en) {                 /* addProof over negs, then poss (equivalence.cuh:100-111) */
        pf_open(c, ABSV(p), 0);
        for (int side = 0; side < 2; side++) {
            const uint32_t lit = side ? p : n;
            const uint32_t* ol = OL(c, lit);
            for (uint32_t i = 0; i < OLSZ(c, lit); i++) {
                Cls* k = &c->cls[ol[i]];
                if (is_orig(k)) pf_line(c, PROOF_ADDED, CL(c, k), k->size);
            }
        }
        pf_close(c);
    }
}

/* find_sfanin (equivalence.cuh:106-122) */
static uint32_t find_sfanin(Ctx* c, uint32_t gate_out, uint32_t lit) {
    uint32_t imp = 0; int nImps = 0;
    const uint32_t* ol = OL(c, lit);
    for (uint32_t i = 0; i < OLSZ(c, lit); i++) {
        Cls* k = &c->cls[ol[i]];
        if (is_orig(k) && k->size == 2) {
            const uint32_t* l = CL(c, k);
            imp = FLIPL(l[0] ^ l[1] ^ gate_out);
            k->molten = 1;
            nImps++;
        }
        if (nImps > 1) return 0;
    }
    return imp;
}

/* find_equ_gate (equivalence.cuh:124-160) */
static uint32_t find_equ_gate(Ctx* c, uint32_t p, uint32_t n) {
    const uint32_t* pl = OL(c, p); const uint32_t* nl = OL(c, n);
    if (c->cls[pl[0]].size > 2 || c->cls[nl[0]].size > 2) return 0;
    uint32_t first = find_sfanin(c, p, p);
    if (first) {
        uint32_t second = n, def = first;
        if (second < def) { first = second; second = def; }
        for (uint32_t i = 0; i < OLSZ(c, n); i++) {
            Cls* k = &c->cls[nl[i]];
            const uint32_t* l = CL(c, k);
            if (is_orig(k) && k->size == 2 && l[0] == first && l[1] == second) {
                k->molten = 1;
                return def;
            }
        }
    }
    freezeBinaries(c, p);
    return 0;
}

/* ---- SUB (subsume.cuh) ---- */
static int subc(Ctx* c, Cls* s, Cls* t) {            /* sub(subsuming, subsumed), subsume.cuh:48-70 */
    const uint32_t* d1 = CL(c, s); const uint32_t* d2 = CL(c, t);
    const uint32_t n1 = s->size, n2 = t->size;
    uint32_t i = 0, j = 0, sub = 0;
    while (i < n1 && j < n2) {
        if (d1[i] < d2[j]) i++;
        else if (d2[j] < d1[i]) j++;
        else { sub++; i++; j++; }
    }
    return sub == n1;
}

static int selfsubc(Ctx* c, uint32_t x, uint32_t fx, Cls* s, Cls* t) {  /* subsume.cuh:126-168 */
    const uint32_t* d1 = CL(c, s); const uint32_t* d2 = CL(c, t);
    const uint32_t n1 = s->size, n2 = t->size;
    uint32_t i = 0, j = 0, sub = 0; int self = 0;
    while (i < n1 && j < n2) {
        const uint32_t l1 = d1[i], l2 = d2[j];
        if (l1 == fx) i++;
        else if (l2 == x) { self = 1; j++; }
        else if (l1 < l2) i++;
        else if (l2 < l1) j++;
        else { sub++; i++; j++; }
    }
    if (sub + 1 == n1) {
        if (self) return 1;
        while (j < n2) { if (d2[j] == x) return 1; j++; }
    }
    return 0;
}

static void bumpShrunken(Cls* k) {                    /* subsume.cuh:216-231 */
    const int old_lbd = (int)k->lbd;
    if (old_lbd <= (int)LBD_TIER1) return;
    const int sz1 = (int)k->size - 1;
    const int new_lbd = sz1 < old_lbd ? sz1 : old_lbd;
    if (new_lbd >= old_lbd) return;
    k->lbd = (uint32_t)new_lbd;
    k->usage = USAGET3;
}

static void strengthen(Ctx* c, Cls* k, uint32_t self) {   /* subsume.cuh:233-291 */
    uint32_t* l = CL(c, k);
    uint32_t j = 0;
    for (uint32_t i = 0; i < k->size; i++) if (l[i] != self) l[j++] = l[i];
    k->size--;
    if (k->size > 1) {
        calcSig(c, k);
        if (is_learnt(k)) bumpShrunken(k);
    }
}

static void updateOL(Ctx* c, uint32_t lit) {             /* subsume.cuh:293-303 */
    uint32_t* ol = OL(c, lit);
    uint32_t j = 0;
    for (uint32_t i = 0; i < OLSZ(c, lit); i++) {
        Cls* k = &c->cls[ol[i]];
        if (k->molten) k->molten = 0;
        else if (!is_deleted(k)) ol[j++] = ol[i];
    }
    OLSZ(c, lit) = j;
}

static void subsume_cand(Ctx* c, uint32_t lit, uint32_t end, Cls* cand) {   /* subsume.cuh:305-342 */
    const uint32_t candsz = cand->size;
    const uint32_t* ol = OL(c, lit);
    for (uint32_t j = 0; j < end; j++) {
        Cls* s = &c->cls[ol[j]];
        if (is_deleted(s)) continue;
        if (cand->molten && s->size > candsz) continue;
        if (s->size > 1 && SUBSIG(s->sig, cand->sig) && subc(c, s, cand)) {
            if (is_learnt(s) && is_orig(cand)) s->st = ST_ORIGINAL;
            cand->st = ST_DELETED;
            break;
        }
    }
}

static void selfsubsume(Ctx* c, uint32_t x, uint32_t fx, uint32_t lit, Cls* cand, uint32_t* nUnits) {  /* subsume.cuh:344-399 */
    const uint32_t candsz = cand->size, candsig = cand->sig;
    const uint32_t* ol = OL(c, lit);
    for (uint32_t j = 0; j < OLSZ(c, lit); j++) {
        Cls* s = &c->cls[ol[j]];
        const uint32_t subsize = s->size;
        if (subsize > candsz) break;
        if (is_deleted(s) || s->molten) continue;
        if (subsize > 1 && selfsub_sig(s->sig, candsig) && selfsubc(c, x, fx, s, cand)) {
            strengthen(c, cand, x);
            cand->molten = 1;
            if (cand->size == 1) (*nUnits)++;
            break;
        }
    }
}

/* sub_k body for one elected variable (subsume.cuh:402-484) */
static void sub_var(Ctx* c, uint32_t x) {
    const uint32_t p = 2 * x, n = p | 1;
    if (OLSZ(c, p) > c->o.sub_max_occurs || OLSZ(c, n) > c->o.sub_max_occurs) return;
    uint32_t nPos = 0, nNeg = 0;
    const uint32_t* pl = OL(c, p);
    for (uint32_t i = 0; i < OLSZ(c, p); i++) {
        Cls* pos = &c->cls[pl[i]];
        if (pos->size > SUB_MAX_CL_SIZE) break;
        if (is_deleted(pos)) continue;
        selfsubsume(c, p, n, n, pos, &nPos);
        subsume_cand(c, p, i, pos);
    }
    const uint32_t* nl = OL(c, n);
    for (uint32_t i = 0; i < OLSZ(c, n); i++) {
        Cls* neg = &c->cls[nl[i]];
        if (neg->size > SUB_MAX_CL_SIZE) break;
        if (is_deleted(neg)) continue;
        selfsubsume(c, n, p, p, neg, &nNeg);
        subsume_cand(c, n, i, neg);
    }
    if (nPos || nNeg) {
        if (nPos) appendUnits(c, p);
        if (nNeg) appendUnits(c, n);
    }
    if (c->o.proof_en) {                 /* saveProof over poss, then negs (subsume.cuh:464-474, proofutils.cuh:180-200) */
        pf_open(c, x, 0);
        for (int side = 0; side < 2; side++) {
            const uint32_t lit = side ? n : p;
            const uint32_t* ol = OL(c, lit);
            for (uint32_t i = 0; i < OLSZ(c, lit); i++) {
                Cls* k = &c->cls[ol[i]];
                if (k->molten) pf_line(c, PROOF_ADDED, CL(c, k), k->size);
                if (is_deleted(k)) pf_line(c, PROOF_DELETED, CL(c, k), k->size);
            }
        }
        pf_close(c);
    }
    updateOL(c, p);
    updateOL(c, n);
}

/* ---- BVE phase 1 (bounded.cuh:282-394, 397-473) ---- */
static void ve_phase1_var(Ctx* c, uint32_t tid, uint32_t x, uint32_t* outs) {
    const uint32_t p = 2 * x, n = p | 1;
    uint32_t pOrgs = 0, nOrgs = 0;
    if (c->o.ve_inprocess) {                       /* in_ve_k_1: countOrgs */
        const uint32_t* pl = OL(c, p); const uint32_t* nl = OL(c, n);
        for (uint32_t i = 0; i < OLSZ(c, p); i++) if (is_orig(&c->cls[pl[i]])) pOrgs++;
        for (uint32_t i = 0; i < OLSZ(c, n); i++) if (is_orig(&c->cls[nl[i]])) nOrgs++;
    } else { pOrgs = OLSZ(c, p); nOrgs = OLSZ(c, n); }
    uint32_t elimType = 0, nE = 0, nC = 0, nL = 0;
    c->type[tid] = 0; c->ucnt[tid] = 0; c->rpos[tid] = 0; c->rref[tid] = 0;
    if (!pOrgs || !nOrgs) {
        toblivionSave(c, p, n, pOrgs, nOrgs);
        c->eliminated[x] |= MELTING_MASK;
        return;
    }
    const uint32_t def = find_equ_gate(c, p, n);
    if (def) {
        saveResolvedOrgs(c, p, n, pOrgs, nOrgs);
        substitute_single(c, p, n, def);
        c->eliminated[x] |= MELTING_MASK;
        return;
    }
    if ((pOrgs == 1 || nOrgs == 1) && countResolventsU(c, x, p, n, &nE, &nC, &nL)) {
        if (nC) {
            c->type[tid] = RES_MASK | (nC << 2) | (nL << 16);
            c->ucnt[tid] = nE; c->rpos[tid] = nC; c->rref[tid] = nL + (uint64_t)NBUCKETS * nC;
        } else {
            toblivionSave(c, p, n, pOrgs, nOrgs);
            c->eliminated[x] |= MELTING_MASK;
        }
        return;
    }
    const uint32_t nClsBefore = pOrgs + nOrgs;
    elimType = 0; nE = 0; nC = 0; nL = 0;
    if (nClsBefore > 2) {
        if (nOrgs < SH_MAX_BVE_OUT1 && find_ao_gate(c, n, p, nClsBefore, outs, &nE, &nC, &nL))
            elimType = AOIX_MASK;
        else if (!nC && pOrgs < SH_MAX_BVE_OUT1 && find_ao_gate(c, p, n, nClsBefore, outs, &nE, &nC, &nL))
            elimType = AOIX_MASK;
    }
    if (!elimType && nClsBefore > 3) {
        if (find_ite_gate(c, p, n, nClsBefore, &nE, &nC, &nL)) elimType = AOIX_MASK;
        else if (!nC && find_ite_gate(c, n, p, nClsBefore, &nE, &nC, &nL)) elimType = AOIX_MASK;
        else if (find_xor_gate(c, p, n, nClsBefore, outs, &nE, &nC, &nL)) elimType = AOIX_MASK;
        else if (!nC && find_xor_gate(c, n, p, nClsBefore, outs, &nE, &nC, &nL)) elimType = AOIX_MASK;
    }
    if (c->varcore_on && !elimType && nClsBefore > 2 && find_fun_gate(c, p, n, nClsBefore, &nE, &nC, &nL))
        elimType = CORE_MASK;
    else if (!elimType && !nC && countResolventsB(c, x, nClsBefore, p, n, &nE, &nC, &nL))
        elimType = RES_MASK;
    if (!nC) {
        toblivionSave(c, p, n, pOrgs, nOrgs);
        c->eliminated[x] |= MELTING_MASK;
    } else if (elimType) {
        c->type[tid] = elimType | (nC << 2) | (nL << 16);
        c->ucnt[tid] = nE; c->rpos[tid] = nC; c->rref[tid] = nL + (uint64_t)NBUCKETS * nC;
    }
}

/* ---- BVE phase 3 emission (bounded.cuh:69-258, 488-544) ---- */
/* scratch for a merge of clauses of sizes a and b (resolvents can be longer
   than any uploaded clause, so the buffer grows with them) */
static uint32_t* merge_buf(Ctx* c, uint64_t a, uint64_t b) {
    const uint64_t need = a + b + 8;
    if (need > c->mcap) {
        c->mcap = 2 * need;
        c->mbuf = (uint32_t*)realloc(c->mbuf, c->mcap * sizeof(uint32_t));
        if (!c->mbuf) { fprintf(stderr, "pfo: out of memory\n"); abort(); }
    }
    return c->mbuf;
}

static void emit_resolvents(Ctx* c, int kind, uint32_t x, uint32_t nAddedCls) {
    const uint32_t p = 2 * x, n = p | 1;
    uint32_t added = 0;
    const uint32_t* ml = OL(c, p); const uint32_t* ot = OL(c, n);
    if (c->o.proof_en) pf_open(c, x, 0);
    for (uint32_t i = 0; i < OLSZ(c, p) && added < nAddedCls; i++) {
        Cls* ci = &c->cls[ml[i]];
        if (is_learnt(ci)) continue;
        for (uint32_t j = 0; j < OLSZ(c, n) && added < nAddedCls; j++) {
            Cls* cj = &c->cls[ot[j]];
            if (is_learnt(cj)) continue;
            if (kind == PAIR_SUBS && ci->molten == cj->molten) continue;
            if (kind == PAIR_CORE && ci->molten && cj->molten) continue;
            uint32_t* buf = merge_buf(c, ci->size, cj->size);
            const int rsize = merge_out(c, x, ci, cj, buf);
            if (!rsize) continue;
            if (c->o.proof_en) pf_line(c, PROOF_ADDED, buf, (uint32_t)rsize);    /* ADD_RESOLVENT's proof line */
            if (rsize == 1) { vpush(&c->units, buf[0]); continue; }
            /* ADD_RESOLVENT (bounded.cuh:69-122): ORIGINAL, added, sig */
            const uint64_t off = push_lits(c, buf, (uint32_t)rsize);
            Cls* k = push_cls(c);
            ci = &c->cls[ml[i]];            /* push_cls may move the array */
            k->off = off; k->size = (uint32_t)rsize; k->st = ST_ORIGINAL; k->added = 1;
            calcSig(c, k);
            added++;
        }
    }
    if (c->o.proof_en) pf_close(c);
    toblivion(c, p, n);
}

static void VE(Ctx* c, uint32_t* outs) {
    const uint32_t E = c->nelected;
    for (uint32_t tid = 0; tid < E; tid++) ve_phase1_var(c, tid, c->elected[tid], outs);
    pf_flush(c);                                                   /* substitution lines (ve_k_1) */
    /* vePhase2: exclusive scans with the current CNF size as init (elimination.cu:74-100) */
    uint64_t pos = c->ncls, ref = c->data_size;
    for (uint32_t tid = 0; tid < E; tid++) {
        const uint64_t a = c->rpos[tid], b = c->rref[tid];
        c->rpos[tid] = pos; c->rref[tid] = ref;
        pos += a; ref += b;
    }
    /* ve_k_2 (bounded.cuh:488-544) */
    int64_t last = -1;
    uint32_t survivors = 0;
    for (uint32_t tid = 0; tid < E; tid++) {
        const uint32_t x = c->elected[tid];
        const uint32_t xinfo = c->type[tid];
        const uint32_t et = xinfo & 3u;
        if (et) {
            const uint32_t p = 2 * x, n = p | 1;
            const uint32_t nAddedCls = (xinfo & 0xFFFCu) >> 2, nAddedLits = xinfo >> 16;
            const uint64_t addedPos = c->rpos[tid], addedRef = c->rref[tid];
            if (addedPos + nAddedCls <= c->cs_cap &&
                addedRef + nAddedLits + (uint64_t)NBUCKETS * nAddedCls <= c->data_cap) {
                if (c->ncls != addedPos) { fprintf(stderr, "pfo: slot mismatch\n"); abort(); }
                saveResolvedLists(c, p, n);
                emit_resolvents(c, et == RES_MASK ? PAIR_RES : (et == CORE_MASK ? PAIR_CORE : PAIR_SUBS),
                                x, nAddedCls);
                c->eliminated[x] |= MELTING_MASK | ADDING_MASK;
                last = tid;
            } else if (et != RES_MASK) {
                freezeClauses(c, p, n);
            }
        }
        if (!c->eliminated[x]) c->elected[survivors++] = x;     /* postVE: DeviceSelect::If */
    }
    pf_flush(c);                                                   /* resolvent lines (ve_k_2) */
    if (last >= 0) {                                               /* resizeCNF_k (cnf.cu:55-80) */
        const uint32_t xinfo = c->type[last];
        const uint64_t nAddedCls = (xinfo & 0xFFFCu) >> 2, nAddedLits = xinfo >> 16;
        c->data_size = c->rref[last] + nAddedLits + NBUCKETS * nAddedCls;
    }
    c->nelected = survivors;
}

/* ---- BCE (blocked.cuh:26-100, elimination.cu:178-291) ---- */
/* isTautology (elimination.cuh:119-138): do c1 and c2 clash on a variable other than x? */
static int is_tautology(Ctx* c, uint32_t x, Cls* c1, Cls* c2) {
    const uint32_t* a = CL(c, c1); const uint32_t* b = CL(c, c2);
    const int n1 = (int)c1->size, n2 = (int)c2->size;
    int i = 0, j = 0;
    while (i < n1 && j < n2) {
        const uint32_t l1 = a[i], l2 = b[j], v1 = ABSV(l1), v2 = ABSV(l2);
        if (v1 == x) i++;
        else if (v2 == x) j++;
        else if ((l1 ^ l2) == 1u) return 1;
        else if (v1 < v2) i++;
        else if (v2 < v1) j++;
        else { i++; j++; }
    }
    return 0;
}

/* blocked_x over the (surviving) elected variables: a non-learnt clause of -x
   whose resolvents with every non-learnt clause of x are tautologies is saved
   with witness -x and deleted */
static void BCE(Ctx* c) {
    for (uint32_t e = 0; e < c->nelected; e++) {
        const uint32_t x = c->elected[e], p = 2 * x, n = p | 1;
        if (OLSZ(c, p) > c->o.bce_max_occurs || OLSZ(c, n) > c->o.bce_max_occurs) continue;
        const uint32_t* pl = OL(c, p); const uint32_t* nl = OL(c, n);
        for (uint32_t i = 0; i < OLSZ(c, n); i++) {
            Cls* ci = &c->cls[nl[i]];
            if (is_deleted(ci) || is_learnt(ci)) continue;
            int all = 1;
            for (uint32_t j = 0; j < OLSZ(c, p) && all; j++) {
                Cls* cj = &c->cls[pl[j]];
                if (is_deleted(cj) || is_learnt(cj)) continue;
                if (!is_tautology(c, x, ci, cj)) all = 0;
            }
            if (all) {
                saveClause(c, ci, n);
                if (c->o.proof_en) {          /* blocked.cuh:67-72 */
                    pf_open(c, x, i);
                    pf_line(c, PROOF_DELETED, CL(c, ci), ci->size);
                    pf_close(c);
                }
                ci->st = ST_DELETED;
            }
        }
    }
    pf_flush(c);
}

/* ---- ERE (redundancy.cuh:27-175) ---- */
static int merge_ere(Ctx* c, uint32_t x, Cls* c1, Cls* c2, uint32_t* out) {
    return merge_out(c, x, c1, c2, out);
}

static void forward_equ(Ctx* c, const uint32_t* m, uint32_t mlen, uint32_t type, uint32_t v, uint32_t* seq) {
    uint32_t best = m[0], msig = MAPHASH(best);
    uint32_t minsize = OLSZ(c, best);
    for (uint32_t k = 1; k < mlen; k++) {
        const uint32_t ls = OLSZ(c, m[k]);
        if (ls < minsize) { minsize = ls; best = m[k]; }
        msig |= MAPHASH(m[k]);
    }
    const uint32_t* ol = OL(c, best);
    for (uint32_t lane = 0; lane < ERE_LANES; lane++) {
        for (uint32_t i = lane; i < minsize; i += ERE_LANES) {
            Cls* k = &c->cls[ol[i]];
            if (mlen == k->size && (is_learnt(k) || k->st == type) && SUBSIG(msig, k->sig) &&
                !is_deleted(k) && isEqual(c, k, m, mlen)) {
                k->st = ST_DELETED;
                if (c->o.proof_en) {          /* redundancy.cuh:122-128 */
                    pf_open(c, v, (*seq)++);
                    pf_line(c, PROOF_DELETED, CL(c, k), k->size);
                    pf_close(c);
                }
                break;
            }
        }
    }
}

static void ERE(Ctx* c) {
    const uint32_t cmax = c->o.ere_clause_max;
    for (uint32_t e = 0; e < c->nelected; e++) {
        const uint32_t v = c->elected[e], p = 2 * v, n = p | 1;
        const uint32_t ds = OLSZ(c, p), fs = OLSZ(c, n);
        if (!(ds && fs && ds <= c->o.ere_max_occurs && fs <= c->o.ere_max_occurs)) continue;
        const uint32_t* pl = OL(c, p); const uint32_t* nl = OL(c, n);
        if (!(c->cls[pl[0]].size <= cmax && c->cls[nl[0]].size <= cmax)) continue;
        uint32_t seq = 0;
        for (uint32_t i = 0; i < ds; i++) {
            Cls* pos = &c->cls[pl[i]];
            if (is_deleted(pos)) continue;
            for (uint32_t j = 0; j < fs; j++) {
                Cls* neg = &c->cls[nl[j]];
                if (is_deleted(neg) || pos->size + neg->size - 2 > cmax) continue;
                uint32_t* buf = merge_buf(c, pos->size, neg->size);
                const int mlen = merge_ere(c, v, pos, neg, buf);
                if (mlen > 1) {
                    const uint32_t type = (is_learnt(pos) || is_learnt(neg)) ? ST_LEARNT : ST_ORIGINAL;
                    forward_equ(c, buf, (uint32_t)mlen, type, v, &seq);
                }
            }
        }
    }
    pf_flush(c);
}

/* ---- option folding (OPTION::init, options.cpp:276-297; GOPTION::init, options.cu:75-88) ---- */
static void resolve_opts(pfg_options* o) {
    o->ve_en = (o->ve_en || o->ve_plus_en) ? 1 : 0;
    if (o->all_en) { o->ve_en = 1; o->ve_plus_en = 1; o->bce_en = 1; o->ere_en = 1; }
    if (!o->phases && (o->ve_en || o->sub_en || o->bce_en)) o->phases = 1;
    if (o->phases && !(o->ve_en || o->sub_en || o->bce_en)) o->phases = 0;
    if (o->phases > 1 && !o->ve_en) o->phases = 1;
    if (o->ere_clause_max > SH_MAX_ERE_OUT) o->ere_clause_max = SH_MAX_ERE_OUT;
    /* "xormaxarity" accepts 2..20 (options.cu:60) */
    if (o->xor_max_arity < 2) o->xor_max_arity = 2;
    if (o->xor_max_arity > 20) o->xor_max_arity = 20;
}

static int cmp_u32(const void* a, const void* b) {
    const uint32_t x = *(const uint32_t*)a, y = *(const uint32_t*)b;
    return x < y ? -1 : (x > y ? 1 : 0);
}

static uint64_t sort_unique(uint32_t* d, uint64_t n) {
    if (!n) return 0;
    qsort(d, n, sizeof(uint32_t), cmp_u32);
    uint64_t j = 1;
    for (uint64_t i = 1; i < n; i++) if (d[i] != d[j - 1]) d[j++] = d[i];
    return j;
}

static void push_round_end(Ctx* c) {
    if (c->nround_ends == c->round_ends_cap) {
        c->round_ends_cap = c->round_ends_cap ? 2 * c->round_ends_cap : 16;
        c->round_ends = (uint64_t*)realloc(c->round_ends, c->round_ends_cap * sizeof(uint64_t));
    }
    c->round_ends[c->nround_ends++] = c->resolved.n;
}

static pfo_round* new_rstat(Ctx* c) {
    if (c->nrstats == c->rstats_cap) {
        c->rstats_cap = c->rstats_cap ? 2 * c->rstats_cap : 16;
        c->rstats = (pfo_round*)realloc(c->rstats, c->rstats_cap * sizeof(pfo_round));
    }
    pfo_round* r = &c->rstats[c->nrstats++];
    memset(r, 0, sizeof(*r));
    return r;
}

int pfo_simplify(const pfg_options* opts, uint32_t max_var, uint64_t ncls,
                 const uint32_t* lits, const uint64_t* cls_off,
                 const uint8_t* cls_learnt, const uint32_t* cls_lbd,
                 const uint8_t* cls_usage, const uint8_t* var_state,
                 const uint8_t* assumed, const uint32_t* vorg,
                 pfo_result** out) {
    if (!opts || !out || !max_var || (ncls && (!lits || !cls_off))) return PFG_INVALID;
    Ctx C; memset(&C, 0, sizeof(C));
    Ctx* c = &C;
    c->o = *opts;
    resolve_opts(&c->o);
    const uint32_t V = max_var;
    c->V = V;
    c->vorg = (uint32_t*)xcalloc(V + 1, sizeof(uint32_t));
    for (uint32_t v = 0; v <= V; v++) c->vorg[v] = vorg ? vorg[v] : v;
    if (var_state) { c->vstate = (uint8_t*)xcalloc(V + 1, 1); memcpy(c->vstate, var_state, V + 1); }
    if (assumed) { c->assumed = (uint8_t*)xcalloc(V + 1, 1); memcpy(c->assumed, assumed, V + 1); }
    const uint64_t nl = 2ull * V + 2;
    c->hist = (uint32_t*)xcalloc(nl, sizeof(uint32_t));
    c->ot_off = (uint64_t*)xcalloc(nl + 1, sizeof(uint64_t));
    c->ot_size = (uint32_t*)xcalloc(nl, sizeof(uint32_t));
    c->eliminated = (uint8_t*)xcalloc(V + 1, 1);
    c->elected = (uint32_t*)xcalloc(V + 1, sizeof(uint32_t));
    c->varcore = (uint32_t*)xcalloc(V + 1, sizeof(uint32_t));
    c->eligible = (uint32_t*)xcalloc(V + 1, sizeof(uint32_t));
    c->scores = (uint32_t*)xcalloc(V + 1, sizeof(uint32_t));
    c->rank = (uint32_t*)xcalloc(V + 1, sizeof(uint32_t));
    c->mstate = (uint32_t*)xcalloc(V + 1, sizeof(uint32_t));
    c->mround = (uint32_t*)xcalloc(V + 1, sizeof(uint32_t));
    c->frozen = (uint8_t*)xcalloc(V + 1, 1);
    c->win = (uint8_t*)xcalloc(V + 1, 1);
    c->type = (uint32_t*)xcalloc(V + 1, sizeof(uint32_t));
    c->ucnt = (uint32_t*)xcalloc(V + 1, sizeof(uint32_t));
    c->rpos = (uint64_t*)xcalloc(V + 1, sizeof(uint64_t));
    c->rref = (uint64_t*)xcalloc(V + 1, sizeof(uint64_t));
    uint32_t* outs = (uint32_t*)xcalloc(SH_MAX_BVE_OUT1 + 8, sizeof(uint32_t));
    uint32_t maxsz = 2;
    /* upload: Solver::extractCNF + SCLAUSE(CLAUSE&) + prep_cnf_k (cnf.cu:45-53,176-184; sclause.cuh:64-78) */
    uint64_t orgCls = 0, orgLits = 0, lrnCls = 0, lrnLits = 0;
    for (uint64_t i = 0; i < ncls; i++) {
        const uint64_t b = cls_off[i], e = cls_off[i + 1];
        const uint32_t sz = (uint32_t)(e - b);
        if (sz < 2) { pfo_free(NULL); return PFG_INVALID; }
        if (sz > maxsz) maxsz = sz;
        const uint64_t off = push_lits(c, lits + b, sz);
        Cls* k = push_cls(c);
        k->off = off; k->size = sz;
        const int learnt = cls_learnt && cls_learnt[i];
        k->st = learnt ? ST_LEARNT : ST_ORIGINAL;
        if (learnt) {
            k->lbd = cls_lbd ? (cls_lbd[i] & MAX_LBD_M) : 0;
            k->usage = cls_usage ? (cls_usage[i] & 3u) : 0;
            lrnCls++; lrnLits += sz;
        } else { orgCls++; orgLits += sz; }
        sort_u32(CL(c, k), sz);
        calcSig(c, k);
    }
    merge_buf(c, maxsz, maxsz);
    c->numClauses = orgCls + lrnCls;
    c->numLiterals = orgLits + lrnLits;
    c->orig_lits_stat = orgLits;
    /* awaken capacities (simplify.cu:83-98, memory.cu:360-375) */
    {
        uint64_t numCls = c->numClauses, numLits = c->numLiterals;
        if (c->o.phases) {
            numCls += c->o.ve_en ? orgCls : 0;
            numLits += c->o.ve_en ? (uint64_t)((double)orgLits * c->o.lits_mul) : 0;
        }
        c->cs_cap = numCls;
        c->data_cap = numCls * NBUCKETS + numLits;
        c->data_size = c->numClauses * NBUCKETS + c->numLiterals;
    }
    c->varcore_on = c->o.ve_fun_en;
    c->status = PFG_UNKNOWN;
    const int disabled = !c->o.phases && !(c->o.all_en | c->o.ere_en);   /* alldisabled() */
    if (!disabled && orgCls) {
        /* round loop (simplify.cu:159-186) */
        int64_t cdiff = INT64_MAX, ldiff = INT64_MAX;
        int64_t clsbefore = (int64_t)c->numClauses, litsbefore = (int64_t)c->numLiterals;
        while (c->numClauses && c->numLiterals && !c->simpstate) {
            const int times = c->phase + 1;
            if (times > 1 && times != c->o.phases && c->o.shrink_rate > 0 && (times % c->o.shrink_rate) == 0)
                compactCNF(c);
            createOT(c);
            if (!prop(c)) { c->status = PFG_UNSAT; break; }
            else if (!c->numClauses) break;
            if (!LCVE(c)) break;
            sortOT(c);
            /* stop() (solver.hpp:748-753) */
            if (c->phase == c->o.phases || (cdiff == 0 && ldiff == 0) ||
                (c->phase > 2 && ldiff <= (int64_t)c->o.phase_lits_min)) {
                if (c->o.ere_en && c->nelected) { ERE(c); c->ere_ran = 1; }
                break;
            }
            pfo_round* rs = new_rstat(c);
            rs->elected = c->nelected;
            rs->mis_rounds = c->mis_rounds;
            rs->clauses_before = c->numClauses;
            rs->literals_before = c->numLiterals;
            const uint64_t ncls0 = c->ncls;
            const uint32_t nel0 = c->nelected;
            if (c->o.sub_en || c->o.ve_plus_en) {
                for (uint32_t e = 0; e < c->nelected; e++) sub_var(c, c->elected[e]);
                pf_flush(c);
            }
            if (c->o.ve_en) VE(c, outs);
            if (c->o.bce_en && c->nelected) BCE(c);
            push_round_end(c);
            countAll(c, &c->numClauses, &c->numLiterals);
            c->nUnits = c->units.n;
            rs->eliminated = nel0 - c->nelected;
            rs->units = (uint32_t)c->units.n;
            rs->resolvents = (uint32_t)(c->ncls - ncls0);
            rs->clauses_after = c->numClauses;
            rs->literals_after = c->numLiterals;
            cdiff = clsbefore - (int64_t)c->numClauses; clsbefore = (int64_t)c->numClauses;
            ldiff = litsbefore - (int64_t)c->numLiterals; litsbefore = (int64_t)c->numLiterals;
            c->phase++; c->multiplier++;
            c->multiplier += (c->phase == c->o.phases);
        }
        if (c->status != PFG_UNSAT && !c->numClauses) c->status = PFG_SAT;
    }
    /* results */
    pfo_result* r = (pfo_result*)xcalloc(1, sizeof(pfo_result));
    r->status = c->status; r->simpstate = c->simpstate; r->rounds = c->phase; r->ere_ran = c->ere_ran;
    r->max_var = V;
    uint64_t live = 0, livel = 0;
    for (uint64_t i = 0; i < c->ncls; i++) if (!is_deleted(&c->cls[i])) { live++; livel += c->cls[i].size; }
    r->ncls = live; r->nlits = livel;
    r->lits = (uint32_t*)xcalloc(livel + 1, sizeof(uint32_t));
    r->cls_off = (uint64_t*)xcalloc(live + 1, sizeof(uint64_t));
    r->cls_learnt = (uint8_t*)xcalloc(live + 1, 1);
    r->cls_lbd = (uint32_t*)xcalloc(live + 1, sizeof(uint32_t));
    r->cls_usage = (uint8_t*)xcalloc(live + 1, 1);
    uint64_t j = 0, lo = 0;
    for (uint64_t i = 0; i < c->ncls; i++) {
        Cls* k = &c->cls[i];
        if (is_deleted(k)) continue;
        r->cls_off[j] = lo;
        memcpy(r->lits + lo, CL(c, k), k->size * sizeof(uint32_t));
        lo += k->size;
        r->cls_learnt[j] = is_learnt(k) ? 1 : 0;
        r->cls_lbd[j] = k->lbd;
        r->cls_usage[j] = k->usage;
        j++;
    }
    r->cls_off[j] = lo;
    r->eliminated = c->eliminated; c->eliminated = NULL;
    r->nunits = sort_unique(c->trail.d, c->trail.n);
    r->units = c->trail.d; c->trail.d = NULL;
    if (!r->units) r->units = (uint32_t*)xcalloc(1, sizeof(uint32_t));
    r->npending = c->nUnits ? sort_unique(c->units.d, c->units.n) : 0;
    r->pending = c->units.d; c->units.d = NULL;
    if (!r->pending) r->pending = (uint32_t*)xcalloc(1, sizeof(uint32_t));
    r->nstack = c->resolved.n;
    r->stack = c->resolved.d; c->resolved.d = NULL;
    if (!r->stack) r->stack = (uint32_t*)xcalloc(1, sizeof(uint32_t));
    r->nround_ends = c->nround_ends;
    r->round_ends = c->round_ends ? c->round_ends : (uint64_t*)xcalloc(1, sizeof(uint64_t));
    c->round_ends = NULL;
    r->nround_stats = c->nrstats;
    r->round_stats = c->rstats ? c->rstats : (pfo_round*)xcalloc(1, sizeof(pfo_round));
    c->rstats = NULL;
    r->nproof = c->nproof;
    r->proof = c->proof ? c->proof : (uint8_t*)xcalloc(1, 1);
    c->proof = NULL;
    /* free context */
    free(c->vorg); free(c->vstate); free(c->assumed); free(c->lits); free(c->cls);
    free(c->hist); free(c->ot_off); free(c->ot_size); free(c->ot_pool); free(c->eliminated);
    free(c->elected); free(c->varcore); free(c->eligible); free(c->scores); free(c->rank);
    free(c->mstate); free(c->mround); free(c->frozen); free(c->win); free(c->type); free(c->ucnt);
    free(c->rpos); free(c->rref); free(c->units.d); free(c->trail.d); free(c->resolved.d);
    free(c->round_ends_v.d); free(outs); free(c->mbuf); free(c->pbuf); free(c->pch);
    *out = r;
    return PFG_OK;
}

void pfo_free(pfo_result* r) {
    if (!r) return;
    free(r->lits); free(r->cls_off); free(r->cls_learnt); free(r->cls_lbd); free(r->cls_usage);
    free(r->eliminated); free(r->units); free(r->pending); free(r->stack); free(r->round_ends);
    free(r->round_stats); free(r->proof);
    free(r);
}

/* ---- canonical form ---- */
typedef struct { const uint32_t* l; uint64_t n; uint8_t learnt, usage; uint32_t lbd; uint64_t idx; } CanonKey;

static int canon_cmp(const void* pa, const void* pb) {
    const CanonKey* a = (const CanonKey*)pa; const CanonKey* b = (const CanonKey*)pb;
    if (a->n != b->n) return a->n < b->n ? -1 : 1;
    for (uint64_t i = 0; i < a->n; i++) if (a->l[i] != b->l[i]) return a->l[i] < b->l[i] ? -1 : 1;
    if (a->learnt != b->learnt) return a->learnt < b->learnt ? -1 : 1;
    if (a->lbd != b->lbd) return a->lbd < b->lbd ? -1 : 1;
    if (a->usage != b->usage) return a->usage < b->usage ? -1 : 1;
    return 0;
}

int pfo_canon_cnf(uint64_t ncls, const uint32_t* lits, const uint64_t* off,
                  const uint8_t* learnt, const uint32_t* lbd, const uint8_t* usage,
                  uint32_t* out_lits, uint64_t* out_off, uint8_t* out_learnt,
                  uint32_t* out_lbd, uint8_t* out_usage) {
    uint32_t* tmp = (uint32_t*)xcalloc(off[ncls] + 1, sizeof(uint32_t));
    memcpy(tmp, lits, off[ncls] * sizeof(uint32_t));
    CanonKey* keys = (CanonKey*)xcalloc(ncls + 1, sizeof(CanonKey));
    for (uint64_t i = 0; i < ncls; i++) {
        const uint64_t n = off[i + 1] - off[i];
        qsort(tmp + off[i], n, sizeof(uint32_t), cmp_u32);
        keys[i].l = tmp + off[i]; keys[i].n = n; keys[i].idx = i;
        keys[i].learnt = learnt ? learnt[i] : 0;
        keys[i].lbd = (learnt && learnt[i] && lbd) ? lbd[i] : 0;
        keys[i].usage = (learnt && learnt[i] && usage) ? usage[i] : 0;
    }
    qsort(keys, ncls, sizeof(CanonKey), canon_cmp);
    uint64_t lo = 0;
    for (uint64_t i = 0; i < ncls; i++) {
        out_off[i] = lo;
        memcpy(out_lits + lo, keys[i].l, keys[i].n * sizeof(uint32_t));
        lo += keys[i].n;
        out_learnt[i] = keys[i].learnt; out_lbd[i] = keys[i].lbd; out_usage[i] = keys[i].usage;
    }
    out_off[ncls] = lo;
    free(keys); free(tmp);
    return 0;
}

typedef struct { uint64_t b, e; uint32_t w, tail; } Block;
static int block_cmp(const void* pa, const void* pb) {
    const Block* a = (const Block*)pa; const Block* b = (const Block*)pb;
    if (a->tail != b->tail) return a->tail < b->tail ? -1 : 1;
    if ((a->w >> 1) != (b->w >> 1)) return (a->w >> 1) < (b->w >> 1) ? -1 : 1;
    return a->b < b->b ? -1 : (a->b > b->b ? 1 : 0);
}

/* A BVE block is [clause*] [witness, 1]; stack words k > 1 are clause lengths.
   BCE saves blocked clauses one by one after the round's BVE blocks, with the
   witness literal first and no [witness, 1] entry (blocked.cuh:64-67): those
   trailing entries are ordered by witness variable, keeping each variable's
   own order. */
int pfo_canon_stack(uint64_t nstack, const uint32_t* stack, uint64_t nrounds,
                    const uint64_t* round_ends, uint32_t* out_stack) {
    Block* blocks = (Block*)xcalloc(nstack / 2 + 2, sizeof(Block));
    uint64_t rb = 0, wo = 0;
    for (uint64_t r = 0; r <= nrounds; r++) {
        const uint64_t re = (r < nrounds) ? round_ends[r] : nstack;
        if (re < rb) { free(blocks); return -1; }
        /* entries are [lits..., k] with the length last, so walk [rb, re) backwards */
        uint64_t nb = 0;
        uint64_t x = re;
        uint64_t bend = re;
        int have = 0;
        uint32_t w = 0;
        while (x > rb) {
            const uint32_t k = stack[x - 1];
            if (k == 0 || x - 1 < rb + k) { free(blocks); return -2; }
            const uint64_t start = x - 1 - k;
            if (k == 1) {
                if (have) { blocks[nb].b = x; blocks[nb].e = bend; blocks[nb].w = w; blocks[nb].tail = 0; nb++; }
                have = 1; w = stack[start]; bend = x;
            } else if (!have) {   /* a BCE entry after the last BVE block */
                blocks[nb].b = start; blocks[nb].e = x; blocks[nb].w = stack[start]; blocks[nb].tail = 1; nb++;
                bend = start;
            }
            x = start;
        }
        if (have) { blocks[nb].b = rb; blocks[nb].e = bend; blocks[nb].w = w; blocks[nb].tail = 0; nb++; }
        qsort(blocks, nb, sizeof(Block), block_cmp);
        for (uint64_t q = 0; q < nb; q++) {
            memcpy(out_stack + wo, stack + blocks[q].b, (blocks[q].e - blocks[q].b) * sizeof(uint32_t));
            wo += blocks[q].e - blocks[q].b;
        }
        rb = re;
    }
    free(blocks);
    return wo == nstack ? 0 : -3;
}

/* MODEL::extend (src/gpu/model.cpp:101-160) */
void pfo_extend_model(uint64_t nstack, const uint32_t* stack, uint8_t* value) {
    if (!nstack) return;
    int64_t x = (int64_t)nstack - 1;
    while (x > 0) {
        uint32_t k = stack[x--];
        int unsat = 1;
        for (; k > 1; k--, x--) {
            const uint32_t l = stack[x];
            const uint8_t vv = value[ABSV(l)];
            if ((SIGNL(l) ? !vv : vv)) { unsat = 0; break; }
        }
        if (unsat) value[ABSV(stack[x])] = SIGNL(stack[x]) ? 0 : 1;
        x -= (int64_t)k;
    }
}

/* ---- small DPLL solver used by the tests to check satisfiability and models ----
   Two watched literals, chronological backtracking; returns 10 (SAT, model in
   value[1..V]), 20 (UNSAT) or 0 (decision budget exhausted). */
/* ---- DRAT RUP check of a simplifier proof (test helper) ----
   Naive unit propagation over all active clauses; enough for the small
   formulas the tests check. */
typedef struct { uint32_t* l; uint32_t n; int active; } RupCls;

static int rup_propagate(RupCls* db, uint64_t n, int8_t* val) {   /* 1 = conflict */
    int changed = 1;
    while (changed) {
        changed = 0;
        for (uint64_t i = 0; i < n; i++) {
            if (!db[i].active) continue;
            uint32_t unset = 0, last = 0; int sat = 0;
            for (uint32_t t = 0; t < db[i].n && !sat; t++) {
                const uint32_t l = db[i].l[t];
                const int8_t v = val[l >> 1];
                if (!v) { unset++; last = l; }
                else if ((v > 0) != ((l & 1u) != 0)) sat = 1;
            }
            if (sat) continue;
            if (!unset) return 1;
            if (unset == 1) { val[last >> 1] = (last & 1u) ? -1 : 1; changed = 1; }
        }
    }
    return 0;
}

static int rup_same(const RupCls* k, const uint32_t* l, uint32_t n) {
    if (k->n != n) return 0;
    for (uint32_t i = 0; i < n; i++) {
        uint32_t f = 0;
        for (uint32_t j = 0; j < n && !f; j++) f = k->l[j] == l[i];
        if (!f) return 0;
    }
    return 1;
}

int64_t pfo_check_rup(uint32_t V, uint64_t ncls, const uint32_t* lits, const uint64_t* off,
                      const uint8_t* proof, uint64_t nproof, uint64_t* missing_deletions) {
    uint64_t cap = ncls + 64, n = 0;
    RupCls* db = (RupCls*)xcalloc(cap, sizeof(RupCls));
    for (uint64_t i = 0; i < ncls; i++) {
        const uint32_t sz = (uint32_t)(off[i + 1] - off[i]);
        db[n].l = (uint32_t*)xcalloc(sz + 1, sizeof(uint32_t));
        memcpy(db[n].l, lits + off[i], sz * sizeof(uint32_t));
        db[n].n = sz; db[n].active = 1; n++;
    }
    int8_t* val = (int8_t*)xcalloc(V + 1, 1);
    uint32_t* line = (uint32_t*)xcalloc(V + 8, sizeof(uint32_t));
    int64_t bad = 0, lineno = 0;
    uint64_t p = 0, missing = 0;
    while (p < nproof && !bad) {
        const uint8_t st = proof[p++];
        uint32_t len = 0;
        lineno++;
        if (st != PROOF_ADDED && st != PROOF_DELETED) { bad = lineno; break; }
        while (p < nproof && proof[p]) {
            uint32_t v = 0, sh = 0; uint8_t b;
            do { b = proof[p++]; v |= (uint32_t)(b & 0x7Fu) << sh; sh += 7; } while ((b & 0x80u) && p < nproof);
            if ((v >> 1) == 0 || (v >> 1) > V || len > V + 4) { bad = lineno; break; }
            line[len++] = v;
        }
        if (bad) break;
        if (p >= nproof) { bad = lineno; break; }
        p++;                                            /* terminator */
        if (st == PROOF_DELETED) {
            uint64_t i = 0;
            for (; i < n; i++) if (db[i].active && rup_same(&db[i], line, len)) break;
            if (i < n) db[i].active = 0; else missing++;
            continue;
        }
        memset(val, 0, V + 1);
        for (uint32_t i = 0; i < len; i++) val[line[i] >> 1] = (line[i] & 1u) ? 1 : -1;   /* negation */
        if (!rup_propagate(db, n, val)) { bad = lineno; break; }
        if (n == cap) { cap *= 2; db = (RupCls*)realloc(db, cap * sizeof(RupCls)); }
        db[n].l = (uint32_t*)xcalloc(len + 1, sizeof(uint32_t));
        memcpy(db[n].l, line, len * sizeof(uint32_t));
        db[n].n = len; db[n].active = 1; n++;
    }
    for (uint64_t i = 0; i < n; i++) free(db[i].l);
    free(db); free(val); free(line);
    if (missing_deletions) *missing_deletions = missing;
    return bad;
}

int pfo_solve(uint32_t V, uint64_t ncls, const uint32_t* lits, const uint64_t* off,
              uint8_t* value, uint64_t max_decisions) {
    const uint64_t nl = 2ull * V + 2;
    int8_t* val = (int8_t*)xcalloc(V + 1, 1);              /* 0 unassigned, 1 true, -1 false */
    uint32_t* cl = (uint32_t*)xcalloc(off[ncls] + 1, sizeof(uint32_t));
    memcpy(cl, lits, off[ncls] * sizeof(uint32_t));
    Vec* watch = (Vec*)xcalloc(nl, sizeof(Vec));
    uint32_t* trail = (uint32_t*)xcalloc(V + 1, sizeof(uint32_t));
    uint8_t* isdec = (uint8_t*)xcalloc(V + 1, 1);
    uint8_t* tried = (uint8_t*)xcalloc(V + 1, 1);
    uint64_t tn = 0, qh = 0, decisions = 0;
    int result = 0;
#define LV(l) (val[(l) >> 1] == 0 ? 0 : (((l) & 1) ? -val[(l) >> 1] : val[(l) >> 1]))
    int conflict = 0;
    for (uint64_t c = 0; c < ncls && !conflict; c++) {
        const uint64_t b = off[c], e = off[c + 1];
        if (e == b) { conflict = 1; break; }
        if (e - b == 1) {
            const uint32_t u = cl[b];
            if (LV(u) == -1) conflict = 1;
            else if (LV(u) == 0) { val[u >> 1] = (u & 1) ? -1 : 1; trail[tn++] = u; }
            continue;
        }
        vpush(&watch[cl[b]], (uint32_t)c);
        vpush(&watch[cl[b + 1]], (uint32_t)c);
    }
    if (conflict) { result = 20; goto done; }
    for (;;) {
        /* propagate */
        conflict = 0;
        while (qh < tn && !conflict) {
            const uint32_t f = trail[qh++] ^ 1u;     /* literal that became false */
            Vec* w = &watch[f];
            uint64_t i = 0, j = 0;
            while (i < w->n) {
                const uint32_t c = w->d[i++];
                uint32_t* l = cl + off[c];
                const uint64_t sz = off[c + 1] - off[c];
                if (l[0] == f) { l[0] = l[1]; l[1] = f; }
                if (LV(l[0]) == 1) { w->d[j++] = c; continue; }
                uint64_t k;
                for (k = 2; k < sz; k++) {
                    if (LV(l[k]) != -1) {
                        l[1] = l[k]; l[k] = f;
                        vpush(&watch[l[1]], c);
                        break;
                    }
                }
                if (k < sz) continue;
                w->d[j++] = c;
                if (LV(l[0]) == -1) {
                    conflict = 1;
                    while (i < w->n) w->d[j++] = w->d[i++];
                } else if (LV(l[0]) == 0) {
                    val[l[0] >> 1] = (l[0] & 1) ? -1 : 1;
                    trail[tn++] = l[0];
                }
            }
            w->n = j;
        }
        if (conflict) {
            /* backtrack to the last decision not yet flipped */
            int64_t t = (int64_t)tn - 1;
            while (t >= 0 && !(isdec[trail[t] >> 1] && !tried[trail[t] >> 1])) {
                const uint32_t v = trail[t] >> 1;
                val[v] = 0; isdec[v] = 0; tried[v] = 0;
                t--;
            }
            if (t < 0) { result = 20; break; }
            const uint32_t d = trail[t];
            const uint32_t v = d >> 1;
            tn = (uint64_t)t;
            val[v] = (d & 1) ? 1 : -1;             /* flipped decision */
            isdec[v] = 1; tried[v] = 1;
            trail[tn++] = d ^ 1u;
            qh = tn - 1;
            continue;
        }
        /* decide */
        uint32_t v = 0;
        for (uint32_t u = 1; u <= V; u++) if (!val[u]) { v = u; break; }
        if (!v) { result = 10; break; }
        if (++decisions > max_decisions) { result = 0; break; }
        val[v] = -1; isdec[v] = 1; tried[v] = 0;
        trail[tn++] = (v << 1) | 1u;
    }
    if (result == 10 && value) for (uint32_t u = 1; u <= V; u++) value[u] = val[u] > 0;
#undef LV
done:
    for (uint64_t l = 0; l < nl; l++) free(watch[l].d);
    free(watch); free(val); free(cl); free(trail); free(isdec); free(tried);
    return result;
}
