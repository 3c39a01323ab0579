// C-ABI and round driver of the GB300 CNF inprocessing engine.
//
// pfg_upload replaces Solver::awaken (src/gpu/simplify.cu:77-134),
// pfg_simplify the round loop of Solver::simplifying (simplify.cu:159-186),
// pfg_download the write-back (cacheCNF cnf.cu:200-236, cacheEliminated
// transfer.cu:69, cacheResolved transfer.cu:83).
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <unordered_map>
#include <vector>

#include "engine.cuh"

struct pfg_ctx {
    pfg::Ctx c;
    std::unordered_map<void*, size_t> sizes;
    size_t allocated = 0;
    size_t budget = 0;
};

namespace pfg {

static pfg_ctx* owner_of(Ctx& c) { return reinterpret_cast<pfg_ctx*>(reinterpret_cast<char*>(&c) - offsetof(pfg_ctx, c)); }

bool cuda_ok(Ctx& c, cudaError_t e, const char* what) {
    if (e == cudaSuccess) return true;
    if (c.err.empty()) {
        c.err = std::string(what) + ": " + cudaGetErrorString(e);
    }
    return false;
}

bool dalloc(Ctx& c, void** p, size_t bytes) {
    *p = nullptr;
    if (bytes == 0) bytes = 16;
    pfg_ctx* o = owner_of(c);
    if (o->budget && o->allocated + bytes > o->budget) {
        c.err = "device pool budget exceeded";
        return false;
    }
    cudaError_t e = cudaMallocAsync(p, bytes, c.s);
    if (e != cudaSuccess) {
        cudaGetLastError();
        *p = nullptr;
        c.err = std::string("device allocation of ") + std::to_string(bytes) + " bytes failed: " + cudaGetErrorString(e);
        return false;
    }
    o->sizes[*p] = bytes;
    o->allocated += bytes;
    return true;
}

void dfree(Ctx& c, void* p) {
    if (!p) return;
    pfg_ctx* o = owner_of(c);
    auto it = o->sizes.find(p);
    if (it != o->sizes.end()) { o->allocated -= it->second; o->sizes.erase(it); }
    cudaFreeAsync(p, c.s);
}

bool ensure_tmp(Ctx& c, size_t bytes) {
    if (c.tmp_cap >= bytes) return true;
    dfree(c, c.tmp);
    c.tmp = nullptr;
    const size_t cap = std::max<size_t>(bytes + bytes / 2, 1 << 20);
    if (!dalloc(c, &c.tmp, cap)) { c.tmp_cap = 0; return false; }
    c.tmp_cap = cap;
    return true;
}

bool ensure_tmp_u32(Ctx& c, uint64_t count) {
    if (c.tmp_u32_cap >= count) return true;
    dfree(c, c.tmp_u32);
    c.tmp_u32 = nullptr;
    const uint64_t cap = std::max<uint64_t>(count + count / 2, 4096);
    if (!dalloc_t(c, &c.tmp_u32, cap)) { c.tmp_u32_cap = 0; return false; }
    c.tmp_u32_cap = cap;
    return true;
}

void sync_counters(Ctx& c) {
    cudaMemcpyAsync(c.hc, c.dc, sizeof(DevCounters), cudaMemcpyDeviceToHost, c.s);
    cuda_ok(c, cudaStreamSynchronize(c.s), "stream synchronize");
    if (c.err.empty() && c.hc->err) {
        char b[128];
        snprintf(b, sizeof(b), "device error flags 0x%x", c.hc->err);
        c.err = b;
    }
}

namespace {

__global__ void init_hdr_k(ClsHdr* hdr, const unsigned long long* off, uint64_t ncls, const uint8_t* learnt,
                           const uint32_t* lbd, const uint8_t* usage) {
    for (uint64_t c = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; c < ncls; c += (uint64_t)gridDim.x * blockDim.x) {
        ClsHdr h;
        h.off = (uint32_t)off[c];
        h.size = (uint32_t)(off[c + 1] - off[c]);
        h.sig = 0;
        const bool l = learnt && learnt[c];
        h.meta = l ? m_make(ST_LEARNT, 0, 0, usage ? (usage[c] & 3u) : 0u, lbd ? (lbd[c] & 0x03FFFFFFu) : 0u)
                   : m_make(ST_ORIGINAL, 0, 0, 0, 0);
        hdr[c] = h;
    }
}

// prep_cnf_k (cnf.cu:45-53): sort literals of every clause, compute its signature
__global__ void prep_k(ClsHdr* hdr, uint32_t* lits, uint64_t ncls) {
    for (uint64_t c = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; c < ncls; c += (uint64_t)gridDim.x * blockDim.x) {
        const ClsHdr h = hdr[c];
        uint32_t* l = lits + h.off;
        for (uint32_t i = 1; i < h.size; i++) {
            const uint32_t t = l[i];
            uint32_t j = i;
            while (j > 0 && t < l[j - 1]) { l[j] = l[j - 1]; j--; }
            l[j] = t;
        }
        if (h.size > 1) {
            uint32_t s = 0;
            for (uint32_t i = 0; i < h.size; i++) s |= MAPHASH(l[i]);
            hdr[c].sig = s;
        }
    }
}

__global__ void identity_k(uint32_t* v, uint32_t n) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) v[i] = i;
}

// sum of list sizes and literal counts over elected variables (C_E, L_E of the byte model)
__global__ void elected_volume_k(const uint32_t* elected, uint32_t n, const ClsHdr* hdr, const uint32_t* ot_off,
                                 const uint32_t* ot_size, const uint32_t* ot_ids, unsigned long long* out) {
    unsigned long long cc = 0, ll = 0;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t v = elected[i];
        for (int s = 0; s < 2; s++) {
            const uint32_t lit = 2 * v + s;
            const uint32_t o = ot_off[lit], sz = ot_size[lit];
            cc += sz;
            for (uint32_t j = 0; j < sz; j++) ll += hdr[ot_ids[o + j]].size;
        }
    }
    for (int d = 16; d > 0; d >>= 1) {
        cc += __shfl_down_sync(0xFFFFFFFFu, cc, d);
        ll += __shfl_down_sync(0xFFFFFFFFu, ll, d);
    }
    if ((threadIdx.x & 31u) == 0 && (cc || ll)) { atomicAdd(&out[0], cc); atomicAdd(&out[1], ll); }
}

// live clauses -> packed host layout
__global__ void out_flags_k(const ClsHdr* hdr, uint64_t ncls, uint32_t* flag, unsigned long long* sz) {
    for (uint64_t c = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; c < ncls; c += (uint64_t)gridDim.x * blockDim.x) {
        const ClsHdr h = hdr[c];
        const bool live = !m_deleted(h.meta);
        flag[c] = live;
        sz[c] = live ? h.size : 0;
    }
}

__global__ void out_pack_k(const ClsHdr* hdr, const uint32_t* lits, uint64_t ncls, const uint32_t* pos,
                           const unsigned long long* loff, uint32_t* olits, unsigned long long* ooff, uint8_t* olearnt,
                           uint32_t* olbd, uint8_t* ousage) {
    const uint64_t warp = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    const unsigned lane = threadIdx.x & 31u;
    for (uint64_t c = warp; c < ncls; c += nwarps) {
        const ClsHdr h = hdr[c];
        if (m_deleted(h.meta)) continue;
        const unsigned long long o = loff[c];
        for (uint32_t k = lane; k < h.size; k += 32) olits[o + k] = lits[h.off + k];
        if (lane == 0) {
            const uint32_t q = pos[c];
            ooff[q] = o;
            const bool l = m_learnt(h.meta);
            olearnt[q] = l;
            olbd[q] = m_lbd(h.meta);
            ousage[q] = (uint8_t)m_usage(h.meta);
        }
    }
}

void free_all(pfg_ctx* o) {
    Ctx& c = o->c;
    std::vector<void*> ptrs;
    for (auto& kv : o->sizes) ptrs.push_back(kv.first);
    for (void* p : ptrs) cudaFreeAsync(p, c.s);
    o->sizes.clear();
    o->allocated = 0;
    if (c.s) cudaStreamSynchronize(c.s);
    Ctx fresh;
    fresh.o = c.o;
    fresh.device = c.device;
    fresh.s = c.s;
    fresh.ev_begin = c.ev_begin; fresh.ev_end = c.ev_end; fresh.ev_a = c.ev_a; fresh.ev_b = c.ev_b;
    fresh.dc = nullptr; fresh.hc = c.hc;
    fresh.launches = c.launches;
    fresh.prof = c.prof;
    c = fresh;
}

struct PassTimer {
    Ctx& c;
    int slot;
    PassTimer(Ctx& cc, int s) : c(cc), slot(s) { cudaEventRecord(c.ev_a, c.s); }
    ~PassTimer() {
        cudaEventRecord(c.ev_b, c.s);
        cudaEventSynchronize(c.ev_b);
        float ms = 0;
        cudaEventElapsedTime(&ms, c.ev_a, c.ev_b);
        c.pass_ms[slot] += ms;
    }
};

}  // namespace
}  // namespace pfg

using namespace pfg;

extern "C" void pfg_abi_sizes(size_t* options, size_t* stats, size_t* result_sizes) {
    if (options) *options = sizeof(pfg_options);
    if (stats) *stats = sizeof(pfg_stats);
    if (result_sizes) *result_sizes = sizeof(pfg_result_sizes);
}

extern "C" void pfg_default_options(pfg_options* o) {
    std::memset(o, 0, sizeof(*o));
    o->phases = 5;
    o->shrink_rate = 2;
    o->lcve_fast = 1;
    o->lcve_min_vars = 2;
    o->lcve_max_occurs = 3000;
    o->lcve_clause_max = 30000;
    o->phase_lits_min = 500;
    o->mu_pos = 32;
    o->mu_neg = 32;
    o->lits_mul = 1.0;
    o->ve_en = 1;
    o->ve_plus_en = 1;
    o->sub_en = 1;
    o->ere_en = 1;
    o->ve_fun_en = 1;
    o->ve_clause_max = 100;
    o->xor_max_arity = 10;
    o->sub_max_occurs = 3000;
    o->ere_max_occurs = 3000;
    o->ere_clause_max = 250;
    o->bce_max_occurs = 3000;
}

extern "C" void pfg_resolve_options(pfg_options* o) {
    // OPTION::init (options.cpp:283-297)
    o->ve_en = (o->ve_en || o->ve_plus_en) ? 1 : 0;
    if (o->all_en) { o->ve_en = 1; o->ve_plus_en = 1; o->bce_en = 1; o->ere_en = 1; }
    if (!o->phases && (o->ve_en || o->sub_en || o->bce_en)) o->phases = 1;
    if (o->phases && !(o->ve_en || o->sub_en || o->bce_en)) o->phases = 0;
    if (o->phases > 1 && !o->ve_en) o->phases = 1;
    // GOPTION::init (options.cu:84): ERE resolvents are staged in SH_MAX_ERE_OUT words
    if (o->ere_clause_max > SH_MAX_ERE_OUT) o->ere_clause_max = SH_MAX_ERE_OUT;
}

extern "C" int pfg_create(pfg_ctx** out, const pfg_options* opts, size_t arena_bytes) {
    if (!out) return PFG_INVALID;
    *out = nullptr;
    pfg_ctx* o = new pfg_ctx();
    Ctx& c = o->c;
    if (opts) c.o = *opts; else pfg_default_options(&c.o);
    pfg_resolve_options(&c.o);
    if (c.o.bce_en || c.o.proof_en) { c.err = "BCE and proof emission are not supported"; }
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) { cudaGetLastError(); delete o; return PFG_CUDA_ERROR; }
    c.device = dev;
    if (cudaStreamCreateWithFlags(&c.s, cudaStreamNonBlocking) != cudaSuccess) { cudaGetLastError(); delete o; return PFG_CUDA_ERROR; }
    cudaEventCreate(&c.ev_begin); cudaEventCreate(&c.ev_end); cudaEventCreate(&c.ev_a); cudaEventCreate(&c.ev_b);
    // keep freed blocks in the device pool: the pool is the engine's arena
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
        uint64_t thr = UINT64_MAX;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
    }
    if (cudaMallocHost((void**)&c.hc, sizeof(DevCounters)) != cudaSuccess) { cudaGetLastError(); delete o; return PFG_CUDA_ERROR; }
    std::memset(c.hc, 0, sizeof(DevCounters));
    if (arena_bytes == 0) {
        size_t fr = 0, tot = 0;
        if (cudaMemGetInfo(&fr, &tot) == cudaSuccess && fr > (256ull << 20)) o->budget = fr - (256ull << 20);
    } else {
        o->budget = arena_bytes;
    }
    if (c.o.bce_en || c.o.proof_en) {
        cudaFreeHost(c.hc);
        cudaStreamDestroy(c.s);
        delete o;
        return PFG_INVALID;
    }
    *out = o;
    return PFG_OK;
}

extern "C" const char* pfg_last_error(pfg_ctx* o) {
    if (!o) return "null context";
    return o->c.err.c_str();
}

extern "C" uint64_t pfg_kernel_launches(pfg_ctx* o) { return o ? o->c.launches : 0; }

extern "C" int pfg_upload(pfg_ctx* o, uint32_t max_var, uint64_t num_clauses, const uint32_t* lits,
                          const uint64_t* cls_off, const uint8_t* cls_learnt, const uint32_t* cls_lbd,
                          const uint8_t* cls_usage, const uint8_t* var_state, const uint8_t* assumed,
                          const uint32_t* vorg) {
    if (!o) return PFG_INVALID;
    Ctx& c = o->c;
    c.err.clear();
    if (max_var == 0 || max_var > 0x7FFFFFF0u || (num_clauses && (!lits || !cls_off))) { c.err = "invalid arguments"; return PFG_INVALID; }
    // validate on the host: literal range, clause size >= 2, no duplicate or complementary literals
    const uint64_t nlits = num_clauses ? cls_off[num_clauses] : 0;
    if (num_clauses && cls_off[0] != 0) { c.err = "cls_off[0] must be 0"; return PFG_INVALID; }
    {
        std::vector<uint64_t> seen(max_var + 1, ~0ull);
        for (uint64_t i = 0; i < num_clauses; i++) {
            const uint64_t b = cls_off[i], e = cls_off[i + 1];
            if (e < b + 2 || e > nlits) { c.err = "clause " + std::to_string(i) + " has fewer than 2 literals"; return PFG_INVALID; }
            for (uint64_t k = b; k < e; k++) {
                const uint32_t l = lits[k], v = l >> 1;
                if (v == 0 || v > max_var) { c.err = "literal out of range in clause " + std::to_string(i); return PFG_INVALID; }
                if (seen[v] == i) { c.err = "repeated variable in clause " + std::to_string(i); return PFG_INVALID; }
                seen[v] = i;
            }
        }
    }
    const uint64_t base_launches = g_launches;
    free_all(o);
    g_prof = &c.prof;
    c.V = max_var;
    c.nlist = 2ull * max_var + 2;
    uint64_t orgCls = 0, orgLits = 0;
    for (uint64_t i = 0; i < num_clauses; i++) {
        if (!(cls_learnt && cls_learnt[i])) { orgCls++; orgLits += cls_off[i + 1] - cls_off[i]; }
    }
    c.orig_cls = orgCls;
    c.orig_lits = orgLits;
    c.numClauses = num_clauses;
    c.numLiterals = nlits;
    c.ncls = num_clauses;
    c.lits_used = nlits;
    // capacities of awaken (simplify.cu:83-98)
    uint64_t numCls = num_clauses, numLits = nlits;
    if (c.o.phases) {
        numCls += c.o.ve_en ? orgCls : 0;
        numLits += c.o.ve_en ? (uint64_t)((double)orgLits * c.o.lits_mul) : 0;
    }
    c.cs_cap = numCls;
    c.data_cap = numCls * NBUCKETS + numLits;
    c.data_size = num_clauses * NBUCKETS + nlits;
    c.hdr_cap = numCls + 1;
    c.lits_cap = c.data_cap - NBUCKETS * num_clauses + 64;
    if (c.lits_cap > 0xFFFFFFF0ull || c.nlist > 0xFFFFFFF0ull) { c.err = "instance exceeds 2^32 literals"; return PFG_CNFALLOC_FAIL; }
    const uint64_t V1 = (uint64_t)max_var + 1;
    c.units_cap = (uint32_t)std::min<uint64_t>(2 * V1 + 1024, 0xFFFFFFF0ull);
    c.trail_cap = (uint32_t)V1;
    c.stack_cap = 2 * (numCls + numLits) + 1024;
    bool ok = cudaMallocAsync((void**)&c.dc, sizeof(DevCounters), c.s) == cudaSuccess;
    if (ok) { o->sizes[c.dc] = sizeof(DevCounters); o->allocated += sizeof(DevCounters); }
    ok = ok && dalloc_t(c, &c.hdr, c.hdr_cap) && dalloc_t(c, &c.lits, c.lits_cap) &&
         dalloc_t(c, &c.hist, c.nlist) && dalloc_t(c, &c.ot_off, c.nlist + 1) &&
         dalloc_t(c, &c.ot_size, c.nlist) && dalloc_t(c, &c.ot_fill, c.nlist) &&
         dalloc_t(c, &c.big_lists, c.nlist) &&
         dalloc_t(c, &c.elim, V1 + 8) && dalloc_t(c, &c.vstate, V1 + 8) && dalloc_t(c, &c.frozen, V1 + 8) &&
         dalloc_t(c, &c.mstate, V1 + 8) && dalloc_t(c, &c.flag8, V1 + 8) && dalloc_t(c, &c.bstate, V1 + 8) &&
         dalloc_t(c, &c.vorg, V1) && dalloc_t(c, &c.scores, V1) && dalloc_t(c, &c.keys_a, V1) &&
         dalloc_t(c, &c.keys_b, V1) && dalloc_t(c, &c.eligible, V1) && dalloc_t(c, &c.eligible_b, V1) &&
         dalloc_t(c, &c.rank, V1) && dalloc_t(c, &c.varcore, V1) && dalloc_t(c, &c.elected, V1) &&
         dalloc_t(c, &c.work, V1) && dalloc_t(c, &c.work_b, V1) && dalloc_t(c, &c.vscan, V1 + 1) &&
         dalloc_t(c, &c.winv, V1 + 8) &&
         dalloc_t(c, &c.type, V1) && dalloc_t(c, &c.ucnt, V1) && dalloc_t(c, &c.rpos, V1) &&
         dalloc_t(c, &c.rref, V1) && dalloc_t(c, &c.units, c.units_cap) && dalloc_t(c, &c.trail, c.trail_cap) &&
         dalloc_t(c, &c.stack, c.stack_cap) && dalloc_t(c, &c.front_a, V1) && dalloc_t(c, &c.front_b, V1);
    if (assumed) ok = ok && dalloc_t(c, &c.assumed, V1 + 8);
    if (!ok) {
        if (c.err.empty()) c.err = "device allocation failed";
        free_all(o);
        return PFG_CNFALLOC_FAIL;
    }
    // H2D: literals are already packed by cls_off
    unsigned long long* d_off = nullptr;
    uint8_t* d_learnt = nullptr;
    uint32_t* d_lbd = nullptr;
    uint8_t* d_usage = nullptr;
    ok = dalloc_t(c, &d_off, num_clauses + 1);
    if (ok && cls_learnt) ok = dalloc_t(c, &d_learnt, num_clauses + 1);
    if (ok && cls_lbd) ok = dalloc_t(c, &d_lbd, num_clauses + 1);
    if (ok && cls_usage) ok = dalloc_t(c, &d_usage, num_clauses + 1);
    if (!ok) { free_all(o); return PFG_CNFALLOC_FAIL; }
    cudaMemcpyAsync(c.lits, lits, nlits * sizeof(uint32_t), cudaMemcpyHostToDevice, c.s);
    cudaMemcpyAsync(d_off, cls_off, (num_clauses + 1) * sizeof(uint64_t), cudaMemcpyHostToDevice, c.s);
    if (cls_learnt) cudaMemcpyAsync(d_learnt, cls_learnt, num_clauses, cudaMemcpyHostToDevice, c.s);
    if (cls_lbd) cudaMemcpyAsync(d_lbd, cls_lbd, num_clauses * sizeof(uint32_t), cudaMemcpyHostToDevice, c.s);
    if (cls_usage) cudaMemcpyAsync(d_usage, cls_usage, num_clauses, cudaMemcpyHostToDevice, c.s);
    if (num_clauses) {
        PFG_LAUNCH(K_UPLOAD, init_hdr_k, grid_for(num_clauses, 256), 256, 0, c.s, c.hdr, d_off, num_clauses, d_learnt, d_lbd, d_usage);
        PFG_LAUNCH(K_UPLOAD, prep_k, grid_for(num_clauses, 128), 128, 0, c.s, c.hdr, c.lits, num_clauses);
    }
    if (var_state) cudaMemcpyAsync(c.vstate, var_state, V1, cudaMemcpyHostToDevice, c.s);
    else cudaMemsetAsync(c.vstate, 0, V1, c.s);
    if (assumed) cudaMemcpyAsync(c.assumed, assumed, V1, cudaMemcpyHostToDevice, c.s);
    if (vorg) cudaMemcpyAsync(c.vorg, vorg, V1 * sizeof(uint32_t), cudaMemcpyHostToDevice, c.s);
    else { PFG_LAUNCH(K_UPLOAD, identity_k, grid_for(V1, 256), 256, 0, c.s, c.vorg, (uint32_t)V1); }
    cudaMemsetAsync(c.elim, 0, V1, c.s);
    cudaMemsetAsync(c.varcore, 0, V1 * sizeof(uint32_t), c.s);
    cudaMemsetAsync(c.dc, 0, sizeof(DevCounters), c.s);
    dfree(c, d_off); dfree(c, d_learnt); dfree(c, d_lbd); dfree(c, d_usage);
    sync_counters(c);
    c.launches += g_launches - base_launches;
    g_prof = nullptr;
    if (!c.err.empty()) return PFG_CUDA_ERROR;
    c.uploaded = true;
    c.simplified = false;
    c.round_ends.clear();
    c.nUnits = 0;
    c.stats = pfg_stats{};
    c.stats.clauses_in = num_clauses;
    c.stats.literals_in = nlits;
    return PFG_OK;
}

static int finish(Ctx& c, pfg_stats* st, uint64_t base_launches, int rc) {
    if (c.prof.on) c.prof.resolve();
    g_prof = nullptr;
    c.launches += g_launches - base_launches;
    if (st) *st = c.stats;
    return rc;
}

extern "C" int pfg_simplify(pfg_ctx* o, pfg_stats* st) {
    if (!o) return PFG_INVALID;
    Ctx& c = o->c;
    if (!c.uploaded) { c.err = "no instance uploaded"; return PFG_INVALID; }
    if (c.simplified) { c.err = "instance already simplified; upload again"; return PFG_INVALID; }
    const uint64_t base_launches = g_launches;
    g_prof = &c.prof;
    c.err.clear();
    for (double& x : c.pass_ms) x = 0;
    c.phase = c.multiplier = c.simpstate = 0;
    c.status = PFG_UNKNOWN;
    c.varcore_on = c.o.ve_fun_en != 0;
    cudaEventRecord(c.ev_begin, c.s);
    uint64_t alg = 0;
    const bool disabled = !c.o.phases && !(c.o.all_en | c.o.ere_en);   // alldisabled (solver.hpp:722)
    if (!disabled && c.orig_cls) {
        int64_t cdiff = INT64_MAX, ldiff = INT64_MAX;
        int64_t clsbefore = (int64_t)c.numClauses, litsbefore = (int64_t)c.numLiterals;
        while (c.numClauses && c.numLiterals && !c.simpstate) {
            const int times = c.phase + 1;
            if (times > 1 && times != c.o.phases && c.o.shrink_rate > 0 && (times % c.o.shrink_rate) == 0) {
                PassTimer t(c, 6);
                if (!compact_cnf(c)) break;
            }
            {
                PassTimer t(c, 0);
                if (!ot_build(c)) break;
            }
            if (c.nUnits) {
                PassTimer t(c, 1);
                bool ok = true;
                if (!bcp_prop(c, ok)) break;
                if (!ok) { c.status = PFG_UNSAT; break; }
                count_live(c);
                sync_counters(c);
                c.numClauses = c.hc->live_cls;
                c.numLiterals = c.hc->live_lits;
                if (!ot_build(c)) break;
                cudaMemsetAsync(&c.dc->nunits, 0, sizeof(uint32_t), c.s);
                c.nUnits = 0;
            }
            if (!c.numClauses) break;
            {
                PassTimer t(c, 2);
                if (!c.o.lcve_fast && !ot_sort(c, true)) break;
                if (!lcve(c)) break;
            }
            if (c.nelected < c.o.lcve_min_vars) break;
            {
                PassTimer t(c, 0);
                if (!ot_sort(c, false)) break;
            }
            // stop() (solver.hpp:748-753)
            if (c.phase == c.o.phases || (cdiff == 0 && ldiff == 0) ||
                (c.phase > 2 && ldiff <= (int64_t)c.o.phase_lits_min)) {
                if (c.o.ere_en && c.nelected) {
                    cudaMemsetAsync(&c.dc->live_cls, 0, 2 * sizeof(unsigned long long), c.s);
                    PFG_LAUNCH(K_MISC, elected_volume_k, grid_for(c.nelected, 256), 256, 0, c.s, c.elected, c.nelected,
                               c.hdr, c.ot_off, c.ot_size, c.ot_ids, &c.dc->live_cls);
                    sync_counters(c);
                    c.prof.bytes[K_ERE] += 4 * (c.hc->live_cls + c.hc->live_lits);
                    PassTimer t(c, 5);
                    ere_pass(c);
                    c.stats.ere_ran = 1;
                }
                break;
            }
            // byte model: C_E, L_E of this round
            cudaMemsetAsync(&c.dc->live_cls, 0, 2 * sizeof(unsigned long long), c.s);
            PFG_LAUNCH(K_MISC, elected_volume_k, grid_for(c.nelected, 256), 256, 0, c.s, c.elected, c.nelected, c.hdr, c.ot_off,
                                                                         c.ot_size, c.ot_ids, &c.dc->live_cls);
            sync_counters(c);
            const uint64_t CE = c.hc->live_cls, LE = c.hc->live_lits;
            const uint64_t Cin = c.numClauses, Lin = c.numLiterals;
            c.prof.bytes[K_SUB] += 4 * (LE + CE);
            c.prof.bytes[K_VE1] += 4 * (LE + CE);
            const uint64_t ncls0 = c.ncls, lits0 = c.lits_used;
            c.stats.clauses_processed += Cin;
            c.stats.literals_processed += Lin;
            if (c.o.sub_en || c.o.ve_plus_en) {
                PassTimer t(c, 3);
                sub_pass(c);
            }
            if (c.o.ve_en) {
                PassTimer t(c, 4);
                if (!ve_pass(c)) break;
            }
            {
                PassTimer t(c, 6);
                count_live(c);
                sync_counters(c);
            }
            c.round_ends.push_back(c.hc->nstack);
            c.numClauses = c.hc->live_cls;
            c.numLiterals = c.hc->live_lits;
            c.nUnits = c.hc->nunits;
            const uint64_t Cres = c.ncls - ncls0, Lres = c.lits_used - lits0;
            c.stats.resolvents += Cres;
            c.prof.bytes[K_VE3] += 4 * (LE + CE) + 4 * (Lres + Cres);
            alg += 4 * (Lin + Cin) + 8 * Lin + 8 * (LE + CE) + 4 * (Lres + Cres) + 4 * (c.numLiterals + c.numClauses);
            cdiff = clsbefore - (int64_t)c.numClauses; clsbefore = (int64_t)c.numClauses;
            ldiff = litsbefore - (int64_t)c.numLiterals; litsbefore = (int64_t)c.numLiterals;
            c.phase++; c.multiplier++;
            c.multiplier += (c.phase == c.o.phases);
            if (!c.err.empty()) break;
        }
        if (c.err.empty()) {   // ERE deletes after the last count (the write-back recounts, cnf.cu:211-224)
            count_live(c);
            sync_counters(c);
            c.numClauses = c.hc->live_cls;
            c.numLiterals = c.hc->live_lits;
        }
        if (c.status != PFG_UNSAT && c.err.empty() && !c.numClauses) c.status = PFG_SAT;
    }
    cudaEventRecord(c.ev_end, c.s);
    sync_counters(c);
    float ms = 0;
    cudaEventElapsedTime(&ms, c.ev_begin, c.ev_end);
    c.simplified = true;
    c.stats.status = c.status;
    c.stats.rounds = c.phase;
    c.stats.simpstate = c.simpstate;
    c.stats.clauses_out = c.numClauses;
    c.stats.literals_out = c.numLiterals;
    c.stats.stack_words = c.hc->nstack;
    c.stats.device_ms = ms;
    for (int i = 0; i < 8; i++) c.stats.pass_ms[i] = c.pass_ms[i];
    c.stats.alg_bytes = alg;
    c.stats.kernel_launches = g_launches - base_launches;
    // eliminated / forced counts are filled in by pfg_download's host copy; compute here cheaply
    {
        std::vector<uint8_t> el(c.V + 1);
        cudaMemcpyAsync(el.data(), c.elim, c.V + 1, cudaMemcpyDeviceToHost, c.s);
        cudaStreamSynchronize(c.s);
        uint64_t ne = 0, nf = 0;
        for (uint32_t v = 1; v <= c.V; v++) {
            if (el[v] & FORCED_MASK) nf++;
            else if (el[v]) ne++;
        }
        c.stats.eliminated = ne;
        c.stats.forced = nf;
    }
    int rc = PFG_OK;
    if (!c.err.empty()) rc = (c.simpstate == PFG_TIMEOUT) ? PFG_TIMEOUT : (c.simpstate ? c.simpstate : PFG_CUDA_ERROR);
    else if (c.simpstate) rc = c.simpstate;
    return finish(c, st, base_launches, rc);
}

extern "C" int pfg_result_sizes_get(pfg_ctx* o, pfg_result_sizes* r) {
    if (!o || !r) return PFG_INVALID;
    Ctx& c = o->c;
    if (!c.uploaded) return PFG_INVALID;
    std::memset(r, 0, sizeof(*r));
    sync_counters(c);
    r->clauses = c.numClauses;
    r->literals = c.numLiterals;
    r->units = c.hc->ntrail;
    r->pending_units = c.nUnits ? std::min<uint64_t>(c.hc->nunits, c.units_cap) : 0;
    r->stack_words = c.hc->nstack;
    r->rounds = c.round_ends.size();
    r->max_var = c.V;
    return PFG_OK;
}

extern "C" int pfg_download(pfg_ctx* o, uint32_t* lits, uint64_t* cls_off, uint8_t* cls_learnt, uint32_t* cls_lbd,
                            uint8_t* cls_usage, uint8_t* eliminated, uint32_t* units, uint32_t* pending_units,
                            uint32_t* stack, uint64_t* round_ends) {
    if (!o) return PFG_INVALID;
    Ctx& c = o->c;
    if (!c.uploaded) return PFG_INVALID;
    const uint64_t base_launches = g_launches;
    g_prof = &c.prof;
    sync_counters(c);
    const uint64_t n = c.ncls;
    if (lits || cls_off || cls_learnt || cls_lbd || cls_usage) {
        uint32_t* flag = nullptr;
        unsigned long long* sz = nullptr;
        uint32_t* olits = nullptr;
        unsigned long long* ooff = nullptr;
        uint8_t* olearnt = nullptr;
        uint32_t* olbd = nullptr;
        uint8_t* ousage = nullptr;
        const uint64_t C = c.numClauses, L = c.numLiterals;
        bool ok = dalloc_t(c, &flag, n + 1) && dalloc_t(c, &sz, n + 1) && dalloc_t(c, &olits, L + 1) &&
                  dalloc_t(c, &ooff, C + 1) && dalloc_t(c, &olearnt, C + 1) && dalloc_t(c, &olbd, C + 1) &&
                  dalloc_t(c, &ousage, C + 1) && ensure_tmp(c, scan_temp_bytes(n + 1));
        if (!ok) { dfree(c, flag); dfree(c, sz); dfree(c, olits); dfree(c, ooff); dfree(c, olearnt); dfree(c, olbd); dfree(c, ousage); return PFG_CNFALLOC_FAIL; }
        if (n) {
            PFG_LAUNCH(K_DOWNLOAD, out_flags_k, grid_for(n, 256), 256, 0, c.s, c.hdr, n, flag, sz);
            exclusive_scan_u32(flag, flag, n, 0u, nullptr, c.tmp, c.s);
            exclusive_scan_u64(sz, sz, n, 0ull, ooff + C, c.tmp, c.s);
            PFG_LAUNCH(K_DOWNLOAD, out_pack_k, grid_for(n * 32, 256), 256, 0, c.s, c.hdr, c.lits, n, flag, sz, olits, ooff, olearnt, olbd, ousage);
        } else {
            cudaMemsetAsync(ooff, 0, sizeof(unsigned long long), c.s);
        }
        if (lits) cudaMemcpyAsync(lits, olits, L * sizeof(uint32_t), cudaMemcpyDeviceToHost, c.s);
        if (cls_off) cudaMemcpyAsync(cls_off, ooff, (C + 1) * sizeof(uint64_t), cudaMemcpyDeviceToHost, c.s);
        if (cls_learnt) cudaMemcpyAsync(cls_learnt, olearnt, C, cudaMemcpyDeviceToHost, c.s);
        if (cls_lbd) cudaMemcpyAsync(cls_lbd, olbd, C * sizeof(uint32_t), cudaMemcpyDeviceToHost, c.s);
        if (cls_usage) cudaMemcpyAsync(cls_usage, ousage, C, cudaMemcpyDeviceToHost, c.s);
        dfree(c, flag); dfree(c, sz); dfree(c, olits); dfree(c, ooff); dfree(c, olearnt); dfree(c, olbd); dfree(c, ousage);
    }
    if (eliminated) cudaMemcpyAsync(eliminated, c.elim, c.V + 1, cudaMemcpyDeviceToHost, c.s);
    if (units && c.hc->ntrail) cudaMemcpyAsync(units, c.trail, c.hc->ntrail * sizeof(uint32_t), cudaMemcpyDeviceToHost, c.s);
    const uint64_t npend = c.nUnits ? std::min<uint64_t>(c.hc->nunits, c.units_cap) : 0;
    if (pending_units && npend) cudaMemcpyAsync(pending_units, c.units, npend * sizeof(uint32_t), cudaMemcpyDeviceToHost, c.s);
    if (stack && c.hc->nstack) cudaMemcpyAsync(stack, c.stack, c.hc->nstack * sizeof(uint32_t), cudaMemcpyDeviceToHost, c.s);
    if (!cuda_ok(c, cudaStreamSynchronize(c.s), "download")) return finish(c, nullptr, base_launches, PFG_CUDA_ERROR);
    if (units && c.hc->ntrail) std::sort(units, units + c.hc->ntrail);
    if (pending_units && npend) std::sort(pending_units, pending_units + npend);
    if (round_ends) for (size_t i = 0; i < c.round_ends.size(); i++) round_ends[i] = c.round_ends[i];
    return finish(c, nullptr, base_launches, PFG_OK);
}

extern "C" int pfg_profile_enable(pfg_ctx* o, int on) {
    if (!o) return PFG_INVALID;
    o->c.prof.on = on != 0;
    return PFG_OK;
}

extern "C" void pfg_profile_reset(pfg_ctx* o) {
    if (o) o->c.prof.reset();
}

extern "C" int pfg_profile_count(void) { return K_NUM; }

extern "C" const char* pfg_profile_name(int id) { return (id >= 0 && id < K_NUM) ? kKernelNames[id] : ""; }

extern "C" int pfg_profile_get(pfg_ctx* o, int id, uint64_t* launches, double* ms, uint64_t* alg_bytes) {
    if (!o || id < 0 || id >= K_NUM) return PFG_INVALID;
    if (launches) *launches = o->c.prof.launches[id];
    if (ms) *ms = o->c.prof.ms[id];
    if (alg_bytes) *alg_bytes = o->c.prof.bytes[id];
    return PFG_OK;
}

extern "C" void pfg_destroy(pfg_ctx* o) {
    if (!o) return;
    Ctx& c = o->c;
    std::vector<void*> ptrs;
    for (auto& kv : o->sizes) ptrs.push_back(kv.first);
    for (void* p : ptrs) cudaFreeAsync(p, c.s);
    if (c.s) { cudaStreamSynchronize(c.s); cudaStreamDestroy(c.s); }
    if (c.ev_begin) cudaEventDestroy(c.ev_begin);
    if (c.ev_end) cudaEventDestroy(c.ev_end);
    if (c.ev_a) cudaEventDestroy(c.ev_a);
    if (c.ev_b) cudaEventDestroy(c.ev_b);
    if (c.hc) cudaFreeHost(c.hc);
    c.prof.destroy();
    cudaGetLastError();
    delete o;
}
