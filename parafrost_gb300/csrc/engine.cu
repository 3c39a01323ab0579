// C-ABI and round driver of the GB300 CNF inprocessing engine.
//
// pfg_upload / pfg_batch_upload replace Solver::awaken (src/gpu/simplify.cu:77-134),
// pfg_simplify the round loop of Solver::simplifying (simplify.cu:159-186),
// pfg_download / pfg_batch_download the write-back (cacheCNF cnf.cu:200-236,
// cacheEliminated transfer.cu:69, cacheResolved transfer.cu:83).
#include <algorithm>
#include <atomic>
#include <cstdio>
#include <cstring>
#include <thread>
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

unsigned sm_count() {
    static const unsigned n = [] {
        int dev = 0, sms = 0;
        cudaGetDevice(&dev);
        if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
            cudaGetLastError();
            sms = 152;
        }
        return (unsigned)std::max(1, sms);
    }();
    return n;
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

// The host waits by polling the stream: the round loop waits for a few bytes
// of counters dozens of times per call, and waking a blocked thread cost more
// than the device work between two such waits.
bool stream_sync(Ctx& c, const char* what) {
    if (c.prof.on) c.prof.close();
    cudaError_t e;
    while ((e = cudaStreamQuery(c.s)) == cudaErrorNotReady) {}
    return cuda_ok(c, e, what);
}

void sync_counters(Ctx& c) {
    cudaMemcpyAsync(c.hc, c.dc, sizeof(DevCounters), cudaMemcpyDeviceToHost, c.s);
    stream_sync(c, "stream synchronize");
    if (c.err.empty() && c.hc->err) {
        char b[128];
        snprintf(b, sizeof(b), "device error flags 0x%x", c.hc->err);
        c.err = b;
    }
}

static size_t align_up(size_t x) { return (x + 255) & ~(size_t)255; }

template <typename T>
static void place(char* base, size_t& off, T** p, size_t count) {
    if (p) *p = base ? reinterpret_cast<T*>(base + off) : nullptr;
    off = align_up(off + count * sizeof(T));
}

size_t inst_in_layout(uint32_t n, char* base, InstIn* p) {
    InstIn dummy;
    InstIn& q = p ? *p : dummy;
    size_t off = 0;
    place(base, off, &q.voff, n + 1);
    place(base, off, &q.seg, n + 1);
    place(base, off, &q.ucap, n);
    place(base, off, &q.tcap, n);
    place(base, off, &q.ubase, n);
    place(base, off, &q.tbase, n);
    place(base, off, &q.sbase, n);
    place(base, off, &q.scap, n);
    place(base, off, &q.acc, 4 * (size_t)n);
    place(base, off, &q.active, n);
    place(base, off, &q.vc_on, n);
    place(base, off, &q.bcp, n);
    place(base, off, &q.mode, n);
    return off;
}

size_t inst_out_layout(uint32_t n, char* base, InstOut* p) {
    InstOut dummy;
    InstOut& q = p ? *p : dummy;
    size_t off = 0;
    place(base, off, &q.conflict, n);
    place(base, off, &q.ucount, n);
    place(base, off, &q.tcount, n);
    place(base, off, &q.nelect, n);
    place(base, off, &q.nfrozen, n);
    place(base, off, &q.fbase, n + 1);
    place(base, off, &q.scount, n);
    place(base, off, &q.cnt, 2 * (size_t)n);
    place(base, off, &q.add, 2 * (size_t)n);
    return off;
}

void push_inst_in(Ctx& c) {
    // the pinned mirror may be rewritten right after this call: wait for the copy
    cudaMemcpyAsync(c.di.voff, c.hi.voff, c.in_bytes, cudaMemcpyHostToDevice, c.s);
    stream_sync(c, "instance inputs");
}

void pull_inst_out(Ctx& c) {
    cudaMemcpyAsync(c.hout.conflict, c.dout.conflict, c.out_bytes, cudaMemcpyDeviceToHost, c.s);
    sync_counters(c);
}

// ---- DRAT proof of a pass (the device side of cuPROOF, src/gpu/proof.cu:184-246) ----
bool proof_prepare(Ctx& c, unsigned long long words) {
    words += 64;
    if (words > c.pf_wcap) {
        dfree(c, c.pf_w);
        dfree(c, c.pf_b);
        c.pf_w = nullptr; c.pf_b = nullptr; c.pf_wcap = 0; c.pf_bcap = 0;
        const unsigned long long cap = words + words / 4;
        const unsigned long long bcap = cap / 2 + 1;   // a block holds a line: 2 words at least
        if (bcap > 0xFFFFFFFFull) { c.err = "proof block table exceeds 2^32 entries"; return false; }
        if (!dalloc_t(c, &c.pf_w, cap) || !dalloc_t(c, &c.pf_b, bcap)) return false;
        c.pf_wcap = cap;
        c.pf_bcap = (uint32_t)bcap;
    }
    cudaMemsetAsync(&c.dc->pf_words, 0, sizeof(unsigned long long), c.s);
    cudaMemsetAsync(&c.dc->pf_blocks, 0, sizeof(uint32_t), c.s);
    return true;
}

// The pass's blocks in (variable, sequence) order; each line becomes 'a' or 'd',
// its literals as 7-bit groups (saveProofLiteral, proofutils.cuh:93-111), and a
// zero byte, appended to the proof of the variable's instance.
bool proof_collect(Ctx& c) {
    sync_counters(c);
    if (!c.err.empty()) return false;
    const unsigned long long nw = c.hc->pf_words;
    const uint32_t nb = c.hc->pf_blocks;
    if (!nb) return true;
    c.pf_hw.resize(nw);
    c.pf_hb.resize(nb);
    cudaMemcpyAsync(c.pf_hw.data(), c.pf_w, nw * sizeof(uint32_t), cudaMemcpyDeviceToHost, c.s);
    cudaMemcpyAsync(c.pf_hb.data(), c.pf_b, nb * sizeof(ulonglong2), cudaMemcpyDeviceToHost, c.s);
    if (!stream_sync(c, "proof copy")) return false;
    // blocks tile [0, nw) in reservation order: their ends are the next starts
    std::vector<ulonglong2>& b = c.pf_hb;
    std::sort(b.begin(), b.end(), [](const ulonglong2& a, const ulonglong2& z) { return a.y < z.y; });
    std::vector<std::pair<unsigned long long, std::pair<unsigned long long, unsigned long long>>> blk(nb);
    for (uint32_t i = 0; i < nb; i++) blk[i] = {b[i].x, {b[i].y, i + 1 < nb ? b[i + 1].y : nw}};
    std::sort(blk.begin(), blk.end());
    uint32_t inst = 0;
    for (const auto& e : blk) {
        const uint32_t x = (uint32_t)(e.first >> 32);
        while (inst + 1 < c.ninst && c.ih[inst + 1].voff < x) inst++;
        std::vector<uint8_t>& out = c.ih[inst].proof;
        for (unsigned long long w = e.second.first; w < e.second.second;) {
            const uint32_t h = c.pf_hw[w];
            if (!h) { w++; continue; }                    // padding
            const uint32_t n = h & 0x7FFFFFFFu;
            if (w + 1 + n > e.second.second) { c.err = "malformed proof block"; return false; }
            out.push_back((h >> 31) ? PROOF_DELETED : PROOF_ADDED);
            for (uint32_t t = 0; t < n; t++) {
                uint32_t v = c.pf_hw[w + 1 + t];
                while (v >= 0x80u) { out.push_back((uint8_t)((v & 0x7Fu) | 0x80u)); v >>= 7; }
                out.push_back((uint8_t)v);
            }
            out.push_back(0);
            w += 1 + n;
        }
    }
    return true;
}

namespace {

// Offsets of every uploaded clause: the first clause of an instance starts at
// 0, every clause ends at least 2 literals after its start and no later than
// the instance's literal count. The smallest failing clause lands in *bad.
__global__ void check_off_k(const unsigned long long* off, uint64_t ncls, const unsigned long long* clsbase,
                            const unsigned long long* litbase, uint32_t ninst, unsigned long long* bad) {
    for (uint64_t c = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; c < ncls; c += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t lo = 0, hi = ninst;
        while (hi - lo > 1) {
            const uint32_t mid = (lo + hi) >> 1;
            if (clsbase[mid] <= c) lo = mid; else hi = mid;
        }
        const uint64_t L = litbase[lo + 1] - litbase[lo];
        const uint64_t b = off[c];
        const uint64_t e = (c + 1 < clsbase[lo + 1]) ? off[c + 1] : L;
        if ((c == clsbase[lo] && b != 0) || e < b + 2 || e > L) atomicMin(bad, (unsigned long long)c);
    }
}

// header of every uploaded clause; literals moved to their instance's variable range
__global__ void init_hdr_k(ClsHdr* hdr, const unsigned long long* off, uint64_t ncls, const uint8_t* learnt,
                           const uint32_t* lbd, const uint8_t* usage, const unsigned long long* clsbase,
                           const unsigned long long* litbase, const uint32_t* voff, uint32_t ninst,
                           const uint32_t* vmax, uint32_t* lits, unsigned long long* bad) {
    for (uint64_t c = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; c < ncls; c += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t lo = 0, hi = ninst;   // largest i with clsbase[i] <= c
        while (hi - lo > 1) {
            const uint32_t mid = (lo + hi) >> 1;
            if (clsbase[mid] <= c) lo = mid; else hi = mid;
        }
        const uint32_t inst = lo;
        const uint64_t b = off[c] + litbase[inst];
        const uint64_t e = (c + 1 < clsbase[inst + 1]) ? off[c + 1] + litbase[inst] : litbase[inst + 1];
        ClsHdr h;
        h.off = (uint32_t)b;
        h.size = (uint32_t)(e - b);
        h.sig = 0;
        const bool l = learnt && learnt[c];
        h.meta = l ? m_make(ST_LEARNT, 0, 0, usage ? (usage[c] & 3u) : 0u, lbd ? (lbd[c] & 0x03FFFFFFu) : 0u)
                   : m_make(ST_ORIGINAL, 0, 0, 0, 0);
        hdr[c] = h;
        const uint32_t shift = 2u * voff[inst], vm = vmax[inst];
        bool ok = true;
        for (uint64_t k = b; k < e; k++) {
            const uint32_t v = lits[k] >> 1;
            ok &= v >= 1 && v <= vm;
            lits[k] += shift;
        }
        if (!ok) atomicMin(bad, (unsigned long long)c);
    }
}

// prep_cnf_k (cnf.cu:45-53): sort literals of every clause, compute its signature
// literals of every clause sorted, signature computed; a variable that occurs
// twice in a clause (repeated literal or a literal and its negation) lands in *bad
__global__ void prep_k(ClsHdr* hdr, uint32_t* lits, uint64_t ncls, unsigned long long* bad) {
    for (uint64_t c = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; c < ncls; c += (uint64_t)gridDim.x * blockDim.x) {
        const ClsHdr h = hdr[c];
        uint32_t* l = lits + h.off;
        for (uint32_t i = 1; i < h.size; i++) {
            const uint32_t t = l[i];
            uint32_t j = i;
            while (j > 0 && t < l[j - 1]) { l[j] = l[j - 1]; j--; }
            l[j] = t;
        }
        for (uint32_t i = 1; i < h.size; i++)
            if ((l[i] >> 1) == (l[i - 1] >> 1)) { atomicMin(bad, (unsigned long long)c); break; }
        if (h.size > 1) {
            uint32_t s = 0;
            for (uint32_t i = 0; i < h.size; i++) s |= MAPHASH(l[i]);
            hdr[c].sig = s;
        }
    }
}

// proof bytes of every literal: 7-bit groups of its original (cnt_proof, proof.cu:49-85)
__global__ void lbyte_k(const uint32_t* vorg, uint32_t V, uint8_t* lbyte) {
    for (uint64_t l = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; l < 2ull * V + 2;
         l += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t v = (uint32_t)(l >> 1);
        lbyte[l] = v ? (uint8_t)varint_len((vorg[v] << 1) | (uint32_t)(l & 1)) : 0u;
    }
}

// instance of every global variable, and its instance-local number (the default vorg)
__global__ void vinst_k(const uint32_t* voff, uint32_t ninst, uint32_t V, uint32_t* vinst, uint32_t* vorg) {
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v <= V; v += gridDim.x * blockDim.x) {
        const uint32_t i = v ? inst_search(voff, ninst, v) : 0u;
        vinst[v] = i;
        vorg[v] = v ? v - voff[i] : 0u;
    }
}

// sum of list sizes and literal counts over a variable set (C_E, L_E of the byte model)
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

// elected variables of the instances in `want` mode
__global__ void mode_flags_k(const uint32_t* elected, uint32_t n, const uint32_t* vinst, const uint8_t* mode,
                             uint8_t want, uint8_t* flag) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        flag[i] = mode[vinst[elected[i]]] == want;
}

// live clauses -> packed host layout (one instance)
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
            olearnt[q] = m_learnt(h.meta);
            olbd[q] = m_lbd(h.meta);
            ousage[q] = (uint8_t)m_usage(h.meta);
        }
    }
}

// batch write-back: live clauses keyed by instance (deleted ones after all instances)
__global__ void cls_inst_keys_k(const ClsHdr* hdr, const uint32_t* lits, uint64_t ncls, const uint32_t* vinst,
                                uint32_t ninst, uint32_t* keys, uint32_t* ids) {
    for (uint64_t c = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; c < ncls; c += (uint64_t)gridDim.x * blockDim.x) {
        const ClsHdr h = hdr[c];
        keys[c] = (m_deleted(h.meta) || !h.size) ? ninst : vinst[ABSV(lits[h.off])];
        ids[c] = (uint32_t)c;
    }
}

__global__ void gathered_sizes_k(const ClsHdr* hdr, const uint32_t* ids, uint64_t n, unsigned long long* sz) {
    for (uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; j < n; j += (uint64_t)gridDim.x * blockDim.x)
        sz[j] = hdr[ids[j]].size;
}

// thread per clause (clauses are short, and neighbouring threads read and
// write neighbouring ranges: the ids are sorted by instance, stably);
// literals back to the instance's own numbering
__global__ void gathered_pack_k(const ClsHdr* __restrict__ hdr, const uint32_t* __restrict__ lits,
                                const uint32_t* __restrict__ ids, const uint32_t* __restrict__ inst, uint64_t n,
                                const unsigned long long* __restrict__ loff, const uint32_t* __restrict__ voff,
                                uint32_t* olits, uint8_t* olearnt, uint32_t* olbd, uint8_t* ousage) {
    for (uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; j < n; j += (uint64_t)gridDim.x * blockDim.x) {
        const ClsHdr h = hdr[ids[j]];
        const uint32_t* l = lits + h.off;
        const uint32_t shift = 2u * voff[inst[j]];
        uint32_t* out = olits + loff[j];
        for (uint32_t k = 0; k < h.size; k++) out[k] = l[k] - shift;
        olearnt[j] = m_learnt(h.meta);
        olbd[j] = m_lbd(h.meta);
        ousage[j] = (uint8_t)m_usage(h.meta);
    }
}

// offsets relative to the instance: minus the instance's first packed literal
__global__ void relative_off_k(const uint32_t* inst_of, uint64_t n, const unsigned long long* lit_base,
                               unsigned long long* off) {
    for (uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; j < n; j += (uint64_t)gridDim.x * blockDim.x)
        off[j] -= lit_base[inst_of[j]];
}

void free_all(pfg_ctx* o) {
    Ctx& c = o->c;
    std::vector<void*> ptrs;
    for (auto& kv : o->sizes) ptrs.push_back(kv.first);
    for (void* p : ptrs) cudaFreeAsync(p, c.s);
    o->sizes.clear();
    o->allocated = 0;
    if (c.s) cudaStreamSynchronize(c.s);
    if (c.in_blob_h) cudaFreeHost(c.in_blob_h);
    if (c.out_blob_h) cudaFreeHost(c.out_blob_h);
    Ctx fresh;
    fresh.o = c.o;
    fresh.device = c.device;
    fresh.s = c.s;
    fresh.tune = c.tune;
    fresh.s_copy = c.s_copy; fresh.ev_copy = c.ev_copy;
    fresh.ev_begin = c.ev_begin; fresh.ev_end = c.ev_end;
    fresh.pass_clock = c.pass_clock;
    fresh.dc = nullptr; fresh.hc = c.hc;
    fresh.launches = c.launches;
    fresh.prof = c.prof;
    fresh.lim_bcp_levels = c.lim_bcp_levels;
    fresh.lim_mis_rounds = c.lim_mis_rounds;
    c = fresh;
}

// Device time of a pass: an event pair on the engine's stream, read when the
// call ends (pfg_simplify), so the host does not wait for the device after
// every pass.
struct PassTimer {
    Ctx& c;
    int slot;
    PassTimer(Ctx& cc, int s) : c(cc), slot(s) { c.pass_clock.begin(slot, c.s); }
    ~PassTimer() { c.pass_clock.end(slot, c.s); }
};

// Host checks of one instance (literal range, clause size >= 2, no duplicate or
// complementary literals); also counts its original clauses and literals.
// Host checks of one instance that cost O(1), plus its original (non-learnt)
// clause and literal counts (a pass over the learnt flags when there are any).
// Offsets, literal ranges and repeated variables are checked on the device
// while the clauses are prepared.
bool valid_instance(uint32_t idx, const pfg_instance& q, std::string& err, uint64_t& orig_cls, uint64_t& orig_lits) {
    const std::string who = "instance " + std::to_string(idx) + ": ";
    orig_cls = orig_lits = 0;
    if (q.max_var == 0 || q.max_var > 0x7FFFFFF0u || (q.num_clauses && (!q.lits || !q.cls_off))) {
        err = who + "invalid arguments";
        return false;
    }
    if (!q.num_clauses) return true;
    if (q.cls_off[0] != 0) { err = who + "cls_off[0] must be 0"; return false; }
    const uint64_t nlits = q.cls_off[q.num_clauses];
    if (!q.cls_learnt) { orig_cls = q.num_clauses; orig_lits = nlits; return true; }
    for (uint64_t i = 0; i < q.num_clauses; i++)
        if (!q.cls_learnt[i]) { orig_cls++; orig_lits += q.cls_off[i + 1] - q.cls_off[i]; }
    return true;
}
bool valid_instances(Ctx& c, uint32_t n, const pfg_instance* in, std::vector<uint64_t>& orig_cls,
                     std::vector<uint64_t>& orig_lits) {
    orig_cls.assign(n, 0);
    orig_lits.assign(n, 0);
    std::vector<std::string> errs(n);
    std::vector<uint8_t> ok(n, 1);
    std::atomic<uint32_t> next{0};
    auto work = [&]() {
        for (uint32_t i = next.fetch_add(1); i < n; i = next.fetch_add(1))
            ok[i] = valid_instance(i, in[i], errs[i], orig_cls[i], orig_lits[i]) ? 1 : 0;
    };
    const uint32_t hw = std::max(1u, std::thread::hardware_concurrency());
    const uint32_t nt = std::min<uint32_t>(n, std::min<uint32_t>(hw, 64));
    if (nt <= 1) {
        work();
    } else {
        std::vector<std::thread> th;
        for (uint32_t t = 0; t < nt; t++) th.emplace_back(work);
        for (std::thread& t : th) t.join();
    }
    for (uint32_t i = 0; i < n; i++)
        if (!ok[i]) { c.err = errs[i]; return false; }
    return true;
}

// Solver::awaken (simplify.cu:77-134) for n instances side by side
int upload_impl(pfg_ctx* o, uint32_t n, const pfg_instance* in) {
    Ctx& c = o->c;
    c.err.clear();
    if (n == 0 || !in) { c.err = "no instances"; return PFG_INVALID; }
    // Instance i owns global variables voff[i]+1 .. voff[i+1]. Every voff is a
    // multiple of 16, so a literal keeps its low 5 bits when it is moved into
    // the global range: clause signatures (1 << (lit & 31)) and with them the
    // occurrence-list order are the ones of the instance alone.
    uint64_t Vtot = 0, Ctot = 0, Ltot = 0;
    std::vector<uint64_t> voffs(n + 1, 0), orig_cls, orig_lits;
    if (!valid_instances(c, n, in, orig_cls, orig_lits)) return PFG_INVALID;
    for (uint32_t i = 0; i < n; i++) {
        Vtot = voffs[i] + in[i].max_var;
        voffs[i + 1] = (i + 1 < n) ? ((Vtot + 15) & ~15ull) : Vtot;
        Ctot += in[i].num_clauses;
        Ltot += in[i].num_clauses ? in[i].cls_off[in[i].num_clauses] : 0;
    }
    if (Vtot > 0x7FFFFFF0ull) { c.err = "total variables exceed 2^31"; return PFG_INVALID; }
    const uint64_t base_launches = g_launches;
    free_all(o);
    g_prof = &c.prof;
    c.ninst = n;
    c.ih.assign(n, InstHost{});
    c.V = (uint32_t)Vtot;
    c.nlist = 2ull * Vtot + 2;
    c.numClauses = Ctot;
    c.numLiterals = Ltot;
    c.ncls = Ctot;
    c.lits_used = Ltot;
    // per-instance capacities of awaken (simplify.cu:83-98)
    std::vector<unsigned long long> clsbase(n + 1), litbase(n + 1);
    std::vector<uint64_t> acc(4 * (size_t)n);
    std::vector<uint32_t> ucap(n), tcap(n);
    std::vector<unsigned long long> ubase(n), tbase(n), sbase(n), scap(n);
    uint64_t hdr_cap = 1, lits_cap = 64;
    bool any_learnt = false, any_lbd = false, any_usage = false, any_assumed = false;
    for (uint32_t i = 0; i < n; i++) {
        const pfg_instance& q = in[i];
        InstHost& h = c.ih[i];
        const uint64_t L = q.num_clauses ? q.cls_off[q.num_clauses] : 0;
        h.V = q.max_var;
        h.voff = (uint32_t)voffs[i];
        h.orig_cls = orig_cls[i];
        h.orig_lits = orig_lits[i];
        h.cls_in = h.numClauses = q.num_clauses;
        h.lits_in = h.numLiterals = L;
        clsbase[i + 1] = clsbase[i] + q.num_clauses;
        litbase[i + 1] = litbase[i] + L;
        uint64_t numCls = q.num_clauses, numLits = L;
        if (c.o.phases) {
            numCls += c.o.ve_en ? h.orig_cls : 0;
            numLits += c.o.ve_en ? (uint64_t)((double)h.orig_lits * c.o.lits_mul) : 0;
        }
        acc[4 * i + 0] = q.num_clauses;
        acc[4 * i + 1] = q.num_clauses * NBUCKETS + L;
        acc[4 * i + 2] = numCls;
        acc[4 * i + 3] = numCls * NBUCKETS + numLits;
        hdr_cap += numCls;
        lits_cap += acc[4 * i + 3] - NBUCKETS * q.num_clauses;
        const uint64_t V1 = (uint64_t)q.max_var + 1;
        ucap[i] = (uint32_t)std::min<uint64_t>(2 * V1 + 1024, 0xFFFFFFF0ull);
        ubase[i] = c.units_total; c.units_total += ucap[i];
        tcap[i] = (uint32_t)V1;
        tbase[i] = c.trail_total; c.trail_total += tcap[i];
        scap[i] = 2 * (numCls + numLits) + 1024;
        sbase[i] = c.stack_total; c.stack_total += scap[i];
        any_learnt |= q.cls_learnt != nullptr;
        any_lbd |= q.cls_lbd != nullptr;
        any_usage |= q.cls_usage != nullptr;
        any_assumed |= q.assumed != nullptr;
    }
    c.hdr_cap = hdr_cap;
    c.lits_cap = lits_cap;
    if (c.lits_cap > 0xFFFFFFF0ull || c.hdr_cap > 0xFFFFFFF0ull || c.nlist > 0xFFFFFFF0ull) {
        c.err = "instances exceed 2^32 literals";
        return PFG_CNFALLOC_FAIL;
    }
    // per-instance blobs (device + pinned mirror)
    c.in_bytes = inst_in_layout(n, nullptr, nullptr);
    c.out_bytes = inst_out_layout(n, nullptr, nullptr);
    if (cudaMallocHost(&c.in_blob_h, c.in_bytes) != cudaSuccess || cudaMallocHost(&c.out_blob_h, c.out_bytes) != cudaSuccess) {
        cudaGetLastError();
        c.err = "pinned host allocation failed";
        free_all(o);
        return PFG_CNFALLOC_FAIL;
    }
    std::memset(c.in_blob_h, 0, c.in_bytes);
    std::memset(c.out_blob_h, 0, c.out_bytes);
    inst_in_layout(n, (char*)c.in_blob_h, &c.hi);
    inst_out_layout(n, (char*)c.out_blob_h, &c.hout);
    const uint64_t V1 = Vtot + 1;
    void* din = nullptr;
    void* dout = nullptr;
    bool ok = cudaMallocAsync((void**)&c.dc, sizeof(DevCounters), c.s) == cudaSuccess;
    if (ok) { o->sizes[c.dc] = sizeof(DevCounters); o->allocated += sizeof(DevCounters); }
    ok = ok && dalloc(c, &din, c.in_bytes) && dalloc(c, &dout, c.out_bytes);
    if (ok) {
        inst_in_layout(n, (char*)din, &c.di);
        inst_out_layout(n, (char*)dout, &c.dout);
    }
    ok = ok && dalloc_t(c, &c.hdr, c.hdr_cap) && dalloc_t(c, &c.lits, c.lits_cap) &&
         dalloc_t(c, &c.hist, c.nlist) && dalloc_t(c, &c.ot_off, c.nlist + 1) &&
         dalloc_t(c, &c.ot_size, c.nlist) && dalloc_t(c, &c.ot_fill, c.nlist) &&
         dalloc_t(c, &c.big_lists, c.nlist) &&
         dalloc_t(c, &c.elim, V1 + 8) && dalloc_t(c, &c.vstate, V1 + 8) && dalloc_t(c, &c.frozen, V1 + 8) &&
         dalloc_t(c, &c.mstate, V1 + 8) && dalloc_t(c, &c.flag8, V1 + 8) && dalloc_t(c, &c.bstate, V1 + 8) &&
         dalloc_t(c, &c.vorg, V1) && dalloc_t(c, &c.vinst, V1) && dalloc_t(c, &c.scores, V1) &&
         dalloc_t(c, &c.keys_a, V1) && dalloc_t(c, &c.keys_b, V1) && dalloc_t(c, &c.eligible, V1) &&
         dalloc_t(c, &c.eligible_b, V1) && dalloc_t(c, &c.rank, V1) && dalloc_t(c, &c.varcore, V1) &&
         dalloc_t(c, &c.elected, V1) && dalloc_t(c, &c.veset, V1) && dalloc_t(c, &c.ereset, V1) &&
         dalloc_t(c, &c.work, V1) && dalloc_t(c, &c.work_b, V1) && dalloc_t(c, &c.vscan, V1 + 1) &&
         dalloc_t(c, &c.winv, V1 + 8) && dalloc_t(c, &c.type, V1) && dalloc_t(c, &c.ucnt, V1) &&
         dalloc_t(c, &c.rpos, V1) && dalloc_t(c, &c.rref, V1) && dalloc_t(c, &c.rslot, V1 + 1) &&
         dalloc_t(c, &c.rlit, V1 + 1) && dalloc_t(c, &c.units, c.units_total) &&
         dalloc_t(c, &c.trail, c.trail_total) && dalloc_t(c, &c.stack, c.stack_total) &&
         dalloc_t(c, &c.front_a, V1) && dalloc_t(c, &c.front_b, V1) && dalloc_t(c, &c.long_a, V1) &&
         dalloc_t(c, &c.long_b, V1) && dalloc_t(c, &c.cnew, c.hdr_cap) && dalloc_t(c, &c.ot_off2, c.nlist + 1) &&
         dalloc_t(c, &c.fcut, (size_t)n + 1);
    if (any_assumed) ok = ok && dalloc_t(c, &c.assumed, V1 + 8);
    if (!ok) {
        if (c.err.empty()) c.err = "device allocation failed";
        free_all(o);
        return PFG_CNFALLOC_FAIL;
    }
    // host-written instance inputs
    for (uint32_t i = 0; i < n; i++) {
        c.hi.voff[i] = c.ih[i].voff;
        c.hi.ucap[i] = ucap[i]; c.hi.tcap[i] = tcap[i];
        c.hi.ubase[i] = ubase[i]; c.hi.tbase[i] = tbase[i];
        c.hi.sbase[i] = sbase[i]; c.hi.scap[i] = scap[i];
        for (int k = 0; k < 4; k++) c.hi.acc[4 * i + k] = acc[4 * i + k];
    }
    c.hi.voff[n] = (uint32_t)Vtot;
    push_inst_in(c);
    cudaMemsetAsync(c.dout.conflict, 0, c.out_bytes, c.s);
    // H2D: each instance's literals and offsets into its slice of the store
    unsigned long long* d_off = nullptr;
    unsigned long long* d_base = nullptr;   // clsbase (n+1) then litbase (n+1)
    uint8_t* d_learnt = nullptr;
    uint32_t* d_lbd = nullptr;
    uint8_t* d_usage = nullptr;
    ok = dalloc_t(c, &d_off, Ctot + 1) && dalloc_t(c, &d_base, 2 * ((size_t)n + 1) + 2 + ((size_t)n + 1) / 2);
    if (ok && any_learnt) ok = dalloc_t(c, &d_learnt, Ctot + 1);
    if (ok && any_lbd) ok = dalloc_t(c, &d_lbd, Ctot + 1);
    if (ok && any_usage) ok = dalloc_t(c, &d_usage, Ctot + 1);
    if (!ok) { free_all(o); return PFG_CNFALLOC_FAIL; }
    if (any_learnt) cudaMemsetAsync(d_learnt, 0, Ctot + 1, c.s);
    if (any_lbd) cudaMemsetAsync(d_lbd, 0, (Ctot + 1) * sizeof(uint32_t), c.s);
    if (any_usage) cudaMemsetAsync(d_usage, 0, Ctot + 1, c.s);
    // d_base: clsbase (n+1), litbase (n+1), two error words (first bad clause of
    // the offset check and of the literal checks), then max_var per instance
    const size_t nb2 = 2 * ((size_t)n + 1);
    unsigned long long* d_bad = d_base + nb2;
    uint32_t* d_vmax = reinterpret_cast<uint32_t*>(d_base + nb2 + 2);
    {
        std::vector<unsigned long long> bases(nb2 + 2 + ((size_t)n + 1) / 2, 0);
        for (uint32_t i = 0; i <= n; i++) { bases[i] = clsbase[i]; bases[n + 1 + i] = litbase[i]; }
        bases[nb2] = bases[nb2 + 1] = ~0ull;
        uint32_t* vm = reinterpret_cast<uint32_t*>(bases.data() + nb2 + 2);
        for (uint32_t i = 0; i < n; i++) vm[i] = in[i].max_var;
        cudaMemcpy(d_base, bases.data(), bases.size() * sizeof(unsigned long long), cudaMemcpyHostToDevice);
    }
    cudaMemsetAsync(c.vstate, 0, V1, c.s);
    if (any_assumed) cudaMemsetAsync(c.assumed, 0, V1, c.s);
    PFG_LAUNCH(K_UPLOAD, vinst_k, grid_for(V1, 256), 256, 0, c.s, c.di.voff, n, c.V, c.vinst, c.vorg);
    for (uint32_t i = 0; i < n; i++) {
        const pfg_instance& q = in[i];
        const uint64_t Ci = q.num_clauses, Li = litbase[i + 1] - litbase[i];
        const uint32_t vo = c.ih[i].voff;
        if (Li) cudaMemcpyAsync(c.lits + litbase[i], q.lits, Li * sizeof(uint32_t), cudaMemcpyHostToDevice, c.s);
        if (Ci) cudaMemcpyAsync(d_off + clsbase[i], q.cls_off, Ci * sizeof(uint64_t), cudaMemcpyHostToDevice, c.s);
        if (Ci && q.cls_learnt) cudaMemcpyAsync(d_learnt + clsbase[i], q.cls_learnt, Ci, cudaMemcpyHostToDevice, c.s);
        if (Ci && q.cls_lbd) cudaMemcpyAsync(d_lbd + clsbase[i], q.cls_lbd, Ci * sizeof(uint32_t), cudaMemcpyHostToDevice, c.s);
        if (Ci && q.cls_usage) cudaMemcpyAsync(d_usage + clsbase[i], q.cls_usage, Ci, cudaMemcpyHostToDevice, c.s);
        if (q.var_state) cudaMemcpyAsync(c.vstate + vo + 1, q.var_state + 1, q.max_var, cudaMemcpyHostToDevice, c.s);
        if (q.assumed) cudaMemcpyAsync(c.assumed + vo + 1, q.assumed + 1, q.max_var, cudaMemcpyHostToDevice, c.s);
        if (q.vorg) cudaMemcpyAsync(c.vorg + vo + 1, q.vorg + 1, q.max_var * sizeof(uint32_t), cudaMemcpyHostToDevice, c.s);
    }
    unsigned long long hbad[2] = {~0ull, ~0ull};
    if (Ctot) {
        // offsets first: the header kernel reads literals between them
        PFG_LAUNCH(K_UPLOAD, check_off_k, grid_for(Ctot, 256), 256, 0, c.s, d_off, Ctot, d_base, d_base + n + 1, n,
                   d_bad);
        cudaMemcpyAsync(hbad, d_bad, sizeof(unsigned long long), cudaMemcpyDeviceToHost, c.s);
        stream_sync(c, "upload");
        if (hbad[0] == ~0ull && c.err.empty()) {
            PFG_LAUNCH(K_UPLOAD, init_hdr_k, grid_for(Ctot, 256), 256, 0, c.s, c.hdr, d_off, Ctot, d_learnt, d_lbd,
                       d_usage, d_base, d_base + n + 1, c.di.voff, n, d_vmax, c.lits, d_bad + 1);
            PFG_LAUNCH(K_UPLOAD, prep_k, grid_for(Ctot, 128), 128, 0, c.s, c.hdr, c.lits, Ctot, d_bad + 1);
            cudaMemcpyAsync(hbad + 1, d_bad + 1, sizeof(unsigned long long), cudaMemcpyDeviceToHost, c.s);
        }
    }
    if (c.o.proof_en) {
        if (!dalloc_t(c, &c.lbyte, 2 * V1)) { free_all(o); return PFG_CNFALLOC_FAIL; }
        PFG_LAUNCH(K_UPLOAD, lbyte_k, grid_for(2 * V1, 256), 256, 0, c.s, c.vorg, c.V, c.lbyte);
    }
    cudaMemsetAsync(c.elim, 0, V1, c.s);
    cudaMemsetAsync(c.cnew, 0, c.hdr_cap, c.s);
    cudaMemsetAsync(c.varcore, 0, V1 * sizeof(uint32_t), c.s);
    cudaMemsetAsync(c.dc, 0, sizeof(DevCounters), c.s);
    dfree(c, d_off); dfree(c, d_base); dfree(c, d_learnt); dfree(c, d_lbd); dfree(c, d_usage);
    sync_counters(c);
    c.launches += g_launches - base_launches;
    g_prof = nullptr;
    if (!c.err.empty()) return PFG_CUDA_ERROR;
    for (int k = 0; k < 2; k++) {
        if (hbad[k] == ~0ull) continue;
        const uint64_t bad = hbad[k];
        const uint32_t i = (uint32_t)(std::upper_bound(clsbase.begin(), clsbase.end(), bad) - clsbase.begin() - 1);
        const std::string msg = "instance " + std::to_string(i) + ": clause " + std::to_string(bad - clsbase[i]) +
                                (k == 0 ? " has fewer than 2 literals or offsets out of order"
                                        : " has a literal out of range or a repeated variable");
        free_all(o);
        c.err = msg;
        return PFG_INVALID;
    }
    c.uploaded = true;
    c.simplified = false;
    c.cache_ready = false;
    c.stats = pfg_stats{};
    c.stats.clauses_in = Ctot;
    c.stats.literals_in = Ltot;
    return PFG_OK;
}

// instances leaving the round loop keep the units of their last round unpropagated
__global__ void regions_all_k(const uint32_t* src, const unsigned long long* src_base,
                              const unsigned long long* dst_base, const uint32_t* shift, uint32_t n, uint64_t total,
                              uint32_t* out);

void retire(Ctx& c, const std::vector<uint32_t>& ids) {
    bool need = false;
    for (uint32_t i : ids) need |= c.ih[i].nUnits > 0;
    if (need) pull_inst_out(c);
    // the unit regions of the leaving instances, gathered back to back on the
    // device and copied in one transfer
    std::vector<uint32_t> with;
    std::vector<unsigned long long> sb, db(1, 0);
    for (uint32_t i : ids) {
        InstHost& h = c.ih[i];
        h.active = false;
        if (!h.nUnits) continue;
        const uint64_t nu = std::min<uint64_t>(c.hout.ucount[i], c.hi.ucap[i]);
        h.pending.resize(nu);
        h.nUnits = 0;
        if (!nu) continue;
        with.push_back(i);
        sb.push_back(c.hi.ubase[i]);
        db.push_back(db.back() + nu);
    }
    if (with.empty()) return;
    const uint32_t m = (uint32_t)with.size();
    const uint64_t total = db.back();
    unsigned long long* dbases = nullptr;
    uint32_t* dout = nullptr;
    if (m > 1 && dalloc_t(c, &dbases, 2 * (size_t)m + 1) && dalloc_t(c, &dout, total)) {
        std::vector<unsigned long long> hb(sb);
        hb.insert(hb.end(), db.begin(), db.end());
        cudaMemcpyAsync(dbases, hb.data(), hb.size() * sizeof(unsigned long long), cudaMemcpyHostToDevice, c.s);
        PFG_LAUNCH(K_MISC, regions_all_k, grid_for(total, 256), 256, 0, c.s, c.units, dbases, dbases + m,
                   (const uint32_t*)nullptr, m, total, dout);
        std::vector<uint32_t> all(total);
        cudaMemcpyAsync(all.data(), dout, total * sizeof(uint32_t), cudaMemcpyDeviceToHost, c.s);
        stream_sync(c, "pending units");
        for (uint32_t q = 0; q < m; q++)
            std::copy(all.begin() + db[q], all.begin() + db[q + 1], c.ih[with[q]].pending.begin());
    } else {
        for (uint32_t q = 0; q < m; q++)
            cudaMemcpy(c.ih[with[q]].pending.data(), c.units + sb[q], (db[q + 1] - db[q]) * sizeof(uint32_t),
                       cudaMemcpyDeviceToHost);
    }
    dfree(c, dbases);
    dfree(c, dout);
}

std::vector<uint32_t> active_ids(const Ctx& c) {
    std::vector<uint32_t> a;
    for (uint32_t i = 0; i < c.ninst; i++) if (c.ih[i].active) a.push_back(i);
    return a;
}

// elected variables of the instances in `want` mode, in order, into `out`
uint32_t select_mode(Ctx& c, uint8_t want, uint32_t*& out) {
    uint64_t total = 0;
    bool exact = true;   // every elected variable belongs to an instance in `want` mode
    for (uint32_t i = 0; i < c.ninst; i++) {
        const InstHost& h = c.ih[i];
        if (h.mode == want) total += h.nelected;
        else if (h.nelected && h.mode != want) exact = false;
    }
    if (!total) return 0;
    if (exact) {                        // the elected list is the set: swap buffers
        std::swap(out, c.elected);
        return c.nelected;
    }
    PFG_LAUNCH(K_MISC, mode_flags_k, grid_for(c.nelected, 256), 256, 0, c.s, c.elected, c.nelected, c.vinst, c.di.mode,
               want, c.flag8);
    if (!ensure_tmp(c, scan_temp_bytes(c.nelected + 1))) return 0;
    select_flagged(c.elected, c.flag8, out, c.nelected, &c.dc->nwork, c.vscan, c.tmp, c.s);
    return (uint32_t)total;
}

}  // namespace
}  // namespace pfg

using namespace pfg;

// Page-locked host memory for callers' input and result buffers: copies from
// and to it run as DMA at link speed instead of through staging buffers
// (cuMM::allocPinned, src/gpu/memory.cu:505-523).
extern "C" void* pfg_host_alloc(size_t bytes) {
    void* p = nullptr;
    if (cudaMallocHost(&p, bytes ? bytes : 1) != cudaSuccess) { cudaGetLastError(); return nullptr; }
    return p;
}

extern "C" void pfg_host_free(void* p) {
    if (p) cudaFreeHost(p);
}

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
    // "xormaxarity" accepts 2..20 (options.cu:60)
    if (o->xor_max_arity < 2) o->xor_max_arity = 2;
    if (o->xor_max_arity > 20) o->xor_max_arity = 20;
}

extern "C" int pfg_create(pfg_ctx** out, const pfg_options* opts, size_t arena_bytes) {
    if (!out) return PFG_INVALID;
    *out = nullptr;
    pfg_ctx* o = new pfg_ctx();
    Ctx& c = o->c;
    if (opts) c.o = *opts; else pfg_default_options(&c.o);
    pfg_resolve_options(&c.o);
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) { cudaGetLastError(); delete o; return PFG_CUDA_ERROR; }
    c.device = dev;
    if (cudaStreamCreateWithFlags(&c.s, cudaStreamNonBlocking) != cudaSuccess) { cudaGetLastError(); delete o; return PFG_CUDA_ERROR; }
    cudaEventCreate(&c.ev_begin); cudaEventCreate(&c.ev_end);
    // keep freed blocks in the device pool: the pool is the engine's arena
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
        uint64_t thr = UINT64_MAX;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
    }
    if (cudaMallocHost((void**)&c.hc, sizeof(DevCounters)) != cudaSuccess) {
        cudaGetLastError();
        cudaStreamDestroy(c.s);
        delete o;
        return PFG_CUDA_ERROR;
    }
    std::memset(c.hc, 0, sizeof(DevCounters));
    if (arena_bytes == 0) {
        size_t fr = 0, tot = 0;
        if (cudaMemGetInfo(&fr, &tot) == cudaSuccess && fr > (256ull << 20)) o->budget = fr - (256ull << 20);
    } else {
        o->budget = arena_bytes;
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
    pfg_instance q;
    std::memset(&q, 0, sizeof(q));
    q.max_var = max_var;
    q.num_clauses = num_clauses;
    q.lits = lits;
    q.cls_off = cls_off;
    q.cls_learnt = cls_learnt;
    q.cls_lbd = cls_lbd;
    q.cls_usage = cls_usage;
    q.var_state = var_state;
    q.assumed = assumed;
    q.vorg = vorg;
    const int rc = upload_impl(o, 1, &q);
    if (rc != PFG_OK && o->c.err.rfind("instance 0: ", 0) == 0) o->c.err = o->c.err.substr(12);
    return rc;
}

extern "C" int pfg_batch_upload(pfg_ctx* o, uint32_t n, const pfg_instance* instances) {
    if (!o) return PFG_INVALID;
    return upload_impl(o, n, instances);
}

extern "C" uint32_t pfg_batch_size(pfg_ctx* o) { return (o && o->c.uploaded) ? o->c.ninst : 0; }

static int finish(Ctx& c, pfg_stats* st, uint64_t base_launches, int rc) {
    if (c.prof.on) c.prof.resolve();
    g_prof = nullptr;
    c.launches += g_launches - base_launches;
    if (st) *st = c.stats;
    return rc;
}

namespace pfg {
namespace {
__global__ void elim_counts_k(const uint8_t* elim, const uint32_t* vinst, uint32_t V, unsigned long long* cnt);
}  // namespace
}  // namespace pfg

// The round loop of Solver::simplifying (simplify.cu:159-186), run for every
// instance at once. All instances still in the loop share the round counter
// and the multiplier; everything else (stop rule, counts, units, accounting)
// is per instance, and an instance leaves the loop exactly where a run of it
// alone would break.
extern "C" int pfg_simplify(pfg_ctx* o, pfg_stats* st) {
    if (!o) return PFG_INVALID;
    Ctx& c = o->c;
    if (!c.uploaded) { c.err = "no instance uploaded"; return PFG_INVALID; }
    if (c.simplified) { c.err = "instance already simplified; upload again"; return PFG_INVALID; }
    const uint64_t base_launches = g_launches;
    g_prof = &c.prof;
    c.err.clear();
    c.pass_clock.reset();
    c.phase = c.multiplier = c.simpstate = 0;
    const uint32_t n = c.ninst;
    cudaEventRecord(c.ev_begin, c.s);
    uint64_t alg = 0;
    const bool disabled = !c.o.phases && !(c.o.all_en | c.o.ere_en);   // alldisabled (solver.hpp:722)
    std::vector<uint8_t> entered(n, 0);
    for (uint32_t i = 0; i < n; i++) {
        InstHost& h = c.ih[i];
        h.status = PFG_UNKNOWN;
        h.varcore_on = c.o.ve_fun_en != 0;
        h.active = !disabled && h.orig_cls > 0;
        entered[i] = h.active;
        h.cdiff = h.ldiff = INT64_MAX;
        h.clsbefore = (int64_t)h.numClauses;
        h.litsbefore = (int64_t)h.numLiterals;
    }
    bool any_entered = false;
    for (uint32_t i = 0; i < n; i++) any_entered |= entered[i] != 0;
    while (true) {
        // while (numClauses && numLiterals && !simpstate)
        {
            std::vector<uint32_t> out;
            for (uint32_t i = 0; i < n; i++) {
                const InstHost& h = c.ih[i];
                if (h.active && (!h.numClauses || !h.numLiterals || c.simpstate)) out.push_back(i);
            }
            retire(c, out);
        }
        std::vector<uint32_t> act = active_ids(c);
        if (act.empty() || !c.err.empty()) break;
        const int times = c.phase + 1;
        // after the first round the table is updated, not rebuilt: pruned on the
        // old clause ids, then moved (through the compaction words) and completed
        if (c.ot_valid) {
            PassTimer t(c, 0);
            if (!ot_prune(c)) break;
        }
        if (times > 1 && times != c.o.phases && c.o.shrink_rate > 0 && (times % c.o.shrink_rate) == 0) {
            PassTimer t(c, 6);
            if (!compact_cnf(c)) break;
        }
        {
            PassTimer t(c, 0);
            if (!(c.ot_valid ? ot_update(c) : ot_build(c))) break;
            dfree(c, c.cbits);
            c.cbits = nullptr;
            c.ot_valid = true;
        }
        bool any_units = false;
        for (uint32_t i = 0; i < n; i++) {
            c.hi.bcp[i] = c.ih[i].active && c.ih[i].nUnits > 0;
            any_units |= c.hi.bcp[i] != 0;
        }
        if (any_units) {
            PassTimer t(c, 1);
            push_inst_in(c);
            if (!bcp_prop(c)) break;      // leaves the live counts as count_live does
            pull_inst_out(c);
            if (!c.err.empty()) break;
            c.numClauses = c.hc->live_cls;
            c.numLiterals = c.hc->live_lits;
            for (uint32_t i = 0; i < n; i++) {
                InstHost& h = c.ih[i];
                h.numClauses = c.hout.cnt[2 * i];
                h.numLiterals = c.hout.cnt[2 * i + 1];
                if (c.hi.bcp[i]) {
                    h.nUnits = 0;
                    if (c.hout.conflict[i]) { h.status = PFG_UNSAT; h.active = false; }
                }
            }
            if (!ot_filter(c, c.bstate)) break;
            cudaMemsetAsync(c.dout.ucount, 0, n * sizeof(uint32_t), c.s);
        }
        for (uint32_t i = 0; i < n; i++)
            if (c.ih[i].active && !c.ih[i].numClauses) c.ih[i].active = false;
        act = active_ids(c);
        if (act.empty()) break;
        for (uint32_t i = 0; i < n; i++) {
            c.hi.active[i] = c.ih[i].active;
            c.hi.vc_on[i] = c.ih[i].active && c.ih[i].varcore_on;
            c.ih[i].nelected = 0;
            c.ih[i].mode = 0;
        }
        push_inst_in(c);
        {
            PassTimer t(c, 2);
            if (!c.o.lcve_fast && !ot_sort(c, true)) break;
            if (!lcve(c)) break;
        }
        for (uint32_t i : act)
            if (c.ih[i].nelected < c.o.lcve_min_vars) c.ih[i].active = false;
        act = active_ids(c);
        if (act.empty()) break;
        // stop() (solver.hpp:748-753) per instance: the last round runs ERE instead of SUB+BVE
        uint32_t nmode1 = 0, nmode2 = 0;
        for (uint32_t i : act) {
            InstHost& h = c.ih[i];
            const bool stop = c.phase == c.o.phases || (h.cdiff == 0 && h.ldiff == 0) ||
                              (c.phase > 2 && h.ldiff <= (int64_t)c.o.phase_lits_min);
            if (stop) {
                h.active = false;
                if (c.o.ere_en && h.nelected) { h.mode = 2; h.ere_ran = true; nmode2++; }
            } else {
                h.mode = 1;
                nmode1++;
            }
        }
        uint32_t acc_seg = 0;
        for (uint32_t i = 0; i < n; i++) {
            c.hi.mode[i] = (uint8_t)c.ih[i].mode;
            c.hi.vc_on[i] = c.ih[i].mode == 1 && c.ih[i].varcore_on;
            c.hi.seg[i] = acc_seg;
            if (c.ih[i].mode == 1) acc_seg += c.ih[i].nelected;
        }
        c.hi.seg[n] = acc_seg;
        push_inst_in(c);
        c.nere = nmode2 ? select_mode(c, 2, c.ereset) : 0;
        c.nve = nmode1 ? select_mode(c, 1, c.veset) : 0;
        // sortOT (segsort.cu:37). Only the elected variables' lists are read in
        // list order (staging, subsumption order, witness and resolvent order;
        // gate lookups search those lists too; ERE finds equal clauses through a
        // hash table), so only they are sorted.
        if (c.nere || c.nve) {
            PassTimer t(c, 0);
            if (c.nere && !ot_sort(c, false, c.ereset, c.nere)) break;
            // the ERE sort just made every clause's key and no clause changed since
            if (c.nve && !ot_sort(c, false, c.veset, c.nve, c.nere != 0)) break;
        }
        if (c.nere) {
            // byte model: the elected lists' clauses and literals, summed on the
            // device (a pass of its own, so only while the profiler is on)
            if (c.prof.on)
                PFG_LAUNCH(K_MISC, elected_volume_k, grid_for(c.nere, 256), 256, 0, c.s, c.ereset, c.nere, c.hdr,
                           c.ot_off, c.ot_size, c.ot_ids, c.dc->vol_ere);
            PassTimer t(c, 5);
            if (!ere_pass(c)) break;
        }
        if (!nmode1) break;
        // byte model: C_E, L_E of the round, summed over the rounds on the
        // device and read when the call ends (only while the profiler is on)
        if (c.prof.on)
            PFG_LAUNCH(K_MISC, elected_volume_k, grid_for(c.nve, 256), 256, 0, c.s, c.veset, c.nve, c.hdr, c.ot_off,
                       c.ot_size, c.ot_ids, c.dc->vol_ve);
        uint64_t Cin = 0, Lin = 0;
        for (uint32_t i = 0; i < n; i++)
            if (c.ih[i].mode == 1) {
                Cin += c.ih[i].numClauses;
                Lin += c.ih[i].numLiterals;
                c.ih[i].processed_cls += c.ih[i].numClauses;
                c.ih[i].processed_lits += c.ih[i].numLiterals;
            }
        const uint64_t ncls0 = c.ncls, lits0 = c.lits_used;
        c.stats.clauses_processed += Cin;
        c.stats.literals_processed += Lin;
        if (c.o.sub_en || c.o.ve_plus_en) {
            PassTimer t(c, 3);
            if (!sub_pass(c)) break;
        }
        if (c.o.ve_en) {
            PassTimer t(c, 4);
            if (!ve_pass(c)) break;
        }
        if (c.o.bce_en) {   // SUB(), VE(), BCE() (simplify.cu:173)
            PassTimer t(c, 7);
            if (!bce_pass(c)) break;
        }
        {
            PassTimer t(c, 6);
            count_live(c);
            pull_inst_out(c);
        }
        if (!c.err.empty()) break;
        c.numClauses = c.hc->live_cls;
        c.numLiterals = c.hc->live_lits;
        for (uint32_t i = 0; i < n; i++) {
            InstHost& h = c.ih[i];
            h.numClauses = c.hout.cnt[2 * i];
            h.numLiterals = c.hout.cnt[2 * i + 1];
            if (h.mode != 1) continue;
            h.round_ends.push_back(c.hout.scount[i]);
            h.nUnits = c.hout.ucount[i];
            h.cdiff = h.clsbefore - (int64_t)h.numClauses; h.clsbefore = (int64_t)h.numClauses;
            h.ldiff = h.litsbefore - (int64_t)h.numLiterals; h.litsbefore = (int64_t)h.numLiterals;
            h.rounds++;
        }
        const uint64_t Cres = c.ncls - ncls0, Lres = c.lits_used - lits0;
        c.stats.resolvents += Cres;
        c.prof.bytes[K_VE3] += 4 * (Lres + Cres);
        alg += 4 * (Lin + Cin) + 8 * Lin + 4 * (Lres + Cres) + 4 * (c.numLiterals + c.numClauses);
        c.phase++; c.multiplier++;
        c.multiplier += (c.phase == c.o.phases);
    }
    retire(c, active_ids(c));
    if (c.err.empty() && any_entered) {   // ERE deletes after the last count (the write-back recounts, cnf.cu:211-224)
        count_live(c);
        pull_inst_out(c);
        c.numClauses = c.hc->live_cls;
        c.numLiterals = c.hc->live_lits;
        for (uint32_t i = 0; i < n; i++) {
            InstHost& h = c.ih[i];
            h.numClauses = c.hout.cnt[2 * i];
            h.numLiterals = c.hout.cnt[2 * i + 1];
            if (entered[i] && h.status != PFG_UNSAT && !h.numClauses) h.status = PFG_SAT;
        }
    }
    cudaEventRecord(c.ev_end, c.s);
    // eliminated / forced variables, counted per instance on the device
    std::vector<unsigned long long> ecnt(2 * (size_t)n, 0);
    {
        unsigned long long* d_ecnt = nullptr;
        if (dalloc_t(c, &d_ecnt, 2 * (size_t)n)) {
            cudaMemsetAsync(d_ecnt, 0, 2 * (size_t)n * sizeof(unsigned long long), c.s);
            PFG_LAUNCH(K_DOWNLOAD, elim_counts_k, grid_for(c.V, 256), 256, 0, c.s, c.elim, c.vinst, c.V, d_ecnt);
            cudaMemcpyAsync(ecnt.data(), d_ecnt, ecnt.size() * sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                            c.s);
            dfree(c, d_ecnt);
        }
    }
    pull_inst_out(c);
    {   // byte model of the elected lists (elected_volume_k), summed over the rounds
        const uint64_t CE = c.hc->vol_ve[0], LE = c.hc->vol_ve[1];
        c.prof.bytes[K_SUB] += 4 * (LE + CE);
        c.prof.bytes[K_VE1] += 4 * (LE + CE);
        c.prof.bytes[K_VE3] += 4 * (LE + CE);
        c.prof.bytes[K_ERE] += 4 * (c.hc->vol_ere[0] + c.hc->vol_ere[1]);
        alg += 8 * (LE + CE);
    }
    float ms = 0;
    cudaEventElapsedTime(&ms, c.ev_begin, c.ev_end);
    c.simplified = true;
    uint64_t tot_e = 0, tot_f = 0, tot_stack = 0;
    uint32_t max_rounds = 0;
    for (uint32_t i = 0; i < n; i++) {
        InstHost& h = c.ih[i];
        tot_e += ecnt[2 * i];
        tot_f += ecnt[2 * i + 1];
        tot_stack += c.hout.scount[i];
        max_rounds = std::max(max_rounds, h.rounds);
    }
    c.stats.status = n == 1 ? c.ih[0].status : PFG_UNKNOWN;
    c.stats.rounds = max_rounds;
    c.stats.ere_ran = 0;
    for (uint32_t i = 0; i < n; i++) c.stats.ere_ran |= c.ih[i].ere_ran ? 1 : 0;
    c.stats.simpstate = c.simpstate;
    c.stats.clauses_out = c.numClauses;
    c.stats.literals_out = c.numLiterals;
    c.stats.stack_words = tot_stack;
    c.stats.device_ms = ms;
    c.pass_clock.resolve();
    for (int i = 0; i < 8; i++) c.stats.pass_ms[i] = c.pass_clock.ms[i];
    c.stats.alg_bytes = alg;
    c.stats.kernel_launches = g_launches - base_launches;
    c.stats.eliminated = tot_e;
    c.stats.forced = tot_f;
    int rc = PFG_OK;
    if (!c.err.empty()) rc = (c.simpstate == PFG_TIMEOUT) ? PFG_TIMEOUT : (c.simpstate ? c.simpstate : PFG_CUDA_ERROR);
    else if (c.simpstate) rc = c.simpstate;
    return finish(c, st, base_launches, rc);
}

extern "C" int pfg_simplify_many(pfg_ctx* const* ctxs, uint32_t k, pfg_stats* stats, float* device_ms) {
    if (!ctxs || !k || !stats) return PFG_INVALID;
    for (uint32_t j = 0; j < k; j++) {
        if (!ctxs[j] || ctxs[j]->c.device != ctxs[0]->c.device) return PFG_INVALID;
        for (uint32_t i = 0; i < j; i++)
            if (ctxs[i] == ctxs[j]) return PFG_INVALID;
    }
    const int dev = ctxs[0]->c.device;
    if (cudaSetDevice(dev) != cudaSuccess) { cudaGetLastError(); return PFG_CUDA_ERROR; }
    cudaEvent_t start = nullptr;
    if (cudaEventCreate(&start) != cudaSuccess) { cudaGetLastError(); return PFG_CUDA_ERROR; }
    cudaEventRecord(start, ctxs[0]->c.s);
    for (uint32_t j = 1; j < k; j++) cudaStreamWaitEvent(ctxs[j]->c.s, start, 0);
    std::vector<int> rc(k, PFG_OK);
    std::vector<std::thread> th;
    th.reserve(k - 1);
    for (uint32_t j = 1; j < k; j++)
        th.emplace_back([&, j] {
            if (cudaSetDevice(dev) != cudaSuccess) { cudaGetLastError(); rc[j] = PFG_CUDA_ERROR; return; }
            rc[j] = pfg_simplify(ctxs[j], &stats[j]);
        });
    rc[0] = pfg_simplify(ctxs[0], &stats[0]);
    for (std::thread& t : th) t.join();
    float ms = 0;
    for (uint32_t j = 0; j < k; j++) {
        if (!ctxs[j]->c.simplified) continue;
        float t = 0;
        if (cudaEventElapsedTime(&t, start, ctxs[j]->c.ev_end) == cudaSuccess) ms = std::max(ms, t);
        else cudaGetLastError();
    }
    cudaEventDestroy(start);
    if (device_ms) *device_ms = ms;
    for (uint32_t j = 0; j < k; j++)
        if (rc[j] != PFG_OK) return rc[j];
    return PFG_OK;
}

namespace pfg {
namespace {
int build_cache(Ctx& c);
}  // namespace
}  // namespace pfg

extern "C" int pfg_batch_stats(pfg_ctx* o, uint32_t i, pfg_stats* st) {
    if (!o || !st) return PFG_INVALID;
    Ctx& c = o->c;
    if (!c.simplified || i >= c.ninst) return PFG_INVALID;
    const InstHost& h = c.ih[i];
    pfg_stats s = c.stats;
    s.status = h.status;
    s.rounds = h.rounds;
    s.ere_ran = h.ere_ran ? 1 : 0;
    s.clauses_in = h.cls_in;
    s.literals_in = h.lits_in;
    s.clauses_out = h.numClauses;
    s.literals_out = h.numLiterals;
    s.clauses_processed = h.processed_cls;
    s.literals_processed = h.processed_lits;
    s.resolvents = h.resolvents;
    s.stack_words = c.hout.scount[i];
    const int rc = build_cache(c);
    if (rc != PFG_OK) return rc;
    s.eliminated = c.cache_elim_cnt[i];
    s.forced = c.cache_forced_cnt[i];
    *st = s;
    return PFG_OK;
}

extern "C" int pfg_result_sizes_get(pfg_ctx* o, pfg_result_sizes* r) {
    if (!o || !r) return PFG_INVALID;
    Ctx& c = o->c;
    if (!c.uploaded) return PFG_INVALID;
    std::memset(r, 0, sizeof(*r));
    pull_inst_out(c);
    r->clauses = c.numClauses;
    r->literals = c.numLiterals;
    uint64_t units = 0, pend = 0, words = 0, rounds = 0;
    for (uint32_t i = 0; i < c.ninst; i++) {
        units += c.hout.tcount[i];
        pend += c.ih[i].pending.size();
        words += c.hout.scount[i];
        rounds = std::max<uint64_t>(rounds, c.ih[i].round_ends.size());
    }
    r->units = units;
    r->pending_units = pend;
    r->stack_words = words;
    r->rounds = rounds;
    r->max_var = c.V;
    for (uint32_t i = 0; i < c.ninst; i++) r->proof_bytes += c.ih[i].proof.size();
    return PFG_OK;
}

// one-instance write-back straight into the caller's buffers
extern "C" int pfg_download(pfg_ctx* o, uint32_t* lits, uint64_t* cls_off, uint8_t* cls_learnt, uint32_t* cls_lbd,
                            uint8_t* cls_usage, uint8_t* eliminated, uint32_t* units, uint32_t* pending_units,
                            uint32_t* stack, uint64_t* round_ends) {
    if (!o) return PFG_INVALID;
    Ctx& c = o->c;
    if (!c.uploaded) return PFG_INVALID;
    if (c.ninst != 1) { c.err = "several instances uploaded: use pfg_batch_download"; return PFG_INVALID; }
    const uint64_t base_launches = g_launches;
    g_prof = &c.prof;
    pull_inst_out(c);
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
    const InstHost& h = c.ih[0];
    const uint32_t ntrail = c.hout.tcount[0];
    const uint64_t nstack = c.hout.scount[0];
    if (eliminated) cudaMemcpyAsync(eliminated, c.elim, c.V + 1, cudaMemcpyDeviceToHost, c.s);
    // forced units ascending: a long trail is radix-sorted on the device (a host
    // sort of millions of literals costs more than the whole simplify call),
    // a short one on the host after the copy
    const uint32_t* usrc = c.trail;
    bool host_sort = units && ntrail;
    uint32_t *uk0 = nullptr, *uk1 = nullptr, *uv0 = nullptr, *uv1 = nullptr;
    if (units && ntrail > 4096) {
        if (dalloc_t(c, &uk0, ntrail) && dalloc_t(c, &uk1, ntrail) && dalloc_t(c, &uv0, ntrail) &&
            dalloc_t(c, &uv1, ntrail) && ensure_tmp(c, radix_temp_bytes(ntrail))) {
            cudaMemcpyAsync(uk0, c.trail, ntrail * sizeof(uint32_t), cudaMemcpyDeviceToDevice, c.s);
            cudaMemsetAsync(uv0, 0, ntrail * sizeof(uint32_t), c.s);
            int bits = 0;
            while (bits < 32 && ((2ull * c.V + 1) >> bits)) bits++;
            usrc = radix_sort_pairs(uk0, uv0, uk1, uv1, ntrail, 0, bits, c.tmp, c.s) ? uk1 : uk0;
            host_sort = false;
        } else {
            c.err.clear();   // no room for the sort buffers: sort on the host instead
        }
    }
    if (units && ntrail) cudaMemcpyAsync(units, usrc, ntrail * sizeof(uint32_t), cudaMemcpyDeviceToHost, c.s);
    if (stack && nstack) cudaMemcpyAsync(stack, c.stack, nstack * sizeof(uint32_t), cudaMemcpyDeviceToHost, c.s);
    const bool synced = stream_sync(c, "download");
    dfree(c, uk0); dfree(c, uk1); dfree(c, uv0); dfree(c, uv1);
    if (!synced) return finish(c, nullptr, base_launches, PFG_CUDA_ERROR);
    if (host_sort) std::sort(units, units + ntrail);
    if (pending_units && !h.pending.empty()) {
        std::copy(h.pending.begin(), h.pending.end(), pending_units);
        std::sort(pending_units, pending_units + h.pending.size());
    }
    if (round_ends) std::copy(h.round_ends.begin(), h.round_ends.end(), round_ends);
    return finish(c, nullptr, base_launches, PFG_OK);
}

namespace pfg {
namespace {

// Packs every instance's live clauses once: grouped by instance (clause order
// kept), literals back in the instance's numbering, offsets relative to the
// instance. Per-instance eliminated / forced counts come from one copy of the
// eliminated bytes.
// per instance: variables eliminated (any bit but FORCED) and forced, with one
// atomic per warp and instance
__global__ void elim_counts_k(const uint8_t* elim, const uint32_t* vinst, uint32_t V, unsigned long long* cnt) {
    const unsigned lane = threadIdx.x & 31u;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t b = (uint64_t)blockIdx.x * blockDim.x; b < (uint64_t)V + 1; b += stride) {
        const uint64_t v = b + threadIdx.x;
        const bool in = v >= 1 && v <= V;
        const uint8_t e = in ? elim[v] : 0u;
        const uint32_t inst = in ? vinst[v] : 0xFFFFFFFFu;
        const unsigned peers = __match_any_sync(0xFFFFFFFFu, inst);
        const unsigned fb = __ballot_sync(0xFFFFFFFFu, (e & FORCED_MASK) != 0) & peers;
        const unsigned eb = __ballot_sync(0xFFFFFFFFu, e && !(e & FORCED_MASK)) & peers;
        if (in && lane == (unsigned)(__ffs(peers) - 1)) {
            if (eb) atomicAdd(&cnt[2 * (uint64_t)inst], (unsigned long long)__popc(eb));
            if (fb) atomicAdd(&cnt[2 * (uint64_t)inst + 1], (unsigned long long)__popc(fb));
        }
    }
}

int build_cache(Ctx& c) {
    if (c.cache_ready) return PFG_OK;
    const uint32_t n = c.ninst;
    pull_inst_out(c);
    const uint64_t N = c.ncls;
    c.cache_cls_base.assign((size_t)n + 1, 0);
    c.cache_lit_base.assign((size_t)n + 1, 0);
    for (uint32_t i = 0; i < n; i++) {
        c.cache_cls_base[i + 1] = c.cache_cls_base[i] + c.ih[i].numClauses;
        c.cache_lit_base[i + 1] = c.cache_lit_base[i] + c.ih[i].numLiterals;
    }
    const uint64_t C = c.cache_cls_base[n];
    dfree(c, c.pk_lits); dfree(c, c.pk_roff); dfree(c, c.pk_learnt); dfree(c, c.pk_lbd); dfree(c, c.pk_usage);
    c.pk_lits = nullptr; c.pk_roff = nullptr; c.pk_learnt = nullptr; c.pk_lbd = nullptr; c.pk_usage = nullptr;
    uint32_t *k0 = nullptr, *v0 = nullptr, *k1 = nullptr, *v1 = nullptr;
    unsigned long long* bases = nullptr;
    bool ok = dalloc_t(c, &k0, N + 1) && dalloc_t(c, &v0, N + 1) && dalloc_t(c, &k1, N + 1) &&
              dalloc_t(c, &v1, N + 1) && dalloc_t(c, &bases, (size_t)n + 1) &&
              dalloc_t(c, &c.pk_roff, C + 1) && dalloc_t(c, &c.pk_lits, c.numLiterals + 1) &&
              dalloc_t(c, &c.pk_lbd, C + 1) && dalloc_t(c, &c.pk_learnt, C + 1) && dalloc_t(c, &c.pk_usage, C + 1) &&
              ensure_tmp(c, std::max(radix_temp_bytes(N + 1), scan_temp_bytes(C + 1)));
    auto release = [&]() { dfree(c, k0); dfree(c, v0); dfree(c, k1); dfree(c, v1); dfree(c, bases); };
    if (!ok) { release(); return PFG_CNFALLOC_FAIL; }
    uint32_t* ids = v0;
    uint32_t* keys = k0;
    if (N) {
        int bits = 0;
        while (bits < 32 && (n >> bits)) bits += 8;
        PFG_LAUNCH(K_DOWNLOAD, cls_inst_keys_k, grid_for(N, 256), 256, 0, c.s, c.hdr, c.lits, N, c.vinst, n, k0, v0);
        const int which = radix_sort_pairs(k0, v0, k1, v1, N, 0, bits, c.tmp, c.s);
        ids = which ? v1 : v0;
        keys = which ? k1 : k0;
    }
    if (C) {
        PFG_LAUNCH(K_DOWNLOAD, gathered_sizes_k, grid_for(C, 256), 256, 0, c.s, c.hdr, ids, C, c.pk_roff);
        exclusive_scan_u64(c.pk_roff, c.pk_roff, C, 0ull, c.pk_roff + C, c.tmp, c.s);
        PFG_LAUNCH(K_DOWNLOAD, gathered_pack_k, grid_for(C, 256), 256, 0, c.s, c.hdr, c.lits, ids, keys, C,
                   c.pk_roff, c.di.voff, c.pk_lits, c.pk_learnt, c.pk_lbd, c.pk_usage);
        cudaMemcpyAsync(bases, c.cache_lit_base.data(), ((size_t)n + 1) * sizeof(uint64_t), cudaMemcpyHostToDevice, c.s);
        PFG_LAUNCH(K_DOWNLOAD, relative_off_k, grid_for(C, 256), 256, 0, c.s, keys, C, bases, c.pk_roff);
    }
    // eliminated and forced variables per instance, counted on the device
    unsigned long long* ecnt = nullptr;
    if (!dalloc_t(c, &ecnt, 2 * (size_t)n)) { release(); return PFG_CNFALLOC_FAIL; }
    cudaMemsetAsync(ecnt, 0, 2 * (size_t)n * sizeof(unsigned long long), c.s);
    PFG_LAUNCH(K_DOWNLOAD, elim_counts_k, grid_for(c.V, 256), 256, 0, c.s, c.elim, c.vinst, c.V, ecnt);
    std::vector<unsigned long long> hcnt(2 * (size_t)n);
    cudaMemcpyAsync(hcnt.data(), ecnt, hcnt.size() * sizeof(unsigned long long), cudaMemcpyDeviceToHost, c.s);
    const bool synced = stream_sync(c, "batch write-back");
    release();
    dfree(c, ecnt);
    if (!synced) return PFG_CUDA_ERROR;
    c.cache_elim_cnt.assign(n, 0);
    c.cache_forced_cnt.assign(n, 0);
    for (uint32_t i = 0; i < n; i++) {
        c.cache_elim_cnt[i] = hcnt[2 * i];
        c.cache_forced_cnt[i] = hcnt[2 * i + 1];
    }
    c.cache_ready = true;
    return PFG_OK;
}

}  // namespace
}  // namespace pfg

extern "C" int pfg_batch_result_sizes(pfg_ctx* o, uint32_t i, pfg_result_sizes* r) {
    if (!o || !r) return PFG_INVALID;
    Ctx& c = o->c;
    if (!c.uploaded || i >= c.ninst) return PFG_INVALID;
    const uint64_t base_launches = g_launches;
    g_prof = &c.prof;
    const int rc = build_cache(c);
    finish(c, nullptr, base_launches, rc);
    if (rc != PFG_OK) return rc;
    const InstHost& h = c.ih[i];
    std::memset(r, 0, sizeof(*r));
    r->clauses = c.cache_cls_base[i + 1] - c.cache_cls_base[i];
    r->literals = c.cache_lit_base[i + 1] - c.cache_lit_base[i];
    r->units = std::min<uint64_t>(c.hout.tcount[i], c.hi.tcap[i]);
    r->pending_units = h.pending.size();
    r->stack_words = c.hout.scount[i];
    r->rounds = h.round_ends.size();
    r->max_var = h.V;
    r->proof_bytes = h.proof.size();
    return PFG_OK;
}

extern "C" int pfg_batch_download_proof(pfg_ctx* o, uint32_t i, uint8_t* out) {
    if (!o) return PFG_INVALID;
    Ctx& c = o->c;
    if (!c.uploaded || i >= c.ninst) return PFG_INVALID;
    const std::vector<uint8_t>& p = c.ih[i].proof;
    if (!p.empty()) {
        if (!out) return PFG_INVALID;
        std::memcpy(out, p.data(), p.size());
    }
    return PFG_OK;
}

extern "C" int pfg_download_proof(pfg_ctx* o, uint8_t* out) {
    if (!o) return PFG_INVALID;
    if (o->c.ninst != 1) return PFG_INVALID;
    return pfg_batch_download_proof(o, 0, out);
}

extern "C" int pfg_batch_download(pfg_ctx* o, uint32_t i, uint32_t* lits, uint64_t* cls_off, uint8_t* cls_learnt,
                                  uint32_t* cls_lbd, uint8_t* cls_usage, uint8_t* eliminated, uint32_t* units,
                                  uint32_t* pending_units, uint32_t* stack, uint64_t* round_ends) {
    if (!o) return PFG_INVALID;
    Ctx& c = o->c;
    if (!c.uploaded || i >= c.ninst) return PFG_INVALID;
    const uint64_t base_launches = g_launches;
    g_prof = &c.prof;
    int rc = build_cache(c);
    if (rc != PFG_OK) return finish(c, nullptr, base_launches, rc);
    const InstHost& h = c.ih[i];
    const uint64_t b = c.cache_cls_base[i], nc = c.cache_cls_base[i + 1] - b;
    const uint64_t lb = c.cache_lit_base[i], nl = c.cache_lit_base[i + 1] - lb;
    const uint64_t nt = std::min<uint64_t>(c.hout.tcount[i], c.hi.tcap[i]);
    const uint64_t ns = c.hout.scount[i];
    // straight from the packed device arrays into the caller's buffers
    if (lits && nl) cudaMemcpyAsync(lits, c.pk_lits + lb, nl * sizeof(uint32_t), cudaMemcpyDeviceToHost, c.s);
    if (cls_off && nc) cudaMemcpyAsync(cls_off, c.pk_roff + b, nc * sizeof(uint64_t), cudaMemcpyDeviceToHost, c.s);
    if (cls_learnt && nc) cudaMemcpyAsync(cls_learnt, c.pk_learnt + b, nc, cudaMemcpyDeviceToHost, c.s);
    if (cls_lbd && nc) cudaMemcpyAsync(cls_lbd, c.pk_lbd + b, nc * sizeof(uint32_t), cudaMemcpyDeviceToHost, c.s);
    if (cls_usage && nc) cudaMemcpyAsync(cls_usage, c.pk_usage + b, nc, cudaMemcpyDeviceToHost, c.s);
    if (eliminated) cudaMemcpyAsync(eliminated + 1, c.elim + h.voff + 1, h.V, cudaMemcpyDeviceToHost, c.s);
    if (units && nt) cudaMemcpyAsync(units, c.trail + c.hi.tbase[i], nt * sizeof(uint32_t), cudaMemcpyDeviceToHost, c.s);
    if (stack && ns) cudaMemcpyAsync(stack, c.stack + c.hi.sbase[i], ns * sizeof(uint32_t), cudaMemcpyDeviceToHost, c.s);
    if (!stream_sync(c, "batch download")) return finish(c, nullptr, base_launches, PFG_CUDA_ERROR);
    if (cls_off) cls_off[nc] = nl;
    if (eliminated) eliminated[0] = 0;
    if (units && nt) {
        // trail literals back to the instance's numbering
        for (uint64_t k = 0; k < nt; k++) units[k] -= 2u * h.voff;
        std::sort(units, units + nt);
    }
    if (pending_units && !h.pending.empty()) {
        for (size_t k = 0; k < h.pending.size(); k++) pending_units[k] = h.pending[k] - 2u * h.voff;
        std::sort(pending_units, pending_units + h.pending.size());
    }
    if (round_ends) std::copy(h.round_ends.begin(), h.round_ends.end(), round_ends);
    return finish(c, nullptr, base_launches, PFG_OK);
}

namespace pfg {
namespace {

// instance of output position q, given the instances' output starts base[0..n]
PFG_D uint32_t region_of(const unsigned long long* base, uint32_t n, uint64_t q) {
    uint32_t lo = 0, hi = n;   // largest i < n with base[i] <= q
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (base[mid] <= q) lo = mid; else hi = mid;
    }
    return lo;
}

// cls_off of all instances back to back, each with its final entry (its literal count)
__global__ void offsets_all_k(const unsigned long long* roff, uint64_t C, const unsigned long long* cls_base,
                              const unsigned long long* lit_base, uint32_t n, unsigned long long* out) {
    for (uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; j < C + n; j += (uint64_t)gridDim.x * blockDim.x) {
        if (j < C) {
            const uint32_t i = region_of(cls_base, n, j);
            out[j + i] = roff[j];
        } else {
            const uint32_t i = (uint32_t)(j - C);
            out[cls_base[i + 1] + i] = lit_base[i + 1] - lit_base[i];
        }
    }
}

// eliminated bytes of all instances back to back, max_var + 1 each, entry 0 zero
__global__ void elim_all_k(const uint8_t* elim, const unsigned long long* ebase, const uint32_t* voff, uint32_t n,
                           uint64_t total, uint8_t* out) {
    for (uint64_t q = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; q < total; q += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t i = region_of(ebase, n, q);
        const uint64_t v = q - ebase[i];
        out[q] = v ? elim[voff[i] + v] : 0;
    }
}

// per-instance regions [src_base[i], +count) back to back; literals moved down by 2 * shift[i]
__global__ void regions_all_k(const uint32_t* src, const unsigned long long* src_base,
                              const unsigned long long* dst_base, const uint32_t* shift, uint32_t n, uint64_t total,
                              uint32_t* out) {
    for (uint64_t q = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; q < total; q += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t i = region_of(dst_base, n, q);
        const uint32_t w = src[src_base[i] + (q - dst_base[i])];
        out[q] = shift ? w - 2u * shift[i] : w;
    }
}

// instance of every gathered unit (its region in dst_base)
__global__ void region_ids_k(const unsigned long long* dst_base, uint32_t n, uint64_t total, uint32_t* out) {
    for (uint64_t q = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; q < total; q += (uint64_t)gridDim.x * blockDim.x)
        out[q] = region_of(dst_base, n, q);
}

uint32_t bits_for(uint64_t x) {
    uint32_t b = 1;
    while (b < 32 && (x >> b)) b++;
    return b;
}

}  // namespace
}  // namespace pfg

extern "C" int pfg_batch_result_sizes_all(pfg_ctx* o, pfg_result_sizes* sizes) {
    if (!o || !sizes) return PFG_INVALID;
    Ctx& c = o->c;
    if (!c.uploaded) return PFG_INVALID;
    for (uint32_t i = 0; i < c.ninst; i++) {
        const int rc = pfg_batch_result_sizes(o, i, sizes + i);
        if (rc != PFG_OK) return rc;
    }
    return PFG_OK;
}

extern "C" int pfg_batch_download_all(pfg_ctx* o, uint32_t* lits, uint64_t* cls_off, uint8_t* cls_learnt,
                                      uint32_t* cls_lbd, uint8_t* cls_usage, uint8_t* eliminated, uint32_t* units,
                                      uint32_t* pending_units, uint32_t* stack, uint64_t* round_ends) {
    if (!o) return PFG_INVALID;
    Ctx& c = o->c;
    if (!c.uploaded) return PFG_INVALID;
    const uint64_t base_launches = g_launches;
    g_prof = &c.prof;
    int rc = build_cache(c);
    if (rc != PFG_OK) return finish(c, nullptr, base_launches, rc);
    const uint32_t n = c.ninst;
    const uint64_t C = c.cache_cls_base[n], L = c.cache_lit_base[n];
    // the packed clauses are complete here: their copies go to the host on a
    // second stream, beside the write-back kernels below
    cudaStream_t cs = c.s;
    if (!c.s_copy && cudaStreamCreateWithFlags(&c.s_copy, cudaStreamNonBlocking) != cudaSuccess) {
        cudaGetLastError();
        c.s_copy = nullptr;
    }
    if (c.s_copy && !c.ev_copy && cudaEventCreateWithFlags(&c.ev_copy, cudaEventDisableTiming) != cudaSuccess) {
        cudaGetLastError();
        c.ev_copy = nullptr;
    }
    if (c.s_copy && c.ev_copy) {
        cudaEventRecord(c.ev_copy, c.s);
        cudaStreamWaitEvent(c.s_copy, c.ev_copy, 0);
        cs = c.s_copy;
    }
    if (lits && L) cudaMemcpyAsync(lits, c.pk_lits, L * sizeof(uint32_t), cudaMemcpyDeviceToHost, cs);
    if (cls_learnt && C) cudaMemcpyAsync(cls_learnt, c.pk_learnt, C, cudaMemcpyDeviceToHost, cs);
    if (cls_lbd && C) cudaMemcpyAsync(cls_lbd, c.pk_lbd, C * sizeof(uint32_t), cudaMemcpyDeviceToHost, cs);
    if (cls_usage && C) cudaMemcpyAsync(cls_usage, c.pk_usage, C, cudaMemcpyDeviceToHost, cs);
    // output starts of every instance: eliminated, units, stack
    std::vector<unsigned long long> hb(6 * ((size_t)n + 1), 0);
    unsigned long long* eb = hb.data();
    unsigned long long* ub = eb + (n + 1);
    unsigned long long* sb = ub + (n + 1);
    unsigned long long* tsrc = sb + (n + 1);
    unsigned long long* ssrc = tsrc + (n + 1);
    unsigned long long* cb = ssrc + (n + 1);
    for (uint32_t i = 0; i < n; i++) {
        eb[i + 1] = eb[i] + c.ih[i].V + 1;
        ub[i + 1] = ub[i] + std::min<uint64_t>(c.hout.tcount[i], c.hi.tcap[i]);
        sb[i + 1] = sb[i] + c.hout.scount[i];
        tsrc[i] = c.hi.tbase[i];
        ssrc[i] = c.hi.sbase[i];
    }
    for (uint32_t i = 0; i <= n; i++) cb[i] = c.cache_cls_base[i];
    std::vector<uint32_t> shift(n);
    for (uint32_t i = 0; i < n; i++) shift[i] = c.ih[i].voff;
    unsigned long long* dbases = nullptr;
    uint32_t* dshift = nullptr;
    unsigned long long* doff = nullptr;
    uint8_t* delim = nullptr;
    uint32_t *dunits = nullptr, *dstack = nullptr;
    bool ok = dalloc_t(c, &dbases, hb.size() + (size_t)n + 1) && dalloc_t(c, &dshift, (size_t)n + 1) &&
              dalloc_t(c, &doff, C + n + 1) && dalloc_t(c, &delim, eb[n] + 1) && dalloc_t(c, &dunits, ub[n] + 1) &&
              dalloc_t(c, &dstack, sb[n] + 1);
    auto release = [&]() {
        if (cs != c.s) cudaStreamSynchronize(cs);    // no copy into the caller's buffers outlives the call
        dfree(c, dbases); dfree(c, dshift); dfree(c, doff); dfree(c, delim); dfree(c, dunits); dfree(c, dstack);
    };
    if (!ok) { release(); return finish(c, nullptr, base_launches, PFG_CNFALLOC_FAIL); }
    cudaMemcpyAsync(dbases, hb.data(), hb.size() * sizeof(unsigned long long), cudaMemcpyHostToDevice, c.s);
    cudaMemcpyAsync(dbases + hb.size(), c.cache_lit_base.data(), ((size_t)n + 1) * sizeof(unsigned long long),
                    cudaMemcpyHostToDevice, c.s);
    cudaMemcpyAsync(dshift, shift.data(), (size_t)n * sizeof(uint32_t), cudaMemcpyHostToDevice, c.s);
    const unsigned long long* d_eb = dbases;
    const unsigned long long* d_ub = d_eb + (n + 1);
    const unsigned long long* d_sb = d_ub + (n + 1);
    const unsigned long long* d_tsrc = d_sb + (n + 1);
    const unsigned long long* d_ssrc = d_tsrc + (n + 1);
    const unsigned long long* d_cb = d_ssrc + (n + 1);
    const unsigned long long* d_lb = dbases + hb.size();
    if (cls_off)
        PFG_LAUNCH(K_DOWNLOAD, offsets_all_k, grid_for(C + n, 256), 256, 0, c.s, c.pk_roff, C, d_cb, d_lb, n, doff);
    if (eliminated)
        PFG_LAUNCH(K_DOWNLOAD, elim_all_k, grid_for(eb[n], 256), 256, 0, c.s, c.elim, d_eb, c.di.voff, n, eb[n], delim);
    uint32_t* units_sorted = dunits;
    uint32_t *uk1 = nullptr, *uv0 = nullptr, *uv1 = nullptr;
    if (units && ub[n]) {
        // every instance's units sorted ascending on the device: a stable sort by
        // literal, then a stable sort by instance
        const uint64_t N = ub[n];
        PFG_LAUNCH(K_DOWNLOAD, regions_all_k, grid_for(N, 256), 256, 0, c.s, c.trail, d_tsrc, d_ub, dshift, n, N,
                   dunits);
        uint32_t vmax = 0;
        for (uint32_t i = 0; i < n; i++) vmax = std::max(vmax, c.ih[i].V);
        if (!dalloc_t(c, &uk1, N) || !dalloc_t(c, &uv0, N) || !dalloc_t(c, &uv1, N) ||
            !ensure_tmp(c, radix_temp_bytes(N))) {
            release(); dfree(c, uk1); dfree(c, uv0); dfree(c, uv1);
            return finish(c, nullptr, base_launches, PFG_CNFALLOC_FAIL);
        }
        PFG_LAUNCH(K_DOWNLOAD, region_ids_k, grid_for(N, 256), 256, 0, c.s, d_ub, n, N, uv0);
        const int r1 = radix_sort_pairs(dunits, uv0, uk1, uv1, N, 0, (int)bits_for(2ull * vmax + 1), c.tmp, c.s);
        uint32_t* lk = r1 ? uk1 : dunits;     // literals, sorted
        uint32_t* li = r1 ? uv1 : uv0;        // their instances
        uint32_t* ak = r1 ? dunits : uk1;     // spare pair
        uint32_t* ai = r1 ? uv0 : uv1;
        const int r2 = radix_sort_pairs(li, lk, ai, ak, N, 0, (int)bits_for(n), c.tmp, c.s);
        units_sorted = r2 ? ak : lk;
    }
    if (stack && sb[n])
        PFG_LAUNCH(K_DOWNLOAD, regions_all_k, grid_for(sb[n], 256), 256, 0, c.s, c.stack, d_ssrc, d_sb,
                   (const uint32_t*)nullptr, n, sb[n], dstack);
    if (cls_off) cudaMemcpyAsync(cls_off, doff, (C + n) * sizeof(uint64_t), cudaMemcpyDeviceToHost, c.s);
    if (eliminated) cudaMemcpyAsync(eliminated, delim, eb[n], cudaMemcpyDeviceToHost, c.s);
    if (units && ub[n]) cudaMemcpyAsync(units, units_sorted, ub[n] * sizeof(uint32_t), cudaMemcpyDeviceToHost, c.s);
    if (stack && sb[n]) cudaMemcpyAsync(stack, dstack, sb[n] * sizeof(uint32_t), cudaMemcpyDeviceToHost, c.s);
    bool synced = stream_sync(c, "batch download");
    if (cs != c.s) synced = cuda_ok(c, cudaStreamSynchronize(cs), "batch download copies") && synced;
    release();
    dfree(c, uk1); dfree(c, uv0); dfree(c, uv1);
    if (!synced) return finish(c, nullptr, base_launches, PFG_CUDA_ERROR);
    uint64_t pend = 0, rends = 0;
    for (uint32_t i = 0; i < n; i++) {
        const InstHost& h = c.ih[i];
        if (pending_units && !h.pending.empty()) {
            for (size_t k = 0; k < h.pending.size(); k++) pending_units[pend + k] = h.pending[k] - 2u * h.voff;
            std::sort(pending_units + pend, pending_units + pend + h.pending.size());
        }
        pend += h.pending.size();
        if (round_ends) std::copy(h.round_ends.begin(), h.round_ends.end(), round_ends + rends);
        rends += h.round_ends.size();
    }
    return finish(c, nullptr, base_launches, PFG_OK);
}

bool pfg::profiling(pfg_ctx* o) { return o && o->c.prof.on; }

void pfg::set_error(pfg_ctx* o, const std::string& e) {
    if (o) o->c.err = e;
}

extern "C" int pfg_tuning_get(pfg_ctx* o, pfg_tuning* out) {
    if (!o || !out) return PFG_INVALID;
    *out = o->c.tune;
    return PFG_OK;
}

extern "C" int pfg_set_loop_limits(pfg_ctx* o, uint32_t max_bcp_levels, uint32_t max_mis_rounds) {
    if (!o) return PFG_INVALID;
    o->c.lim_bcp_levels = max_bcp_levels;
    o->c.lim_mis_rounds = max_mis_rounds;
    return PFG_OK;
}

extern "C" int pfg_tuning_set(pfg_ctx* o, const pfg_tuning* t) {
    if (!o || !t) return PFG_INVALID;
    auto threads_ok = [](uint32_t v) { return v == 0 || (v % 32 == 0 && v <= 1024); };
    if (t->sub_blocks_per_sm > 64 || t->ve1_blocks_per_sm > 64 || t->ve3_blocks_per_sm > 64 ||
        t->bcp_blocks_per_sm > 64 || t->ve3_ticket > 65536 || !threads_ok(t->mis_threads) ||
        !threads_ok(t->list_threads)) {
        o->c.err = "tuning field out of range (blocks per SM <= 64, ticket <= 65536, threads a multiple of 32 "
                   "up to 1024)";
        return PFG_INVALID;
    }
    o->c.tune = *t;
    return PFG_OK;
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
    if (g_prof == &c.prof) g_prof = nullptr;   // the calling thread's launches no longer mark this profiler
    std::vector<void*> ptrs;
    for (auto& kv : o->sizes) ptrs.push_back(kv.first);
    for (void* p : ptrs) cudaFreeAsync(p, c.s);
    if (c.s) { cudaStreamSynchronize(c.s); cudaStreamDestroy(c.s); }
    if (c.s_copy) { cudaStreamSynchronize(c.s_copy); cudaStreamDestroy(c.s_copy); }
    if (c.ev_copy) cudaEventDestroy(c.ev_copy);
    if (c.ev_begin) cudaEventDestroy(c.ev_begin);
    if (c.ev_end) cudaEventDestroy(c.ev_end);
    c.pass_clock.destroy();
    if (c.hc) cudaFreeHost(c.hc);
    if (c.in_blob_h) cudaFreeHost(c.in_blob_h);
    if (c.out_blob_h) cudaFreeHost(c.out_blob_h);
    c.prof.destroy();
    cudaGetLastError();
    delete o;
}

// ---- allocation-free write-back into caller-owned device buffers ----
namespace pfg {
namespace {

// Scratch of pfg_download_device_noalloc: per clause slot a u32 flag and a u64
// size (each region 256-byte aligned), then the tile sums of the scans.
constexpr size_t NOALLOC_SCRATCH_BYTES = 16ull << 20;
static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_SCRATCH_BYTES];

size_t noalloc_bytes(uint64_t n) {
    return align_up(4 * (n + 1)) + align_up(8 * (n + 1)) + scan_temp_bytes(n + 1);
}

// the largest clause store (slots, live or deleted) the scratch covers
uint64_t noalloc_max_slots() {
    uint64_t lo = 0, hi = NOALLOC_SCRATCH_BYTES / 12;
    while (lo < hi) {
        const uint64_t mid = (lo + hi + 1) / 2;
        if (noalloc_bytes(mid) <= NOALLOC_SCRATCH_BYTES) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// Device address of the scratch array in the current context. The lookup is
// made on every call (it allocates nothing once the module is loaded), so an
// address never outlives the context it belongs to (a device reset or a
// re-created primary context gives the array a new address).
bool noalloc_scratch(Ctx& c, char** out) {
    int dev = -1;
    if (!cuda_ok(c, cudaGetDevice(&dev), "cudaGetDevice")) return false;
    if (dev != c.device) { c.err = "the context's device is not the current device"; return false; }
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
        cudaGetLastError();
        c.err = std::string("cudaGetSymbolAddress of the download scratch failed: ") + cudaGetErrorString(e);
        return false;
    }
    *out = (char*)p;
    return true;
}

// out_pack_k that skips the outputs the caller did not ask for
__global__ void out_pack_opt_k(const ClsHdr* hdr, const uint32_t* lits, uint64_t ncls, const uint32_t* pos,
                               const unsigned long long* loff, uint32_t* olits, unsigned long long* ooff,
                               uint8_t* olearnt, uint32_t* olbd, uint8_t* ousage) {
    const uint64_t warp = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    const unsigned lane = threadIdx.x & 31u;
    for (uint64_t c = warp; c < ncls; c += nwarps) {
        const ClsHdr h = hdr[c];
        if (m_deleted(h.meta)) continue;
        const unsigned long long o = loff[c];
        if (olits)
            for (uint32_t k = lane; k < h.size; k += 32) olits[o + k] = lits[h.off + k];
        if (lane == 0) {
            const uint32_t q = pos[c];
            if (ooff) ooff[q] = o;
            if (olearnt) olearnt[q] = m_learnt(h.meta);
            if (olbd) olbd[q] = m_lbd(h.meta);
            if (ousage) ousage[q] = (uint8_t)m_usage(h.meta);
        }
    }
}

}  // namespace
}  // namespace pfg

extern "C" int pfg_download_device_noalloc(pfg_ctx* o, uint32_t* d_lits, uint64_t* d_cls_off, uint8_t* d_cls_learnt,
                                           uint32_t* d_cls_lbd, uint8_t* d_cls_usage) {
    if (!o) return PFG_INVALID;
    Ctx& c = o->c;
    c.err.clear();
    if (!c.uploaded) { c.err = "no instance uploaded"; return PFG_INVALID; }
    if (c.ninst != 1) { c.err = "several instances uploaded: the allocation-free download takes one"; return PFG_INVALID; }
    const uint64_t n = c.ncls, C = c.numClauses;
    if (noalloc_bytes(n) > NOALLOC_SCRATCH_BYTES) {
        c.err = "the clause store has " + std::to_string(n) + " clause slots; the allocation-free download handles at most " +
                std::to_string(noalloc_max_slots()) + " (its scratch is a fixed 16 MiB device array)";
        return PFG_INVALID;
    }
    char* scratch = nullptr;
    if (!noalloc_scratch(c, &scratch)) return PFG_CUDA_ERROR;
    uint32_t* flag = (uint32_t*)scratch;
    unsigned long long* sz = (unsigned long long*)(scratch + align_up(4 * (n + 1)));
    void* tmp = scratch + align_up(4 * (n + 1)) + align_up(8 * (n + 1));
    unsigned long long* ooff = reinterpret_cast<unsigned long long*>(d_cls_off);
    const uint64_t base_launches = g_launches;
    if (n) {
        PFG_LAUNCH(K_DOWNLOAD, out_flags_k, grid_for(n, 256), 256, 0, c.s, c.hdr, n, flag, sz);
        exclusive_scan_u32(flag, flag, n, 0u, nullptr, tmp, c.s);
        exclusive_scan_u64(sz, sz, n, 0ull, ooff ? ooff + C : nullptr, tmp, c.s);
        PFG_LAUNCH(K_DOWNLOAD, out_pack_opt_k, grid_for(n * 32, 256), 256, 0, c.s, c.hdr, c.lits, n, flag, sz, d_lits,
                   ooff, d_cls_learnt, d_cls_lbd, d_cls_usage);
    } else if (ooff) {
        cudaMemsetAsync(ooff, 0, sizeof(unsigned long long), c.s);
    }
    const bool ok = stream_sync(c, "allocation-free download");
    c.launches += g_launches - base_launches;
    return ok ? PFG_OK : PFG_CUDA_ERROR;
}
