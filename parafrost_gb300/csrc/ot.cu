// Occurrence-table construction and sorting.
//
// Replaces histSimp (full sort of all literals, histogram.cu:54-71),
// resizeOTAsync/assignListPtrs (memory.cu:421-466), create_ot_k
// (occurrence.cu:50-62) and the moderngpu segmented sort of sortOT
// (segsort.cu:37-47) with:
//   1. a literal histogram by atomics over live clauses,
//   2. an exclusive scan into CSR offsets,
//   3. an atomic scatter of clause ids,
//   4. a size-tiered segmented sort by the OLIST_CMP key (key.cuh:67-85):
//      insertion sort, a thread per list (<= 16 entries); shuffle bitonic
//      network, a warp per list (<= 64); block bitonic sort in shared
//      memory (<= 2048); chunk sort + merge-path passes for longer lists.
#include <algorithm>
#include <vector>

#include "engine.cuh"

namespace pfg {
namespace {

constexpr uint32_t SMALL_MAX = 16;
// The list passes give a warp 32 consecutive lists; a list longer than this
// (the hub literals of skewed instances) is handed to a whole block instead,
// so one warp does not walk it 32 entries at a time while the grid waits.
constexpr uint32_t OT_LONG = 1024;
constexpr int LONG_THREADS = 1024;
constexpr uint32_t WARP_MAX = 64;
constexpr uint32_t MID_MAX = 2048;
constexpr int MID_THREADS = 256;

__global__ void hist_k(const ClsHdr* __restrict__ hdr, const uint32_t* __restrict__ lits, uint64_t ncls,
                       uint32_t* hist) {
    for (uint64_t c = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; c < ncls; c += (uint64_t)gridDim.x * blockDim.x) {
        const ClsHdr h = hdr[c];
        if (m_deleted(h.meta)) continue;
        for (uint32_t k = 0; k < h.size; k++) atomicAdd(&hist[lits[h.off + k]], 1u);
    }
}

// One clause's entries: its literals are loaded FILL_BURST at a time and their
// cursor increments issued together, so the atomics' round trips to L2
// overlap instead of each one waiting for the previous store.
constexpr uint32_t FILL_BURST = 8;

PFG_D void fill_clause(const ClsHdr& h, const uint32_t* __restrict__ lits, uint32_t c, uint32_t* fill,
                       uint32_t* ids) {
    for (uint32_t k0 = 0; k0 < h.size; k0 += FILL_BURST) {
        uint32_t l[FILL_BURST], pos[FILL_BURST];
#pragma unroll
        for (uint32_t q = 0; q < FILL_BURST; q++) l[q] = k0 + q < h.size ? lits[h.off + k0 + q] : 0u;
#pragma unroll
        for (uint32_t q = 0; q < FILL_BURST; q++)
            if (k0 + q < h.size) pos[q] = atomicAdd(&fill[l[q]], 1u);
#pragma unroll
        for (uint32_t q = 0; q < FILL_BURST; q++)
            if (k0 + q < h.size) ids[pos[q]] = c;
    }
}

__global__ void fill_k(const ClsHdr* __restrict__ hdr, const uint32_t* __restrict__ lits, uint64_t ncls,
                       uint32_t* fill, uint32_t* ids) {
    for (uint64_t c = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; c < ncls; c += (uint64_t)gridDim.x * blockDim.x) {
        const ClsHdr h = hdr[c];
        if (m_deleted(h.meta)) continue;
        fill_clause(h, lits, (uint32_t)c, fill, ids);
    }
}

// ---- incremental update between rounds ----
// occurrences of the flagged (added or rewritten) live clauses
__global__ void new_hist_k(const ClsHdr* __restrict__ hdr, const uint32_t* __restrict__ lits, uint64_t ncls,
                           const uint8_t* __restrict__ cnew, uint32_t* hist) {
    for (uint64_t c = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; c < ncls; c += (uint64_t)gridDim.x * blockDim.x) {
        if (!cnew[c]) continue;
        const ClsHdr h = hdr[c];
        if (m_deleted(h.meta)) continue;
        for (uint32_t k = 0; k < h.size; k++) atomicAdd(&hist[lits[h.off + k]], 1u);
    }
}

__global__ void fill_new_k(const ClsHdr* __restrict__ hdr, const uint32_t* __restrict__ lits, uint64_t ncls,
                           const uint8_t* __restrict__ cnew, uint32_t* fill, uint32_t* ids) {
    for (uint64_t c = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; c < ncls; c += (uint64_t)gridDim.x * blockDim.x) {
        if (!cnew[c]) continue;
        const ClsHdr h = hdr[c];
        if (m_deleted(h.meta)) continue;
        fill_clause(h, lits, (uint32_t)c, fill, ids);
    }
}

// Lists are processed 32 at a time by one warp: the lanes walk the entries of
// the 32 lists back to back (the lists lie next to each other in the id array,
// so the reads are nearly coalesced and a long list does not hold up one
// thread), each lane finding its entry's list by a binary search over the
// lists' starts.
PFG_D uint32_t owner_lane(uint32_t pre, uint32_t e) {
    uint32_t lo = 0, hi = 31;   // last lane whose list starts at or before e
#pragma unroll
    for (int it = 0; it < 5; it++) {
        const uint32_t mid = (lo + hi + 1) >> 1;
        const uint32_t pm = __shfl_sync(0xFFFFFFFFu, pre, mid);
        if (pm <= e) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// flag[c] |= deleted: the list filters then read one byte per entry (an array
// that stays in L2) instead of a clause header
__global__ void mark_dead_k(const ClsHdr* __restrict__ hdr, uint64_t ncls, uint8_t* flag) {
    for (uint64_t c = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; c < ncls; c += (uint64_t)gridDim.x * blockDim.x)
        if (m_deleted(hdr[c].meta)) flag[c] = 1;
}

// After unit propagation (bcp_apply_k) a list of an assigned variable is empty:
// a true literal's clauses are satisfied and deleted, a false literal was
// stripped from its clauses. Other lists lose the clauses flagged in `drop`
// (deleted ones; between rounds also the added and rewritten ones, listed again
// by ot_update). `assigned` is then the eliminated-byte array: an eliminated
// variable's lists are emptied. In place, order kept.
__global__ void ot_filter_w_k(uint64_t nlist, const uint32_t* __restrict__ off, uint32_t* size, uint32_t* hist,
                              uint32_t* ids, const uint8_t* __restrict__ assigned, const uint8_t* __restrict__ drop,
                              uint32_t* longs, uint32_t* nlong) {
    const unsigned lane = threadIdx.x & 31u;
    const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    for (uint64_t w = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; w * 32 < nlist; w += nwarps) {
        const uint64_t l = w * 32 + lane;
        uint32_t n = 0, o = 0;
        bool is_long = false;
        if (l < nlist) {
            n = size[l];
            if (n && assigned[l >> 1]) n = 0;
            o = off[l];
            if (n > OT_LONG) {   // ot_filter_long_k filters it
                longs[atomicAdd(nlong, 1u)] = (uint32_t)l;
                is_long = true;
                n = 0;
            }
        }
        uint32_t incl = n;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint32_t t = __shfl_up_sync(0xFFFFFFFFu, incl, d);
            if (lane >= (unsigned)d) incl += t;
        }
        const uint32_t pre = incl - n, T = __shfl_sync(0xFFFFFFFFu, incl, 31);
        uint32_t kept = 0;
        // the ids of the next chunk are loaded while this one is decided (every
        // write goes to a position at or before the entry it keeps, so no write
        // of a chunk reaches a later chunk's entries)
        uint32_t nj = owner_lane(pre, lane);
        uint32_t nsj = __shfl_sync(0xFFFFFFFFu, pre, nj);
        uint32_t noj = __shfl_sync(0xFFFFFFFFu, o, nj);
        uint32_t nc = lane < T ? ids[noj + (lane - nsj)] : 0u;
        for (uint32_t e0 = 0; e0 < T; e0 += 32) {
            const uint32_t e = e0 + lane;
            const uint32_t j = nj, sj = nsj, oj = noj, c = nc;
            const uint32_t kj = __shfl_sync(0xFFFFFFFFu, kept, j);
            const bool valid = e < T;
            if (e0 + 32 < T) {
                const uint32_t e2 = e + 32;
                nj = owner_lane(pre, e2);
                nsj = __shfl_sync(0xFFFFFFFFu, pre, nj);
                noj = __shfl_sync(0xFFFFFFFFu, o, nj);
                nc = e2 < T ? ids[noj + (e2 - nsj)] : 0u;
            }
            const bool keep = valid && !drop[c];
            const unsigned bal = __ballot_sync(0xFFFFFFFFu, keep);
            // lanes of list j in this chunk start at lane max(sj - e0, 0)
            const uint32_t first = sj > e0 ? sj - e0 : 0u;
            const unsigned mine = ((1u << lane) - 1u) & ~((1u << first) - 1u);
            // an entry with no dropped entry before it in its list stays where it is
            const uint32_t to = oj + kj + __popc(bal & mine);
            if (keep && to != oj + (e - sj)) ids[to] = c;
            // this lane's own list: its entries in this chunk
            const int64_t a = (int64_t)pre - (int64_t)e0, b = a + (int64_t)n;
            const int lo = a < 0 ? 0 : (a > 32 ? 32 : (int)a);
            const int hi = b < 0 ? 0 : (b > 32 ? 32 : (int)b);
            if (hi > lo) {
                const unsigned m = (hi - lo == 32) ? 0xFFFFFFFFu : (((1u << (hi - lo)) - 1u) << lo);
                kept += __popc(bal & m);
            }
        }
        if (l < nlist && !is_long) { size[l] = kept; hist[l] = kept; }
    }
}

// Exclusive prefix of one flag per thread over a block of LONG_THREADS
// threads; *total gets the block's count. `sh` holds 33 words.
PFG_D uint32_t block_flag_scan(bool f, uint32_t* sh, uint32_t* total) {
    const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const unsigned bal = __ballot_sync(0xFFFFFFFFu, f);
    if (lane == 0) sh[warp] = __popc(bal);
    __syncthreads();
    if (warp == 0) {
        const uint32_t v = lane < (blockDim.x >> 5) ? sh[lane] : 0u;
        uint32_t incl = v;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint32_t t = __shfl_up_sync(0xFFFFFFFFu, incl, d);
            if (lane >= (unsigned)d) incl += t;
        }
        sh[lane] = incl - v;
        if (lane == 31) sh[32] = incl;
    }
    __syncthreads();
    const uint32_t pre = sh[warp] + __popc(bal & ((1u << lane) - 1u));
    *total = sh[32];
    __syncthreads();
    return pre;
}

// The long lists ot_filter_w_k handed over: one block per list, a tile of
// LONG_THREADS entries at a time, order kept. In place: a tile's entries are
// read before any of its kept entries is written, and they go to positions
// at or before their own.
__global__ void __launch_bounds__(LONG_THREADS) ot_filter_long_k(const uint32_t* __restrict__ off, uint32_t* size,
                                                                 uint32_t* hist, uint32_t* ids,
                                                                 const uint8_t* __restrict__ drop,
                                                                 const uint32_t* longs, const uint32_t* nlong) {
    __shared__ uint32_t sh[33];
    const uint32_t count = *nlong;
    for (uint32_t b = blockIdx.x; b < count; b += gridDim.x) {
        const uint32_t l = longs[b];
        const uint32_t n = size[l], o = off[l];
        uint32_t kept = 0;
        for (uint32_t t0 = 0; t0 < n; t0 += blockDim.x) {
            const uint32_t i = t0 + threadIdx.x;
            const uint32_t c = i < n ? ids[o + i] : 0u;
            const bool keep = i < n && !drop[c];
            uint32_t total;
            const uint32_t pre = block_flag_scan(keep, sh, &total);   // synchronises after the reads
            if (keep && kept + pre != i) ids[o + kept + pre] = c;      // moved entries only
            kept += total;
        }
        if (threadIdx.x == 0) { size[l] = kept; hist[l] = kept; }
        __syncthreads();
    }
}

// sizes of the update before the drops are known: a list's old size (nothing
// for an eliminated variable's lists), new_hist_k adds the flagged clauses
__global__ void hist_init_k(uint64_t nlist, const uint32_t* __restrict__ size, const uint8_t* __restrict__ elim,
                            uint32_t* hist) {
    for (uint64_t l = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; l < nlist; l += (uint64_t)gridDim.x * blockDim.x)
        hist[l] = elim[l >> 1] ? 0u : size[l];
}

// Whether the table update keeps clause c, and its id in the new store: after
// a compaction from the words of drop_bits_k (kept bit; live clauses before
// the word plus the live bits below c), else from the drop bytes (id kept).
PFG_D bool entry_kept(const uint8_t* __restrict__ drop, const uint4* __restrict__ bits, uint32_t c, uint32_t& id) {
    if (bits) {
        const uint4 b = bits[c >> 5];
        const uint32_t bit = c & 31u;
        id = b.z + __popc(b.x & ((1u << bit) - 1u));
        return (b.y >> bit) & 1u;
    }
    id = c;
    return !drop[c];
}

// Prune and move in one pass: the entries of every list that `drop` keeps
// (not deleted, not flagged) go in order to the list's new offset, renumbered
// through the compaction words when the store was compacted; an eliminated variable's lists
// keep nothing. The new offsets were sized for the whole old list, so a list
// ends with the gap of its dropped entries; its size (and histogram count,
// which the election reads) becomes the kept entries plus its flagged clauses,
// and its append cursor starts behind the kept ones. Same warp layout as the
// in-place filter, but reads and writes go to different arrays.
__global__ void prune_move_w_k(uint64_t nlist, const uint32_t* __restrict__ off, uint32_t* size, uint32_t* hist,
                               const uint32_t* __restrict__ ids, const uint8_t* __restrict__ elim,
                               const uint8_t* __restrict__ drop, const uint32_t* __restrict__ off2,
                               uint32_t* __restrict__ ids2, const uint4* __restrict__ bits, uint32_t* fill,
                               uint32_t* longs, uint32_t* nlong) {
    const unsigned lane = threadIdx.x & 31u;
    const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    for (uint64_t w = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; w * 32 < nlist; w += nwarps) {
        const uint64_t l = w * 32 + lane;
        uint32_t n = 0, o = 0, o2 = 0;
        bool is_long = false;
        if (l < nlist) {
            n = size[l];
            if (n && elim[l >> 1]) n = 0;
            o = off[l];
            o2 = off2[l];
            if (n > OT_LONG) {   // prune_move_long_k moves it
                longs[atomicAdd(nlong, 1u)] = (uint32_t)l;
                is_long = true;
                n = 0;
            }
        }
        uint32_t incl = n;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint32_t t = __shfl_up_sync(0xFFFFFFFFu, incl, d);
            if (lane >= (unsigned)d) incl += t;
        }
        const uint32_t pre = incl - n, T = __shfl_sync(0xFFFFFFFFu, incl, 31);
        uint32_t kept = 0;
        uint32_t nj = owner_lane(pre, lane);
        uint32_t nsj = __shfl_sync(0xFFFFFFFFu, pre, nj);
        uint32_t noj = __shfl_sync(0xFFFFFFFFu, o, nj);
        uint32_t nc = lane < T ? ids[noj + (lane - nsj)] : 0u;
        for (uint32_t e0 = 0; e0 < T; e0 += 32) {
            const uint32_t e = e0 + lane;
            const uint32_t j = nj, sj = nsj, c = nc;
            const uint32_t kj = __shfl_sync(0xFFFFFFFFu, kept, j);
            const uint32_t o2j = __shfl_sync(0xFFFFFFFFu, o2, j);
            const bool valid = e < T;
            if (e0 + 32 < T) {
                const uint32_t e2 = e + 32;
                nj = owner_lane(pre, e2);
                nsj = __shfl_sync(0xFFFFFFFFu, pre, nj);
                noj = __shfl_sync(0xFFFFFFFFu, o, nj);
                nc = e2 < T ? ids[noj + (e2 - nsj)] : 0u;
            }
            uint32_t id = c;
            const bool keep = valid && entry_kept(drop, bits, c, id);
            const unsigned bal = __ballot_sync(0xFFFFFFFFu, keep);
            const uint32_t first = sj > e0 ? sj - e0 : 0u;
            const unsigned mine = ((1u << lane) - 1u) & ~((1u << first) - 1u);
            if (keep) ids2[o2j + kj + __popc(bal & mine)] = id;
            const int64_t a = (int64_t)pre - (int64_t)e0, b = a + (int64_t)n;
            const int lo = a < 0 ? 0 : (a > 32 ? 32 : (int)a);
            const int hi = b < 0 ? 0 : (b > 32 ? 32 : (int)b);
            if (hi > lo) {
                const unsigned m = (hi - lo == 32) ? 0xFFFFFFFFu : (((1u << (hi - lo)) - 1u) << lo);
                kept += __popc(bal & m);
            }
        }
        if (l < nlist && !is_long) {
            const uint32_t total = kept + (hist[l] - n);
            size[l] = total;
            hist[l] = total;
            fill[l] = o2 + kept;
        }
    }
}

// The long lists prune_move_w_k handed over: one block per list, a tile of
// LONG_THREADS entries at a time, order kept, into the new layout.
__global__ void __launch_bounds__(LONG_THREADS) prune_move_long_k(const uint32_t* __restrict__ off, uint32_t* size,
                                                                  uint32_t* hist, const uint32_t* __restrict__ ids,
                                                                  const uint8_t* __restrict__ drop,
                                                                  const uint32_t* __restrict__ off2,
                                                                  uint32_t* __restrict__ ids2,
                                                                  const uint4* __restrict__ bits, uint32_t* fill,
                                                                  const uint32_t* longs, const uint32_t* nlong) {
    __shared__ uint32_t sh[33];
    const uint32_t count = *nlong;
    for (uint32_t b = blockIdx.x; b < count; b += gridDim.x) {
        const uint32_t l = longs[b];
        const uint32_t n = size[l], o = off[l], o2 = off2[l];
        uint32_t kept = 0;
        for (uint32_t t0 = 0; t0 < n; t0 += blockDim.x) {
            const uint32_t i = t0 + threadIdx.x;
            const uint32_t c = i < n ? ids[o + i] : 0u;
            uint32_t id = c;
            const bool keep = i < n && entry_kept(drop, bits, c, id);
            uint32_t total;
            const uint32_t pre = block_flag_scan(keep, sh, &total);
            if (keep) ids2[o2 + kept + pre] = id;
            kept += total;
        }
        if (threadIdx.x == 0) {
            // the list's old size n was counted in hist by hist_init_k
            const uint32_t total = kept + (hist[l] - n);
            size[l] = total;
            hist[l] = total;
            fill[l] = o2 + kept;
        }
        __syncthreads();
    }
}

// OLIST_CMP key of every live clause, computed once per sort in clause order
__global__ void ckeys_k(const ClsHdr* __restrict__ hdr, const uint32_t* __restrict__ lits, uint64_t ncls,
                        uint4* keys, bool by_id) {
    for (uint64_t c = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; c < ncls; c += (uint64_t)gridDim.x * blockDim.x) {
        const ClsHdr h = hdr[c];
        if (m_deleted(h.meta)) continue;
        keys[c] = by_id ? make_uint4(0, 0, 0, 0) : make_uint4(h.size, lits[h.off], lits[h.off + h.size - 1], h.sig);
    }
}

PFG_D uint4 ckey(const uint4* keys, uint32_t c) { return keys[c]; }

// OLIST_CMP: (size, first, last, sig, ref)
PFG_D bool kless(const uint4& a, uint32_t ia, const uint4& b, uint32_t ib) {
    if (a.x != b.x) return a.x < b.x;
    if (a.y != b.y) return a.y < b.y;
    if (a.z != b.z) return a.z < b.z;
    if (a.w != b.w) return a.w < b.w;
    return ia < ib;
}

// All lists (vlist null, count = number of lists) or the two lists of each
// variable of vlist[0..count/2).
__global__ void sort_small_k(const uint4* keys, const uint32_t* vlist, uint64_t count,
                             const uint32_t* off, const uint32_t* size, uint32_t* ids,
                             uint32_t* mid_desc, uint32_t* mid_cnt, uint32_t* big_lists, uint32_t* big_cnt,
                             uint32_t* warp_desc, uint32_t* warp_cnt) {
    for (uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; t < count; t += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t l = vlist ? 2ull * vlist[t >> 1] + (t & 1) : t;
        const uint32_t n = size[l];
        if (n < 2) continue;
        if (n > SMALL_MAX) {
            if (n <= WARP_MAX) {
                const uint32_t q = atomicAdd(warp_cnt, 1u);
                warp_desc[2 * q] = off[l];
                warp_desc[2 * q + 1] = n;
            } else if (n <= MID_MAX) {
                const uint32_t q = atomicAdd(mid_cnt, 1u);
                mid_desc[2 * q] = off[l];
                mid_desc[2 * q + 1] = n;
            } else {
                big_lists[atomicAdd(big_cnt, 1u)] = (uint32_t)l;
            }
            continue;
        }
        uint32_t* L = ids + off[l];
        uint4 k[SMALL_MAX];
        uint32_t id[SMALL_MAX];
        for (uint32_t i = 0; i < n; i++) { id[i] = L[i]; k[i] = ckey(keys, id[i]); }
        for (uint32_t i = 1; i < n; i++) {
            const uint4 tk = k[i];
            const uint32_t ti = id[i];
            uint32_t j = i;
            while (j > 0 && kless(tk, ti, k[j - 1], id[j - 1])) { k[j] = k[j - 1]; id[j] = id[j - 1]; j--; }
            k[j] = tk; id[j] = ti;
        }
        for (uint32_t i = 0; i < n; i++) L[i] = id[i];
    }
}

// One list of 17..64 entries per warp: lane holds positions lane and lane+32;
// a bitonic network with shuffles for partners in the same half.
PFG_D void warp_cx(uint4& k, uint32_t& id, int j, bool keep_min) {
    uint4 o;
    o.x = __shfl_xor_sync(0xFFFFFFFFu, k.x, j);
    o.y = __shfl_xor_sync(0xFFFFFFFFu, k.y, j);
    o.z = __shfl_xor_sync(0xFFFFFFFFu, k.z, j);
    o.w = __shfl_xor_sync(0xFFFFFFFFu, k.w, j);
    const uint32_t oid = __shfl_xor_sync(0xFFFFFFFFu, id, j);
    const bool other_less = kless(o, oid, k, id);
    if (other_less == keep_min) { k = o; id = oid; }
}

__global__ void sort_warp_k(const uint4* keys, const uint32_t* desc, const uint32_t* count, uint32_t* ids) {
    const unsigned lane = threadIdx.x & 31u;
    const uint32_t nd = *count;
    const uint4 pad = make_uint4(0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu);
    for (uint32_t q = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; q < nd; q += (gridDim.x * blockDim.x) >> 5) {
        const uint32_t o = desc[2 * q], n = desc[2 * q + 1];
        uint32_t* L = ids + o;
        uint32_t ia = lane < n ? L[lane] : 0xFFFFFFFFu;
        uint32_t ib = lane + 32 < n ? L[lane + 32] : 0xFFFFFFFFu;
        uint4 ka = lane < n ? keys[ia] : pad;
        uint4 kb = lane + 32 < n ? keys[ib] : pad;
#pragma unroll
        for (int sz = 2; sz <= 64; sz <<= 1) {
#pragma unroll
            for (int j = sz >> 1; j > 0; j >>= 1) {
                const bool asc_a = (lane & sz) == 0;          // position lane
                const bool asc_b = ((lane + 32) & sz) == 0;   // position lane + 32
                if (j == 32) {
                    // partners in the same lane: a (lower position) keeps the min when ascending
                    const bool sw = asc_a ? kless(kb, ib, ka, ia) : kless(ka, ia, kb, ib);
                    if (sw) {
                        const uint4 tk = ka; ka = kb; kb = tk;
                        const uint32_t ti = ia; ia = ib; ib = ti;
                    }
                } else {
                    const bool lower = (lane & j) == 0;
                    warp_cx(ka, ia, j, lower == asc_a);
                    warp_cx(kb, ib, j, lower == asc_b);
                }
            }
        }
        if (lane < n) L[lane] = ia;
        if (lane + 32 < n) L[lane + 32] = ib;
    }
}

// Bitonic sort of one segment (<= MID_MAX) in shared memory.
PFG_D void bitonic_smem(uint4* sk, uint32_t* sid, uint32_t P) {
    for (uint32_t k = 2; k <= P; k <<= 1) {
        for (uint32_t j = k >> 1; j > 0; j >>= 1) {
            for (uint32_t i = threadIdx.x; i < P; i += blockDim.x) {
                const uint32_t ixj = i ^ j;
                if (ixj > i) {
                    const bool asc = (i & k) == 0;
                    const bool gt = kless(sk[ixj], sid[ixj], sk[i], sid[i]);
                    if (gt == asc) {
                        const uint4 tk = sk[i]; sk[i] = sk[ixj]; sk[ixj] = tk;
                        const uint32_t ti = sid[i]; sid[i] = sid[ixj]; sid[ixj] = ti;
                    }
                }
            }
            __syncthreads();
        }
    }
}

__global__ void __launch_bounds__(MID_THREADS) sort_mid_k(const uint4* keys, const uint32_t* desc, uint32_t* ids) {
    __shared__ uint4 sk[MID_MAX];
    __shared__ uint32_t sid[MID_MAX];
    const uint32_t o = desc[2 * blockIdx.x], n = desc[2 * blockIdx.x + 1];
    uint32_t P = 1;
    while (P < n) P <<= 1;
    for (uint32_t i = threadIdx.x; i < P; i += blockDim.x) {
        if (i < n) { sid[i] = ids[o + i]; sk[i] = ckey(keys, sid[i]); }
        else { sid[i] = 0xFFFFFFFFu; sk[i] = make_uint4(0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu); }
    }
    __syncthreads();
    bitonic_smem(sk, sid, P);
    for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) ids[o + i] = sid[i];
}

// Big lists: gather into a contiguous area with precomputed keys.
__global__ void big_gather_k(const uint4* keys, const uint32_t* big_lists, uint32_t nbig,
                             const uint32_t* off, const uint32_t* size, const uint32_t* boff,
                             const uint32_t* ids, uint4* bk, uint32_t* bid) {
    for (uint32_t b = blockIdx.x; b < nbig; b += gridDim.x) {
        const uint32_t l = big_lists[b], n = size[l], o = off[l], a = boff[b];
        for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
            const uint32_t c = ids[o + i];
            bid[a + i] = c;
            bk[a + i] = ckey(keys, c);
        }
    }
}

// chunk sort of big lists: block (b, chunk)
__global__ void __launch_bounds__(MID_THREADS) big_chunk_k(const uint32_t* big_lists, uint32_t nbig, const uint32_t* size,
                                                          const uint32_t* boff, uint4* bk, uint32_t* bid) {
    __shared__ uint4 sk[MID_MAX];
    __shared__ uint32_t sid[MID_MAX];
    for (uint32_t b = blockIdx.y; b < nbig; b += gridDim.y) {
    const uint32_t n = size[big_lists[b]];
    const uint32_t cs = blockIdx.x * MID_MAX;
    if (cs >= n) continue;
    const uint32_t m = min(MID_MAX, n - cs);
    const uint32_t a = boff[b] + cs;
    uint32_t P = 1;
    while (P < m) P <<= 1;
    for (uint32_t i = threadIdx.x; i < P; i += blockDim.x) {
        if (i < m) { sid[i] = bid[a + i]; sk[i] = bk[a + i]; }
        else { sid[i] = 0xFFFFFFFFu; sk[i] = make_uint4(0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu); }
    }
    __syncthreads();
    bitonic_smem(sk, sid, P);
    for (uint32_t i = threadIdx.x; i < m; i += blockDim.x) { bid[a + i] = sid[i]; bk[a + i] = sk[i]; }
    __syncthreads();
    }
}

// one merge pass: runs of length R merged pairwise (element-parallel binary search)
__global__ void big_merge_k(const uint32_t* big_lists, uint32_t nbig, const uint32_t* size, const uint32_t* boff,
                            uint32_t R, const uint4* bk, const uint32_t* bid, uint4* bk2, uint32_t* bid2) {
    for (uint32_t b = blockIdx.y; b < nbig; b += gridDim.y) {
    const uint32_t n = size[big_lists[b]];
    const uint32_t a = boff[b];
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t r = i / R, s = r * R;
        uint32_t ps, pe;
        if (r & 1u) { ps = s - R; pe = s; }
        else { ps = s + R; pe = min(s + 2 * R, n); if (ps > n) ps = n; }
        const uint4 mk = bk[a + i];
        const uint32_t mi = bid[a + i];
        // count partner elements less than me
        uint32_t lo = ps, hi = pe;
        while (lo < hi) {
            const uint32_t mid = (lo + hi) >> 1;
            if (kless(bk[a + mid], bid[a + mid], mk, mi)) lo = mid + 1;
            else hi = mid;
        }
        const uint32_t pair = (r & ~1u) * R;
        const uint32_t dst = pair + (i - s) + (lo - ps);
        bk2[a + dst] = mk;
        bid2[a + dst] = mi;
    }
    }
}

__global__ void big_scatter_k(const uint32_t* big_lists, uint32_t nbig, const uint32_t* off, const uint32_t* size,
                              const uint32_t* boff, const uint32_t* bid, uint32_t* ids) {
    for (uint32_t b = blockIdx.x; b < nbig; b += gridDim.x) {
        const uint32_t l = big_lists[b], n = size[l], o = off[l], a = boff[b];
        for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) ids[o + i] = bid[a + i];
    }
}

__global__ void big_sizes_k(const uint32_t* big_lists, uint32_t nbig, const uint32_t* size, uint32_t* out) {
    for (uint32_t b = blockIdx.x * blockDim.x + threadIdx.x; b < nbig; b += gridDim.x * blockDim.x)
        out[b] = size[big_lists[b]];
}

}  // namespace

bool ot_build(Ctx& c) {
    const uint64_t nl = c.nlist;
    if (c.numLiterals > 0xFFFFFFF0ull) { c.simpstate = PFG_OTALLOC_FAIL; c.err = "occurrence table exceeds 2^32 entries"; return false; }
    if (c.ot_cap < c.numLiterals) {
        dfree(c, c.ot_ids);
        c.ot_ids = nullptr;
        const uint64_t cap = c.numLiterals + c.numLiterals / 4 + 1024;
        if (!dalloc_t(c, &c.ot_ids, cap)) { c.simpstate = PFG_OTALLOC_FAIL; c.ot_cap = 0; return false; }
        c.ot_cap = cap;
    }
    c.prof.bytes[K_HIST] += 4 * (c.numLiterals + c.numClauses);
    c.prof.bytes[K_FILL] += 4 * (c.numLiterals + c.numClauses) + 4 * c.numLiterals;
    cudaMemsetAsync(c.hist, 0, nl * sizeof(uint32_t), c.s);
    PFG_LAUNCH(K_HIST, hist_k, grid_for(c.ncls, 256), 256, 0, c.s, c.hdr, c.lits, c.ncls, c.hist);
    if (!ensure_tmp(c, scan_temp_bytes(nl))) return false;
    exclusive_scan_u32(c.hist, c.ot_off, nl, 0u, c.ot_off + nl, c.tmp, c.s);
    cudaMemcpyAsync(c.ot_fill, c.ot_off, nl * sizeof(uint32_t), cudaMemcpyDeviceToDevice, c.s);
    cudaMemcpyAsync(c.ot_size, c.hist, nl * sizeof(uint32_t), cudaMemcpyDeviceToDevice, c.s);
    PFG_LAUNCH(K_FILL, fill_k, grid_for(c.ncls, 256), 256, 0, c.s, c.hdr, c.lits, c.ncls, c.ot_fill, c.ot_ids);
    cudaMemsetAsync(c.cnew, 0, c.ncls, c.s);
    return cuda_ok(c, cudaGetLastError(), "ot_build");
}

bool ot_filter(Ctx& c, const uint8_t* assigned) {
    PFG_LAUNCH(K_FILL, mark_dead_k, grid_for(c.ncls, 256), 256, 0, c.s, c.hdr, c.ncls, c.cnew);
    const unsigned lt = tuned(c.tune.list_threads, LIST_THREADS);
    cudaMemsetAsync(&c.dc->ot_long, 0, sizeof(uint32_t), c.s);
    PFG_LAUNCH(K_FILL, ot_filter_w_k, grid_for((c.nlist + 31) / 32 * 32, lt), lt, 0, c.s, c.nlist, c.ot_off,
               c.ot_size, c.hist, c.ot_ids, assigned, c.cnew, c.big_lists, &c.dc->ot_long);
    PFG_LAUNCH(K_FILL, ot_filter_long_k, 2 * sm_count(), LONG_THREADS, 0, c.s, c.ot_off, c.ot_size, c.hist,
               c.ot_ids, c.cnew, c.big_lists, &c.dc->ot_long);
    return cuda_ok(c, cudaGetLastError(), "ot_filter");
}

bool ot_prune(Ctx& c) {
    // the deleted clauses join the flagged ones in the drop bytes; the lists
    // are filtered when they move (ot_update), after any compaction
    PFG_LAUNCH(K_FILL, mark_dead_k, grid_for(c.ncls, 256), 256, 0, c.s, c.hdr, c.ncls, c.cnew);
    return cuda_ok(c, cudaGetLastError(), "ot_prune");
}

bool ot_update(Ctx& c) {
    const uint64_t nl = c.nlist;
    if (c.numLiterals > 0xFFFFFFF0ull) { c.simpstate = PFG_OTALLOC_FAIL; c.err = "occurrence table exceeds 2^32 entries"; return false; }
    c.prof.bytes[K_HIST] += 4 * (c.numLiterals + c.numClauses);
    c.prof.bytes[K_FILL] += 4 * (c.numLiterals + c.numClauses) + 4 * c.numLiterals;
    // room: the old entries of every list plus the occurrences of the flagged clauses
    PFG_LAUNCH(K_HIST, hist_init_k, grid_for(nl, 256), 256, 0, c.s, nl, c.ot_size, c.elim, c.hist);
    PFG_LAUNCH(K_HIST, new_hist_k, grid_for(c.ncls, 256), 256, 0, c.s, c.hdr, c.lits, c.ncls, c.cnew, c.hist);
    if (!ensure_tmp(c, scan_temp_bytes(nl))) return false;
    exclusive_scan_u32(c.hist, c.ot_off2, nl, 0u, c.ot_off2 + nl, c.tmp, c.s);
    uint32_t total = 0;
    cudaMemcpyAsync(&total, c.ot_off2 + nl, sizeof(uint32_t), cudaMemcpyDeviceToHost, c.s);
    if (!stream_sync(c, "ot_update")) return false;
    if (c.ot_cap2 < total) {   // the kept entries stay in ot_ids; only the target grows
        dfree(c, c.ot_ids2);
        c.ot_ids2 = nullptr;
        const uint64_t cap = (uint64_t)total + total / 4 + 1024;
        if (!dalloc_t(c, &c.ot_ids2, cap)) { c.simpstate = PFG_OTALLOC_FAIL; c.ot_cap2 = 0; return false; }
        c.ot_cap2 = cap;
    }
    // kept entries move to the new offsets (after a compaction the table is
    // still on the old ids: which entries stay and their new ids come from
    // c.cbits, while c.cnew is already on the new ids); the flagged clauses
    // are appended behind them
    const unsigned lt = tuned(c.tune.list_threads, LIST_THREADS);
    const uint8_t* drop = c.cbits ? nullptr : c.cnew;
    cudaMemsetAsync(&c.dc->ot_long, 0, sizeof(uint32_t), c.s);
    PFG_LAUNCH(K_FILL, prune_move_w_k, grid_for((nl + 31) / 32 * 32, lt), lt, 0, c.s, nl, c.ot_off, c.ot_size,
               c.hist, c.ot_ids, c.elim, drop, c.ot_off2, c.ot_ids2, c.cbits, c.ot_fill, c.big_lists,
               &c.dc->ot_long);
    PFG_LAUNCH(K_FILL, prune_move_long_k, 2 * sm_count(), LONG_THREADS, 0, c.s, c.ot_off, c.ot_size, c.hist,
               c.ot_ids, drop, c.ot_off2, c.ot_ids2, c.cbits, c.ot_fill, c.big_lists, &c.dc->ot_long);
    PFG_LAUNCH(K_FILL, fill_new_k, grid_for(c.ncls, 256), 256, 0, c.s, c.hdr, c.lits, c.ncls, c.cnew, c.ot_fill,
               c.ot_ids2);
    cudaMemsetAsync(c.cnew, 0, c.ncls, c.s);
    std::swap(c.ot_ids, c.ot_ids2);
    std::swap(c.ot_cap, c.ot_cap2);
    std::swap(c.ot_off, c.ot_off2);
    return cuda_ok(c, cudaGetLastError(), "ot_update");
}

bool ot_sort(Ctx& c, bool by_id, const uint32_t* vlist, uint32_t nv, bool keys_ready) {
    const uint64_t nl = c.nlist;
    const uint64_t count = vlist ? 2ull * nv : nl;
    // worst case: every list is mid-sized
    const uint64_t want_desc = std::max<uint64_t>(1024, c.numLiterals / (SMALL_MAX + 1) + 1);
    if (c.mid_desc_cap < want_desc) {
        dfree(c, c.mid_desc);
        dfree(c, c.warp_desc);
        c.mid_desc = c.warp_desc = nullptr;
        if (!dalloc_t(c, &c.mid_desc, 2 * want_desc) || !dalloc_t(c, &c.warp_desc, 2 * want_desc)) {
            c.simpstate = PFG_OTALLOC_FAIL;
            c.mid_desc_cap = 0;
            return false;
        }
        c.mid_desc_cap = want_desc;
    }
    if (c.ckeys_cap < c.ncls) {
        dfree(c, c.ckeys);
        c.ckeys = nullptr;
        const uint64_t cap = c.hdr_cap > c.ncls ? c.hdr_cap : c.ncls;
        if (!dalloc_t(c, &c.ckeys, cap)) { c.simpstate = PFG_OTALLOC_FAIL; c.ckeys_cap = 0; return false; }
        c.ckeys_cap = cap;
    }
    if (!keys_ready)
        PFG_LAUNCH(K_SORT_SMALL, ckeys_k, grid_for(c.ncls, 256), 256, 0, c.s, c.hdr, c.lits, c.ncls, c.ckeys, by_id);
    cudaMemsetAsync(&c.dc->nwin, 0, sizeof(uint32_t), c.s);
    cudaMemsetAsync(&c.dc->big_lists, 0, sizeof(uint32_t), c.s);
    cudaMemsetAsync(&c.dc->sort_warp, 0, sizeof(uint32_t), c.s);
    PFG_LAUNCH(K_SORT_SMALL, sort_small_k, grid_for(count, 256), 256, 0, c.s, c.ckeys, vlist, count, c.ot_off,
               c.ot_size, c.ot_ids, c.mid_desc, &c.dc->nwin, c.big_lists, &c.dc->big_lists, c.warp_desc,
               &c.dc->sort_warp);
    // lists of 17..64 entries: a warp each; the grid walks the device-side count
    PFG_LAUNCH(K_SORT_MID, sort_warp_k, grid_for(c.numLiterals * 32 / (SMALL_MAX + 1) + 32, 256, 16), 256, 0, c.s,
               c.ckeys, c.warp_desc, &c.dc->sort_warp, c.ot_ids);
    sync_counters(c);
    const uint32_t nmid = c.hc->nwin, nbig = c.hc->big_lists;
    if (nmid) {
        PFG_LAUNCH(K_SORT_MID, sort_mid_k, nmid, MID_THREADS, 0, c.s, c.ckeys, c.mid_desc, c.ot_ids);
    }
    if (nbig) {
        // sizes and area offsets of the big lists
        uint32_t* bsz = c.tmp_u32;  // nbig + 1 entries needed twice
        if (!ensure_tmp_u32(c, 2ull * nbig + 4)) return false;
        bsz = c.tmp_u32;
        uint32_t* boff = c.tmp_u32 + nbig + 2;
        PFG_LAUNCH(K_SORT_BIG, big_sizes_k, grid_for(nbig, 256), 256, 0, c.s, c.big_lists, nbig, c.ot_size, bsz);
        if (!ensure_tmp(c, scan_temp_bytes(nbig))) return false;
        exclusive_scan_u32(bsz, boff, nbig, 0u, boff + nbig, c.tmp, c.s);
        std::vector<uint32_t> hs(nbig + 1);
        cudaMemcpyAsync(hs.data(), bsz, nbig * sizeof(uint32_t), cudaMemcpyDeviceToHost, c.s);
        cudaMemcpyAsync(&hs[nbig], boff + nbig, sizeof(uint32_t), cudaMemcpyDeviceToHost, c.s);
        if (!stream_sync(c, "ot_sort big sizes")) return false;
        const uint64_t total = hs[nbig];
        uint32_t maxn = 0;
        for (uint32_t i = 0; i < nbig; i++) maxn = std::max(maxn, hs[i]);
        if (c.big_cap < total) {
            dfree(c, c.big_keys); dfree(c, c.big_keys_alt); dfree(c, c.big_ids); dfree(c, c.big_ids_alt);
            c.big_keys = c.big_keys_alt = nullptr; c.big_ids = c.big_ids_alt = nullptr;
            const uint64_t cap = total + total / 4 + 1024;
            if (!dalloc_t(c, &c.big_keys, cap) || !dalloc_t(c, &c.big_keys_alt, cap) ||
                !dalloc_t(c, &c.big_ids, cap) || !dalloc_t(c, &c.big_ids_alt, cap)) {
                c.simpstate = PFG_OTALLOC_FAIL; c.big_cap = 0; return false;
            }
            c.big_cap = cap;
        }
        PFG_LAUNCH(K_SORT_BIG, big_gather_k, std::min<uint32_t>(nbig, 4096), 256, 0, c.s, c.ckeys, c.big_lists, nbig,
                   c.ot_off, c.ot_size, boff, c.ot_ids, c.big_keys, c.big_ids);
        const uint32_t nchunks = (maxn + MID_MAX - 1) / MID_MAX;
        const uint32_t gy = std::min<uint32_t>(nbig, 65535);
        PFG_LAUNCH(K_SORT_BIG, big_chunk_k, dim3(nchunks, gy), MID_THREADS, 0, c.s, c.big_lists, nbig, c.ot_size, boff, c.big_keys, c.big_ids);
        uint4* k0 = c.big_keys; uint4* k1 = c.big_keys_alt;
        uint32_t* i0 = c.big_ids; uint32_t* i1 = c.big_ids_alt;
        for (uint32_t R = MID_MAX; R < maxn; R <<= 1) {
            const uint32_t gx = std::min<uint32_t>((maxn + 255) / 256, 1024);
            PFG_LAUNCH(K_SORT_BIG, big_merge_k, dim3(gx, gy), 256, 0, c.s, c.big_lists, nbig, c.ot_size, boff, R, k0, i0, k1, i1);
            std::swap(k0, k1); std::swap(i0, i1);
        }
        PFG_LAUNCH(K_SORT_BIG, big_scatter_k, std::min<uint32_t>(nbig, 4096), 256, 0, c.s, c.big_lists, nbig, c.ot_off, c.ot_size,
                                                                      boff, i0, c.ot_ids);
    }
    return cuda_ok(c, cudaGetLastError(), "ot_sort");
}

}  // namespace pfg
