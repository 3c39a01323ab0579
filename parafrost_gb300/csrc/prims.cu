// Device-wide scan, stable radix sort and compaction (see prims.cuh).
#include "prims.cuh"

namespace pfg {

thread_local uint64_t g_launches = 0;
thread_local Profiler* g_prof = nullptr;

const char* const kKernelNames[K_NUM] = {
    "ot_hist", "ot_fill", "ot_sort_small", "ot_sort_mid", "ot_sort_big", "scan", "radix_sort", "select",
    "lcve", "mis_win", "mis_apply", "sub", "ve_phase1", "ve_phase1_fun", "ve_phase3", "thread_fallback", "ere", "bcp", "count", "compact",
    "upload", "download", "misc", "bce",
};

uint32_t Profiler::record(cudaStream_t s) {
    if (used == pool.size()) {
        cudaEvent_t e;
        cudaEventCreate(&e);
        pool.push_back(e);
    }
    cudaEventRecord(pool[used], s);
    return (uint32_t)used++;
}

void Profiler::launch(int id, cudaStream_t s) {
    if (open_id == id && open_s == s) return;
    const uint32_t ev = record(s);
    if (open_id >= 0) spans.push_back({open_id, open_b, open_s == s ? ev : record(open_s)});
    open_id = id;
    open_s = s;
    open_b = ev;
}

void Profiler::after(int id) {
    if (id == K_UPLOAD || id == K_DOWNLOAD) close();
}

void Profiler::close() {
    if (open_id < 0) return;
    spans.push_back({open_id, open_b, record(open_s)});
    open_id = -1;
}

void Profiler::begin(int, cudaStream_t s) { pair_b = record(s); }

void Profiler::end(int id, cudaStream_t s) { spans.push_back({id, pair_b, record(s)}); }

void Profiler::resolve() {
    close();
    for (const Span& sp : spans) {
        float t = 0;
        cudaEventSynchronize(pool[sp.e]);
        if (cudaEventElapsedTime(&t, pool[sp.b], pool[sp.e]) == cudaSuccess) ms[sp.id] += t;
        else cudaGetLastError();
    }
    spans.clear();
    used = 0;
}

void Profiler::reset() {
    spans.clear();
    open_id = -1;
    used = 0;
    for (int i = 0; i < K_NUM; i++) { ms[i] = 0; launches[i] = 0; bytes[i] = 0; }
}

void Profiler::destroy() {
    for (cudaEvent_t e : pool) cudaEventDestroy(e);
    pool.clear();
    spans.clear();
    open_id = -1;
    used = 0;
}

namespace {

constexpr int SCAN_THREADS = 256;
constexpr int SCAN_ITEMS = 8;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;

template <typename T>
__device__ __forceinline__ T warp_incl_scan(T v) {
    const unsigned lane = threadIdx.x & 31u;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        T o = __shfl_up_sync(0xFFFFFFFFu, v, d);
        if (lane >= (unsigned)d) v += o;
    }
    return v;
}

// Block-wide exclusive scan of one value per thread; returns the block total.
template <typename T>
__device__ __forceinline__ T block_excl_scan(T v, T& total) {
    __shared__ T warp_tot[SCAN_THREADS / 32];
    const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    T incl = warp_incl_scan(v);
    if (lane == 31) warp_tot[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        T w = (lane < SCAN_THREADS / 32) ? warp_tot[lane] : T(0);
        T wi = warp_incl_scan(w);
        if (lane < SCAN_THREADS / 32) warp_tot[lane] = wi - w;
    }
    __syncthreads();
    T excl = incl - v + warp_tot[warp];
    // block total = last thread's inclusive value
    __shared__ T tot;
    if (threadIdx.x == SCAN_THREADS - 1) tot = excl + v;
    __syncthreads();
    total = tot;
    __syncthreads();
    return excl;
}

// Arrays above SCAN_SINGLE_MAX_TILES tiles: reduce, then scan. Phase 1 sums
// each tile; phase 2 scans the tile sums into tile offsets; phase 3 scans
// each tile again with its offset. The input is read twice and the output
// written once (a scan-then-add pass wrote it twice and read it back).
template <typename T>
__global__ void __launch_bounds__(SCAN_THREADS) scan_reduce_k(const T* in, uint64_t n, T* tile_sums) {
    const uint64_t base = (uint64_t)blockIdx.x * SCAN_TILE;
    T sum = 0;
#pragma unroll
    for (int i = 0; i < SCAN_ITEMS; i++) {
        const uint64_t idx = base + (uint64_t)i * SCAN_THREADS + threadIdx.x;
        if (idx < n) sum += in[idx];
    }
    T total;
    block_excl_scan<T>(sum, total);
    if (threadIdx.x == 0) tile_sums[blockIdx.x] = total;
}

// Phase 2: one block scans the tile sums, SCAN_ITEMS consecutive sums per
// thread, carrying the prefix across chunks of SCAN_TILE sums.
template <typename T>
__global__ void __launch_bounds__(SCAN_THREADS) scan_sums_k(T* sums, uint64_t nt, T init, T* total_out) {
    T carry = init;
    for (uint64_t b = 0; b < nt; b += SCAN_TILE) {
        const uint64_t first = b + (uint64_t)threadIdx.x * SCAN_ITEMS;
        T loc[SCAN_ITEMS];
        T sum = 0;
#pragma unroll
        for (int i = 0; i < SCAN_ITEMS; i++) {
            const T v = first + i < nt ? sums[first + i] : T(0);
            loc[i] = sum;
            sum += v;
        }
        T tot;
        const T ex = block_excl_scan<T>(sum, tot);
#pragma unroll
        for (int i = 0; i < SCAN_ITEMS; i++)
            if (first + i < nt) sums[first + i] = carry + ex + loc[i];
        carry += tot;
    }
    if (threadIdx.x == 0 && total_out) *total_out = carry;
}

// Phase 3: scan each tile locally from its offset (in and out may alias: a
// block reads its whole tile before it writes).
template <typename T>
__global__ void __launch_bounds__(SCAN_THREADS) scan_tiles_k(const T* in, T* out, uint64_t n, const T* offsets) {
    const uint64_t base = (uint64_t)blockIdx.x * SCAN_TILE;
    __shared__ T sh[SCAN_TILE];
    // coalesced striped load into shared memory
#pragma unroll
    for (int i = 0; i < SCAN_ITEMS; i++) {
        const uint64_t idx = base + (uint64_t)i * SCAN_THREADS + threadIdx.x;
        sh[i * SCAN_THREADS + threadIdx.x] = idx < n ? in[idx] : T(0);
    }
    __syncthreads();
    T loc[SCAN_ITEMS];
    T sum = 0;
#pragma unroll
    for (int i = 0; i < SCAN_ITEMS; i++) {
        loc[i] = sum;
        sum += sh[threadIdx.x * SCAN_ITEMS + i];
    }
    T total;
    const T excl = block_excl_scan<T>(sum, total) + offsets[blockIdx.x];
#pragma unroll
    for (int i = 0; i < SCAN_ITEMS; i++) sh[threadIdx.x * SCAN_ITEMS + i] = loc[i] + excl;
    __syncthreads();
#pragma unroll
    for (int i = 0; i < SCAN_ITEMS; i++) {
        const uint64_t idx = base + (uint64_t)i * SCAN_THREADS + threadIdx.x;
        if (idx < n) out[idx] = sh[i * SCAN_THREADS + threadIdx.x];
    }
}

// Small arrays: one block walks the tiles in order, carrying the prefix (one launch).
template <typename T>
__global__ void __launch_bounds__(SCAN_THREADS) scan_single_k(const T* in, T* out, uint64_t n, T init, T* total_out) {
    __shared__ T sh[SCAN_TILE];
    T carry = init;
    for (uint64_t base = 0; base < n; base += SCAN_TILE) {
#pragma unroll
        for (int i = 0; i < SCAN_ITEMS; i++) {
            const uint64_t idx = base + (uint64_t)i * SCAN_THREADS + threadIdx.x;
            sh[i * SCAN_THREADS + threadIdx.x] = idx < n ? in[idx] : T(0);
        }
        __syncthreads();
        T loc[SCAN_ITEMS];
        T sum = 0;
#pragma unroll
        for (int i = 0; i < SCAN_ITEMS; i++) {
            loc[i] = sum;
            sum += sh[threadIdx.x * SCAN_ITEMS + i];
        }
        T total;
        const T excl = block_excl_scan<T>(sum, total);
#pragma unroll
        for (int i = 0; i < SCAN_ITEMS; i++) sh[threadIdx.x * SCAN_ITEMS + i] = carry + loc[i] + excl;
        __syncthreads();
#pragma unroll
        for (int i = 0; i < SCAN_ITEMS; i++) {
            const uint64_t idx = base + (uint64_t)i * SCAN_THREADS + threadIdx.x;
            if (idx < n) out[idx] = sh[i * SCAN_THREADS + threadIdx.x];
        }
        carry += total;
        __syncthreads();
    }
    if (threadIdx.x == 0 && total_out) *total_out = carry;
}

constexpr uint64_t SCAN_SINGLE_MAX_TILES = 16;

template <typename T>
void excl_scan(const T* in, T* out, uint64_t n, T init, T* total_out, void* tmp, cudaStream_t s) {
    if (g_prof) g_prof->bytes[K_SCAN] += 2 * n * sizeof(T);   // byte model: the input read, the output written
    if (n == 0) {
        if (total_out) cudaMemcpyAsync(total_out, &init, sizeof(T), cudaMemcpyHostToDevice, s);
        return;
    }
    const uint64_t nt = (n + SCAN_TILE - 1) / SCAN_TILE;
    if (nt <= SCAN_SINGLE_MAX_TILES) {
        PFG_LAUNCH(K_SCAN, scan_single_k<T>, 1, SCAN_THREADS, 0, s, in, out, n, init, total_out);
        return;
    }
    T* sums = (T*)tmp;
    PFG_LAUNCH(K_SCAN, scan_reduce_k<T>, (unsigned)nt, SCAN_THREADS, 0, s, in, n, sums);
    PFG_LAUNCH(K_SCAN, scan_sums_k<T>, 1, SCAN_THREADS, 0, s, sums, nt, init, total_out);
    PFG_LAUNCH(K_SCAN, scan_tiles_k<T>, (unsigned)nt, SCAN_THREADS, 0, s, in, out, n, sums);
}

// ---------------- radix sort ----------------
constexpr int RS_THREADS = 256;
constexpr int RS_ROUNDS = 8;
constexpr int RS_TILE = RS_THREADS * RS_ROUNDS;
constexpr int RS_WARPS = RS_THREADS / 32;

__global__ void __launch_bounds__(RS_THREADS) radix_hist_k(const uint32_t* keys, uint64_t n, int shift,
                                                          uint32_t* hist, uint32_t nblocks) {
    __shared__ uint32_t cnt[256];
    cnt[threadIdx.x] = 0;
    __syncthreads();
    const uint64_t base = (uint64_t)blockIdx.x * RS_TILE;
#pragma unroll
    for (int r = 0; r < RS_ROUNDS; r++) {
        const uint64_t idx = base + (uint64_t)r * RS_THREADS + threadIdx.x;
        if (idx < n) atomicAdd(&cnt[(keys[idx] >> shift) & 0xFFu], 1u);
    }
    __syncthreads();
    hist[(uint64_t)threadIdx.x * nblocks + blockIdx.x] = cnt[threadIdx.x];
}

__global__ void __launch_bounds__(RS_THREADS) radix_scatter_k(const uint32_t* keys, const uint32_t* vals,
                                                             uint32_t* kout, uint32_t* vout, uint64_t n,
                                                             int shift, const uint32_t* offs, uint32_t nblocks) {
    __shared__ uint32_t tab[RS_WARPS][257];
    __shared__ uint32_t run[256];
    __shared__ uint32_t gbase[256];
    gbase[threadIdx.x] = offs[(uint64_t)threadIdx.x * nblocks + blockIdx.x];
    run[threadIdx.x] = 0;
    const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    unsigned lt;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(lt));
    const uint64_t base = (uint64_t)blockIdx.x * RS_TILE;
    for (int r = 0; r < RS_ROUNDS; r++) {
        for (int i = threadIdx.x; i < RS_WARPS * 257; i += RS_THREADS) (&tab[0][0])[i] = 0;
        __syncthreads();
        const uint64_t idx = base + (uint64_t)r * RS_THREADS + threadIdx.x;
        const bool valid = idx < n;
        uint32_t k = 0, v = 0, d = 256;
        if (valid) { k = keys[idx]; v = vals[idx]; d = (k >> shift) & 0xFFu; }
        const unsigned peers = __match_any_sync(0xFFFFFFFFu, d);
        const unsigned wrank = __popc(peers & lt);
        if (wrank == 0 && d != 256) tab[warp][d] = __popc(peers);
        __syncthreads();
        {   // per-digit exclusive prefix over warps, continuing the running totals
            const uint32_t dg = threadIdx.x;
            uint32_t acc = run[dg];
#pragma unroll
            for (int w = 0; w < RS_WARPS; w++) {
                const uint32_t t = tab[w][dg];
                tab[w][dg] = acc;
                acc += t;
            }
            run[dg] = acc;
        }
        __syncthreads();
        if (valid) {
            const uint32_t dst = gbase[d] + tab[warp][d] + wrank;
            kout[dst] = k;
            vout[dst] = v;
        }
        __syncthreads();
    }
}

// ---------------- compaction ----------------
__global__ void flags_to_u32_k(const uint8_t* flags, uint32_t* out, uint64_t n) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        out[i] = flags[i] ? 1u : 0u;
}

__global__ void select_scatter_k(const uint32_t* in, const uint8_t* flags, const uint32_t* pos, uint32_t* out, uint64_t n) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        if (flags[i]) out[pos[i]] = in ? in[i] : (uint32_t)i;
}

}  // namespace

size_t scan_temp_bytes(uint64_t n) {
    return ((n + SCAN_TILE - 1) / SCAN_TILE + 1) * sizeof(unsigned long long) + 256;
}

size_t radix_temp_bytes(uint64_t n) {
    const uint64_t nb = (n + RS_TILE - 1) / RS_TILE;
    const uint64_t h = 256 * nb;
    return h * sizeof(uint32_t) + scan_temp_bytes(h) + 512;
}

void exclusive_scan_u32(const uint32_t* in, uint32_t* out, uint64_t n, uint32_t init,
                        uint32_t* total_out, void* tmp, cudaStream_t s) {
    excl_scan<uint32_t>(in, out, n, init, total_out, tmp, s);
}

void exclusive_scan_u64(const unsigned long long* in, unsigned long long* out, uint64_t n,
                        unsigned long long init, unsigned long long* total_out, void* tmp,
                        cudaStream_t s) {
    excl_scan<unsigned long long>(in, out, n, init, total_out, tmp, s);
}

int radix_sort_pairs(uint32_t* k0, uint32_t* v0, uint32_t* k1, uint32_t* v1, uint64_t n,
                     int begin_bit, int end_bit, void* tmp, cudaStream_t s) {
    if (n <= 1) return 0;
    const uint64_t nb = (n + RS_TILE - 1) / RS_TILE;
    uint32_t* hist = (uint32_t*)tmp;
    void* stmp = (void*)(((uintptr_t)(hist + 256 * nb) + 255) & ~(uintptr_t)255);
    int cur = 0;
    // byte model: every 8-bit pass reads and writes the (key, value) pairs once
    if (g_prof) g_prof->bytes[K_RADIX] += 16 * n * (uint64_t)((end_bit - begin_bit + 7) / 8);
    for (int sh = begin_bit; sh < end_bit; sh += 8) {
        const uint32_t* ki = cur ? k1 : k0;
        const uint32_t* vi = cur ? v1 : v0;
        uint32_t* ko = cur ? k0 : k1;
        uint32_t* vo = cur ? v0 : v1;
        PFG_LAUNCH(K_RADIX, radix_hist_k, (unsigned)nb, RS_THREADS, 0, s, ki, n, sh, hist, (uint32_t)nb);
        excl_scan<uint32_t>(hist, hist, 256 * nb, 0u, nullptr, stmp, s);
        PFG_LAUNCH(K_RADIX, radix_scatter_k, (unsigned)nb, RS_THREADS, 0, s, ki, vi, ko, vo, n, sh, hist, (uint32_t)nb);
        cur ^= 1;
    }
    return cur;
}

void select_flagged(const uint32_t* in, const uint8_t* flags, uint32_t* out, uint64_t n,
                    uint32_t* count_out, uint32_t* scan_buf, void* tmp, cudaStream_t s) {
    if (n == 0) {
        cudaMemsetAsync(count_out, 0, sizeof(uint32_t), s);
        return;
    }
    // byte model: flags and input read (the kept output is not known on the host)
    if (g_prof) g_prof->bytes[K_SELECT] += 5 * n;
    PFG_LAUNCH(K_SELECT, flags_to_u32_k, grid_for(n, 256), 256, 0, s, flags, scan_buf, n);
    excl_scan<uint32_t>(scan_buf, scan_buf, n, 0u, count_out, tmp, s);
    PFG_LAUNCH(K_SELECT, select_scatter_k, grid_for(n, 256), 256, 0, s, in, flags, scan_buf, out, n);
}

}  // namespace pfg
