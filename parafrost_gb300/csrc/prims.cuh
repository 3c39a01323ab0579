// Device-wide primitives of the engine: exclusive scans, stable LSD radix
// sort and stream compaction. They replace the reference's CUB/Thrust calls
// (DeviceScan: elimination.cu:85-92, memory.cu:429-430, recycle.cu:84-93;
// DeviceSelect: elimination.cu:253-256, cnf.cu:218-222; thrust::sort:
// lcve.cu:294, histogram.cu:65).
#pragma once

#include <cstddef>
#include <cstdint>
#include <vector>
#include <cuda_runtime.h>

namespace pfg {

// Kernel groups timed by the profiler.
enum KernelId : int {
    K_HIST = 0, K_FILL, K_SORT_SMALL, K_SORT_MID, K_SORT_BIG, K_SCAN, K_RADIX, K_SELECT,
    K_LCVE, K_MIS_WIN, K_MIS_APPLY, K_SUB, K_VE1, K_VE1B, K_VE3, K_BIGVAR, K_ERE, K_BCP, K_COUNT, K_COMPACT,
    K_UPLOAD, K_DOWNLOAD, K_MISC, K_BCE, K_NUM
};
extern const char* const kKernelNames[K_NUM];

// Device time per kernel group from CUDA events. Consecutive launches of one
// group on one stream share one span: an event is recorded only where the
// group (or the stream) changes, one event ending the last span and starting
// the next, and the open span is closed at every host synchronisation, so a
// span never covers the host's side of a wait. Upload and download kernels sit
// between large host copies, so each of their launches is a span of its own.
// (One event pair per launch added ~2.5 % to the batched step.) begin/end
// time explicit pairs instead.
struct Profiler {
    struct Span {
        int id;
        uint32_t b, e;    // event indices in the pool
    };
    bool on = false;
    std::vector<cudaEvent_t> pool;
    size_t used = 0;
    std::vector<Span> spans;
    int open_id = -1;
    cudaStream_t open_s = nullptr;
    uint32_t open_b = 0, pair_b = 0;
    double ms[K_NUM] = {0};
    uint64_t launches[K_NUM] = {0};
    uint64_t bytes[K_NUM] = {0};
    uint32_t record(cudaStream_t s);
    void launch(int id, cudaStream_t s);   // before a launch of group id on s
    void after(int id);                    // after it: upload and download launches end their span
    void close();                          // ends the open span
    void begin(int id, cudaStream_t s);
    void end(int id, cudaStream_t s);
    void resolve();                        // closes, synchronizes and accumulates the spans
    void reset();
    void destroy();
};

// Every launcher counts its kernel launches here (per host thread) and, when
// a profiler is installed for the calling thread, marks the launch's group.
extern thread_local uint64_t g_launches;
extern thread_local Profiler* g_prof;

#define PFG_LAUNCH(ID, KERNEL, GRID, BLOCK, SMEM, STREAM, ...)                  \
    do {                                                                        \
        ::pfg::Profiler* _pp = ::pfg::g_prof;                                   \
        if (_pp && _pp->on) _pp->launch(::pfg::ID, (STREAM));                   \
        KERNEL<<<(GRID), (BLOCK), (SMEM), (STREAM)>>>(__VA_ARGS__);             \
        ::pfg::g_launches++;                                                    \
        if (_pp) { _pp->launches[::pfg::ID]++;                                  \
                   if (_pp->on) _pp->after(::pfg::ID); }                        \
    } while (0)

// Scratch bytes needed by the scans / sorts below for n elements.
size_t scan_temp_bytes(uint64_t n);
size_t radix_temp_bytes(uint64_t n);

// out[i] = init + sum(in[0..i)); optional *total_out (device) = init + sum(in).
// in and out may alias.
void exclusive_scan_u32(const uint32_t* in, uint32_t* out, uint64_t n, uint32_t init,
                        uint32_t* total_out, void* tmp, cudaStream_t s);
void exclusive_scan_u64(const unsigned long long* in, unsigned long long* out, uint64_t n,
                        unsigned long long init, unsigned long long* total_out, void* tmp,
                        cudaStream_t s);

// Stable LSD radix sort of (key, value) pairs on bits [begin_bit, end_bit).
// Ping-pongs between (k0, v0) and (k1, v1); returns 0 if the result is in
// (k0, v0), 1 if in (k1, v1).
int radix_sort_pairs(uint32_t* k0, uint32_t* v0, uint32_t* k1, uint32_t* v1, uint64_t n,
                     int begin_bit, int end_bit, void* tmp, cudaStream_t s);

// Stable compaction: out[j] = in[i] for flags[i] != 0 in order (i itself
// when in is null); *count_out (device) = number kept. `scan_buf` holds n+1
// uint32.
void select_flagged(const uint32_t* in, const uint8_t* flags, uint32_t* out, uint64_t n,
                    uint32_t* count_out, uint32_t* scan_buf, void* tmp, cudaStream_t s);

// Grid size helper: enough blocks to cover n with `threads`, capped at 152 SMs x `per_sm`.
inline unsigned grid_for(uint64_t n, unsigned threads, unsigned per_sm = 32) {
    uint64_t b = (n + threads - 1) / threads;
    const uint64_t cap = 152ull * per_sm;
    if (b > cap) b = cap;
    if (b < 1) b = 1;
    return (unsigned)b;
}

}  // namespace pfg
