/*
 * cuarena/allocator.cuh - stand-in for the cuArena device-pool library
 * (TEST INFRASTRUCTURE ONLY).
 *
 * The reference GPU simplifier includes <cuarena/allocator.cuh>, a git
 * submodule (https://github.com/muhos/cuArena) that is not part of the
 * reference tree. This header implements exactly the surface the reference
 * calls (src/gpu/memory.cuh:81-146, src/gpu/memory.cu:99-546,
 * src/gpu/cache.cu:27-86, src/gpu/simplify.cu:219-220) so that the unmodified
 * reference sources compile into the oracle's reference binary:
 *
 *   DeviceArena::create_gpu_pool / create_cpu_pool / destroy_gpu_pool,
 *   allocate<T>(n, Region), allocate_pinned<T>(n), deallocate,
 *   deallocate_pinned, compact_gpu_dynamic, gpu_capacity, gpu_available,
 *   gpu_stable_available, gpu_peak_used, cpu_used, align_up, alignment,
 *   and the exceptions gpu_memory_error / cpu_memory_error.
 *
 * Design: the pool sizes given at creation are budgets, not reservations.
 * Each allocation is its own cudaMalloc / cudaMallocHost, counted against the
 * budget of its region, so a block never moves and compaction has nothing to
 * do. Over-budget requests throw like the library does. Device memory held
 * is what the reference actually uses, not the free memory it sizes its pool
 * from.
 */
#ifndef PFG_REFGPU_CUARENA_ALLOCATOR_CUH
#define PFG_REFGPU_CUARENA_ALLOCATOR_CUH

#include <cuda_runtime.h>
#include <cstddef>
#include <cstdint>
#include <map>
#include <stdexcept>
#include <string>

namespace cuArena {

enum class Region { Stable, Dynamic };
enum class GPUMemoryType { Device, Managed };
enum class CPUMemoryType { Pinned, Pageable };

struct gpu_memory_error : std::runtime_error {
    explicit gpu_memory_error(const std::string& m) : std::runtime_error(m) {}
};
struct cpu_memory_error : std::runtime_error {
    explicit cpu_memory_error(const std::string& m) : std::runtime_error(m) {}
};

class DeviceArena {
    static constexpr size_t kAlign = 256;
    size_t gpu_cap_ = 0, stable_cap_ = 0;
    size_t stable_used_ = 0, dynamic_used_ = 0, peak_ = 0;
    size_t cpu_cap_ = 0, cpu_used_ = 0;
    struct Block { size_t bytes; Region region; };
    std::map<void*, Block> dev_;
    std::map<void*, size_t> host_;

public:
    DeviceArena() = default;
    DeviceArena(const DeviceArena&) = delete;
    DeviceArena& operator=(const DeviceArena&) = delete;
    ~DeviceArena() { destroy_gpu_pool(); destroy_cpu_pool(); }

    size_t alignment() const { return kAlign; }
    size_t align_up(size_t n) const { return (n + kAlign - 1) / kAlign * kAlign; }

    /* `stable_bytes` of `bytes` form the stable region; the rest is dynamic. */
    bool create_gpu_pool(size_t bytes, GPUMemoryType, int device, size_t stable_bytes) {
        if (gpu_cap_) return true;
        if (cudaSetDevice(device) != cudaSuccess) return false;
        gpu_cap_ = bytes;
        stable_cap_ = stable_bytes < bytes ? stable_bytes : bytes;
        return true;
    }
    bool create_cpu_pool(size_t bytes, CPUMemoryType) {
        cpu_cap_ = bytes;
        return true;
    }
    void destroy_gpu_pool() {
        for (auto& kv : dev_) cudaFree(kv.first);
        dev_.clear();
        gpu_cap_ = stable_cap_ = stable_used_ = dynamic_used_ = 0;
    }
    void destroy_cpu_pool() {
        for (auto& kv : host_) cudaFreeHost(kv.first);
        host_.clear();
        cpu_cap_ = cpu_used_ = 0;
    }

    size_t gpu_capacity() const { return gpu_cap_; }
    size_t gpu_stable_available() const { return stable_cap_ - stable_used_; }
    size_t gpu_available() const {
        const size_t dyn_cap = gpu_cap_ - stable_cap_;
        return dyn_cap > dynamic_used_ ? dyn_cap - dynamic_used_ : 0;
    }
    size_t gpu_peak_used() const { return peak_; }
    size_t cpu_used() const { return cpu_used_; }

    template <class T>
    T* allocate(size_t n, Region region) {
        const size_t bytes = align_up(n * sizeof(T));
        if (!bytes) throw gpu_memory_error("zero-byte device allocation");
        const size_t avail = region == Region::Stable ? gpu_stable_available() : gpu_available();
        if (bytes > avail) throw gpu_memory_error("device pool budget exceeded");
        void* p = nullptr;
        if (cudaMalloc(&p, bytes) != cudaSuccess) {
            cudaGetLastError();
            throw gpu_memory_error("cudaMalloc failed");
        }
        dev_[p] = Block{bytes, region};
        (region == Region::Stable ? stable_used_ : dynamic_used_) += bytes;
        if (stable_used_ + dynamic_used_ > peak_) peak_ = stable_used_ + dynamic_used_;
        return static_cast<T*>(p);
    }
    void deallocate(void* p) {
        auto it = dev_.find(p);
        if (it == dev_.end()) return;
        (it->second.region == Region::Stable ? stable_used_ : dynamic_used_) -= it->second.bytes;
        cudaFree(p);
        dev_.erase(it);
    }
    /* Blocks never move, so there is nothing to compact. */
    void compact_gpu_dynamic(cudaStream_t) {}

    template <class T>
    T* allocate_pinned(size_t n) {
        const size_t bytes = align_up(n * sizeof(T));
        if (cpu_used_ + bytes > cpu_cap_) throw cpu_memory_error("pinned pool budget exceeded");
        void* p = nullptr;
        if (cudaMallocHost(&p, bytes) != cudaSuccess) {
            cudaGetLastError();
            throw cpu_memory_error("cudaMallocHost failed");
        }
        host_[p] = bytes;
        cpu_used_ += bytes;
        return static_cast<T*>(p);
    }
    void deallocate_pinned(void* p) {
        auto it = host_.find(p);
        if (it == host_.end()) return;
        cpu_used_ -= it->second;
        cudaFreeHost(p);
        host_.erase(it);
    }
};

}  // namespace cuArena

#endif
