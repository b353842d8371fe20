// hc_pool.h -- device memory for batched instances.
//
// Admitting and retiring solves must not call cudaMalloc / cudaFree each
// time: cudaFree waits for the whole device, which would stall every live
// solve at each retirement, and cudaMalloc costs tens of microseconds per
// call.  The pool takes device memory in large arenas and hands out 256-byte
// aligned ranges first-fit, merging neighbouring free ranges on release.
//
// A released range is only handed out again to work issued later on the same
// stream as its previous user, so stream order keeps the last reader of the
// old contents ahead of the first writer of the new ones; releasing needs no
// synchronisation.  Arenas are returned to the driver only by trim() (after
// a synchronisation, when an allocation would otherwise fail) and by the
// destructor.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <iterator>
#include <map>
#include <vector>

namespace hc {

// Where arenas come from: the CUDA runtime (a host-only test substitutes
// plain host memory).
struct CudaArenas {
    static cudaError_t alloc(void** p, size_t bytes) { return cudaMalloc(p, bytes); }
    static void free(void* p) { cudaFree(p); }
    static void clear_error() { cudaGetLastError(); }
};

template <class Backend>
class DevicePoolT {
public:
    static constexpr size_t kAlign = 256;

    explicit DevicePoolT(size_t arena_bytes = (size_t)1 << 30) : arena_bytes_(arena_bytes) {}
    ~DevicePoolT() { release_all(); }
    DevicePoolT(const DevicePoolT&) = delete;
    DevicePoolT& operator=(const DevicePoolT&) = delete;

    // A range of at least `bytes` bytes; cudaSuccess or the allocation error.
    cudaError_t alloc(size_t bytes, void** out) {
        size_t const need = round(bytes);
        if (take(need, out)) return cudaSuccess;
        cudaError_t e = grow(need);
        if (e != cudaSuccess) {
            // return whole free arenas to the driver and try once more
            Backend::clear_error();
            if (trim() == 0) return e;
            e = grow(need);
            if (e != cudaSuccess) return e;
        }
        return take(need, out) ? cudaSuccess : cudaErrorMemoryAllocation;
    }

    void release(void* p, size_t bytes) {
        if (!p) return;
        size_t const len = round(bytes);
        for (Arena& a : arenas_) {
            char* const c = static_cast<char*>(p);
            if (c < a.base || c >= a.base + a.size) continue;
            size_t off = (size_t)(c - a.base), n = len;
            auto next = a.free.lower_bound(off);
            if (next != a.free.end() && off + n == next->first) {
                n += next->second;
                next = a.free.erase(next);
            }
            if (next != a.free.begin()) {
                auto prev = std::prev(next);
                if (prev->first + prev->second == off) {
                    prev->second += n;
                    return;
                }
            }
            a.free.emplace(off, n);
            return;
        }
    }

    // Frees every arena with nothing handed out; returns the bytes freed.
    // Synchronises the device (cudaFree does).
    size_t trim() {
        size_t freed = 0;
        for (size_t k = 0; k < arenas_.size();) {
            Arena& a = arenas_[k];
            if (a.free.size() == 1 && a.free.begin()->first == 0 && a.free.begin()->second == a.size) {
                Backend::free(a.base);
                freed += a.size;
                arenas_.erase(arenas_.begin() + (long)k);
            } else {
                ++k;
            }
        }
        return freed;
    }

    void release_all() {
        for (Arena& a : arenas_) Backend::free(a.base);
        arenas_.clear();
    }

    size_t reserved() const {
        size_t s = 0;
        for (const Arena& a : arenas_) s += a.size;
        return s;
    }

    size_t free_bytes() const {
        size_t s = 0;
        for (const Arena& a : arenas_)
            for (const auto& kv : a.free) s += kv.second;
        return s;
    }

    size_t num_arenas() const { return arenas_.size(); }

private:
    struct Arena {
        char* base;
        size_t size;
        std::map<size_t, size_t> free;   // offset -> length
    };

    static size_t round(size_t b) { return (b + kAlign - 1) / kAlign * kAlign; }

    bool take(size_t need, void** out) {
        for (Arena& a : arenas_)
            for (auto it = a.free.begin(); it != a.free.end(); ++it) {
                if (it->second < need) continue;
                size_t const off = it->first, len = it->second;
                a.free.erase(it);
                if (len > need) a.free.emplace(off + need, len - need);
                *out = a.base + off;
                return true;
            }
        return false;
    }

    cudaError_t grow(size_t need) {
        size_t size = need > arena_bytes_ ? need : arena_bytes_;
        void* p = nullptr;
        cudaError_t e = Backend::alloc(&p, size);
        if (e != cudaSuccess && size > need) {
            // not enough room for a whole arena: take just what is asked
            Backend::clear_error();
            size = need;
            e = Backend::alloc(&p, size);
        }
        if (e != cudaSuccess) return e;
        Arena a{static_cast<char*>(p), size, {}};
        a.free.emplace(0, size);
        arenas_.push_back(std::move(a));
        return cudaSuccess;
    }

    size_t arena_bytes_;
    std::vector<Arena> arenas_;
};

using DevicePool = DevicePoolT<CudaArenas>;

}  // namespace hc
