// Per-call device scratch shared by the host orchestration files.
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <string>
#include <vector>

#include "model.h"

namespace cg {

void cuda_check(cudaError_t e, const char* what);
#define CK(x) ::cg::cuda_check((x), #x)

// The stream-ordered pool that per-call scratch comes from: one per device, made on
// first use (with that device current) and kept until the process exits.  It keeps
// up to 32 GiB of freed scratch mapped across synchronisations; a pool that returns
// freed memory to the driver at every synchronisation has to map each row block's
// work lists again, which cost tens of milliseconds per block of a streamed
// assembly when the rest of device memory was busy.
cudaMemPool_t scratch_pool(int device);
// Return the pool's unused memory to the driver (before sizing a cache from the
// device's free memory).
void scratch_pool_trim(int device);

// Per-call scratch: stream-ordered device allocations from scratch_pool() released
// at the end of the call, or -- for the no-allocation entry point -- a bump
// allocator over the static device array below (256-byte aligned sub-buffers,
// capacity checked).
struct Scratch {
    cudaStream_t s;
    unsigned char* base = nullptr;
    size_t cap = 0, used = 0;
    std::vector<void*> ptrs;
    cudaMemPool_t pool = nullptr;
    explicit Scratch(cudaStream_t st) : s(st) {
        int dev = 0;
        CK(cudaGetDevice(&dev));
        pool = scratch_pool(dev);
    }
    Scratch(cudaStream_t st, void* static_base, size_t capacity)
        : s(st), base(reinterpret_cast<unsigned char*>(static_base)), cap(capacity) {}
    template <typename T>
    T* get(size_t n) {
        const size_t bytes = std::max<size_t>(n, 1) * sizeof(T);
        if (base) {
            const size_t off = (used + 255) & ~size_t(255);
            if (off + bytes > cap)
                throw Error(4, "input exceeds the no-allocation scratch capacity of " +
                                   std::to_string(cap >> 20) + " MiB; use cg_assemble_device");
            used = off + bytes;
            return reinterpret_cast<T*>(base + off);
        }
        void* p = nullptr;
        CK(cudaMallocFromPoolAsync(&p, bytes, pool, s));
        ptrs.push_back(p);
        return reinterpret_cast<T*>(p);
    }
    ~Scratch() {
        for (void* p : ptrs) cudaFreeAsync(p, s);
    }
};


}  // namespace cg
