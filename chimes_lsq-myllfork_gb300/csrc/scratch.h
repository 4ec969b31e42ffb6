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

// Per-call scratch: stream-ordered device allocations released at the end of the
// call, or -- for the no-allocation entry point -- a bump allocator over the
// static device array below (256-byte aligned sub-buffers, capacity checked).
struct Scratch {
    cudaStream_t s;
    unsigned char* base = nullptr;
    size_t cap = 0, used = 0;
    std::vector<void*> ptrs;
    explicit Scratch(cudaStream_t st) : s(st) {}
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
        CK(cudaMallocAsync(&p, bytes, s));
        ptrs.push_back(p);
        return reinterpret_cast<T*>(p);
    }
    ~Scratch() {
        for (void* p : ptrs) cudaFreeAsync(p, s);
    }
};


}  // namespace cg
