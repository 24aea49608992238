// Batch transfers through the library's own page-locked host allocations (transfer.cu).
#pragma once
#include <cuda_runtime.h>
#include <cstddef>
#include <cstdint>
#include "kernels.hpp"

namespace ann {

// the registry of page-locked host allocations made by ann_host_alloc (and the context's status
// word); only ranges inside one of them are read or written by the copy kernel
void host_register(void* p, size_t bytes);
void host_unregister(void* p);
// the device-side address of [p, p + bytes) when the whole range lies in a registered allocation,
// else nullptr (the caller then uses cudaMemcpyAsync)
void* host_device_view(const void* p, size_t bytes);

constexpr int CP_MAXSEG = 4;
struct CopySeg {
    const unsigned char* src;
    unsigned char* dst;
    int unit;                    // bytes moved per element: 16, 8, 4 or 1
};
struct CopyPlan {
    CopySeg seg[CP_MAXSEG];
    uint64_t start[CP_MAXSEG + 1] = {0, 0, 0, 0, 0};   // first element of each segment
    int n = 0;
    bool add(const void* src, void* dst, size_t bytes);  // false: the plan is full
};
// one kernel for every segment of the plan (device addresses on both sides)
void launch_copy_plan(const CopyPlan& p, int nsm, cudaStream_t st);

}  // namespace ann
