// Host <-> device transfers of a batch through page-locked buffers that this library allocated
// (ann_host_alloc). On this node the GPU reaches page-locked host memory directly over the
// coherent chip-to-chip link, and one kernel with many loads in flight moves a batch's inputs
// (positions, types, cells) or results (energies, forces, virials, status) faster than one
// copy-engine transfer per array. Ranges are taken only from the library's own registry of
// allocations (base, size), so that a copy can never reach outside an allocation; any other
// pointer goes through cudaMemcpyAsync.
#include <cuda_runtime.h>
#include <algorithm>
#include <cstdint>
#include <map>
#include <mutex>
#include "transfer.hpp"

namespace ann {

namespace {
struct HostAlloc { size_t bytes; void* dev; };
std::mutex g_mu;
std::map<uintptr_t, HostAlloc> g_allocs;   // base address -> allocation
}

void host_register(void* p, size_t bytes) {
    if (!p || bytes == 0) return;
    void* dev = nullptr;
    if (cudaHostGetDevicePointer(&dev, p, 0) != cudaSuccess) { cudaGetLastError(); return; }
    std::lock_guard<std::mutex> g(g_mu);
    g_allocs[(uintptr_t)p] = HostAlloc{bytes, dev};
}
void host_unregister(void* p) {
    std::lock_guard<std::mutex> g(g_mu);
    g_allocs.erase((uintptr_t)p);
}
void* host_device_view(const void* p, size_t bytes) {
    if (!p) return nullptr;
    std::lock_guard<std::mutex> g(g_mu);
    auto it = g_allocs.upper_bound((uintptr_t)p);
    if (it == g_allocs.begin()) return nullptr;
    --it;
    const uintptr_t base = it->first, q = (uintptr_t)p;
    if (q < base || q - base > it->second.bytes || bytes > it->second.bytes - (q - base)) return nullptr;
    return static_cast<unsigned char*>(it->second.dev) + (q - base);
}

// up to CP_MAXSEG segments in one launch; each segment moves in units of 16, 8, 4 or 1 bytes
// (the largest that divides both addresses and the length)
__global__ void __launch_bounds__(256) k_copy_segs(const __grid_constant__ CopyPlan p) {
    const uint64_t total = p.start[p.n];
    for (uint64_t u = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; u < total; u += (uint64_t)gridDim.x * blockDim.x) {
        int k = 0;
        while (k + 1 < p.n && u >= p.start[k + 1]) ++k;
        const uint64_t v = u - p.start[k];
        const CopySeg& s = p.seg[k];
        switch (s.unit) {
            case 16: reinterpret_cast<uint4*>(s.dst)[v] = reinterpret_cast<const uint4*>(s.src)[v]; break;
            case 8: reinterpret_cast<uint2*>(s.dst)[v] = reinterpret_cast<const uint2*>(s.src)[v]; break;
            case 4: reinterpret_cast<uint32_t*>(s.dst)[v] = reinterpret_cast<const uint32_t*>(s.src)[v]; break;
            default: s.dst[v] = s.src[v]; break;
        }
    }
}

bool CopyPlan::add(const void* src, void* dst, size_t bytes) {
    if (bytes == 0) return true;
    if (n >= CP_MAXSEG) return false;
    const uintptr_t a = (uintptr_t)src | (uintptr_t)dst | (uintptr_t)bytes;
    const int unit = (a % 16 == 0) ? 16 : (a % 8 == 0) ? 8 : (a % 4 == 0) ? 4 : 1;
    seg[n] = CopySeg{static_cast<const unsigned char*>(src), static_cast<unsigned char*>(dst), unit};
    start[n + 1] = start[n] + bytes / unit;
    ++n;
    return true;
}

void launch_copy_plan(const CopyPlan& p, int nsm, cudaStream_t st) {
    const uint64_t total = p.start[p.n];
    if (total == 0) return;
    const uint64_t want = (total + 255) / 256;
    const int grid = (int)std::min<uint64_t>(want, (uint64_t)std::max(nsm, 1) * 8);
    ++::ann::g_launch_counter;
    k_copy_segs<<<grid, 256, 0, st>>>(p);
}

}  // namespace ann
