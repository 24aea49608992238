// PTX helpers of the tcgen05 network kernels (inference, mlp_tc.cu; training, mlp_tc_train.cu):
// mbarriers with bounded waits, shared-memory matrix descriptors, tcgen05.mma of kind::f16 with
// FP32 accumulators in TMEM, TMEM loads / stores, and BF16 hi / lo splits of operand rows.
#pragma once
#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <cstdint>
#include "mlp_tc.hpp"

namespace ann {

static __device__ __forceinline__ uint32_t su32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// ---------------------------------------------------------------- mbarrier / bulk copy
static __device__ __forceinline__ void tc_mbar_init(uint64_t* bar) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(su32(bar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
static __device__ __forceinline__ bool tc_try_wait(uint64_t* bar, uint32_t phase) {
    uint32_t ok;
    asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
                 : "=r"(ok) : "r"(su32(bar)), "r"(phase) : "memory");
    return ok != 0;
}
static __device__ __forceinline__ bool tc_test_wait(uint64_t* bar, uint32_t phase) {   // non-blocking poll
    uint32_t ok;
    asm volatile("{\n .reg .pred p;\n mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
                 : "=r"(ok) : "r"(su32(bar)), "r"(phase) : "memory");
    return ok != 0;
}
// bounded by 2^22 potentially blocking polls, or (polls > 0, testing the timeout path) by
// polls - 1 non-blocking ones; the drains after a timeout always take the full bound
static __device__ __forceinline__ bool tc_wait(uint64_t* bar, uint32_t phase, int polls = 0) {
    if (polls > 0) {
        for (int it = 1; it < polls; ++it) if (tc_test_wait(bar, phase)) return true;
        return false;
    }
    for (int it = 0; it < (1 << 22); ++it) if (tc_try_wait(bar, phase)) return true;
    return false;
}

// ---------------------------------------------------------------- tcgen05
// shared-memory matrix descriptor: start address, leading (K) and stride (8-row group) byte
// offsets, fixed 0b001 at bits 46-48, no swizzle
static __device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}
// instruction descriptor of kind::f16: D FP32, A and B BF16, A K-major (aT = false) or MN-major
// (aT = true, bit 15), B K-major (bT = false) or MN-major (bT = true, bit 16), N and M=128
static __device__ __forceinline__ uint32_t idesc_bf16(int N, bool bT, bool aT = false) {
    return (1u << 4) | (1u << 7) | (1u << 10) | (aT ? (1u << 15) : 0u) | (bT ? (1u << 16) : 0u) | ((uint32_t)(N >> 3) << 17) |
           ((uint32_t)(TC_M >> 4) << 24);
}
static __device__ __forceinline__ void tc_mma(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t accum) {
    asm volatile("{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n"
                 ::"r"(d), "l"(a), "l"(b), "r"(idesc), "r"(accum) : "memory");
}
static __device__ __forceinline__ void tc_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(su32(bar)) : "memory");
}
static __device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
static __device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
static __device__ __forceinline__ void tc_ld16(uint32_t taddr, float (&v)[16]) {
    uint32_t r[16];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                   "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
                 : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

static __device__ __forceinline__ void tc_ld8(uint32_t taddr, float (&v)[8]) {
    uint32_t r[8];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
                 : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 8; ++i) v[i] = __uint_as_float(r[i]);
}

// 8 consecutive values of row r into the A tiles (hi, and lo = remainder when lo != nullptr)
static __device__ __forceinline__ void put8(uint8_t* hi, uint8_t* lo, int r, int c0, uint32_t sbo, const float* v) {
    const uint32_t off = (uint32_t)(r >> 3) * sbo + (uint32_t)(c0 >> 3) * 128u + (uint32_t)(r & 7) * 16u;
    uint32_t h[4], l[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const __nv_bfloat16 a0 = __float2bfloat16_rn(v[2 * q]), a1 = __float2bfloat16_rn(v[2 * q + 1]);
        h[q] = (uint32_t)__bfloat16_as_ushort(a0) | ((uint32_t)__bfloat16_as_ushort(a1) << 16);
        if (lo) {
            const __nv_bfloat16 b0 = __float2bfloat16_rn(v[2 * q] - __bfloat162float(a0));
            const __nv_bfloat16 b1 = __float2bfloat16_rn(v[2 * q + 1] - __bfloat162float(a1));
            l[q] = (uint32_t)__bfloat16_as_ushort(b0) | ((uint32_t)__bfloat16_as_ushort(b1) << 16);
        }
    }
    *reinterpret_cast<uint4*>(hi + off) = make_uint4(h[0], h[1], h[2], h[3]);
    if (lo) *reinterpret_cast<uint4*>(lo + off) = make_uint4(l[0], l[1], l[2], l[3]);
}

static __device__ __forceinline__ void tc_st16(uint32_t taddr, const float (&v)[16]) {
    asm volatile("tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, %16};"
                 ::"r"(taddr), "r"(__float_as_uint(v[0])), "r"(__float_as_uint(v[1])), "r"(__float_as_uint(v[2])), "r"(__float_as_uint(v[3])),
                   "r"(__float_as_uint(v[4])), "r"(__float_as_uint(v[5])), "r"(__float_as_uint(v[6])), "r"(__float_as_uint(v[7])),
                   "r"(__float_as_uint(v[8])), "r"(__float_as_uint(v[9])), "r"(__float_as_uint(v[10])), "r"(__float_as_uint(v[11])),
                   "r"(__float_as_uint(v[12])), "r"(__float_as_uint(v[13])), "r"(__float_as_uint(v[14])), "r"(__float_as_uint(v[15]))
                 : "memory");
    asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
}

}  // namespace ann
