// K3 on the 5th-generation tensor cores: per-element networks (forward, energy, backward to dE/dG)
// over tiles of 128 atoms of one type, as tcgen05 BF16 GEMMs with FP32 accumulators in TMEM.
//
// Reference: NN::ANN::fpbp (src/ml/nn.cpp:1343-1409), NN::DODZ::grad (nn.cpp:1801-1824) and
// NNH::energy (src/nnp/nnh.cpp:118-121), the same computation as the SIMT kernel in mlp.cu.
//
// Per CTA (128 x G threads: G warps per TMEM lane quadrant, G = 1, 2 or 4 so that 4 / G CTAs share
// an SM when tensor memory allows and the type has tiles enough; tile row r <-> TMEM lane r),
// persistent over the type's tiles:
//   weights   : one bulk asynchronous copy (cp.async.bulk + mbarrier) of the type's image
//               (B operands W_l in the canonical K-major no-swizzle layout, BF16 hi/lo; the
//               backward GEMMs read the same bytes as the MN-major operand W_l^T).
//   per tile  : A0 = inpw*(G+inpb) split into BF16 hi+lo rows, then for every hidden layer
//               D = A W_l^T (tcgen05.mma kind::f16, M=128, issued by one thread, completion via
//               tcgen05.commit on an mbarrier); the epilogue (tcgen05.ld, bias, activation, next A)
//               is split by 16-column chunks over the warps sharing a quadrant, and f'(z) is
//               written back over z (tcgen05.st). The last hidden layer's epilogue forms the
//               energy and delta = outw w_last f'(z); the backward GEMMs D = delta W_l multiply by
//               the stored f'(z_{l-1}), down to dE/dG = D inpw.
//   split     : A = A_hi + A_lo and W = W_hi + W_lo accumulate 3 MMAs per k-step, giving close
//               to FP32 products from BF16 operands.
// Every wait is bounded; on a timeout the CTA records ST_TIMEOUT, drains, frees TMEM and returns.
#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <algorithm>
#include <cstdint>
#include "dev_math.cuh"
#include "kernels.hpp"
#include "mlp_tc.hpp"
#include "tcgen05.cuh"

namespace ann {

// the other activation forms of nn.cpp:149-810 with full-accuracy functions, out of line so that
// the epilogue code of the common forms stays compact
static __device__ __noinline__ void act_other(int neuron, float c, float z, float& a, float& d) {
    float d2;
    act_fd<float>(neuron, c, z, a, d, d2);
}
// activation value and first derivative: sigmoid, tanh and softplus with the hardware
// approximations (exp2 / log2 / rcp; absolute errors ~1e-7, far inside the FP32 path's tolerance)
static __device__ __forceinline__ void act_fast(int neuron, float c, float z, float& a, float& d) {
    switch (neuron) {
        case N_SIGMOID: {
            const float e = __expf(-c * fabsf(z)), r = __frcp_rn(1.0f + e);
            a = (z >= 0.0f) ? r : e * r;
            d = c * e * r * r;
            return;
        }
        case N_TANH: {
            const float e = __expf(-2.0f * c * fabsf(z));
            const float t = copysignf((1.0f - e) * __frcp_rn(1.0f + e), z);
            a = t;
            d = c * (1.0f - t * t);
            return;
        }
        case N_SOFTPLUS: {
            const float e = __expf(-c * fabsf(z)), r = __frcp_rn(1.0f + e);
            a = fmaxf(z, 0.0f) + (__logf(1.0f + e) - (float)kLOG2) / c;
            d = (z > 0.0f) ? r : e * r;
            return;
        }
        default: act_other(neuron, c, z, a, d); return;
    }
}

// G warps share each TMEM lane quadrant (warp w: rows 32*(w%4).., column chunks c with
// c % G == w / 4), so an epilogue runs on G * 4 warps; 4 / G CTAs share an SM (tc_groups)
template <int G>
__global__ void __launch_bounds__(TC_M * G, 4 / G) k_mlp_tc(const __grid_constant__ TcType tt, const TcArgs a) {
    extern __shared__ __align__(1024) uint8_t sm[];
    const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
    const int quad = warp & 3, grp = warp >> 2;
    const int r = quad * 32 + lane;                 // the thread's row of the tile (= TMEM lane)
    const int a0 = a.tstart[a.type], cnt = a.tstart[a.type + 1] - a0;
    const int ntiles = (cnt + TC_M - 1) / TC_M;
    if ((int)blockIdx.x >= ntiles) return;

    uint8_t* img = sm;
    const uint32_t abytes = (uint32_t)TC_M * tt.wmax * 2;
    uint8_t* Ahi = sm + ((tt.img_bytes + 127) / 128) * 128;
    uint8_t* Alo = (tt.split >= 2) ? Ahi + abytes : nullptr;
    uint64_t* bar = reinterpret_cast<uint64_t*>(Ahi + abytes * (tt.split >= 2 ? 2 : 1));
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bar + 2);
    float* ered = reinterpret_cast<float*>(bar + 4);      // [G][TC_M] energy partial sums
    const uint32_t asbo = (uint32_t)tt.wmax * 16u;   // (wmax / 8) * 128

    if (t == 0) { tc_mbar_init(&bar[0]); tc_mbar_init(&bar[1]); }
    __syncthreads();
    if (t == 0) {
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(su32(&bar[0])), "r"(tt.img_bytes) : "memory");
        asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                     ::"r"(su32(img)), "l"(a.image + tt.img_off), "r"(tt.img_bytes), "r"(su32(&bar[0])) : "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(su32(tmem_slot)), "r"((uint32_t)tt.tmem_cols) : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    bool good = tc_wait(&bar[0], 0, a.wait_polls);
    tc_fence_before();
    good = __syncthreads_and(good);
    const bool image_ok = good;
    bool mma_pending = false;       // an MMA group whose completion was not observed
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;
    const uint32_t lane_off = (uint32_t)(quad * 32) << 16;
    uint32_t mphase = 0;

    const float* inpw = reinterpret_cast<const float*>(img + tt.inpw);
    const float* inpb = reinterpret_cast<const float*>(img + tt.inpb);
    const float* wlast = reinterpret_cast<const float*>(img + tt.wlast);
    const float c = tt.c;
    const uint32_t img_s = su32(img), ahi_s = su32(Ahi), alo_s = Alo ? su32(Alo) : 0u;

    // one GEMM: D[tmem col] = A (rows x K) . B^T, accumulating the hi/lo parts. Forward (bT false):
    // B is W (N x K) in the canonical K-major layout. Backward (bT true): B is W^T (N = the layer's
    // inputs, K = its outputs), read from the same image of W as an MN-major operand: there the 8
    // contiguous elements of a core matrix run along N and its 8 rows along K, core matrices are
    // 128 B apart along N (stride byte offset) and N/8 * 128 B apart along K (leading byte offset)
    auto gemm = [&](uint32_t b_hi, uint32_t b_lo, int K, int N, uint32_t dcol, bool bT) -> bool {
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        tc_fence_before();
        __syncthreads();
        tc_fence_after();
        if (t == 0) {
            const uint32_t idesc = idesc_bf16(N, bT);
            const uint32_t bk = bT ? (uint32_t)(N / 8) * 128u : 128u;           // between core matrices along K
            const uint32_t bn = bT ? 128u : (uint32_t)(K / 8) * 128u;           // between core matrices along N
            for (int s = 0; s < K / 16; ++s) {
                const uint64_t ad = smem_desc(ahi_s + 256u * s, 128u, asbo);
                const uint64_t bd = smem_desc(img_s + b_hi + 2u * bk * s, bk, bn);
                tc_mma(tmem + dcol, ad, bd, idesc, s > 0 ? 1u : 0u);
                if (tt.split >= 2) tc_mma(tmem + dcol, smem_desc(alo_s + 256u * s, 128u, asbo), bd, idesc, 1u);
                if (tt.split >= 3) tc_mma(tmem + dcol, ad, smem_desc(img_s + b_lo + 2u * bk * s, bk, bn), idesc, 1u);
            }
            tc_commit(&bar[1]);
        }
        const bool ok = __syncthreads_and(tc_wait(&bar[1], mphase, a.wait_polls));
        tc_fence_after();
        if (ok) mphase ^= 1u;
        else mma_pending = true;
        return ok;
    };

    for (int tile = blockIdx.x; tile < ntiles && good; tile += gridDim.x) {
        const int row = tile * TC_M + r;
        const int at = (row < cnt) ? a.tlist[a0 + row] : -1;
        const float* Grow = a.G + (size_t)(at >= 0 ? at : 0) * a.imax;
        // ---- A0 = inpw * (G + inpb), 8-column chunks shared out over the groups
        // rows 16-byte aligned (row length and base pointers): vector loads / stores of full chunks
        const bool vec = (a.imax & 3) == 0 && ((reinterpret_cast<uintptr_t>(a.G) | reinterpret_cast<uintptr_t>(a.dEdG)) & 15) == 0;
        for (int c0 = grp * 8; c0 < tt.K0; c0 += 8 * G) {
            float v[8];
            if (vec && at >= 0 && c0 + 8 <= tt.nin) {
                const float4 g0 = *reinterpret_cast<const float4*>(Grow + c0), g1 = *reinterpret_cast<const float4*>(Grow + c0 + 4);
                const float gg[8] = {g0.x, g0.y, g0.z, g0.w, g1.x, g1.y, g1.z, g1.w};
#pragma unroll
                for (int q = 0; q < 8; ++q) v[q] = inpw[c0 + q] * (gg[q] + inpb[c0 + q]);
            } else {
#pragma unroll
                for (int q = 0; q < 8; ++q) {
                    const int k = c0 + q;
                    v[q] = (at >= 0 && k < tt.nin) ? inpw[k] * (Grow[k] + inpb[k]) : 0.0f;
                }
            }
            put8(Ahi, Alo, r, c0, asbo, v);
        }
        // ---- forward; f'(z) replaces z in TMEM for the backward pass
        float epart = 0.0f;
        for (int l = 0; l < tt.nhidden && good; ++l) {
            const int Kin = (l == 0) ? tt.K0 : tt.width[l - 1];
            const int N = tt.width[l];
            good = gemm(tt.fwd_hi[l], tt.fwd_lo[l], Kin, N, (uint32_t)tt.fwd_col[l], false);
            if (!good) break;
            const float* bias = reinterpret_cast<const float*>(img + tt.bias[l]);
            const bool last = (l == tt.nhidden - 1);
            for (int c0 = grp * 16; c0 < N; c0 += 16 * G) {
                float v[16], o[16];
                const uint32_t ta = tmem + lane_off + (uint32_t)(tt.fwd_col[l] + c0);
                tc_ld16(ta, v);
#pragma unroll
                for (int q = 0; q < 16; ++q) {
                    const int col = c0 + q;
                    float av, d1;
                    act_fast(tt.neuron, c, v[q] + bias[col], av, d1);
                    if (col >= tt.nodes[l]) { av = 0.0f; d1 = 0.0f; }
                    if (last) { epart += wlast[col] * av; o[q] = tt.outw * wlast[col] * d1; }
                    else o[q] = av;
                    v[q] = d1;
                }
                if (!last) tc_st16(ta, v);
                put8(Ahi, Alo, r, c0, asbo, o);
                put8(Ahi, Alo, r, c0 + 8, asbo, o + 8);
            }
        }
        if (!good) break;
        ered[grp * TC_M + r] = epart;
        // ---- backward: A holds delta of hidden layer l
        for (int l = tt.nhidden - 1; l >= 0 && good; --l) {
            const int Nout = (l == 0) ? tt.K0 : tt.width[l - 1];
            good = gemm(tt.fwd_hi[l], tt.fwd_lo[l], tt.width[l], Nout, (uint32_t)tt.bwd_col, true);
            if (!good) break;
            if (l == tt.nhidden - 1 && grp == 0 && at >= 0) {   // ered is complete after the GEMM's barrier
                float e = 0.0f;
#pragma unroll
                for (int g = 0; g < G; ++g) e += ered[g * TC_M + r];
                const float blast = *reinterpret_cast<const float*>(img + tt.blast);
                a.Eatom[at] = (double)(tt.outb + tt.outw * (e + blast)) + tt.evac;
            }
            for (int c0 = grp * 16; c0 < Nout; c0 += 16 * G) {
                float gv[16];
                tc_ld16(tmem + lane_off + (uint32_t)(tt.bwd_col + c0), gv);
                if (l > 0) {
                    float dz[16], o[16];
                    tc_ld16(tmem + lane_off + (uint32_t)(tt.fwd_col[l - 1] + c0), dz);
#pragma unroll
                    for (int q = 0; q < 16; ++q) o[q] = gv[q] * dz[q];   // f' is zero in padded columns
                    put8(Ahi, Alo, r, c0, asbo, o);
                    put8(Ahi, Alo, r, c0 + 8, asbo, o + 8);
                } else if (at >= 0) {
                    float* drow = a.dEdG + (size_t)at * a.imax;
                    if (vec && c0 + 16 <= a.imax) {
                        float o[16];
#pragma unroll
                        for (int q = 0; q < 16; ++q) o[q] = (c0 + q < tt.nin) ? gv[q] * inpw[c0 + q] : 0.0f;
#pragma unroll
                        for (int q = 0; q < 16; q += 4) *reinterpret_cast<float4*>(drow + c0 + q) = make_float4(o[q], o[q + 1], o[q + 2], o[q + 3]);
                    } else {
#pragma unroll
                        for (int q = 0; q < 16; ++q) {
                            const int col = c0 + q;
                            if (col < a.imax) drow[col] = (col < tt.nin) ? gv[q] * inpw[col] : 0.0f;
                        }
                    }
                }
            }
            if (l == 0 && at >= 0 && grp == 0)
                for (int col = tt.K0; col < a.imax; ++col) a.dEdG[(size_t)at * a.imax + col] = 0.0f;
        }
    }
    if (!good) {
        if (t == 0) atomicOr(a.status, (int)ST_TIMEOUT);
        // drain what may still be in flight before the shared memory and TMEM go away (bounded)
        if (!image_ok) tc_wait(&bar[0], 0);
        if (mma_pending) tc_wait(&bar[1], mphase);
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"((uint32_t)tt.tmem_cols) : "memory");
}

void launch_mlp_tc(const TcType& tt, const TcArgs& a, long long est_atoms, int groups, size_t smem, int nsm, cudaStream_t st) {
    if (a.natoms <= 0) return;
    // a forced split cannot oversubscribe tensor memory: smem_bytes admits at most 512 / tmem_cols
    // CTAs per SM whatever their width
    nsm = std::max(1, nsm);
    const int g = groups ? groups : tc_groups(tt, est_atoms, nsm);
    int grid = (a.natoms + TC_M - 1) / TC_M;
    grid = std::min(grid, nsm * (4 / g));
    ++::ann::g_launch_counter;
    if (g == 1) k_mlp_tc<1><<<grid, TC_M, smem, st>>>(tt, a);
    else if (g == 2) k_mlp_tc<2><<<grid, TC_M * 2, smem, st>>>(tt, a);
    else k_mlp_tc<4><<<grid, TC_M * 4, smem, st>>>(tt, a);
}
void configure_mlp_tc(int maxsmem) {
    set_max_dynamic_smem(k_mlp_tc<1>, maxsmem);
    set_max_dynamic_smem(k_mlp_tc<2>, maxsmem);
    set_max_dynamic_smem(k_mlp_tc<4>, maxsmem);
}

}  // namespace ann
