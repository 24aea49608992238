// K6a on the 5th-generation tensor cores: the training pass of the per-element networks,
// d/dp [ ce E + ct (dE/dG . u) ] summed over the atoms, as tcgen05 BF16 GEMMs with FP32 accumulators
// in TMEM, one CTA per tile of 128 atoms of one type.
//
// Reference: NN::Cost::grad (src/ml/nn.cpp:1712-1770) for the energy term and the mixed second
// derivative of NN::D2ODZDI (nn.cpp:2012-2100) contracted with the tangent u (the force term of
// nnptef.cpp:1748-1820), here as forward-over-reverse: the same result as k_mlp_train (mlp.cu).
//
// Per tile (row r of every operand = atom r = TMEM lane r of the row-major accumulators):
//   forward   for each hidden layer l: Z_l = H_l W_l^T and Zd_l = Hd_l W_l^T (GEMMs, B = the weight
//             image of the inference kernel), kept in TMEM; H_{l+1} = f(Z_l + b_l) and
//             Hd_{l+1} = f'(.) Zd_l written to shared memory as BF16 hi / lo for the next layer.
//   last      zbar = ce outw, zdbar = ct outw per atom; its weight gradient is the GEMM below with
//             a 16-column delta of which column 0 is used; abar / adbar of the last hidden layer are
//             the rank-1 products zbar w_last, zdbar w_last, formed in the epilogue.
//   backward  for l from the last hidden layer down: zbar_l = f'(z) abar + f''(z) zd adbar and
//             zdbar_l = f'(z) adbar (epilogue, from TMEM); then
//             GW_l^T += H_l^T zbar_l + Hd_l^T zdbar_l  (M = 128 rows m of the layer's inputs, N = its
//             outputs, K = the 128 atoms; H and zbar are the row-major tiles read as MN-major
//             operands, H carrying a column of ones at index n_in so that row n_in is the bias
//             gradient) and, for l >= 1, abar_{l-1} = zbar_l W_l, adbar_{l-1} = zdbar_l W_l (the
//             inference kernel's backward GEMM, W read as the MN-major W^T). H_l is rebuilt from
//             Z_{l-1} in TMEM (or from G and U for l = 0) before its gradient GEMM.
//   output    the tile's gradient of every parameter of its type, read from TMEM (lane m = input
//             m of the layer) and stored as one row of the per-tile sums that k_grad_blocks adds in
//             tile order.
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

constexpr int TT_G = 4;                       // warps per TMEM lane quadrant (512 threads)

// activation value and first and second derivatives: sigmoid, tanh and softplus (ln 2 shifted)
// with the hardware approximations of the inference kernel (exp2 / log2 / rcp; absolute errors
// ~1e-7), the second derivative from the first (sigmoid c s (1 - s) (1 - 2 s), tanh -2 c t f',
// softplus c f' (1 - f')); the other forms of nn.cpp:149-810 at full accuracy, out of line
static __device__ __noinline__ void act_other3(int neuron, float c, float z, float& a, float& d, float& d2) {
    act_fd<float>(neuron, c, z, a, d, d2);
}
static __device__ __forceinline__ void act_fast3(int neuron, float c, float z, float& a, float& d, float& d2) {
    switch (neuron) {
        case N_SIGMOID: {
            const float e = __expf(-c * fabsf(z)), r = __frcp_rn(1.0f + e);
            const float s = (z >= 0.0f) ? r : e * r;
            a = s; d = c * s * (1.0f - s); d2 = c * d * (1.0f - 2.0f * s);
            return;
        }
        case N_TANH: {
            const float e = __expf(-2.0f * c * fabsf(z));
            const float t = copysignf((1.0f - e) * __frcp_rn(1.0f + e), z);
            a = t; d = c * (1.0f - t * t); d2 = -2.0f * c * t * d;
            return;
        }
        case N_SOFTPLUS: {
            const float e = __expf(-c * fabsf(z)), r = __frcp_rn(1.0f + e);
            a = fmaxf(z, 0.0f) + (__logf(1.0f + e) - (float)kLOG2) / c;
            d = (z > 0.0f) ? r : e * r;
            d2 = c * d * (1.0f - d);
            return;
        }
        default: act_other3(neuron, c, z, a, d, d2); return;
    }
}

struct TcTrainPlan {
    TcType t[MAXT];
    TcTrainLayout lay[MAXT];
};

// the tile of a CTA: tiles of type 0 first, then type 1, ...
static __device__ __forceinline__ bool train_tile(const TcTrainArgs& a, int& type, int& a0, int& cnt) {
    int b = blockIdx.x;
    for (int t = 0; t < a.ntypes; ++t) {
        const int c = a.tstart[t + 1] - a.tstart[t];
        const int tiles = (c + TC_M - 1) / TC_M;
        if (b < tiles) { type = t; a0 = a.tstart[t] + b * TC_M; cnt = min(TC_M, c - b * TC_M); return true; }
        b -= tiles;
    }
    return false;
}

__global__ void __launch_bounds__(TC_M * TT_G, 1) k_mlp_train_tc(const __grid_constant__ TcTrainPlan plan, const TcTrainArgs a) {
    extern __shared__ __align__(1024) uint8_t sm[];
    const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
    const int quad = warp & 3, grp = warp >> 2;
    const int r = quad * 32 + lane;                 // row of the tile (atom) = TMEM lane
    int type, a0, cnt;
    if (!train_tile(a, type, a0, cnt)) return;
    const TcType& tt = plan.t[type];
    const TcTrainLayout& ly = plan.lay[type];
    const int nh = tt.nhidden;

    uint8_t* img = sm;
    const uint32_t hb = (uint32_t)TC_M * ly.WH * 2, zb = (uint32_t)TC_M * ly.WZ * 2;
    uint8_t* Hh = sm + ly.o_h;                      // H hi, H lo, Hd hi, Hd lo, then the delta tiles
    uint8_t* Hl = Hh + hb;
    uint8_t* Dh = Hl + hb;
    uint8_t* Dl = Dh + hb;
    uint8_t* Bh = sm + ly.o_z;                      // zbar hi, zbar lo, zdbar hi, zdbar lo
    uint8_t* Bl = Bh + zb;
    uint8_t* Ch = Bl + zb;
    uint8_t* Cl = Ch + zb;
    uint64_t* bar = reinterpret_cast<uint64_t*>(sm + ly.o_tail);
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bar + 2);
    const bool lo_a = tt.split >= 2;                // activation rows split hi + lo
    const uint32_t hsbo = (uint32_t)ly.WH * 16u, zsbo = (uint32_t)ly.WZ * 16u;

    if (t == 0) { tc_mbar_init(&bar[0]); tc_mbar_init(&bar[1]); }
    __syncthreads();
    if (t == 0) {
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(su32(&bar[0])), "r"(tt.img_bytes) : "memory");
        asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                     ::"r"(su32(img)), "l"(a.image + tt.img_off), "r"(tt.img_bytes), "r"(su32(&bar[0])) : "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(su32(tmem_slot)), "r"((uint32_t)ly.tmem_cols) : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    bool good = tc_wait(&bar[0], 0, a.wait_polls);
    tc_fence_before();
    good = __syncthreads_and(good);
    const bool image_ok = good;
    bool mma_pending = false;
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;
    const uint32_t lane_off = (uint32_t)(quad * 32) << 16;
    uint32_t mphase = 0;
    const uint32_t img_s = su32(img);
    const float c = tt.c;
    const float* inpw = reinterpret_cast<const float*>(img + tt.inpw);
    const float* inpb = reinterpret_cast<const float*>(img + tt.inpb);
    const float* wlast = reinterpret_cast<const float*>(img + tt.wlast);
    const int row = r;
    const int at = (row < cnt) ? a.tlist[a0 + row] : -1;
    const float cer = (at >= 0) ? (float)(a.ce[at] * (double)tt.outw) : 0.0f;   // zbar of the output per atom
    const float ctr = (at >= 0) ? a.ct * tt.outw : 0.0f;                        // zdbar of the output per atom

    // issue the MMAs of `body` (thread 0), commit, and wait for them (all threads)
    auto mma_round = [&](auto body) -> bool {
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        tc_fence_before();
        __syncthreads();
        tc_fence_after();
        if (t == 0) {
            body();
            tc_commit(&bar[1]);
        }
        const bool ok = __syncthreads_and(tc_wait(&bar[1], mphase, a.wait_polls));
        tc_fence_after();
        if (ok) mphase ^= 1u;
        else mma_pending = true;
        return ok;
    };
    // D = A B^T over K, A and B in the canonical no-swizzle layouts with split hi / lo parts:
    // aT / bT select MN-major operands; (lbo, sbo) per operand; kstep = bytes between k-steps
    auto mma_gemm = [&](uint32_t dcol, int N, int K, uint32_t ahi, uint32_t alo, uint32_t albo, uint32_t asbo, uint32_t astep, bool aT,
                        uint32_t bhi, uint32_t blo, uint32_t blbo, uint32_t bsbo, uint32_t bstep, bool bT, bool lo_b, bool accumulate) {
        const uint32_t idesc = idesc_bf16(N, bT, aT);
        for (int s = 0; s < K / 16; ++s) {
            const uint64_t ad = smem_desc(ahi + astep * s, albo, asbo);
            const uint64_t bd = smem_desc(bhi + bstep * s, blbo, bsbo);
            tc_mma(tmem + dcol, ad, bd, idesc, (accumulate || s > 0) ? 1u : 0u);
            if (lo_a) tc_mma(tmem + dcol, smem_desc(alo + astep * s, albo, asbo), bd, idesc, 1u);
            if (lo_b) tc_mma(tmem + dcol, ad, smem_desc(blo + bstep * s, blbo, bsbo), idesc, 1u);
        }
    };
    // H_0 = inpw (G + inpb) and Hd_0 = inpw U of this row into the H tiles, a one at column nin
    auto build_inputs = [&]() {
        const float* Grow = a.G + (size_t)(at >= 0 ? at : 0) * a.imax;
        const float* Urow = a.U + (size_t)(at >= 0 ? at : 0) * a.imax;
        // rows 16-byte aligned (row length and base pointers): full chunks by vector loads
        const bool vec = (a.imax & 3) == 0 && ((reinterpret_cast<uintptr_t>(a.G) | reinterpret_cast<uintptr_t>(a.U)) & 15) == 0;
        for (int c0 = grp * 8; c0 < ly.WH; c0 += 8 * TT_G) {
            float v[8], d[8];
            if (vec && at >= 0 && c0 + 8 <= tt.nin) {
                const float4 g0 = *reinterpret_cast<const float4*>(Grow + c0), g1 = *reinterpret_cast<const float4*>(Grow + c0 + 4);
                const float4 u0 = *reinterpret_cast<const float4*>(Urow + c0), u1 = *reinterpret_cast<const float4*>(Urow + c0 + 4);
                const float gg[8] = {g0.x, g0.y, g0.z, g0.w, g1.x, g1.y, g1.z, g1.w};
                const float uu[8] = {u0.x, u0.y, u0.z, u0.w, u1.x, u1.y, u1.z, u1.w};
#pragma unroll
                for (int q = 0; q < 8; ++q) { v[q] = inpw[c0 + q] * (gg[q] + inpb[c0 + q]); d[q] = inpw[c0 + q] * uu[q]; }
            } else {
#pragma unroll
                for (int q = 0; q < 8; ++q) {
                    const int k = c0 + q;
                    const bool in = at >= 0 && k < tt.nin;
                    v[q] = in ? inpw[k] * (Grow[k] + inpb[k]) : (k == tt.nin ? 1.0f : 0.0f);
                    d[q] = in ? inpw[k] * Urow[k] : 0.0f;
                }
            }
            put8(Hh, lo_a ? Hl : nullptr, r, c0, hsbo, v);
            put8(Dh, lo_a ? Dl : nullptr, r, c0, hsbo, d);
        }
    };
    // H_{l+1} = f(Z_l + b_l), Hd_{l+1} = f'(.) Zd_l from TMEM into the H tiles, a one at column nodes[l]
    auto build_hidden = [&](int l) {
        const float* bias = reinterpret_cast<const float*>(img + tt.bias[l]);
        for (int c0 = grp * 8; c0 < ly.WH; c0 += 8 * TT_G) {
            float z[8], zd[8], v[8], d[8];
            const bool inside = c0 < tt.width[l];
            if (inside) {
                tc_ld8(tmem + lane_off + (uint32_t)(ly.zc[l] + c0), z);
                tc_ld8(tmem + lane_off + (uint32_t)(ly.zdc[l] + c0), zd);
            }
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                const int col = c0 + q;
                if (inside && col < tt.nodes[l]) {
                    float av, f1, f2;
                    act_fast3(tt.neuron, c, z[q] + bias[col], av, f1, f2);
                    v[q] = av; d[q] = f1 * zd[q];
                } else {
                    v[q] = (col == tt.nodes[l]) ? 1.0f : 0.0f; d[q] = 0.0f;
                }
            }
            put8(Hh, lo_a ? Hl : nullptr, r, c0, hsbo, v);
            put8(Dh, lo_a ? Dl : nullptr, r, c0, hsbo, d);
        }
    };

    // ---- forward
    build_inputs();
    for (int l = 0; l < nh && good; ++l) {
        const int Kin = (l == 0) ? tt.K0 : tt.width[l - 1];
        const uint32_t bk = (uint32_t)(Kin / 8) * 128u;
        good = mma_round([&] {
            mma_gemm((uint32_t)ly.zc[l], tt.width[l], Kin, su32(Hh), su32(Hl), 128u, hsbo, 256u, false,
                     img_s + tt.fwd_hi[l], img_s + tt.fwd_lo[l], 128u, bk, 256u, false, tt.split >= 3, false);
            mma_gemm((uint32_t)ly.zdc[l], tt.width[l], Kin, su32(Dh), su32(Dl), 128u, hsbo, 256u, false,
                     img_s + tt.fwd_hi[l], img_s + tt.fwd_lo[l], 128u, bk, 256u, false, tt.split >= 3, false);
        });
        if (!good) break;
        build_hidden(l);
    }
    // ---- output layer: its deltas (column 0 of a 16-column delta tile) and its weight gradient
    if (good) {
        for (int c0 = grp * 8; c0 < 16; c0 += 8 * TT_G) {
            float v[8], d[8];
#pragma unroll
            for (int q = 0; q < 8; ++q) { v[q] = (c0 + q == 0) ? cer : 0.0f; d[q] = (c0 + q == 0) ? ctr : 0.0f; }
            put8(Bh, lo_a ? Bl : nullptr, r, c0, zsbo, v);
            put8(Ch, lo_a ? Cl : nullptr, r, c0, zsbo, d);
        }
        good = mma_round([&] {
            mma_gemm((uint32_t)ly.gwl, 16, TC_M, su32(Hh), su32(Hl), hsbo, 128u, 2u * hsbo, true,
                     su32(Bh), su32(Bl), zsbo, 128u, 2u * zsbo, true, lo_a, false);
            mma_gemm((uint32_t)ly.gwl, 16, TC_M, su32(Dh), su32(Dl), hsbo, 128u, 2u * hsbo, true,
                     su32(Ch), su32(Cl), zsbo, 128u, 2u * zsbo, true, lo_a, true);
        });
    }
    // ---- backward through the hidden layers
    for (int l = nh - 1; l >= 0 && good; --l) {
        const float* bias = reinterpret_cast<const float*>(img + tt.bias[l]);
        const bool top = (l == nh - 1);
        for (int c0 = grp * 8; c0 < ly.WZ; c0 += 8 * TT_G) {
            float zb[8], zdb[8];
            if (c0 < tt.width[l]) {
                float z[8], zd[8], ab[8], adb[8];
                tc_ld8(tmem + lane_off + (uint32_t)(ly.zc[l] + c0), z);
                tc_ld8(tmem + lane_off + (uint32_t)(ly.zdc[l] + c0), zd);
                if (!top) {   // abar / adbar of this layer's outputs: the GEMMs of layer l + 1
                    tc_ld8(tmem + lane_off + (uint32_t)(ly.zc[l + 1] + c0), ab);
                    tc_ld8(tmem + lane_off + (uint32_t)(ly.zc[l + 1] + tt.width[l] + c0), adb);
                }
#pragma unroll
                for (int q = 0; q < 8; ++q) {
                    const int col = c0 + q;
                    if (col < tt.nodes[l]) {
                        float av, f1, f2;
                        act_fast3(tt.neuron, c, z[q] + bias[col], av, f1, f2);
                        const float abv = top ? cer * wlast[col] : ab[q];
                        const float adbv = top ? ctr * wlast[col] : adb[q];
                        zb[q] = f1 * abv + f2 * zd[q] * adbv;
                        zdb[q] = f1 * adbv;
                    } else {
                        zb[q] = 0.0f; zdb[q] = 0.0f;
                    }
                }
            } else {
#pragma unroll
                for (int q = 0; q < 8; ++q) { zb[q] = 0.0f; zdb[q] = 0.0f; }
            }
            put8(Bh, lo_a ? Bl : nullptr, r, c0, zsbo, zb);
            put8(Ch, lo_a ? Cl : nullptr, r, c0, zsbo, zdb);
        }
        // the layer's inputs (the H tiles held H_{l+1} until the previous round completed)
        if (l == 0) build_inputs();
        else build_hidden(l - 1);
        const int Nin = (l == 0) ? tt.K0 : tt.width[l - 1];
        const uint32_t bn = (uint32_t)(tt.width[l] / 8) * 128u;   // W_l^T as MN-major B: see mlp_tc.cu
        const uint32_t bkk = (uint32_t)(Nin / 8) * 128u;
        good = mma_round([&] {
            mma_gemm((uint32_t)ly.gw[l], tt.width[l], TC_M, su32(Hh), su32(Hl), hsbo, 128u, 2u * hsbo, true,
                     su32(Bh), su32(Bl), zsbo, 128u, 2u * zsbo, true, lo_a, false);
            mma_gemm((uint32_t)ly.gw[l], tt.width[l], TC_M, su32(Dh), su32(Dl), hsbo, 128u, 2u * hsbo, true,
                     su32(Ch), su32(Cl), zsbo, 128u, 2u * zsbo, true, lo_a, true);
            if (l >= 1) {
                mma_gemm((uint32_t)ly.zc[l], Nin, tt.width[l], su32(Bh), su32(Bl), 128u, zsbo, 256u, false,
                         img_s + tt.fwd_hi[l], img_s + tt.fwd_lo[l], bkk, 128u, 2u * bkk, true, tt.split >= 3, false);
                mma_gemm((uint32_t)(ly.zc[l] + Nin), Nin, tt.width[l], su32(Ch), su32(Cl), 128u, zsbo, 256u, false,
                         img_s + tt.fwd_hi[l], img_s + tt.fwd_lo[l], bkk, 128u, 2u * bkk, true, tt.split >= 3, false);
            }
        });
        (void)bn;
    }
    // ---- the tile's gradient: TMEM lane m = input m of the layer (m = n_in: the bias)
    if (good) {
        double* gp = a.gpart + (size_t)blockIdx.x * a.pstride;
        int bias_at = 0, wt_at = 0;
        for (int l = 0; l <= nh; ++l) wt_at += (l < nh) ? tt.nodes[l] : 1;
        for (int l = 0; l < nh; ++l) {
            const int ni = (l == 0) ? tt.nin : tt.nodes[l - 1], no = tt.nodes[l];
            for (int c0 = grp * 16; c0 < tt.width[l]; c0 += 16 * TT_G) {
                float g[16];
                tc_ld16(tmem + lane_off + (uint32_t)(ly.gw[l] + c0), g);
#pragma unroll
                for (int q = 0; q < 16; ++q) {
                    const int n = c0 + q;
                    if (n >= no) continue;
                    if (r < ni) gp[wt_at + r * no + n] = (double)g[q];
                    else if (r == ni) gp[bias_at + n] = (double)g[q];
                }
            }
            bias_at += no;
            wt_at += ni * no;
        }
        if (grp == 0) {
            float g[16];
            tc_ld16(tmem + lane_off + (uint32_t)ly.gwl, g);
            const int ni = tt.nodes[nh - 1];
            if (r < ni) gp[wt_at + r] = (double)g[0];
            else if (r == ni) gp[bias_at] = (double)g[0];
        }
    }
    if (!good) {
        if (t == 0) atomicOr(a.status, (int)ST_TIMEOUT);
        if (!image_ok) tc_wait(&bar[0], 0);
        if (mma_pending) tc_wait(&bar[1], mphase);
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"((uint32_t)ly.tmem_cols) : "memory");
}

// the layout of a type in the training kernel; false if its networks do not fit
bool plan_tc_train(const TcType& tt, int max_smem, TcTrainLayout& ly) {
    ly = TcTrainLayout{};
    const int nh = tt.nhidden;
    if (nh < 1 || tt.img_bytes == 0) return false;
    int wh = tt.K0, wz = 16;
    if (tt.nin + 1 > TC_M) return false;                     // inputs + the ones row within M = 128
    wh = std::max(wh, (tt.nin + 1 + 15) / 16 * 16);
    for (int l = 0; l < nh; ++l) {
        if (tt.nodes[l] + 1 > TC_M) return false;
        wh = std::max(wh, (tt.nodes[l] + 1 + 15) / 16 * 16);
        wz = std::max(wz, tt.width[l]);
        if (l >= 1 && tt.width[l - 1] > tt.width[l]) return false;   // abar / adbar reuse layer l's columns
    }
    ly.WH = wh; ly.WZ = wz;
    int col = 0;
    for (int l = 0; l < nh; ++l) { ly.zc[l] = col; ly.zdc[l] = col + tt.width[l]; col += 2 * tt.width[l]; }
    for (int l = 0; l < nh; ++l) { ly.gw[l] = col; col += tt.width[l]; }
    ly.gwl = col; col += 16;
    ly.tmem_cols = 32;
    while (ly.tmem_cols < col) ly.tmem_cols *= 2;
    if (ly.tmem_cols > 512) return false;
    const size_t hb = (size_t)TC_M * wh * 2, zb = (size_t)TC_M * wz * 2;
    const int hparts = tt.split >= 2 ? 2 : 1;
    ly.o_h = (uint32_t)(((size_t)tt.img_bytes + 1023) / 1024 * 1024);
    // four H tiles (hi / lo of H and Hd; the lo tiles unused without the split), then the delta
    // tiles: the MN-major reads of an H tile run past its end into what follows (rows beyond the
    // layer's inputs, whose results are not used), so the delta tiles must follow it
    ly.o_z = ly.o_h + (uint32_t)(4 * hb);
    ly.o_tail = ly.o_z + (uint32_t)(4 * zb);
    ly.smem = ly.o_tail + 64 + 2048;     // barriers and TMEM slot, then room for the overreads
    (void)hparts;
    return ly.smem + 1024 <= (uint32_t)max_smem;
}

void launch_mlp_train_tc(const TcPlan& tc, const TcTrainLayout* lay, const TcTrainArgs& a, cudaStream_t st) {
    if (a.natoms <= 0) return;
    TcTrainPlan p{};
    uint32_t smem = 0;
    for (int t = 0; t < a.ntypes; ++t) { p.t[t] = tc.t[t]; p.lay[t] = lay[t]; smem = std::max(smem, lay[t].smem); }
    const int grid = (a.natoms + TC_M - 1) / TC_M + a.ntypes;
    ++::ann::g_launch_counter;
    k_mlp_train_tc<<<grid, TC_M * TT_G, smem, st>>>(p, a);
}
void configure_mlp_train_tc(int maxsmem) { set_max_dynamic_smem(k_mlp_train_tc, maxsmem); }

}  // namespace ann
