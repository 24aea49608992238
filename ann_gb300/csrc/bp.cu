// K2 / K4 / K6b: symmetry functions, forces + virial, and the symmetry-function tangent
// (training), one warp per centre atom.
//
// Reference: NNP::symm (src/nnp/nnp.cpp:333-375), NNP::force / NNP::compute (nnp.cpp:461-736),
// BasisR::symm/force (src/nnp/basis_radial.cpp:263-376), BasisA::symm/force
// (src/nnp/basis_angular.cpp:371-563), Cutoff::cutf/cutg (src/nnp/cutoff.cpp:62-114).
//
// Per centre atom i (one warp):
//  1. its neighbour row (type-sorted by the list builder) is staged into shared memory with a
//     bulk asynchronous copy (cp.async.bulk + mbarrier), then compacted to d < rc and turned
//     into per-neighbour records: (unit vector, 1/d), d, cutoff f and f', and for every damping
//     group g of the angular GAUSS functions D_g = f exp(-d^2/eta_g^2) and its d-derivative.
//  2. radial functions: lanes own neighbours and keep the block's functions in registers
//     (symmetry functions / tangents, then a transposing warp reduction), or own neighbours and
//     loop over functions (force pass).
//  3. angular functions of each (J,K) type block. In the fast path (GAUSS, lambda=+-1,
//     zeta=2^k) the reference's exp(-(rij^2+rik^2)/eta^2) factorises into D_g(j) D_g(k) and
//     |1/2 +- cos/2|^zeta comes from a squaring chain (symmetry functions) or from a degree-8
//     polynomial in cos (force pass), so no transcendental is evaluated per triplet. There the
//     neighbours of a type range are split into ceil(n/32) chunks of nearly equal size and lane L
//     owns element L of every chunk; a chunk's triangle and each pair of chunks are walked along
//     rotations (partner = own + step mod n), so the lane's own record stays in registers. Lanes
//     without an element, and partner slots past a chunk's end, read a zero record (index cap),
//     whose terms vanish, so the walk carries no per-step masks. The generic path and the tangent
//     pass hand out (j,k) triplets to lanes instead.
//  4. force pass: per triplet the vectors v_j = -dE_i/dr_ij, v_k = -dE_i/dr_ik are summed per
//     neighbour. Fast path: lanes own neighbours (the chunks above) and visit their
//     partners along a rotation, keeping their own sums in registers and shuffling the partner's
//     share to its owner lane (no atomics). Generic path: triplets along diagonals with shared
//     atomics. F_i = sum_j v_j, F_j -= v_j (Newton's third law, nnp.cpp:491,509-516) and the
//     virial W += r_ij (x) v_j are formed once per neighbour.
#include <cuda_runtime.h>
#include <algorithm>
#include <cstdint>
#include <type_traits>
#include "dev_math.cuh"
#include "kernels.hpp"

namespace ann {

enum { PASS_SYMM = 0, PASS_FORCE = 1, PASS_JVP = 2 };
constexpr int BP_WARPS = 4;
#ifndef ANN_BP_MIN_BLOCKS
#define ANN_BP_MIN_BLOCKS 5         // resident blocks per SM the symmetry / tangent passes are bounded for
#endif
#ifndef ANN_BP_MIN_BLOCKS_FORCE
#define ANN_BP_MIN_BLOCKS_FORCE 4   // the force pass with two or more damping groups (114-126 registers
#endif                              // without spills; bounded for five it spills)
// With one damping group the atoms have few neighbours (the 262,144-atom argon box) and the passes
// need the occupancy: the force pass fits five blocks without spills (92 registers), the symmetry
// and tangent passes six (84 registers; bounded for five they take 89 and lose a block per SM:
// 0.340 -> 0.395 ms on that box)
// (fast-path kernels; the generic path keeps five)
// The FP32 force pass with up to two damping groups is bounded for five blocks (96 registers, a
// 36-byte spill), which its shared memory allows at the row capacities of ~100 that a learned
// capacity gives on the bench batch (0.621 -> 0.614 ms there; the symmetry pass bounded for six,
// 80 registers, took 0.334 -> 0.342 ms and keeps five). The FP64 kernels and four damping groups
// keep the older bounds.
constexpr int bp_min_blocks(int pass, int ng, bool fast, bool fp64) {
    return (fp64 || ng > 2) ? (pass == PASS_FORCE ? (ng > 1 ? ANN_BP_MIN_BLOCKS_FORCE : ANN_BP_MIN_BLOCKS)
                                                  : (ng == 1 && fast ? ANN_BP_MIN_BLOCKS + 1 : ANN_BP_MIN_BLOCKS))
                : (pass == PASS_FORCE ? ANN_BP_MIN_BLOCKS : (ng == 1 && fast ? ANN_BP_MIN_BLOCKS + 1 : ANN_BP_MIN_BLOCKS));
}
constexpr int CHUNK = 16;   // functions per register chunk (radial and generic angular)

// ---------------------------------------------------------------- PTX helpers (bulk copy + mbarrier)
static __device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
static __device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
static __device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
static __device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                 ::"r"(smem_u32(dst)), "l"(src), "r"(bytes), "r"(smem_u32(bar)) : "memory");
}
static __device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t phase) {
    uint32_t ok;
    asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
                 : "=r"(ok) : "r"(smem_u32(bar)), "r"(phase) : "memory");
    return ok != 0;
}
static __device__ __forceinline__ bool mbar_test_wait(uint64_t* bar, uint32_t phase) {   // non-blocking poll
    uint32_t ok;
    asm volatile("{\n .reg .pred p;\n mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
                 : "=r"(ok) : "r"(smem_u32(bar)), "r"(phase) : "memory");
    return ok != 0;
}
// the wait for a staged row: bounded by 2^24 potentially blocking polls, or (testing, polls > 0)
// by polls - 1 non-blocking ones
static __device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t phase, int polls) {
    if (polls > 0) {
        for (int it = 1; it < polls; ++it) if (mbar_test_wait(bar, phase)) return true;
        return false;
    }
    for (int it = 0; it < (1 << 24); ++it) if (mbar_try_wait(bar, phase)) return true;
    return false;
}
static __device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// ---------------------------------------------------------------- warp reductions
// transposing butterfly: on return lane l holds the warp sum of slot (l >> (5-log2 S)) & (S-1)
template <typename real, int S>
__device__ __forceinline__ real warp_slot_reduce(real (&v)[S], int lane) {
    constexpr int LOGS = (S == 1) ? 0 : (S == 2) ? 1 : (S == 4) ? 2 : (S == 8) ? 3 : (S == 16) ? 4 : 5;
#pragma unroll
    for (int h = 0; h < LOGS; ++h) {
        const int off = 16 >> h;
        const int half = S >> (h + 1);
        const bool upper = (lane & off) != 0;
#pragma unroll
        for (int i = 0; i < half; ++i) {
            const real send = upper ? v[i] : v[i + half];
            const real keep = upper ? v[i + half] : v[i];
            v[i] = keep + __shfl_xor_sync(0xffffffffu, send, off);
        }
    }
#pragma unroll
    for (int off = (16 >> LOGS); off >= 1; off >>= 1) v[0] += __shfl_xor_sync(0xffffffffu, v[0], off);
    return v[0];
}
template <int S> struct SlotShift { static constexpr int v = (S == 8) ? 2 : (S == 16) ? 1 : (S == 32) ? 0 : 3; };
template <typename real>
__device__ __forceinline__ real warp_sum(real v) {
#pragma unroll
    for (int off = 16; off >= 1; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    return v;
}

// ---------------------------------------------------------------- triplet enumeration
// pairs j<k of [0,n), lane-strided by 32. ROWS: row-major (row j, then k) -- the warp shares j.
// otherwise diagonal-major (k-j fixed, then j) -- every lane has a different j and k.
template <bool ROWS>
struct TriIter {
    int r, c, len;
    __device__ __forceinline__ void init(int n, int t) { r = 0; len = n - 1; c = t; while (len > 0 && c >= len) { c -= len; ++r; --len; } }
    __device__ __forceinline__ void adv() { c += 32; while (len > 0 && c >= len) { c -= len; ++r; --len; } }
    __device__ __forceinline__ int j() const { return ROWS ? r : c; }
    __device__ __forceinline__ int k() const { return ROWS ? r + 1 + c : c + r + 1; }
};
// pairs of [0,nJ) x [0,nK), lane-strided by 32. ROWS: row-major. otherwise rotated:
// t -> (d = t / nJ, j = t % nJ, k = (j + d) mod nK), distinct j and k within a warp step.
template <bool ROWS>
struct RectIter {
    int q, c, nJ, nK;
    __device__ __forceinline__ void init(int nj, int nk, int t) {
        nJ = nj; nK = nk;
        if (ROWS) { q = t / nk; c = t - q * nk; }
        else { const int d = t / nj; q = t - d * nj; c = (q + d) % nk; }
    }
    __device__ __forceinline__ void adv() {
        if (ROWS) { c += 32; while (c >= nK) { c -= nK; ++q; } }
        else {
            q += 32; c += 32;
            while (q >= nJ) { q -= nJ; c -= nJ - 1; }
            while (c >= nK) c -= nK;
            while (c < 0) c += nK;
        }
    }
};

// ---------------------------------------------------------------- shared-memory layout of one warp
constexpr int TS_ZERO = 64;   // chunk-task scratch: 2 x 32 slots, then the zero record
template <typename real, int NG, int PASS>
struct WarpMem {
    typedef typename V4<real>::T R4;
    R4* geo;             // (ux, uy, uz, 1/d)
    real* dp;            // [e][2*NG]: D_0, D_1, ..., Dp_0, Dp_1, ...
    real *d, *fc, *fcg;
    real *ax, *ay, *az;  // force accumulators (FORCE)
    R4* tg;              // tangent of the pair vector (drx, dry, drz, dd) (JVP)
    real* dE;            // dE/dG row (FORCE); dE + imax: the second staging buffer
    R4* stage;
    int32_t *stagej, *stagej2;   // staged neighbour indices (two buffers); after compaction the
                                 // current one holds j per record (-1: no Newton-3rd share, FORCE)
    uint64_t* bar;       // two mbarriers, one per staging buffer
    // chunk-task scratch (symmetry and force passes): the partner chunk twice over, partner slots
    // without an element as zeros, so that rotation step st reads slot lane + st with no wrap; a
    // zero record at TS_ZERO
    R4* sg;
    real* sd;
    static constexpr int NDP = 2 * NG;
    static __host__ __device__ size_t align(size_t x, size_t a) { return (x + a - 1) / a * a; }
    static __host__ __device__ size_t layout(int cap, int imax, WarpMem* w, unsigned char* base) {
        size_t off = 0;
        auto take = [&](size_t bytes, size_t al) { off = align(off, al); const size_t o = off; off += bytes; return o; };
        // geo / stage / tg / dp hold cap records plus a zero record at index cap (see force_task)
        const size_t o_geo = take(sizeof(R4) * (cap + 1), 32);
        const size_t o_stage = take(sizeof(R4) * (cap + 1), 32);
        const size_t o_tg = (PASS == PASS_JVP) ? take(sizeof(R4) * (cap + 1), 32) : 0;
        const size_t o_dp = take(sizeof(real) * NDP * (cap + 1), 16);
        const size_t o_d = take(sizeof(real) * cap, 16), o_fc = take(sizeof(real) * cap, 16), o_fcg = take(sizeof(real) * cap, 16);
        size_t o_ax = 0, o_ay = 0, o_az = 0, o_dE = 0;
        if (PASS == PASS_FORCE) {
            o_ax = take(sizeof(real) * cap, 16); o_ay = take(sizeof(real) * cap, 16); o_az = take(sizeof(real) * cap, 16);
            o_dE = take(sizeof(real) * imax * 2, 16);   // two rows: the next atom's arrives with its neighbour row
        }
        const size_t o_sj = take(sizeof(int32_t) * cap, 16);
        const size_t o_sj2 = take(sizeof(int32_t) * cap, 16);
        const size_t o_bar = take(16, 16);
        const bool tasks = (PASS != PASS_JVP);
        const size_t o_sg = tasks ? take(sizeof(R4) * (TS_ZERO + 1), 32) : 0;
        const size_t o_sd = tasks ? take(sizeof(real) * NDP * (TS_ZERO + 1), 16) : 0;
        if (w) {
            w->geo = reinterpret_cast<R4*>(base + o_geo); w->stage = reinterpret_cast<R4*>(base + o_stage);
            w->tg = reinterpret_cast<R4*>(base + o_tg); w->dp = reinterpret_cast<real*>(base + o_dp);
            w->d = reinterpret_cast<real*>(base + o_d); w->fc = reinterpret_cast<real*>(base + o_fc); w->fcg = reinterpret_cast<real*>(base + o_fcg);
            w->ax = reinterpret_cast<real*>(base + o_ax); w->ay = reinterpret_cast<real*>(base + o_ay); w->az = reinterpret_cast<real*>(base + o_az);
            w->dE = reinterpret_cast<real*>(base + o_dE);
            w->stagej = reinterpret_cast<int32_t*>(base + o_sj);
            w->stagej2 = reinterpret_cast<int32_t*>(base + o_sj2);
            w->bar = reinterpret_cast<uint64_t*>(base + o_bar);
            w->sg = reinterpret_cast<R4*>(base + o_sg); w->sd = reinterpret_cast<real*>(base + o_sd);
        }
        return align(off, 128);
    }
    static __host__ __device__ size_t bytes(int cap, int imax) { return layout(cap, imax, nullptr, nullptr); }
};

// D/Dp pairs of one neighbour for the fast path
template <typename real, int NG>
struct DampRec {
    alignas(16) real v[2 * NG];
    // records are 2*NG reals at a 2*NG-real stride from a 16-byte aligned base: vector loads
    __device__ __forceinline__ void load(const real* p) {
        constexpr int B = 2 * NG * (int)sizeof(real);
        if constexpr (B % 16 == 0) {
#pragma unroll
            for (int k = 0; k < B / 16; ++k) reinterpret_cast<float4*>(v)[k] = reinterpret_cast<const float4*>(p)[k];
        } else if constexpr (B == 8) {
            *reinterpret_cast<float2*>(v) = *reinterpret_cast<const float2*>(p);
        } else {
#pragma unroll
            for (int q = 0; q < 2 * NG; ++q) v[q] = p[q];
        }
    }
    __device__ __forceinline__ void zero() {
#pragma unroll
        for (int q = 0; q < 2 * NG; ++q) v[q] = real(0);
    }
    __device__ __forceinline__ real D(int g) const { return v[g]; }        // record: D_0..D_{NG-1}, Dp_0..Dp_{NG-1}
    __device__ __forceinline__ real Dp(int g) const { return v[NG + g]; }
};

// ---------------------------------------------------------------- force pass, fast path
// One triplet (i; j, k) of a fast-path angular block: v_j = -dE_i/dr_ij and v_k = -dE_i/dr_ik
// (BasisA::force, basis_angular.cpp:430-563, with the damping factorised per group).
// The block's weighted sum over slots, A_g(cos) = sum_s dE/dG_s |1/2 + lambda_s cos/2|^zeta_s,
// is a polynomial of degree 8 in cos (zeta = 1,2,4,8; the bases are never negative for
// |cos| <= 1); al[g][p] holds its coefficients and Horner's rule gives A_g and dA_g/dcos together.
// two FP32 lanes per register pair (packed FMA of sm_100+), used for the two damping groups
static __device__ __forceinline__ uint64_t pk2(float lo, float hi) {
    uint64_t r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
    return r;
}
static __device__ __forceinline__ float hsum2(uint64_t v) {
    float lo, hi;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
    return lo + hi;
}
static __device__ __forceinline__ uint64_t fma2(uint64_t a, uint64_t b, uint64_t c) {
    uint64_t d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}
static __device__ __forceinline__ uint64_t mul2(uint64_t a, uint64_t b) {
    uint64_t d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}

// The triplet's forces in the frame of its two unit vectors: v_j = cj u_j + bj u_k and
// v_k = ck u_k + bk u_j (u = r / |r| of the entry, gj.w = 1 / |r_ij|).
template <typename real, int NG>
__device__ __forceinline__ void triplet_force(const typename V4<real>::T& gj, const DampRec<real, NG>& dj,
                                              const typename V4<real>::T& gk, const DampRec<real, NG>& dk,
                                              const real (&al)[NG][9], real& cj, real& bj, real& ck, real& bk) {
    const real cs = gj.x * gk.x + gj.y * gk.y + gj.z * gk.z;
    real phi = real(0), e0 = real(0), e1 = real(0);
#pragma unroll
    for (int g = 0; g < NG; ++g) {
        real A = al[g][8], B = real(0);
#pragma unroll
        for (int p = 7; p >= 0; --p) { B = B * cs + A; A = A * cs + al[g][p]; }
        const real DD = dj.D(g) * dk.D(g);
        phi -= B * DD;
        e0 -= A * dj.Dp(g) * dk.D(g);
        e1 -= A * dj.D(g) * dk.Dp(g);
    }
    const real idj = gj.w, idk = gk.w;
    cj = -phi * cs * idj + e0; bj = phi * idj;
    ck = -phi * cs * idk + e1; bk = phi * idk;
}

// the same for FP32 and two damping groups, both groups at once in packed FP32 pairs (group 0 in
// the low half): alp[p] = (al[0][p], al[1][p])
__device__ __forceinline__ void triplet_force2(const Vec4f& gj, const DampRec<float, 2>& dj, const Vec4f& gk, const DampRec<float, 2>& dk,
                                               const uint64_t (&alp)[9], float& cj, float& bj, float& ck, float& bk) {
    const float cs = gj.x * gk.x + gj.y * gk.y + gj.z * gk.z;
    const uint64_t c2 = pk2(cs, cs);
    uint64_t B = alp[8];
    uint64_t A = fma2(B, c2, alp[7]);
#pragma unroll
    for (int p = 6; p >= 0; --p) { B = fma2(B, c2, A); A = fma2(A, c2, alp[p]); }
    const uint64_t Dj = pk2(dj.v[0], dj.v[1]), Dpj = pk2(dj.v[2], dj.v[3]);
    const uint64_t Dk = pk2(dk.v[0], dk.v[1]), Dpk = pk2(dk.v[2], dk.v[3]);
    const float phi = -hsum2(mul2(B, mul2(Dj, Dk)));
    const float e0 = -hsum2(mul2(mul2(A, Dpj), Dk));
    const float e1 = -hsum2(mul2(mul2(A, Dj), Dpk));
    const float idj = gj.w, idk = gk.w;
    cj = -phi * cs * idj + e0; bj = phi * idj;
    ck = -phi * cs * idk + e1; bk = phi * idk;
}

// coefficients of A_g(cos) from the block's dE/dG per slot (slot g*8 + 2q + (lambda < 0), zeta = 2^q):
// ((1 +- x)/2)^zeta = 2^-zeta sum_p C(zeta, p) (+-x)^p
template <typename real, int NG>
__device__ __forceinline__ void angular_poly(const real* dE, const int32_t* slot2ref, int sidx, real (&al)[NG][9]) {
#pragma unroll
    for (int g = 0; g < NG; ++g) {
#pragma unroll
        for (int p = 0; p < 9; ++p) al[g][p] = real(0);
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int rp = slot2ref[sidx + g * 8 + 2 * q], rm = slot2ref[sidx + g * 8 + 2 * q + 1];
            const real cp = (rp >= 0) ? dE[rp] : real(0), cm = (rm >= 0) ? dE[rm] : real(0);
            const int z = 1 << q;
            real binom = real(1);                      // C(z, p)
            const real scale = real(1) / real(1 << z);
#pragma unroll
            for (int p = 0; p <= 8; ++p) {
                if (p <= z) al[g][p] += scale * binom * ((p & 1) ? cp - cm : cp + cm);
                binom = binom * real(z - p) / real(p + 1);
            }
        }
    }
}

// One chunk task of the force pass: the neighbours of an atom are split, per type range, into
// chunks of at most 32, and lane L owns element L of every chunk (chunk start + L). A task is
// either the triangle of one chunk (tri: pairs a < b of [p0, p0+np)) or the rectangle of two
// chunks P x Q (np >= nq). Partners follow a rotation (b = a + step mod n), so in every step the
// 32 lanes touch 32 different partners and each partner is the target of exactly one lane. A
// lane keeps the forces on its own element as c u_own + s (scalar c, vector s); the partner's
// share (ck, bk) goes to the partner's owner lane by two shuffles, and the owner adds ck to its
// scalar and bk times the sender's unit vector (read from shared memory) to its vector. Each
// owner adds its totals to the element's shared-memory accumulator once per task. No atomics;
// every unordered pair is evaluated once.
// A slot without a partner (a lane beyond the chunk, a rectangle partner beyond the shorter chunk,
// the second visit of a pair in the last step of an even triangle) reads the zero record at index
// `zr`: D = D' = 0 and a zero unit vector make every term of the triplet exactly zero, so the loop
// carries no per-step masking of its results. Lanes beyond the owning chunk own the zero record.
// the task scratch for a partner chunk of n elements at qb, of which the first nv have records:
// slot k < 2n holds element k mod n (zeros from nv on). Slots at and beyond 2n keep finite older
// values: only lanes beyond the owning chunk read them, and those lanes own the zero record, so
// their terms vanish.
template <typename WM>
__device__ __forceinline__ void fill_task_scratch(const WM& w, int lane, int qb, int n, int nv) {
    typedef typename WM::R4 R4;
    constexpr int NDP = WM::NDP;
    typedef typename std::remove_pointer<decltype(w.sd)>::type real;
    for (int k = lane; k < 2 * n; k += 32) {
        const int m = (k < n) ? k : k - n;
        R4 g;
        real d[NDP];
        if (m < nv) {
            g = w.geo[qb + m];
#pragma unroll
            for (int q = 0; q < NDP; ++q) d[q] = w.dp[(qb + m) * NDP + q];
        } else {
            g.x = g.y = g.z = g.w = real(0);
#pragma unroll
            for (int q = 0; q < NDP; ++q) d[q] = real(0);
        }
        w.sg[k] = g;
#pragma unroll
        for (int q = 0; q < NDP; ++q) w.sd[k * NDP + q] = d[q];
    }
    __syncwarp();
}

// one rotation step of a force-pass chunk task: the triplet of the lane's own element with the
// element at e, and the share sent by lane src (whose element es is the lane's partner's sender)
template <typename real, int NG, bool PACKED, bool TRI, typename WM, typename R4>
__device__ __forceinline__ void force_step(const WM& w, const R4& ga, const DampRec<real, NG>& da, const real (&al)[NG][9],
                                           const uint64_t (&alp)[9], int e, int es, int src, real& ca, real& cb, real (&sa)[3],
                                           real (&sb)[3]) {
    constexpr int NDP = 2 * NG;
    const R4 gb = w.sg[e];                             // partner (task scratch slot)
    DampRec<real, NG> db;
    db.load(w.sd + e * NDP);
    const R4 gs = TRI ? w.sg[es] : w.geo[es];          // the sending lane's own element
    real cj, bj, ck, bk;
    if constexpr (PACKED) triplet_force2(ga, da, gb, db, alp, cj, bj, ck, bk);
    else triplet_force<real, NG>(ga, da, gb, db, al, cj, bj, ck, bk);
    ca += cj;
    sa[0] += bj * gb.x; sa[1] += bj * gb.y; sa[2] += bj * gb.z;
    const real rc = __shfl_sync(0xffffffffu, ck, src & 31);
    const real rb = __shfl_sync(0xffffffffu, bk, src & 31);
    if (TRI) { ca += rc; sa[0] += rb * gs.x; sa[1] += rb * gs.y; sa[2] += rb * gs.z; }
    else { cb += rc; sb[0] += rb * gs.x; sb[1] += rb * gs.y; sb[2] += rb * gs.z; }
}

template <typename real, int NG, int PASS, bool TRI>
__device__ __forceinline__ void force_task(const WarpMem<real, NG, PASS>& w, const real (&al)[NG][9], int lane,
                                           int p0, int np, int q0, int nq, int zr) {
    typedef typename V4<real>::T R4;
    constexpr int NDP = 2 * NG;
    const bool ownP = lane < np, ownQ = !TRI && lane < nq;
    const int ea = ownP ? p0 + lane : zr;
    const R4 ga = w.geo[ea];
    DampRec<real, NG> da;
    da.load(w.dp + ea * NDP);
    real ca = real(0), cb = real(0);                                       // along the owned unit vectors
    real sa[3] = {real(0), real(0), real(0)}, sb[3] = {real(0), real(0), real(0)};
    constexpr bool PACKED = std::is_same<real, float>::value && NG == 2;
    uint64_t alp[9];
    if constexpr (PACKED) {
#pragma unroll
        for (int p = 0; p < 9; ++p) alp[p] = pk2(al[0][p], al[NG - 1][p]);
    }
    const int n = np;
    const int steps = TRI ? np / 2 : np;      // triangle: steps 1..n/2, rectangle: 0..n-1
    // the partner chunk (the owning one for a triangle) twice over in the task scratch, so that
    // step st reads slot lane + st: partner (lane + st) mod n, or zeros where Q has no element; the
    // sender of step st, lane src = (lane - st) mod n, owns slot n + lane - st of a triangle's
    // scratch, or element p0 + src of a rectangle's owning chunk
    fill_task_scratch(w, lane, TRI ? p0 : q0, n, TRI ? n : nq);
    int src = TRI ? lane - 1 : lane;          // sending lane (lane - step) mod n
    if (src < 0) src += n;
    if (src >= n) src = 0;                    // lanes beyond the chunk: any element of it
    // an even triangle's last step (n/2) visits every pair twice: lanes below n/2 take it, apart
    // from the loop so that the loop body needs no per-lane test
    const bool peel = TRI && (n & 1) == 0 && steps > 0;
    int st = TRI ? 1 : 0;
#pragma unroll 1
    for (; st < (TRI ? steps + (peel ? 0 : 1) : steps); ++st) {
        force_step<real, NG, PACKED, TRI>(w, ga, da, al, alp, lane + st, TRI ? n + lane - st : p0 + src, src, ca, cb, sa, sb);
        src = (src == 0) ? n - 1 : src - 1;
    }
    if (peel) force_step<real, NG, PACKED, TRI>(w, ga, da, al, alp, lane < steps ? lane + st : TS_ZERO, n + lane - st, src, ca, cb, sa, sb);   // (triangles only)
    if (ownP) {
        w.ax[p0 + lane] += ca * ga.x + sa[0]; w.ay[p0 + lane] += ca * ga.y + sa[1]; w.az[p0 + lane] += ca * ga.z + sa[2];
    }
    if (ownQ) {
        const R4 gq = w.geo[q0 + lane];
        w.ax[q0 + lane] += cb * gq.x + sb[0]; w.ay[q0 + lane] += cb * gq.y + sb[1]; w.az[q0 + lane] += cb * gq.z + sb[2];
    }
}

// one rotation step of a symmetry-function chunk task: the triplet of the lane's own element (ga,
// da) with the element at e. FP32 with at most two damping groups: the slot pair (lambda = +1,
// lambda = -1) of each zeta in one packed register, (|1/2 + cos/2|^zeta, |1/2 - cos/2|^zeta) by
// packed squaring, accumulated by packed FMA
template <typename real, int NG, int S, typename WM, typename R4>
__device__ __forceinline__ void symm_step2(const WM& w, const R4& ga, const DampRec<real, NG>& da, int e, uint64_t (&acc2)[S / 2]) {
    constexpr int NDP = 2 * NG;
    const R4 gb = w.sg[e];                 // partner (task scratch slot)
    DampRec<real, NG> db;
    db.load(w.sd + e * NDP);
    const float cs = ga.x * gb.x + ga.y * gb.y + ga.z * gb.z;
    uint64_t pw[4];
    pw[0] = pk2(fabsf(0.5f + 0.5f * cs), fabsf(0.5f - 0.5f * cs));
    pw[1] = mul2(pw[0], pw[0]); pw[2] = mul2(pw[1], pw[1]); pw[3] = mul2(pw[2], pw[2]);
#pragma unroll
    for (int g = 0; g < NG; ++g) {
        const float DD = da.D(g) * db.D(g);          // zero for the zero record
        const uint64_t D2 = pk2(DD, DD);
#pragma unroll
        for (int q = 0; q < 4; ++q) acc2[g * 4 + q] = fma2(pw[q], D2, acc2[g * 4 + q]);
    }
}
template <typename real, int NG, int S, typename WM, typename R4>
__device__ __forceinline__ void symm_step(const WM& w, const R4& ga, const DampRec<real, NG>& da, int e, real (&acc)[S]) {
    constexpr int NDP = 2 * NG;
    const R4 gb = w.sg[e];                 // partner (task scratch slot)
    DampRec<real, NG> db;
    db.load(w.sd + e * NDP);
    const real cs = ga.x * gb.x + ga.y * gb.y + ga.z * gb.z;
    const real cwp = fabs(real(0.5) + real(0.5) * cs), cwm = fabs(real(0.5) - real(0.5) * cs);
    real pp[4], pm[4];
    pp[0] = cwp; pp[1] = cwp * cwp; pp[2] = pp[1] * pp[1]; pp[3] = pp[2] * pp[2];
    pm[0] = cwm; pm[1] = cwm * cwm; pm[2] = pm[1] * pm[1]; pm[3] = pm[2] * pm[2];
#pragma unroll
    for (int g = 0; g < NG; ++g) {
        const real DD = da.D(g) * db.D(g);
#pragma unroll
        for (int q = 0; q < 4; ++q) { acc[g * 8 + 2 * q] += pp[q] * DD; acc[g * 8 + 2 * q + 1] += pm[q] * DD; }
    }
}

// The same chunk tasks for the symmetry functions of a fast-path block: the lane's own neighbour
// stays in registers and only the partner's record is read per pair; acc[s] collects slot s. The
// partner walk is that of force_task (zero record for lanes beyond the chunk, an even triangle's
// last step apart from the loop).
template <typename real, int NG, int S, int PASS, bool TRI>
__device__ __forceinline__ void symm_task(const WarpMem<real, NG, PASS>& w, real (&acc)[S], int lane, int p0, int np, int q0, int nq,
                                          int zr) {
    typedef typename V4<real>::T R4;
    constexpr int NDP = 2 * NG;
    const bool ownP = lane < np;
    const int ea = ownP ? p0 + lane : zr;     // lanes beyond the chunk own the zero record
    const R4 ga = w.geo[ea];
    DampRec<real, NG> da;
    da.load(w.dp + ea * NDP);
    const int n = np;
    const int steps = TRI ? np / 2 : np;
    fill_task_scratch(w, lane, TRI ? p0 : q0, n, TRI ? n : nq);
    const bool peel = TRI && (n & 1) == 0 && steps > 0;
    const int st0 = TRI ? 1 : 0, st_end = TRI ? steps + (peel ? 0 : 1) : steps;
    const int elast = lane < steps ? lane + st_end : TS_ZERO;   // the peeled step's slot
    if constexpr (std::is_same<real, float>::value && NG <= 2) {
        uint64_t acc2[S / 2];
#pragma unroll
        for (int k = 0; k < S / 2; ++k) acc2[k] = pk2(acc[2 * k], acc[2 * k + 1]);
#pragma unroll 2   // two independent triplets per iteration
        for (int st = st0; st < st_end; ++st) symm_step2<real, NG, S>(w, ga, da, lane + st, acc2);
        if (peel) symm_step2<real, NG, S>(w, ga, da, elast, acc2);
#pragma unroll
        for (int k = 0; k < S / 2; ++k) {
            float lo, hi;
            asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(acc2[k]));
            acc[2 * k] = lo; acc[2 * k + 1] = hi;
        }
    } else {
#pragma unroll 2   // two independent triplets per iteration
        for (int st = st0; st < st_end; ++st) symm_step<real, NG, S>(w, ga, da, lane + st, acc);
        if (peel) symm_step<real, NG, S>(w, ga, da, elast, acc);
    }
}

// per-type neighbour ranges of the current atom (at most MAXT = 4): held in registers and read by
// selects (symmetry-function and tangent passes), or as a small array (force pass, whose register
// budget goes to the triplet loop; measured 0.650 vs 0.664 ms on the 74,710-atom batch)
struct TypeRangesReg {
    int v0 = 0, v1 = 0, v2 = 0, v3 = 0;
    __device__ __forceinline__ int get(int t) const { return t == 0 ? v0 : t == 1 ? v1 : t == 2 ? v2 : v3; }
    __device__ __forceinline__ void set(int t, int x) { v0 = t == 0 ? x : v0; v1 = t == 1 ? x : v1; v2 = t == 2 ? x : v2; v3 = t == 3 ? x : v3; }
};
struct TypeRangesArr {
    int v[4];
    __device__ __forceinline__ int get(int t) const { return v[t]; }
    __device__ __forceinline__ void set(int t, int x) { v[t] = x; }
};
static_assert(MAXT == 4, "the type ranges hold four types");

// Shared table of a fast-path force block: the potential's radial parameters (eta, rs) and the
// slot map of the angular blocks, copied once per block so that the force pass's radial loop
// (per neighbour, every function of the block) and coefficient set-up read them from shared
// memory rather than global memory (0.656 -> 0.650 ms; the symmetry pass, which reads each
// parameter once per lane, gains nothing and keeps global loads)
template <typename real>
__host__ __device__ inline size_t bp_table_bytes(const DevPot& pot) {   // force pass, fast path
    const size_t r = ((size_t)2 * pot.nrad * sizeof(real) + 15) / 16 * 16;
    return r + ((size_t)pot.nslot * sizeof(int32_t) + 15) / 16 * 16;
}

// ---------------------------------------------------------------- the kernel
template <typename real, int NG, bool FAST, int PASS>
__global__ void __launch_bounds__(BP_WARPS * 32, bp_min_blocks(PASS, NG, FAST, std::is_same<real, double>::value)) k_bp(const __grid_constant__ DevPot pot, const BpArgs<real> a) {
    typedef typename V4<real>::T R4;
    extern __shared__ __align__(128) unsigned char bsm[];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int cap = a.cap, imax = pot.imax, T = a.ntypes;
    const size_t wbytes = WarpMem<real, NG, PASS>::bytes(cap, imax);
    WarpMem<real, NG, PASS> w;
    WarpMem<real, NG, PASS>::layout(cap, imax, &w, bsm + (size_t)wid * wbytes);
    constexpr int NDP = 2 * NG;
    // force pass, fast path: radial parameters and slot map in shared memory (after the warps' regions)
    const real* t_reta = a.prm.reta;
    const real* t_rs = a.prm.rs;
    const int32_t* t_slot = a.prm.slot2ref;
    if constexpr (FAST && PASS == PASS_FORCE) {
        real* s_reta = reinterpret_cast<real*>(bsm + (size_t)BP_WARPS * wbytes);
        real* s_rs = s_reta + pot.nrad;
        int32_t* s_slot = reinterpret_cast<int32_t*>(bsm + (size_t)BP_WARPS * wbytes + ((size_t)2 * pot.nrad * sizeof(real) + 15) / 16 * 16);
        for (int k = threadIdx.x; k < pot.nrad; k += blockDim.x) { s_reta[k] = a.prm.reta[k]; s_rs[k] = a.prm.rs[k]; }
        for (int k = threadIdx.x; k < pot.nslot; k += blockDim.x) s_slot[k] = a.prm.slot2ref[k];
        __syncthreads();
        t_reta = s_reta; t_rs = s_rs; t_slot = s_slot;
    }
    if (lane == 0) { mbar_init(&w.bar[0], 1); mbar_init(&w.bar[1], 1); }
    // the zero record (index cap) of both staging buffers and of the damping records: a partner
    // slot outside a chunk task reads it and contributes exactly zero
    if (lane < 4) {
        reinterpret_cast<real*>(&w.geo[cap])[lane] = real(0);
        reinterpret_cast<real*>(&w.stage[cap])[lane] = real(0);
    }
    if (lane < NDP) w.dp[(size_t)cap * NDP + lane] = real(0);
    if constexpr (PASS != PASS_JVP) {
        // the task scratch starts as zeros, so that slots no task wrote hold finite values
        for (int k = lane; k < 4 * (TS_ZERO + 1); k += 32) reinterpret_cast<real*>(w.sg)[k] = real(0);
        for (int k = lane; k < NDP * (TS_ZERO + 1); k += 32) w.sd[k] = real(0);
    }
    __syncwarp();
    uint32_t phase = 0;   // bit b: parity of the next phase of barrier b
    const unsigned lt = (1u << lane) - 1u;
    constexpr int S = NG * 8;

    // ---- 1. neighbour rows are staged by bulk asynchronous copies into two buffers: the row of
    //         the next atom is in flight while the current one is processed. A staged row is
    //         compacted in place, so a buffer serves as stage and then as the atom's records.
    R4* const gbuf0 = w.geo;
    R4* const gbuf1 = w.stage;
    int32_t* const jbuf0 = w.stagej;
    int32_t* const jbuf1 = w.stagej2;
    real* const ebuf0 = w.dE;
    real* const ebuf1 = w.dE + imax;
    // force pass: the dE/dG row travels with the neighbour row when rows are whole 16-byte units
    const bool dE_bulk = (PASS == PASS_FORCE) && ((size_t)imax * sizeof(real)) % 16 == 0;
    auto next_atom = [&]() {
        int v = 0;
        if (lane == 0) v = (int)atomicAdd(a.counter, 1u);
        return __shfl_sync(0xffffffffu, v, 0);
    };
    // the next atom's scalars, loaded a whole atom ahead of their use: type, entries, and the
    // entries per neighbour type in lanes 0..T-1
    struct AtomScalars { int type, nn, ntc; };
    auto load_scalars = [&](int i) {
        AtomScalars v{0, 0, 0};
        if (i < a.natoms) {
            v.type = a.type[i];
            v.nn = a.nn[i];
            if (lane < T) v.ntc = a.ntc[(size_t)i * T + lane];
        }
        return v;
    };
    auto stage_row = [&](int i, int b, int nn) -> bool {   // false: nothing was issued
        if (i >= a.natoms) return false;
        const int nin = min(nn, cap);
        if (nin <= 0) return false;
        if (lane == 0) {
            const size_t row = (size_t)i * cap;
            const uint32_t b1 = (uint32_t)(nin * sizeof(R4));
            const uint32_t b2 = (uint32_t)(((nin + 3) / 4) * 16);
            const uint32_t b3 = dE_bulk ? (uint32_t)(imax * sizeof(real)) : 0u;
            fence_proxy_async();
            mbar_expect_tx(&w.bar[b], b1 + b2 + b3);
            bulk_g2s(b ? gbuf1 : gbuf0, reinterpret_cast<const R4*>(a.nr) + row, b1, &w.bar[b]);
            bulk_g2s(b ? jbuf1 : jbuf0, a.nj + row, b2, &w.bar[b]);
            if (dE_bulk) bulk_g2s(b ? ebuf1 : ebuf0, a.dEdG + (size_t)i * imax, b3, &w.bar[b]);
        }
        return true;
    };
    int nx_i = next_atom(), nx_b = 0;
    AtomScalars nx_s = load_scalars(nx_i);
    bool nx_issued = stage_row(nx_i, 0, nx_s.nn);

    for (;;) {
        const int i = nx_i, cb = nx_b;
        const bool issued = nx_issued;
        const AtomScalars cur = nx_s;
        if (i >= a.natoms) break;
        nx_i = next_atom();
        nx_b = cb ^ 1;
        nx_s = load_scalars(nx_i);
        nx_issued = stage_row(nx_i, nx_b, nx_s.nn);
        if (issued) {
            const bool done = mbar_wait_bounded(&w.bar[cb], (phase >> cb) & 1u, a.wait_polls);
            if (!__all_sync(0xffffffffu, done)) {  // bounded wait gave up: report, drain (full bound), stop
                if (lane == 0) atomicOr(a.status, (int)ST_TIMEOUT);
                for (int it = 0; it < (1 << 24); ++it) if (mbar_try_wait(&w.bar[cb], (phase >> cb) & 1u)) break;
                if (nx_issued)
                    for (int it = 0; it < (1 << 24); ++it) if (mbar_try_wait(&w.bar[nx_b], (phase >> nx_b) & 1u)) break;
                return;
            }
            phase ^= 1u << cb;
        }
        w.geo = cb ? gbuf1 : gbuf0;
        w.stagej = cb ? jbuf1 : jbuf0;
        if (PASS == PASS_FORCE) w.dE = cb ? ebuf1 : ebuf0;
        // the symmetry pass clears the atom's force accumulator for the force pass that follows
        if (PASS == PASS_SYMM && lane < 3) a.F[3 * (size_t)i + lane] = real(0);
        const int I = cur.type;
        if (I < 0 || I >= T) { if (lane == 0) atomicOr(a.status, (int)ST_BAD_TYPE); continue; }
        const DevType& TT = pot.t[I];
        const int nin = min(cur.nn, cap);
        const size_t row = (size_t)i * cap;
        // ---- compaction to d < rc, per-type active ranges, per-neighbour records ---------------
        const real rc = (real)TT.rc;
        real ie2[NG];
#pragma unroll
        for (int q = 0; q < NG; ++q) ie2[q] = (real)TT.ietar2[q];
        typename std::conditional<PASS == PASS_FORCE, TypeRangesArr, TypeRangesReg>::type tstart, tcnt;
        int pos = 0, base_in = 0;
        for (int t = 0; t < T; ++t) {
            const int cin = __shfl_sync(0xffffffffu, cur.ntc, t);
            tstart.set(t, pos);
            for (int e0 = 0; e0 < cin; e0 += 32) {
                const int e = base_in + e0 + lane;
                bool keep = false;
                R4 r4;
                int j = 0;
                if (e0 + lane < cin && e < nin) { r4 = w.geo[e]; j = w.stagej[e]; keep = r4.w < rc; }
                const unsigned msk = __ballot_sync(0xffffffffu, keep);
                __syncwarp();   // records are compacted in place (o <= e): all reads of the chunk first
                if (keep) {
                    const int o = pos + __popc(msk & lt);
                    const real dd = r4.w, idd = real(1) / dd;
                    R4 g4; g4.x = r4.x * idd; g4.y = r4.y * idd; g4.z = r4.z * idd; g4.w = idd;
                    w.geo[o] = g4;
                    w.d[o] = dd;
                    real f, g;
                    cutoff_fg<real>(TT.cut, rc, dd, f, g);
                    w.fc[o] = f; w.fcg[o] = g;
                    if (FAST) {
#pragma unroll
                        for (int q = 0; q < NG; ++q) {
                            const real ex = M<real>::bexp(-dd * dd * ie2[q]);
                            w.dp[o * NDP + q] = f * ex;
                            w.dp[o * NDP + NG + q] = ex * (g - real(2) * dd * f * ie2[q]);
                        }
                    }
                    if (PASS == PASS_FORCE) {
                        w.stagej[o] = (a.newton_untranslated && a.nimg[row + e] != 0) ? -1 : j;
                        w.ax[o] = real(0); w.ay[o] = real(0); w.az[o] = real(0);
                    }
                    if (PASS == PASS_JVP) {
                        const real lx = a.lam[3 * (size_t)i] - a.lam[3 * (size_t)j];
                        const real ly = a.lam[3 * (size_t)i + 1] - a.lam[3 * (size_t)j + 1];
                        const real lz = a.lam[3 * (size_t)i + 2] - a.lam[3 * (size_t)j + 2];
                        R4 t4; t4.x = lx; t4.y = ly; t4.z = lz; t4.w = g4.x * lx + g4.y * ly + g4.z * lz;
                        w.tg[o] = t4;
                    }
                }
                pos += __popc(msk);
            }
            tcnt.set(t, pos - tstart.get(t));
            base_in += cin;
        }
        if (PASS == PASS_FORCE && !(dE_bulk && issued)) {
            for (int m = lane; m < TT.nInput; m += 32) w.dE[m] = a.dEdG[(size_t)i * imax + m];
        }
        __syncwarp();

        real* Gout = (PASS == PASS_SYMM) ? a.G + (size_t)i * imax : (PASS == PASS_JVP) ? a.U + (size_t)i * imax : nullptr;

        // ---- 2. radial. Symmetry functions / tangents: lanes own functions. The blocks' functions
        //         are numbered one after the other (block J's function m is slot off_J + m), lane
        //         L takes slots L, L + 32, ... and sums its function over the block's neighbour
        //         range in shared memory, so every slot is one lane's sequential sum (no reduction).
        //         Force pass: lanes own neighbours and loop over the block's functions with
        //         uniform loads ------------------------------------------------------------------
        if (PASS == PASS_FORCE) {
            for (int J = 0; J < T; ++J) {
                const DevRadial& R = TT.R[J];
                if (R.n == 0) continue;
                const int e0 = tstart.get(J), e1 = e0 + tcnt.get(J);
                auto block = [&](auto form) {
                    constexpr int NAME = decltype(form)::value;
                    for (int e = e0 + lane; e < e1; e += 32) {
                        const real dd = w.d[e], f = w.fc[e], g = w.fcg[e];
                        real amp = real(0);
#pragma unroll 4
                        for (int m = 0; m < R.n; ++m) {
                            real val, der;
                            radial_vd_t<NAME, real>(R.name, t_reta[R.pidx + m], t_rs[R.pidx + m], dd, f, g, val, der);
                            amp -= w.dE[R.off + m] * der;
                        }
                        const R4 g4 = w.geo[e];
                        w.ax[e] += amp * g4.x; w.ay[e] += amp * g4.y; w.az[e] += amp * g4.z;
                    }
                };
                if (R.name == R_GAUSSIAN) block(std::integral_constant<int, R_GAUSSIAN>{});
                else block(std::integral_constant<int, -1>{});
            }
        } else {
            int nslot = 0;
            for (int J = 0; J < T; ++J) nslot += TT.R[J].n;
            for (int q = lane; q < nslot; q += 32) {
                int J = 0, m = q, e0 = 0, ne = 0;
#pragma unroll
                for (int t = 0; t < MAXT; ++t) {      // the lane's block, with constant indices only
                    if (t < T && J == t && m >= TT.R[t].n) { m -= TT.R[t].n; J = t + 1; }
                }
                e0 = tstart.get(J); ne = tcnt.get(J);
                const DevRadial& R = TT.R[J];
                const real eta = t_reta[R.pidx + m], rs = t_rs[R.pidx + m];
                real acc = real(0);
                auto block = [&](auto form) {
                    constexpr int NAME = decltype(form)::value;
                    for (int e = e0; e < e0 + ne; ++e) {
                        real val, der;
                        radial_vd_t<NAME, real>(R.name, eta, rs, w.d[e], w.fc[e], w.fcg[e], val, der);
                        acc += (PASS == PASS_SYMM) ? val : der * w.tg[e].w;
                    }
                };
                if (R.name == R_GAUSSIAN) block(std::integral_constant<int, R_GAUSSIAN>{});
                else block(std::integral_constant<int, -1>{});
                Gout[R.off + m] = acc;
            }
        }
        __syncwarp();

        // ---- 3. angular ---------------------------------------------------------------------------
        for (int J = 0; J < T; ++J) {
            for (int K = J; K < T; ++K) {
                const int blk = tri_index(J, K);
                const DevAngular& A = TT.A[blk];
                if (A.n == 0) continue;
                const int nJ = tcnt.get(J), nK = tcnt.get(K), aJ = tstart.get(J), aK = tstart.get(K);
                const int total = (J == K) ? nJ * (nJ - 1) / 2 : nJ * nK;
                constexpr bool ROWS = (PASS != PASS_FORCE);
                if (FAST) {
                    // ------------------------------------------------ fast path (GAUSS, zeta=2^k)
                    real acc[S];
#pragma unroll
                    for (int s = 0; s < S; ++s) acc[s] = real(0);
                    if (PASS != PASS_JVP) {
                        // chunk tasks: triangles of each chunk, rectangles of chunk pairs (larger first)
                        real al[NG][9];
                        if (PASS == PASS_FORCE) angular_poly<real, NG>(w.dE + A.off, t_slot, A.sidx, al);
                        auto task = [&](int p0, int np, int q0, int nq, bool tri) {
                            if (PASS == PASS_FORCE) {
                                if (tri) force_task<real, NG, PASS, true>(w, al, lane, p0, np, q0, nq, cap);
                                else force_task<real, NG, PASS, false>(w, al, lane, p0, np, q0, nq, cap);
                            } else {
                                if (tri) symm_task<real, NG, S, PASS, true>(w, acc, lane, p0, np, q0, nq, cap);
                                else symm_task<real, NG, S, PASS, false>(w, acc, lane, p0, np, q0, nq, cap);
                            }
                        };
                        // a range of n neighbours in ceil(n / 32) chunks of nearly equal size: a
                        // rectangle task of chunks P x Q takes max(|P|, |Q|) steps, so an even split
                        // (35 -> 18 + 17, not 32 + 3) keeps its lanes busy
                        auto chunk = [](int n, int c, int& c0, int& cn) {
                            const int k = (n + 31) >> 5, base = n / k, rem = n - base * k;
                            c0 = c * base + min(c, rem);
                            cn = base + (c < rem ? 1 : 0);
                        };
                        const int kJ = (nJ + 31) >> 5, kK = (nK + 31) >> 5;
                        if (J == K) {
                            for (int ca = 0; ca < kJ; ++ca) {
                                int c0, n0;
                                chunk(nJ, ca, c0, n0);
                                task(aJ + c0, n0, 0, 0, true);
                                for (int cb = ca + 1; cb < kJ; ++cb) {
                                    int c1, n1;
                                    chunk(nJ, cb, c1, n1);
                                    if (n0 >= n1) task(aJ + c0, n0, aJ + c1, n1, false);
                                    else task(aJ + c1, n1, aJ + c0, n0, false);
                                }
                            }
                        } else {
                            for (int ca = 0; ca < kJ; ++ca) {
                                int c0, n0;
                                chunk(nJ, ca, c0, n0);
                                for (int cb = 0; cb < kK; ++cb) {
                                    int c1, n1;
                                    chunk(nK, cb, c1, n1);
                                    if (n0 >= n1) task(aJ + c0, n0, aK + c1, n1, false);
                                    else task(aK + c1, n1, aJ + c0, n0, false);
                                }
                            }
                        }
                    }
                    TriIter<ROWS> ti; RectIter<ROWS> ri;
                    if (PASS == PASS_JVP) { if (J == K) ti.init(nJ, lane); else ri.init(max(nJ, 1), max(nK, 1), lane); }
                    if constexpr (PASS == PASS_JVP && std::is_same<real, float>::value && NG <= 2) {
                        // FP32: the (lambda = +1, lambda = -1) pair of each zeta in one packed
                        // register; d|1/2 +- cos/2|^zeta = +-(zeta/2) |.|^(zeta-1) dcos
                        uint64_t acc2[S / 2];
#pragma unroll
                        for (int k2 = 0; k2 < S / 2; ++k2) acc2[k2] = pk2(acc[2 * k2], acc[2 * k2 + 1]);
                        for (int t = lane; t < total; t += 32) {
                            int j, k;
                            if (J == K) { j = aJ + ti.j(); k = aJ + ti.k(); ti.adv(); }
                            else { j = aJ + ri.q; k = aK + ri.c; ri.adv(); }
                            const R4 gj = w.geo[j], gk = w.geo[k];
                            DampRec<real, NG> dj, dk;
                            dj.load(w.dp + j * NDP); dk.load(w.dp + k * NDP);
                            const float cs = gj.x * gk.x + gj.y * gk.y + gj.z * gk.z;
                            uint64_t pw[4], kq[4];
                            pw[0] = pk2(fabsf(0.5f + 0.5f * cs), fabsf(0.5f - 0.5f * cs));
                            pw[1] = mul2(pw[0], pw[0]); pw[2] = mul2(pw[1], pw[1]); pw[3] = mul2(pw[2], pw[2]);
                            kq[0] = pk2(0.5f, -0.5f);                                  // (zeta/2) cw^(zeta-1), zeta = 1
                            kq[1] = mul2(pw[0], pk2(1.0f, -1.0f));                     // zeta = 2
                            kq[2] = mul2(mul2(pw[0], pw[1]), pk2(2.0f, -2.0f));        // zeta = 4
                            kq[3] = mul2(mul2(mul2(pw[0], pw[1]), pw[2]), pk2(4.0f, -4.0f));   // zeta = 8
                            const R4 tj = w.tg[j], tk = w.tg[k];
                            const float idj = gj.w, idk = gk.w;
                            const float dcos = (tj.x * gk.x + tj.y * gk.y + tj.z * gk.z) * idj +
                                               (tk.x * gj.x + tk.y * gj.y + tk.z * gj.z) * idk - cs * (tj.w * idj + tk.w * idk);
#pragma unroll
                            for (int g = 0; g < NG; ++g) {
                                const float DD = dj.D(g) * dk.D(g);
                                const float dDD = dj.Dp(g) * dk.D(g) * tj.w + dj.D(g) * dk.Dp(g) * tk.w;
                                const uint64_t a2 = pk2(DD * dcos, DD * dcos), b2 = pk2(dDD, dDD);
#pragma unroll
                                for (int q = 0; q < 4; ++q) acc2[g * 4 + q] = fma2(kq[q], a2, fma2(pw[q], b2, acc2[g * 4 + q]));
                            }
                        }
#pragma unroll
                        for (int k2 = 0; k2 < S / 2; ++k2) {
                            float lo, hi;
                            asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(acc2[k2]));
                            acc[2 * k2] = lo; acc[2 * k2 + 1] = hi;
                        }
                    } else {
                    for (int t = lane; PASS == PASS_JVP && t < total; t += 32) {
                        int j, k;
                        if (J == K) { j = aJ + ti.j(); k = aJ + ti.k(); ti.adv(); }
                        else { j = aJ + ri.q; k = aK + ri.c; ri.adv(); }
                        const R4 gj = w.geo[j], gk = w.geo[k];
                        DampRec<real, NG> dj, dk;
                        dj.load(w.dp + j * NDP); dk.load(w.dp + k * NDP);
                        const real cs = gj.x * gk.x + gj.y * gk.y + gj.z * gk.z;
                        const real cwp = fabs(real(0.5) + real(0.5) * cs), cwm = fabs(real(0.5) - real(0.5) * cs);
                        real pp[4], pm[4];
                        pp[0] = cwp; pp[1] = cwp * cwp; pp[2] = pp[1] * pp[1]; pp[3] = pp[2] * pp[2];
                        pm[0] = cwm; pm[1] = cwm * cwm; pm[2] = pm[1] * pm[1]; pm[3] = pm[2] * pm[2];
                        // tangents (training): row order, the warp shares j
                        real qp[4], qm[4];   // cw^(zeta-1) for zeta = 1,2,4,8
                        qp[0] = real(1); qp[1] = cwp; qp[2] = cwp * pp[1]; qp[3] = qp[2] * pp[2];
                        qm[0] = real(1); qm[1] = cwm; qm[2] = cwm * pm[1]; qm[3] = qm[2] * pm[2];
                        const R4 tj = w.tg[j], tk = w.tg[k];
                        const real idj = gj.w, idk = gk.w;
                        const real dcos = (tj.x * gk.x + tj.y * gk.y + tj.z * gk.z) * idj +
                                          (tk.x * gj.x + tk.y * gj.y + tk.z * gj.z) * idk - cs * (tj.w * idj + tk.w * idk);
#pragma unroll
                        for (int g = 0; g < NG; ++g) {
                            const real DD = dj.D(g) * dk.D(g);
                            const real dDD = dj.Dp(g) * dk.D(g) * tj.w + dj.D(g) * dk.Dp(g) * tk.w;
#pragma unroll
                            for (int q = 0; q < 4; ++q) {
                                const real z = real(1 << q);
                                acc[g * 8 + 2 * q] += z * real(0.5) * qp[q] * DD * dcos + pp[q] * dDD;
                                acc[g * 8 + 2 * q + 1] += -z * real(0.5) * qm[q] * DD * dcos + pm[q] * dDD;
                            }
                        }
                    }
                    }
                    if (PASS != PASS_FORCE) {
                        const real v = warp_slot_reduce<real, S>(acc, lane);
                        constexpr int SH = SlotShift<S>::v;
                        if ((lane & ((1 << SH) - 1)) == 0) {
                            const int s = (lane >> SH) & (S - 1);
                            const int ref = t_slot[A.sidx + s];
                            if (ref >= 0) Gout[A.off + ref] = v;
                        }
                    }
                } else {
                    // ------------------------------------------------ generic path (any BasisA)
                    if (PASS == PASS_FORCE) {
                        TriIter<false> ti; RectIter<false> ri;
                        if (J == K) ti.init(nJ, lane); else ri.init(max(nJ, 1), max(nK, 1), lane);
                        for (int t = lane; t < total; t += 32) {
                            int j, k;
                            if (J == K) { j = aJ + ti.j(); k = aJ + ti.k(); ti.adv(); }
                            else { j = aJ + ri.q; k = aK + ri.c; ri.adv(); }
                            const R4 gj = w.geo[j], gk = w.geo[k];
                            const real cs = gj.x * gk.x + gj.y * gk.y + gj.z * gk.z;
                            const real dj = w.d[j], dk = w.d[k];
                            const real r2s = dj * dj + dk * dk;
                            const real fj = w.fc[j], fk = w.fc[k], gjj = w.fcg[j], gkk = w.fcg[k];
                            real phi = real(0), e0 = real(0), e1 = real(0);
                            for (int m = 0; m < A.n; ++m) {
                                const real eta = a.prm.aeta[A.pidx + m], zeta = a.prm.zeta[A.pidx + m];
                                const real lf = real(0.5) * a.prm.alam[A.pidx + m];
                                const real iex = real(1) / (eta * eta);
                                real h, dq;
                                angular_damp<real>(A.name, iex, r2s, h, dq);
                                const real cw = fabs(real(0.5) + lf * cs);
                                const real ga = w.dE[A.off + m] * M<real>::pow(cw, zeta - real(1)) * h;
                                const real fa = cw * ga;
                                phi -= zeta * lf * ga;
                                e0 -= fa * (-dq * real(2) * dj * fj + gjj);
                                e1 -= fa * (-dq * real(2) * dk * fk + gkk);
                            }
                            phi *= fj * fk; e0 *= fk; e1 *= fj;
                            const real idj = gj.w, idk = gk.w;
                            const real cj = -phi * cs * idj + e0, bj = phi * idj;
                            const real ck = -phi * cs * idk + e1, bk = phi * idk;
                            atomicAdd(&w.ax[j], cj * gj.x + bj * gk.x); atomicAdd(&w.ay[j], cj * gj.y + bj * gk.y); atomicAdd(&w.az[j], cj * gj.z + bj * gk.z);
                            atomicAdd(&w.ax[k], ck * gk.x + bk * gj.x); atomicAdd(&w.ay[k], ck * gk.y + bk * gj.y); atomicAdd(&w.az[k], ck * gk.z + bk * gj.z);
                        }
                    } else {
                        for (int m0 = 0; m0 < A.n; m0 += CHUNK) {
                            real acc[CHUNK];
#pragma unroll
                            for (int s = 0; s < CHUNK; ++s) acc[s] = real(0);
                            TriIter<true> ti; RectIter<true> ri;
                            if (J == K) ti.init(nJ, lane); else ri.init(max(nJ, 1), max(nK, 1), lane);
                            for (int t = lane; t < total; t += 32) {
                                int j, k;
                                if (J == K) { j = aJ + ti.j(); k = aJ + ti.k(); ti.adv(); }
                                else { j = aJ + ri.q; k = aK + ri.c; ri.adv(); }
                                const R4 gj = w.geo[j], gk = w.geo[k];
                                const real cs = gj.x * gk.x + gj.y * gk.y + gj.z * gk.z;
                                const real dj = w.d[j], dk = w.d[k];
                                const real r2s = dj * dj + dk * dk;
                                const real fj = w.fc[j], fk = w.fc[k], gjj = w.fcg[j], gkk = w.fcg[k];
                                real dcos = real(0), ddj = real(0), ddk = real(0);
                                if (PASS == PASS_JVP) {
                                    const R4 tj = w.tg[j], tk = w.tg[k];
                                    const real idj = gj.w, idk = gk.w;
                                    ddj = tj.w; ddk = tk.w;
                                    dcos = (tj.x * gk.x + tj.y * gk.y + tj.z * gk.z) * idj + (tk.x * gj.x + tk.y * gj.y + tk.z * gj.z) * idk -
                                           cs * (ddj * idj + ddk * idk);
                                }
#pragma unroll
                                for (int s = 0; s < CHUNK; ++s) {
                                    const int m = m0 + s;
                                    if (m < A.n) {
                                        const real eta = a.prm.aeta[A.pidx + m], zeta = a.prm.zeta[A.pidx + m];
                                        const real lf = real(0.5) * a.prm.alam[A.pidx + m];
                                        const real iex = real(1) / (eta * eta);
                                        real h, dq;
                                        angular_damp<real>(A.name, iex, r2s, h, dq);
                                        const real cw = fabs(real(0.5) + lf * cs);
                                        if (PASS == PASS_SYMM) {
                                            acc[s] += M<real>::pow(cw, zeta) * h * fj * fk;
                                        } else {
                                            const real ga = M<real>::pow(cw, zeta - real(1)) * h;
                                            const real fa = cw * ga;
                                            const real fphi = zeta * lf * ga * fj * fk;
                                            const real fe0 = fa * (-dq * real(2) * dj * fj + gjj) * fk;
                                            const real fe1 = fa * (-dq * real(2) * dk * fk + gkk) * fj;
                                            acc[s] += fphi * dcos + fe0 * ddj + fe1 * ddk;
                                        }
                                    }
                                }
                            }
                            const real v = warp_slot_reduce<real, CHUNK>(acc, lane);
                            if ((lane & 1) == 0) {
                                const int m = m0 + ((lane >> 1) & (CHUNK - 1));
                                if (m < A.n) Gout[A.off + m] = v;
                            }
                        }
                    }
                }
            }
        }
        __syncwarp();

        // ---- 4. force pass: per-neighbour totals ---------------------------------------------------
        if (PASS == PASS_FORCE) {
            real fx = 0, fy = 0, fz = 0;
            real W9[9];
#pragma unroll
            for (int q = 0; q < 9; ++q) W9[q] = real(0);
            for (int e = lane; e < pos; e += 32) {
                const real vx = w.ax[e], vy = w.ay[e], vz = w.az[e];
                fx += vx; fy += vy; fz += vz;
                const R4 g4 = w.geo[e];
                const real dd = w.d[e];
                const real rx = g4.x * dd, ry = g4.y * dd, rz = g4.z * dd;
                W9[0] += rx * vx; W9[1] += rx * vy; W9[2] += rx * vz;
                W9[3] += ry * vx; W9[4] += ry * vy; W9[5] += ry * vz;
                W9[6] += rz * vx; W9[7] += rz * vy; W9[8] += rz * vz;
                const int j = w.stagej[e];
                if (j >= 0) {
                    atomicAdd(&a.F[3 * (size_t)j], -vx); atomicAdd(&a.F[3 * (size_t)j + 1], -vy); atomicAdd(&a.F[3 * (size_t)j + 2], -vz);
                }
            }
            fx = warp_sum(fx); fy = warp_sum(fy); fz = warp_sum(fz);
#pragma unroll
            for (int q = 0; q < 9; ++q) W9[q] = warp_sum(W9[q]);
            if (lane == 0) {
                const size_t ic = a.self ? (size_t)a.self[i] : (size_t)i;
                atomicAdd(&a.F[3 * ic], fx); atomicAdd(&a.F[3 * ic + 1], fy); atomicAdd(&a.F[3 * ic + 2], fz);
#pragma unroll
                for (int q = 0; q < 9; ++q) a.W[9 * (size_t)i + q] = W9[q];
            }
        }
        __syncwarp();
    }
}

// G / U rows must start at zero (blocks without neighbours or triplets are not visited)
template <typename real>
__global__ void k_zero(real* p, size_t n) {
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x) p[k] = real(0);
}

template <typename real>
void launch_zero_rows(real* p, size_t n, cudaStream_t st) {
    if (n == 0) return;
    ++::ann::g_launch_counter, k_zero<real><<<1024, 256, 0, st>>>(p, n);
}
template void launch_zero_rows<float>(float*, size_t, cudaStream_t);
template void launch_zero_rows<double>(double*, size_t, cudaStream_t);

template <typename real, int PASS>
static void launch_pass(const DevPot& pot, const BpArgs<real>& a, cudaStream_t st) {
    if (a.natoms <= 0) return;
    if (PASS != PASS_FORCE && !a.out_zeroed)
        launch_zero_rows<real>((PASS == PASS_SYMM) ? a.G : a.U, (size_t)a.natoms * pot.imax, st);
    cudaMemsetAsync(a.counter, 0, sizeof(uint32_t), st);
    auto go = [&](auto kern, size_t wb, size_t table) {
        const size_t smem = wb * BP_WARPS + table;
        int per_sm = (int)std::max<size_t>(1, (size_t)(227 * 1024) / std::max<size_t>(smem, 1));
        per_sm = std::min(per_sm, 16);
        if (a.grid_per_sm > 0) per_sm = std::min(per_sm, (int)a.grid_per_sm);
        int grid = (a.natoms + BP_WARPS - 1) / BP_WARPS;
        grid = std::min(grid, std::max(1, (int)a.nsm) * per_sm);
        ++::ann::g_launch_counter, kern<<<grid, BP_WARPS * 32, smem, st>>>(pot, a);
    };
    const size_t tb = (PASS == PASS_FORCE) ? bp_table_bytes<real>(pot) : 0;
    if (pot.fast) {
        if (pot.fastNG == 1) go(k_bp<real, 1, true, PASS>, WarpMem<real, 1, PASS>::bytes(a.cap, pot.imax), tb);
        else if (pot.fastNG == 2) go(k_bp<real, 2, true, PASS>, WarpMem<real, 2, PASS>::bytes(a.cap, pot.imax), tb);
        else go(k_bp<real, 4, true, PASS>, WarpMem<real, 4, PASS>::bytes(a.cap, pot.imax), tb);
    } else {
        go(k_bp<real, 1, false, PASS>, WarpMem<real, 1, PASS>::bytes(a.cap, pot.imax), 0);
    }
}

template <typename real, int PASS>
static void configure_pass(int maxsmem) {
    set_max_dynamic_smem(k_bp<real, 1, true, PASS>, maxsmem);
    set_max_dynamic_smem(k_bp<real, 2, true, PASS>, maxsmem);
    set_max_dynamic_smem(k_bp<real, 4, true, PASS>, maxsmem);
    set_max_dynamic_smem(k_bp<real, 1, false, PASS>, maxsmem);
    // residency is bounded by shared memory (neighbour records and task scratch per warp)
    prefer_max_shared(k_bp<real, 1, true, PASS>);
    prefer_max_shared(k_bp<real, 2, true, PASS>);
    prefer_max_shared(k_bp<real, 4, true, PASS>);
    prefer_max_shared(k_bp<real, 1, false, PASS>);
}
void configure_bp(int maxsmem) {
    configure_pass<float, PASS_SYMM>(maxsmem); configure_pass<float, PASS_FORCE>(maxsmem); configure_pass<float, PASS_JVP>(maxsmem);
    configure_pass<double, PASS_SYMM>(maxsmem); configure_pass<double, PASS_FORCE>(maxsmem); configure_pass<double, PASS_JVP>(maxsmem);
}
// the largest per-block shared memory any pass needs for this potential and capacity
size_t bp_smem_bytes(const DevPot& pot, int cap, bool fp64) {
    const int ng = pot.fast ? pot.fastNG : 1;
    auto b = [&](auto tag) -> size_t {
        using real = decltype(tag);
        if (ng == 1) return std::max({WarpMem<real, 1, PASS_SYMM>::bytes(cap, pot.imax), WarpMem<real, 1, PASS_FORCE>::bytes(cap, pot.imax), WarpMem<real, 1, PASS_JVP>::bytes(cap, pot.imax)});
        if (ng == 2) return std::max({WarpMem<real, 2, PASS_SYMM>::bytes(cap, pot.imax), WarpMem<real, 2, PASS_FORCE>::bytes(cap, pot.imax), WarpMem<real, 2, PASS_JVP>::bytes(cap, pot.imax)});
        return std::max({WarpMem<real, 4, PASS_SYMM>::bytes(cap, pot.imax), WarpMem<real, 4, PASS_FORCE>::bytes(cap, pot.imax), WarpMem<real, 4, PASS_JVP>::bytes(cap, pot.imax)});
    };
    const size_t table = pot.fast ? (fp64 ? bp_table_bytes<double>(pot) : bp_table_bytes<float>(pot)) : 0;
    return (fp64 ? b(double()) : b(float())) * BP_WARPS + table;
}

template <typename real> void launch_symm(const DevPot& pot, const BpArgs<real>& a, cudaStream_t st) { launch_pass<real, PASS_SYMM>(pot, a, st); }
template <typename real> void launch_force(const DevPot& pot, const BpArgs<real>& a, cudaStream_t st) { launch_pass<real, PASS_FORCE>(pot, a, st); }
template <typename real> void launch_jvp(const DevPot& pot, const BpArgs<real>& a, cudaStream_t st) { launch_pass<real, PASS_JVP>(pot, a, st); }

template void launch_symm<float>(const DevPot&, const BpArgs<float>&, cudaStream_t);
template void launch_symm<double>(const DevPot&, const BpArgs<double>&, cudaStream_t);
template void launch_force<float>(const DevPot&, const BpArgs<float>&, cudaStream_t);
template void launch_force<double>(const DevPot&, const BpArgs<double>&, cudaStream_t);
template void launch_jvp<float>(const DevPot&, const BpArgs<float>&, cudaStream_t);
template void launch_jvp<double>(const DevPot&, const BpArgs<double>&, cudaStream_t);

}  // namespace ann
