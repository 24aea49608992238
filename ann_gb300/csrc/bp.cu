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
//     into per-neighbour quantities: unit vector, 1/d, cutoff f and f', and for every damping
//     group g of the angular GAUSS functions D_g = f * exp(-d^2/eta_g^2) and its d-derivative.
//  2. radial functions: lanes own functions, loop over the neighbours of each type block.
//  3. angular functions: lanes own (j,k) triplets of each (J,K) type block. In the fast path
//     (GAUSS, lambda=+-1, zeta=2^k) the reference's exp(-(rij^2+rik^2)/eta^2) factorises into
//     D_g(j) D_g(k) and |1/2 +- cos/2|^zeta comes from a squaring chain, so no transcendental
//     is evaluated per triplet. Per-slot sums are reduced across the warp by a transposing
//     butterfly (each lane ends up owning one slot).
//  4. force pass: per triplet the vectors v_j = -dE_i/dr_ij, v_k = -dE_i/dr_ik are added to
//     per-neighbour shared-memory accumulators; F_i = sum_j v_j, F_j -= v_j (Newton's third law,
//     nnp.cpp:491,509-516) and the virial W += r_ij (x) v_j are then formed once per neighbour.
#include <cuda_runtime.h>
#include <cstdint>
#include "dev_math.cuh"
#include "kernels.hpp"

namespace ann {

enum { PASS_SYMM = 0, PASS_FORCE = 1, PASS_JVP = 2 };
constexpr int BP_WARPS = 4;
constexpr int GEN_CHUNK = 16;

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
template <typename real>
__device__ __forceinline__ real warp_sum(real v) {
#pragma unroll
    for (int off = 16; off >= 1; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    return v;
}

// ---------------------------------------------------------------- triplet enumeration
struct TriIter {      // pairs j<k of [0,n) in row-major order, lane-strided by 32
    int r, c, len;
    __device__ __forceinline__ void init(int n, int t) { r = 0; len = n - 1; c = t; while (len > 0 && c >= len) { c -= len; ++r; --len; } }
    __device__ __forceinline__ void adv() { c += 32; while (len > 0 && c >= len) { c -= len; ++r; --len; } }
    __device__ __forceinline__ int j() const { return r; }
    __device__ __forceinline__ int k() const { return r + 1 + c; }
};
struct RectIter {     // pairs (q, c) of [0,nJ) x [0,nK), lane-strided by 32
    int q, c, nK;
    __device__ __forceinline__ void init(int nk, int t) { nK = nk; q = t / nk; c = t - q * nk; }
    __device__ __forceinline__ void adv() { c += 32; while (c >= nK) { c -= nK; ++q; } }
};

// ---------------------------------------------------------------- shared-memory layout of one warp
template <typename real, int NG>
struct WarpMem {
    real *ux, *uy, *uz, *d, *id, *fc, *fcg, *D, *Dp, *ax, *ay, *az, *drx, *dry, *drz, *dd, *dE;
    typename V4<real>::T* stage;
    int32_t *jj, *img, *stagej;
    uint64_t* bar;
    static __host__ __device__ size_t bytes(int cap, int imax) {
        size_t r = (size_t)(7 + 2 * NG + 3 + 4) * cap + (size_t)imax;
        size_t b = ((r * sizeof(real) + 31) / 32) * 32;
        b += (size_t)cap * sizeof(typename V4<real>::T);
        b += (size_t)3 * cap * sizeof(int32_t);
        b = ((b + 15) / 16) * 16 + 16;
        return ((b + 31) / 32) * 32;
    }
    __device__ void carve(unsigned char* base, int cap, int imax) {
        real* p = reinterpret_cast<real*>(base);
        ux = p; p += cap; uy = p; p += cap; uz = p; p += cap; d = p; p += cap; id = p; p += cap; fc = p; p += cap; fcg = p; p += cap;
        D = p; p += NG * cap; Dp = p; p += NG * cap; ax = p; p += cap; ay = p; p += cap; az = p; p += cap;
        drx = p; p += cap; dry = p; p += cap; drz = p; p += cap; dd = p; p += cap; dE = p; p += imax;
        size_t off = (size_t)(7 + 2 * NG + 3 + 4) * cap + (size_t)imax;
        off = ((off * sizeof(real) + 31) / 32) * 32;
        stage = reinterpret_cast<typename V4<real>::T*>(base + off);
        off += (size_t)cap * sizeof(typename V4<real>::T);
        jj = reinterpret_cast<int32_t*>(base + off); img = jj + cap; stagej = img + cap;
        off += (size_t)3 * cap * sizeof(int32_t);
        off = ((off + 15) / 16) * 16;
        bar = reinterpret_cast<uint64_t*>(base + off);
    }
};

// ---------------------------------------------------------------- the kernel
template <typename real, int NG, bool FAST, int PASS>
__global__ void __launch_bounds__(BP_WARPS * 32) k_bp(const __grid_constant__ DevPot pot, const BpArgs<real> a) {
    extern __shared__ __align__(128) unsigned char bsm[];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int cap = a.cap, imax = pot.imax, T = a.ntypes;
    const size_t wbytes = WarpMem<real, NG>::bytes(cap, imax);
    WarpMem<real, NG> w;
    w.carve(bsm + (size_t)wid * wbytes, cap, imax);
    if (lane == 0) mbar_init(w.bar, 1);
    __syncwarp();
    uint32_t phase = 0;
    const unsigned lt = (1u << lane) - 1u;
    constexpr int S = NG * 8;

    for (;;) {
        int i = 0;
        if (lane == 0) i = (int)atomicAdd(a.counter, 1u);
        i = __shfl_sync(0xffffffffu, i, 0);
        if (i >= a.natoms) break;
        const int I = a.type[i];
        if (I < 0 || I >= T) { if (lane == 0) atomicOr(a.status, (int)ST_BAD_TYPE); continue; }
        const DevType& TT = pot.t[I];
        const int nin = min(a.nn[i], cap);
        const size_t row = (size_t)i * cap;

        // ---- 1. stage the neighbour row (bulk async copy) -----------------------------------
        if (nin > 0) {
            if (lane == 0) {
                const uint32_t b1 = (uint32_t)(nin * sizeof(typename V4<real>::T));
                const uint32_t b2 = (uint32_t)(((nin + 3) / 4) * 16);
                fence_proxy_async();
                mbar_expect_tx(w.bar, b1 + b2);
                bulk_g2s(w.stage, reinterpret_cast<const typename V4<real>::T*>(a.nr) + row, b1, w.bar);
                bulk_g2s(w.stagej, a.nj + row, b2, w.bar);
            }
            bool done = false;
            for (int it = 0; it < (1 << 24) && !done; ++it) done = mbar_try_wait(w.bar, phase);
            if (!__all_sync(0xffffffffu, done)) {  // bounded wait gave up: report, drain (bounded), stop
                if (lane == 0) atomicOr(a.status, (int)ST_TIMEOUT);
                for (int it = 0; it < (1 << 24); ++it) if (mbar_try_wait(w.bar, phase)) break;
                return;
            }
            phase ^= 1u;
        }
        // ---- compaction to d < rc, per-type active ranges ---------------------------------------
        const real rc = (real)TT.rc;
        int tstart[MAXT], tcnt[MAXT];
        int pos = 0, base_in = 0;
        for (int t = 0; t < T; ++t) {
            const int cin = a.ntc[(size_t)i * T + t];
            tstart[t] = pos;
            for (int e0 = 0; e0 < cin; e0 += 32) {
                const int e = base_in + e0 + lane;
                bool keep = false;
                typename V4<real>::T r4;
                if (e0 + lane < cin && e < nin) { r4 = w.stage[e]; keep = r4.w < rc; }
                const unsigned msk = __ballot_sync(0xffffffffu, keep);
                if (keep) {
                    const int o = pos + __popc(msk & lt);
                    const real dd = r4.w, idd = real(1) / dd;
                    w.ux[o] = r4.x * idd; w.uy[o] = r4.y * idd; w.uz[o] = r4.z * idd;
                    w.d[o] = dd; w.id[o] = idd;
                    real f, g;
                    cutoff_fg<real>(TT.cut, rc, dd, f, g);
                    w.fc[o] = f; w.fcg[o] = g;
                    if (FAST) {
#pragma unroll
                        for (int q = 0; q < NG; ++q) {
                            const real ie2 = (real)TT.ietar2[q];
                            const real ex = M<real>::bexp(-dd * dd * ie2);
                            w.D[q * cap + o] = f * ex;
                            w.Dp[q * cap + o] = ex * (g - real(2) * dd * f * ie2);
                        }
                    }
                    const int j = w.stagej[e];
                    w.jj[o] = j;
                    if (PASS == PASS_FORCE) {
                        w.ax[o] = real(0); w.ay[o] = real(0); w.az[o] = real(0);
                        w.img[o] = a.newton_untranslated ? a.nimg[row + e] : 0;
                    }
                    if (PASS == PASS_JVP) {
                        const real lx = a.lam[3 * (size_t)i] - a.lam[3 * (size_t)j];
                        const real ly = a.lam[3 * (size_t)i + 1] - a.lam[3 * (size_t)j + 1];
                        const real lz = a.lam[3 * (size_t)i + 2] - a.lam[3 * (size_t)j + 2];
                        w.drx[o] = lx; w.dry[o] = ly; w.drz[o] = lz;
                        w.dd[o] = w.ux[o] * lx + w.uy[o] * ly + w.uz[o] * lz;
                    }
                }
                pos += __popc(msk);
            }
            tcnt[t] = pos - tstart[t];
            base_in += cin;
        }
        if (PASS == PASS_FORCE) {
            for (int m = lane; m < TT.nInput; m += 32) w.dE[m] = a.dEdG[(size_t)i * imax + m];
        }
        __syncwarp();

        real* Gout = (PASS == PASS_SYMM) ? a.G + (size_t)i * imax : (PASS == PASS_JVP) ? a.U + (size_t)i * imax : nullptr;

        // ---- 2. radial ----------------------------------------------------------------------------
        for (int J = 0; J < T; ++J) {
            const DevRadial& R = TT.R[J];
            if (R.n == 0) continue;
            const int e0 = tstart[J], e1 = e0 + tcnt[J];
            if (PASS == PASS_FORCE) {
                for (int e = e0 + lane; e < e1; e += 32) {
                    const real dd = w.d[e], f = w.fc[e], g = w.fcg[e];
                    real amp = real(0);
                    for (int m = 0; m < R.n; ++m) {
                        real val, der;
                        radial_vd<real>(R.name, a.prm.reta[R.pidx + m], a.prm.rs[R.pidx + m], dd, f, g, val, der);
                        amp -= w.dE[R.off + m] * der;
                    }
                    w.ax[e] += amp * w.ux[e]; w.ay[e] += amp * w.uy[e]; w.az[e] += amp * w.uz[e];
                }
            } else {
                for (int m0 = 0; m0 < R.n; m0 += 32) {
                    const int m = m0 + lane;
                    if (m < R.n) {
                        const real eta = a.prm.reta[R.pidx + m], rs = a.prm.rs[R.pidx + m];
                        real acc = real(0);
                        for (int e = e0; e < e1; ++e) {
                            real val, der;
                            radial_vd<real>(R.name, eta, rs, w.d[e], w.fc[e], w.fcg[e], val, der);
                            acc += (PASS == PASS_SYMM) ? val : der * w.dd[e];
                        }
                        Gout[R.off + m] = acc;
                    }
                }
            }
        }
        __syncwarp();

        // ---- 3. angular ---------------------------------------------------------------------------
        for (int J = 0; J < T; ++J) {
            for (int K = J; K < T; ++K) {
                const int blk = tri_index(J, K);
                const DevAngular& A = TT.A[blk];
                if (A.n == 0) continue;
                const int nJ = tcnt[J], nK = tcnt[K], aJ = tstart[J], aK = tstart[K];
                const int total = (J == K) ? nJ * (nJ - 1) / 2 : nJ * nK;
                if (FAST) {
                    // ------------------------------------------------ fast path (GAUSS, zeta=2^k)
                    real acc[S];
                    real cA[S], cB[S];
#pragma unroll
                    for (int s = 0; s < S; ++s) {
                        acc[s] = real(0);
                        if (PASS == PASS_FORCE) {
                            const int ref = a.prm.slot2ref[A.sidx + s];
                            const real dv = (ref >= 0) ? w.dE[A.off + ref] : real(0);
                            const int k = (s & 7) >> 1;
                            cA[s] = dv;
                            cB[s] = dv * real(1 << k) * ((s & 1) ? real(-0.5) : real(0.5));
                        }
                    }
                    TriIter ti; RectIter ri;
                    if (J == K) ti.init(nJ, lane); else ri.init(max(nK, 1), lane);
                    for (int t = lane; t < total; t += 32) {
                        int j, k;
                        if (J == K) { j = aJ + ti.j(); k = aJ + ti.k(); ti.adv(); }
                        else { j = aJ + ri.q; k = aK + ri.c; ri.adv(); }
                        const real ujx = w.ux[j], ujy = w.uy[j], ujz = w.uz[j];
                        const real ukx = w.ux[k], uky = w.uy[k], ukz = w.uz[k];
                        const real cs = ujx * ukx + ujy * uky + ujz * ukz;
                        const real cwp = fabs(real(0.5) + real(0.5) * cs), cwm = fabs(real(0.5) - real(0.5) * cs);
                        real pp[4], pm[4];
                        pp[0] = cwp; pp[1] = cwp * cwp; pp[2] = pp[1] * pp[1]; pp[3] = pp[2] * pp[2];
                        pm[0] = cwm; pm[1] = cwm * cwm; pm[2] = pm[1] * pm[1]; pm[3] = pm[2] * pm[2];
                        if (PASS == PASS_SYMM) {
#pragma unroll
                            for (int g = 0; g < NG; ++g) {
                                const real DD = w.D[g * cap + j] * w.D[g * cap + k];
#pragma unroll
                                for (int q = 0; q < 4; ++q) { acc[g * 8 + 2 * q] += pp[q] * DD; acc[g * 8 + 2 * q + 1] += pm[q] * DD; }
                            }
                        } else {
                            real qp[4], qm[4];   // cw^(zeta-1) for zeta = 1,2,4,8
                            qp[0] = real(1); qp[1] = cwp; qp[2] = cwp * pp[1]; qp[3] = qp[2] * pp[2];
                            qm[0] = real(1); qm[1] = cwm; qm[2] = cwm * pm[1]; qm[3] = qm[2] * pm[2];
                            if (PASS == PASS_FORCE) {
                                real phi = real(0), e0 = real(0), e1 = real(0);
#pragma unroll
                                for (int g = 0; g < NG; ++g) {
                                    real Ag = real(0), Bg = real(0);
#pragma unroll
                                    for (int q = 0; q < 4; ++q) {
                                        Ag += cA[g * 8 + 2 * q] * pp[q] + cA[g * 8 + 2 * q + 1] * pm[q];
                                        Bg += cB[g * 8 + 2 * q] * qp[q] + cB[g * 8 + 2 * q + 1] * qm[q];
                                    }
                                    const real Dj = w.D[g * cap + j], Dk = w.D[g * cap + k];
                                    phi -= Bg * Dj * Dk;
                                    e0 -= Ag * w.Dp[g * cap + j] * Dk;
                                    e1 -= Ag * Dj * w.Dp[g * cap + k];
                                }
                                const real idj = w.id[j], idk = w.id[k];
                                const real cj = -phi * cs * idj + e0, bj = phi * idj;
                                const real ck = -phi * cs * idk + e1, bk = phi * idk;
                                atomicAdd(&w.ax[j], cj * ujx + bj * ukx); atomicAdd(&w.ay[j], cj * ujy + bj * uky); atomicAdd(&w.az[j], cj * ujz + bj * ukz);
                                atomicAdd(&w.ax[k], ck * ukx + bk * ujx); atomicAdd(&w.ay[k], ck * uky + bk * ujy); atomicAdd(&w.az[k], ck * ukz + bk * ujz);
                            } else {  // PASS_JVP
                                const real idj = w.id[j], idk = w.id[k];
                                const real ddj = w.dd[j], ddk = w.dd[k];
                                const real dcos = (w.drx[j] * ukx + w.dry[j] * uky + w.drz[j] * ukz) * idj +
                                                  (w.drx[k] * ujx + w.dry[k] * ujy + w.drz[k] * ujz) * idk - cs * (ddj * idj + ddk * idk);
#pragma unroll
                                for (int g = 0; g < NG; ++g) {
                                    const real Dj = w.D[g * cap + j], Dk = w.D[g * cap + k];
                                    const real DD = Dj * Dk;
                                    const real dDD = w.Dp[g * cap + j] * Dk * ddj + Dj * w.Dp[g * cap + k] * ddk;
#pragma unroll
                                    for (int q = 0; q < 4; ++q) {
                                        const real z = real(1 << q);
                                        acc[g * 8 + 2 * q] += z * real(0.5) * qp[q] * DD * dcos + pp[q] * dDD;
                                        acc[g * 8 + 2 * q + 1] += -z * real(0.5) * qm[q] * DD * dcos + pm[q] * dDD;
                                    }
                                }
                            }
                        }
                    }
                    if (PASS != PASS_FORCE) {
                        const real v = warp_slot_reduce<real, S>(acc, lane);
                        constexpr int SH = (S == 8) ? 2 : (S == 16) ? 1 : 0;
                        if ((lane & ((1 << SH) - 1)) == 0) {
                            const int s = (lane >> SH) & (S - 1);
                            const int ref = a.prm.slot2ref[A.sidx + s];
                            if (ref >= 0) Gout[A.off + ref] = v;
                        }
                    }
                } else {
                    // ------------------------------------------------ generic path (any BasisA)
                    if (PASS == PASS_FORCE) {
                        TriIter ti; RectIter ri;
                        if (J == K) ti.init(nJ, lane); else ri.init(max(nK, 1), lane);
                        for (int t = lane; t < total; t += 32) {
                            int j, k;
                            if (J == K) { j = aJ + ti.j(); k = aJ + ti.k(); ti.adv(); }
                            else { j = aJ + ri.q; k = aK + ri.c; ri.adv(); }
                            const real ujx = w.ux[j], ujy = w.uy[j], ujz = w.uz[j];
                            const real ukx = w.ux[k], uky = w.uy[k], ukz = w.uz[k];
                            const real cs = ujx * ukx + ujy * uky + ujz * ukz;
                            const real dj = w.d[j], dk = w.d[k];
                            const real r2s = dj * dj + dk * dk;
                            const real fj = w.fc[j], fk = w.fc[k], gj = w.fcg[j], gk = w.fcg[k];
                            real phi = real(0), e0 = real(0), e1 = real(0);
                            for (int m = 0; m < A.n; ++m) {
                                const real eta = a.prm.aeta[A.pidx + m], zeta = a.prm.zeta[A.pidx + m];
                                const real lf = real(0.5) * a.prm.alam[A.pidx + m];
                                const real ie2 = real(1) / (eta * eta);
                                real h, dq;
                                angular_damp<real>(A.name, ie2, r2s, h, dq);
                                const real cw = fabs(real(0.5) + lf * cs);
                                const real ga = w.dE[A.off + m] * M<real>::pow(cw, zeta - real(1)) * h;
                                const real fa = cw * ga;
                                phi -= zeta * lf * ga;
                                e0 -= fa * (-dq * real(2) * dj * fj + gj);
                                e1 -= fa * (-dq * real(2) * dk * fk + gk);
                            }
                            phi *= fj * fk; e0 *= fk; e1 *= fj;
                            const real idj = w.id[j], idk = w.id[k];
                            const real cj = -phi * cs * idj + e0, bj = phi * idj;
                            const real ck = -phi * cs * idk + e1, bk = phi * idk;
                            atomicAdd(&w.ax[j], cj * ujx + bj * ukx); atomicAdd(&w.ay[j], cj * ujy + bj * uky); atomicAdd(&w.az[j], cj * ujz + bj * ukz);
                            atomicAdd(&w.ax[k], ck * ukx + bk * ujx); atomicAdd(&w.ay[k], ck * uky + bk * ujy); atomicAdd(&w.az[k], ck * ukz + bk * ujz);
                        }
                    } else {
                        for (int m0 = 0; m0 < A.n; m0 += GEN_CHUNK) {
                            real acc[GEN_CHUNK];
#pragma unroll
                            for (int s = 0; s < GEN_CHUNK; ++s) acc[s] = real(0);
                            TriIter ti; RectIter ri;
                            if (J == K) ti.init(nJ, lane); else ri.init(max(nK, 1), lane);
                            for (int t = lane; t < total; t += 32) {
                                int j, k;
                                if (J == K) { j = aJ + ti.j(); k = aJ + ti.k(); ti.adv(); }
                                else { j = aJ + ri.q; k = aK + ri.c; ri.adv(); }
                                const real ujx = w.ux[j], ujy = w.uy[j], ujz = w.uz[j];
                                const real ukx = w.ux[k], uky = w.uy[k], ukz = w.uz[k];
                                const real cs = ujx * ukx + ujy * uky + ujz * ukz;
                                const real dj = w.d[j], dk = w.d[k];
                                const real r2s = dj * dj + dk * dk;
                                const real fj = w.fc[j], fk = w.fc[k], gj = w.fcg[j], gk = w.fcg[k];
                                real dcos = real(0), ddj = real(0), ddk = real(0);
                                if (PASS == PASS_JVP) {
                                    const real idj = w.id[j], idk = w.id[k];
                                    ddj = w.dd[j]; ddk = w.dd[k];
                                    dcos = (w.drx[j] * ukx + w.dry[j] * uky + w.drz[j] * ukz) * idj +
                                           (w.drx[k] * ujx + w.dry[k] * ujy + w.drz[k] * ujz) * idk - cs * (ddj * idj + ddk * idk);
                                }
#pragma unroll
                                for (int s = 0; s < GEN_CHUNK; ++s) {
                                    const int m = m0 + s;
                                    if (m < A.n) {
                                        const real eta = a.prm.aeta[A.pidx + m], zeta = a.prm.zeta[A.pidx + m];
                                        const real lf = real(0.5) * a.prm.alam[A.pidx + m];
                                        const real ie2 = real(1) / (eta * eta);
                                        real h, dq;
                                        angular_damp<real>(A.name, ie2, r2s, h, dq);
                                        const real cw = fabs(real(0.5) + lf * cs);
                                        if (PASS == PASS_SYMM) {
                                            acc[s] += M<real>::pow(cw, zeta) * h * fj * fk;
                                        } else {
                                            const real ga = M<real>::pow(cw, zeta - real(1)) * h;
                                            const real fa = cw * ga;
                                            const real fphi = zeta * lf * ga * fj * fk;
                                            const real fe0 = fa * (-dq * real(2) * dj * fj + gj) * fk;
                                            const real fe1 = fa * (-dq * real(2) * dk * fk + gk) * fj;
                                            acc[s] += fphi * dcos + fe0 * ddj + fe1 * ddk;
                                        }
                                    }
                                }
                            }
                            const real v = warp_slot_reduce<real, GEN_CHUNK>(acc, lane);
                            if ((lane & 1) == 0) {
                                const int m = m0 + ((lane >> 1) & (GEN_CHUNK - 1));
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
                const real rx = w.ux[e] * w.d[e], ry = w.uy[e] * w.d[e], rz = w.uz[e] * w.d[e];
                W9[0] += rx * vx; W9[1] += rx * vy; W9[2] += rx * vz;
                W9[3] += ry * vx; W9[4] += ry * vy; W9[5] += ry * vz;
                W9[6] += rz * vx; W9[7] += rz * vy; W9[8] += rz * vz;
                if (!a.newton_untranslated || w.img[e] == 0) {
                    const int j = w.jj[e];
                    atomicAdd(&a.F[3 * (size_t)j], -vx); atomicAdd(&a.F[3 * (size_t)j + 1], -vy); atomicAdd(&a.F[3 * (size_t)j + 2], -vz);
                }
            }
            fx = warp_sum(fx); fy = warp_sum(fy); fz = warp_sum(fz);
#pragma unroll
            for (int q = 0; q < 9; ++q) W9[q] = warp_sum(W9[q]);
            if (lane == 0) {
                atomicAdd(&a.F[3 * (size_t)i], fx); atomicAdd(&a.F[3 * (size_t)i + 1], fy); atomicAdd(&a.F[3 * (size_t)i + 2], fz);
#pragma unroll
                for (int q = 0; q < 9; ++q) a.W[9 * (size_t)i + q] = W9[q];
            }
        }
        // symmetry functions of angular blocks with no triplets stay as written by the zero fill
        __syncwarp();
    }
}

// G / U rows must start at zero (blocks without neighbours or triplets are not visited)
template <typename real>
__global__ void k_zero(real* p, size_t n) {
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x) p[k] = real(0);
}

template <typename real, int PASS>
static void launch_pass(const DevPot& pot, const BpArgs<real>& a, cudaStream_t st) {
    if (a.natoms <= 0) return;
    if (PASS != PASS_FORCE) {
        real* out = (PASS == PASS_SYMM) ? a.G : a.U;
        ++::ann::g_launch_counter, k_zero<real><<<1024, 256, 0, st>>>(out, (size_t)a.natoms * pot.imax);
    }
    cudaMemsetAsync(a.counter, 0, sizeof(uint32_t), st);
    int grid = (a.natoms + BP_WARPS - 1) / BP_WARPS;
    grid = std::min(grid, 152 * 16);
    auto go = [&](auto kern, size_t wb) {
        const size_t smem = wb * BP_WARPS;
        ++::ann::g_launch_counter, kern<<<grid, BP_WARPS * 32, smem, st>>>(pot, a);
    };
    if (pot.fast) {
        if (pot.fastNG == 1) go(k_bp<real, 1, true, PASS>, WarpMem<real, 1>::bytes(a.cap, pot.imax));
        else if (pot.fastNG == 2) go(k_bp<real, 2, true, PASS>, WarpMem<real, 2>::bytes(a.cap, pot.imax));
        else go(k_bp<real, 4, true, PASS>, WarpMem<real, 4>::bytes(a.cap, pot.imax));
    } else {
        go(k_bp<real, 1, false, PASS>, WarpMem<real, 1>::bytes(a.cap, pot.imax));
    }
}

template <typename real, int PASS>
static void configure_pass(int maxsmem) {
    set_max_dynamic_smem(k_bp<real, 1, true, PASS>, maxsmem);
    set_max_dynamic_smem(k_bp<real, 2, true, PASS>, maxsmem);
    set_max_dynamic_smem(k_bp<real, 4, true, PASS>, maxsmem);
    set_max_dynamic_smem(k_bp<real, 1, false, PASS>, maxsmem);
}
void configure_bp(int maxsmem) {
    configure_pass<float, PASS_SYMM>(maxsmem); configure_pass<float, PASS_FORCE>(maxsmem); configure_pass<float, PASS_JVP>(maxsmem);
    configure_pass<double, PASS_SYMM>(maxsmem); configure_pass<double, PASS_FORCE>(maxsmem); configure_pass<double, PASS_JVP>(maxsmem);
}
size_t bp_smem_bytes(const DevPot& pot, int cap, bool fp64) {
    const int ng = pot.fast ? pot.fastNG : 1;
    auto b = [&](auto tag) -> size_t {
        using real = decltype(tag);
        return ng == 1 ? WarpMem<real, 1>::bytes(cap, pot.imax) : ng == 2 ? WarpMem<real, 2>::bytes(cap, pot.imax) : WarpMem<real, 4>::bytes(cap, pot.imax);
    };
    return (fp64 ? b(double()) : b(float())) * BP_WARPS;
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
