// Rows of the symmetry-function / force kernels from a neighbour list that the caller owns: the
// full list of an MD engine with ghost atoms (LAMMPS `pair_style nn` with a full neighbour list
// and newton_pair on; the reference's pair style is used at examples/Ar/Ar_md_npt.in:22-23, its
// source is not part of the reference). It is also the shape of NNP::compute(nnp, struc, nlist)
// (src/nnp/nnp.cpp:601-665), where the caller builds the NeighborList.
//
// One warp per row (one centre atom). The row's entries are read from the caller's list, the pair
// vector r = x_centre - x_neighbour is formed from the given positions (ghost atoms carry their
// image shift already), entries with |r| >= rc are dropped (a list built with a skin holds them),
// and the rest are written type-sorted, as the list builder writes its rows: per neighbour type a
// contiguous range, ntc[row*T + t] entries long, in list order inside the range.
//
// The FP64 form forms r in FP64. The mixed form forms it in FP32 from positions split once per
// call into FP32 hi and lo parts (k_split_positions): r = (hi_i - hi_j) + (lo_i - lo_j). The hi
// difference and the final sum each round by at most half an FP32 ulp of |r|, and the lo parts
// carry the coordinates' own rounding to 24 bits, so for entries within 8 A every component lies
// within 5e-7 A of the exact difference at coordinates up to 2e7 A, and within one FP32 ulp of
// |r| at coordinates up to 1000 A (the FP64 difference rounded to FP32, the mixed rows' format, is
// within half an ulp). No FP64 arithmetic is done per entry: this part issues FP64 at a small
// fraction of its FP32 rate, and the per-entry FP64 difference, norm and test bounded the kernel.
#include <cuda_runtime.h>
#include <cstdint>
#include <cmath>
#include "kernels.hpp"

namespace ann {

constexpr int LR_WARPS = 8;

// the mixed form's hi / lo parts of every position, and the type bits beside the hi part
__global__ void __launch_bounds__(256) k_split_positions(int n, const double* x, const int32_t* type, float4* xh, float4* xl) {
    for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < n; a += gridDim.x * blockDim.x) {
        float h[3], l[3];
        for (int d = 0; d < 3; ++d) {
            const double v = x[3 * (size_t)a + d];
            h[d] = __double2float_rn(v);
            l[d] = __double2float_rn(v - (double)h[d]);
        }
        xh[a] = make_float4(h[0], h[1], h[2], __int_as_float(type[a]));
        xl[a] = make_float4(l[0], l[1], l[2], 0.0f);
    }
}

template <bool FP64>
__global__ void __launch_bounds__(LR_WARPS * 32) k_list_rows(ListArgs a) {
    const int lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
    const int T = a.ntypes, cap = a.cap;
    for (int r = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < a.nrows; r += (gridDim.x * blockDim.x) >> 5) {
        const int i = a.ilist ? a.ilist[r] : r;
        bool bad = (i < 0 || i >= a.nall);
        const int I = bad ? -1 : a.type[i];
        double xi[3] = {0.0, 0.0, 0.0};
        if (!bad) { xi[0] = a.x[3 * (size_t)i]; xi[1] = a.x[3 * (size_t)i + 1]; xi[2] = a.x[3 * (size_t)i + 2]; }
        float4 hi = make_float4(0.f, 0.f, 0.f, 0.f), lo = hi;
        if (!FP64 && !bad) { hi = a.xh[i]; lo = a.xl[i]; }
        if (lane == 0) {
            a.rtype[r] = I;   // an out-of-range type is reported by the symmetry-function kernel
            if (bad) atomicOr(a.status, (int)ST_BAD_INDEX);
            else if (!(isfinite(xi[0]) && isfinite(xi[1]) && isfinite(xi[2]))) atomicOr(a.status, (int)ST_NONFINITE);
        }
        const int64_t b0 = a.noff[r];
        const int cin = bad ? 0 : (int)(a.noff[r + 1] - b0);
        const size_t row = (size_t)r * cap;
        int base = 0;   // entries kept so far (before the capacity clamp)
        for (int t = 0; t < T; ++t) {
            int ct = 0;
            for (int e0 = 0; e0 < cin; e0 += 32) {
                const int e = e0 + lane;
                bool keep = false;
                int j = -1;
                double rx = 0.0, ry = 0.0, rz = 0.0, d2 = 0.0;
                float fx = 0.f, fy = 0.f, fz = 0.f, fd2 = 0.f;
                if (e < cin) {
                    j = a.neigh[b0 + e];
                    if (j < 0 || j >= a.nall) {
                        if (t == 0) atomicOr(a.status, (int)ST_BAD_INDEX);
                    } else {
                        float4 hj;
                        if (!FP64) hj = a.xh[j];
                        const int tj = FP64 ? a.type[j] : __float_as_int(hj.w);
                        if (t == 0 && (tj < 0 || tj >= T)) atomicOr(a.status, (int)ST_BAD_TYPE);
                        if (tj == t || t == 0) {   // the first pass also checks every neighbour's position
                            if (FP64) {
                                rx = xi[0] - a.x[3 * (size_t)j];
                                ry = xi[1] - a.x[3 * (size_t)j + 1];
                                rz = xi[2] - a.x[3 * (size_t)j + 2];
                                d2 = rx * rx + ry * ry + rz * rz;
                                if (t == 0 && !isfinite(d2)) atomicOr(a.status, (int)ST_NONFINITE);
                                keep = tj == t && d2 < a.rc2 && d2 > 0.0;
                            } else {
                                const float4 lj = a.xl[j];
                                fx = (hi.x - hj.x) + (lo.x - lj.x);
                                fy = (hi.y - hj.y) + (lo.y - lj.y);
                                fz = (hi.z - hj.z) + (lo.z - lj.z);
                                fd2 = fx * fx + fy * fy + fz * fz;
                                if (t == 0 && !isfinite(fd2)) atomicOr(a.status, (int)ST_NONFINITE);
                                keep = tj == t && fd2 < a.rc2f && fd2 > 0.0f;
                            }
                        }
                    }
                }
                const unsigned msk = __ballot_sync(0xffffffffu, keep);
                const int o = base + ct + __popc(msk & lt);
                if (keep && o < cap) {
                    a.nj[row + o] = j;
                    if (FP64) reinterpret_cast<Vec4d*>(a.nr)[row + o] = Vec4d{rx, ry, rz, sqrt(d2)};
                    else reinterpret_cast<Vec4f*>(a.nr)[row + o] = Vec4f{fx, fy, fz, sqrtf(fd2)};
                }
                ct += __popc(msk);
            }
            // the stored range stops at the capacity; an overflowing row is recomputed with a
            // larger capacity, so the clamped rows are never used for results
            if (lane == 0) a.ntc[(size_t)r * T + t] = min(base + ct, cap) - min(base, cap);
            base += ct;
        }
        if (lane == 0) {
            a.nn[r] = min(base, cap);
            if (base > cap) { atomicOr(a.status, (int)ST_NBR_OVERFLOW); atomicMax(a.status + 1, base); }
            if (base > a.hint) atomicMax(a.status + 2, base);
        }
    }
}

void launch_list_rows(const ListArgs& a, bool fp64, cudaStream_t st) {
    if (a.nrows <= 0) return;
    if (!fp64 && a.nall > 0) {
        const int g = std::min((a.nall + 255) / 256, std::max(1, (int)a.nsm) * 8);
        ++::ann::g_launch_counter, k_split_positions<<<g, 256, 0, st>>>(a.nall, a.x, a.type, a.xh, a.xl);
    }
    const int threads = LR_WARPS * 32;
    int grid = (a.nrows + LR_WARPS - 1) / LR_WARPS;
    grid = std::min(grid, std::max(1, (int)a.nsm) * 8);
    if (fp64) ++::ann::g_launch_counter, k_list_rows<true><<<grid, threads, 0, st>>>(a);
    else ++::ann::g_launch_counter, k_list_rows<false><<<grid, threads, 0, st>>>(a);
}

template <typename real>
__global__ void k_to_double(size_t n, const real* in, double* out) {
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x) out[k] = (double)in[k];
}
template <typename real>
void launch_to_double(size_t n, const real* in, double* out, int nsm, cudaStream_t st) {
    if (n == 0) return;
    const int grid = (int)std::min<size_t>((n + 255) / 256, (size_t)std::max(1, nsm) * 16);
    ++::ann::g_launch_counter, k_to_double<real><<<grid, 256, 0, st>>>(n, in, out);
}
template void launch_to_double<float>(size_t, const float*, double*, int, cudaStream_t);
template void launch_to_double<double>(size_t, const double*, double*, int, cudaStream_t);

}  // namespace ann
