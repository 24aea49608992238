// Rows of the symmetry-function / force kernels from a neighbour list that the caller owns: the
// full list of an MD engine with ghost atoms (LAMMPS `pair_style nn` with a full neighbour list
// and newton_pair on; the reference's pair style is used at examples/Ar/Ar_md_npt.in:22-23, its
// source is not part of the reference). It is also the shape of NNP::compute(nnp, struc, nlist)
// (src/nnp/nnp.cpp:601-665), where the caller builds the NeighborList.
//
// One warp per row (one centre atom). The row's entries are read from the caller's list, the pair
// vector r = x_centre - x_neighbour is formed in FP64 from the given positions (ghost atoms carry
// their image shift already), entries with |r| >= rc are dropped (a list built with a skin holds
// them), and the rest are written type-sorted, as the list builder writes its rows: per neighbour
// type a contiguous range, ntc[row*T + t] entries long, in list order inside the range.
#include <cuda_runtime.h>
#include <cstdint>
#include <cmath>
#include "kernels.hpp"

namespace ann {

constexpr int LR_WARPS = 8;

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
                if (e < cin) {
                    j = a.neigh[b0 + e];
                    if (j < 0 || j >= a.nall) {
                        if (t == 0) atomicOr(a.status, (int)ST_BAD_INDEX);
                    } else {
                        const int tj = a.type[j];
                        if (t == 0 && (tj < 0 || tj >= T)) atomicOr(a.status, (int)ST_BAD_TYPE);
                        if (tj == t || t == 0) {   // the first pass also checks every neighbour's position
                            rx = xi[0] - a.x[3 * (size_t)j];
                            ry = xi[1] - a.x[3 * (size_t)j + 1];
                            rz = xi[2] - a.x[3 * (size_t)j + 2];
                            d2 = rx * rx + ry * ry + rz * rz;
                            if (t == 0 && !isfinite(d2)) atomicOr(a.status, (int)ST_NONFINITE);
                            keep = tj == t && d2 < a.rc2 && d2 > 0.0;
                        }
                    }
                }
                const unsigned msk = __ballot_sync(0xffffffffu, keep);
                const int o = base + ct + __popc(msk & lt);
                if (keep && o < cap) {
                    a.nj[row + o] = j;
                    if (FP64) {
                        reinterpret_cast<Vec4d*>(a.nr)[row + o] = Vec4d{rx, ry, rz, sqrt(d2)};
                    } else {
                        const float fx = (float)rx, fy = (float)ry, fz = (float)rz;
                        reinterpret_cast<Vec4f*>(a.nr)[row + o] = Vec4f{fx, fy, fz, sqrtf(fx * fx + fy * fy + fz * fz)};
                    }
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
