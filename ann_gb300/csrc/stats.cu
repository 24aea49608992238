// Input statistics of a training set on the device (the reference's set-up of the input
// pre-conditioning, nnptefr2.cpp:686-775): per type and input, the max, min, sum of 1/G, sum of
// G, sum of squared deviations from the mean and sum of G^2 over every atom of every batch
// accumulated. The host turns them into max, min, harmonic mean, mean, deviation and rms.
//
// A batch is cut, per type, into chunks of STAT_CHUNK atoms of the type list: one block per
// (chunk, type) forms the chunk's partials (its own two-pass mean / squared deviations), then one
// block per type merges the chunks into the accumulators in chunk order (Chan, Golub and LeVeque's
// pairwise update of the squared deviations). The order is fixed, so the result does not depend on
// the launch.
#include <cuda_runtime.h>
#include <cfloat>
#include <cstdint>
#include "kernels.hpp"

namespace ann {

constexpr int STAT_CHUNK = 256;
constexpr int STAT_THREADS = 128;

int stats_chunks_per_type(int natoms) { return (natoms + STAT_CHUNK - 1) / STAT_CHUNK; }

// part[((t * maxch + c) * 6 + q) * imax + k], q = max, min, sum 1/G, sum G, squared deviations, sum G^2
template <typename real>
__global__ void __launch_bounds__(STAT_THREADS) k_stats_chunks(const real* G, int imax, const int32_t* tstart, const int32_t* tlist,
                                                               int maxch, double* part, int32_t* pcount) {
    const int c = blockIdx.x, t = blockIdx.y;
    const int a0 = tstart[t] + c * STAT_CHUNK;
    const int a1 = min(a0 + STAT_CHUNK, tstart[t + 1]);
    const int n = max(0, a1 - a0);
    if (threadIdx.x == 0) pcount[t * maxch + c] = n;
    if (n == 0) return;
    double* p = part + (size_t)(t * maxch + c) * 6 * imax;
    for (int k = threadIdx.x; k < imax; k += blockDim.x) {
        double mx = -DBL_MAX, mn = DBL_MAX, si = 0.0, s = 0.0, sq = 0.0;
        for (int q = a0; q < a1; ++q) {
            const double g = (double)G[(size_t)tlist[q] * imax + k];
            if (g > mx) mx = g;
            if (g < mn) mn = g;
            si += 1.0 / g; s += g; sq += g * g;
        }
        const double mean = s / n;
        double m2 = 0.0;
        for (int q = a0; q < a1; ++q) {
            const double d = (double)G[(size_t)tlist[q] * imax + k] - mean;
            m2 += d * d;
        }
        p[k] = mx; p[imax + k] = mn; p[2 * imax + k] = si; p[3 * imax + k] = s; p[4 * imax + k] = m2; p[5 * imax + k] = sq;
    }
}

// acc[(t * 6 + q) * imax + k] as the partials; accn[t] atoms accumulated so far
__global__ void __launch_bounds__(STAT_THREADS) k_stats_merge(int imax, int maxch, const double* part, const int32_t* pcount,
                                                              double* acc, double* accn) {
    const int t = blockIdx.x;
    for (int k = threadIdx.x; k < imax; k += blockDim.x) {
        double* a = acc + (size_t)t * 6 * imax;
        double mx = a[k], mn = a[imax + k], si = a[2 * imax + k], s = a[3 * imax + k], m2 = a[4 * imax + k], sq = a[5 * imax + k];
        double nA = accn[t];
        for (int c = 0; c < maxch; ++c) {
            const double nB = (double)pcount[t * maxch + c];
            if (nB == 0.0) continue;
            const double* p = part + (size_t)(t * maxch + c) * 6 * imax;
            if (p[k] > mx) mx = p[k];
            if (p[imax + k] < mn) mn = p[imax + k];
            si += p[2 * imax + k];
            const double sB = p[3 * imax + k];
            if (nA > 0.0) {
                const double d = sB / nB - s / nA;
                m2 += p[4 * imax + k] + d * d * (nA * nB / (nA + nB));
            } else {
                m2 = p[4 * imax + k];
            }
            s += sB; sq += p[5 * imax + k]; nA += nB;
        }
        a[k] = mx; a[imax + k] = mn; a[2 * imax + k] = si; a[3 * imax + k] = s; a[4 * imax + k] = m2; a[5 * imax + k] = sq;
    }
    double n = accn[t];
    if (threadIdx.x == 0) for (int c = 0; c < maxch; ++c) n += (double)pcount[t * maxch + c];
    __syncthreads();   // every thread has read accn[t]
    if (threadIdx.x == 0) accn[t] = n;
}

template <typename real>
void launch_input_stats(int natoms, int ntypes, int imax, const real* G, const int32_t* tstart, const int32_t* tlist, double* part,
                        int32_t* pcount, double* acc, double* accn, cudaStream_t st) {
    const int maxch = stats_chunks_per_type(natoms);
    if (maxch == 0 || ntypes == 0) return;
    ++::ann::g_launch_counter, k_stats_chunks<real><<<dim3(maxch, ntypes), STAT_THREADS, 0, st>>>(G, imax, tstart, tlist, maxch, part, pcount);
    ++::ann::g_launch_counter, k_stats_merge<<<ntypes, STAT_THREADS, 0, st>>>(imax, maxch, part, pcount, acc, accn);
}
template void launch_input_stats<float>(int, int, int, const float*, const int32_t*, const int32_t*, double*, int32_t*, double*, double*,
                                        cudaStream_t);
template void launch_input_stats<double>(int, int, int, const double*, const int32_t*, const int32_t*, double*, int32_t*, double*,
                                         double*, cudaStream_t);

}  // namespace ann
