// Small device kernels: exclusive scan, per-type atom lists, and the per-structure segmented
// reductions (K5) that turn per-atom energies / virials / force accumulators into the FP64
// per-structure results (the reference sums NNP energies per structure, nnp.cpp:436-447, and
// MPI_Reduce-s them across ranks; here fixed-size chunks of each structure are summed in a
// fixed order and the chunk partials added in chunk order, so the result is deterministic).
#include <cuda_runtime.h>
#include <cstdint>
#include "kernels.hpp"

namespace ann {

thread_local int64_t g_launch_counter = 0;

// ---------------------------------------------------------------- exclusive scan (3 phases)
constexpr int SCAN_T = 1024, SCAN_PER = 4, SCAN_BLK = SCAN_T * SCAN_PER;

__global__ void k_scan_blocks(const int32_t* in, int32_t* out, int n, int32_t* bsum) {
    __shared__ int32_t s[SCAN_T];
    const int base = blockIdx.x * SCAN_BLK + threadIdx.x * SCAN_PER;
    int32_t v[SCAN_PER];
    int32_t tot = 0;
#pragma unroll
    for (int k = 0; k < SCAN_PER; ++k) { v[k] = (base + k < n) ? in[base + k] : 0; tot += v[k]; }
    s[threadIdx.x] = tot;
    __syncthreads();
    for (int off = 1; off < SCAN_T; off <<= 1) {
        const int32_t t = (threadIdx.x >= off) ? s[threadIdx.x - off] : 0;
        __syncthreads();
        s[threadIdx.x] += t;
        __syncthreads();
    }
    int32_t run = s[threadIdx.x] - tot;
#pragma unroll
    for (int k = 0; k < SCAN_PER; ++k) { if (base + k < n) out[base + k] = run; run += v[k]; }
    if (threadIdx.x == SCAN_T - 1) bsum[blockIdx.x] = s[SCAN_T - 1];
}
__global__ void k_scan_sums(int32_t* bsum, int nb) {  // single block, serial over chunks
    __shared__ int32_t s[SCAN_T];
    int32_t carry = 0;
    for (int c0 = 0; c0 < nb; c0 += SCAN_T) {
        const int i = c0 + threadIdx.x;
        const int32_t v = (i < nb) ? bsum[i] : 0;
        s[threadIdx.x] = v;
        __syncthreads();
        for (int off = 1; off < SCAN_T; off <<= 1) {
            const int32_t t = (threadIdx.x >= off) ? s[threadIdx.x - off] : 0;
            __syncthreads();
            s[threadIdx.x] += t;
            __syncthreads();
        }
        if (i < nb) bsum[i] = carry + s[threadIdx.x] - v;
        const int32_t last = s[SCAN_T - 1];
        __syncthreads();
        carry += last;
    }
}
__global__ void k_scan_add(int32_t* out, int n, const int32_t* bsum) {
    const int i = blockIdx.x * SCAN_BLK + threadIdx.x;
    const int32_t add = bsum[blockIdx.x];
    for (int k = 0; k < SCAN_PER; ++k) {
        const int j = i + k * SCAN_T;
        if (j < n) out[j] += add;
    }
}
size_t scan_tmp_ints(int n) { return (size_t)(n + SCAN_BLK - 1) / SCAN_BLK + 1; }
void launch_exclusive_scan(const int32_t* in, int32_t* out, int n, int32_t* tmp, cudaStream_t st) {
    if (n <= 0) return;
    const int nb = (n + SCAN_BLK - 1) / SCAN_BLK;
    ++::ann::g_launch_counter, k_scan_blocks<<<nb, SCAN_T, 0, st>>>(in, out, n, tmp);
    ++::ann::g_launch_counter, k_scan_sums<<<1, SCAN_T, 0, st>>>(tmp, nb);
    ++::ann::g_launch_counter, k_scan_add<<<nb, SCAN_T, 0, st>>>(out, n, tmp);
}

// ---------------------------------------------------------------- structure of every atom
__global__ void k_fill_sid(const int32_t* off, int32_t* sid) {
    const int s = blockIdx.x;
    for (int i = off[s] + threadIdx.x; i < off[s + 1]; i += blockDim.x) sid[i] = s;
}
void launch_fill_sid(int nstruc, const int32_t* off, int32_t* sid, cudaStream_t st) {
    if (nstruc > 0) ++::ann::g_launch_counter, k_fill_sid<<<nstruc, 128, 0, st>>>(off, sid);
}

// ---------------------------------------------------------------- per-type atom lists
// slots within each type: lanes of a warp with the same type are counted together
// (match + popc), the block's counts go to global memory with one atomic per type
__global__ void k_type_count(int n, int ntypes, const int32_t* type, int32_t* tcount, int32_t* slot, int32_t* status) {
    __shared__ int32_t hist[MAXT], base[MAXT];
    if (threadIdx.x < MAXT) hist[threadIdx.x] = 0;
    __syncthreads();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    int t = (i < n) ? type[i] : -1;
    if (i < n && (t < 0 || t >= ntypes)) { atomicOr(status, (int)ST_BAD_TYPE); t = -1; }
    const unsigned peers = __match_any_sync(0xffffffffu, t);
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(peers) - 1;
    int first = 0;
    if (t >= 0 && lane == leader) first = atomicAdd(&hist[t], __popc(peers));
    first = __shfl_sync(0xffffffffu, first, leader);
    const int local = first + __popc(peers & ((1u << lane) - 1u));
    __syncthreads();
    if (threadIdx.x < ntypes) base[threadIdx.x] = hist[threadIdx.x] ? atomicAdd(&tcount[threadIdx.x], hist[threadIdx.x]) : 0;
    __syncthreads();
    if (i < n) slot[i] = (t >= 0) ? base[t] + local : -1;
}
__global__ void k_type_start(int ntypes, const int32_t* tcount, int32_t* tstart) {
    if (threadIdx.x == 0) { int32_t r = 0; for (int t = 0; t < ntypes; ++t) { tstart[t] = r; r += tcount[t]; } tstart[ntypes] = r; }
}
__global__ void k_type_scatter(int n, const int32_t* type, const int32_t* slot, const int32_t* tstart, int32_t* tlist) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || slot[i] < 0) return;
    tlist[tstart[type[i]] + slot[i]] = i;
}
// tlist doubles as the slot scratch (slot[i] is consumed before tlist is written in another kernel)
void launch_type_lists(int natoms, int ntypes, const int32_t* type, int32_t* tcount, int32_t* tstart, int32_t* tlist,
                       int32_t* status, cudaStream_t st) {
    cudaMemsetAsync(tcount, 0, sizeof(int32_t) * (ntypes + 1), st);
    if (natoms <= 0) { ++::ann::g_launch_counter, k_type_start<<<1, 32, 0, st>>>(ntypes, tcount, tstart); return; }
    int32_t* slot = tcount + ntypes + 1;  // caller sizes tcount as ntypes+1+natoms
    const int nb = (natoms + 255) / 256;
    ++::ann::g_launch_counter, k_type_count<<<nb, 256, 0, st>>>(natoms, ntypes, type, tcount, slot, status);
    ++::ann::g_launch_counter, k_type_start<<<1, 32, 0, st>>>(ntypes, tcount, tstart);
    ++::ann::g_launch_counter, k_type_scatter<<<nb, 256, 0, st>>>(natoms, type, slot, tstart, tlist);
}

// ---------------------------------------------------------------- per-structure reductions
// Structures are cut into chunks of at most RED_CHUNK atoms (table built on the host with the
// batch): one block per chunk sums E and W in a fixed order into a partial row, then one block
// per structure adds its chunks' partials in a fixed order. The result does not depend on the
// launch geometry, and a 262k-atom structure is spread over 1,024 blocks instead of one.
constexpr int RED_THREADS = 128;
template <typename real>
__global__ void k_reduce_chunks(const int32_t* chunk, const double* Eatom, const real* W, const real* F, double* partial,
                                double* Fout) {
    const int c = blockIdx.x;
    const int a0 = chunk[3 * c + 1], a1 = chunk[3 * c + 2];
    __shared__ double red[10][RED_THREADS];
    double acc[10];
#pragma unroll
    for (int k = 0; k < 10; ++k) acc[k] = 0.0;
    for (int i = a0 + threadIdx.x; i < a1; i += blockDim.x) {
        acc[0] += Eatom[i];
        if (W) {
#pragma unroll
            for (int k = 0; k < 9; ++k) acc[1 + k] += (double)W[9 * (size_t)i + k];
        }
        if (Fout) {
            Fout[3 * (size_t)i] = (double)F[3 * (size_t)i];
            Fout[3 * (size_t)i + 1] = (double)F[3 * (size_t)i + 1];
            Fout[3 * (size_t)i + 2] = (double)F[3 * (size_t)i + 2];
        }
    }
#pragma unroll
    for (int k = 0; k < 10; ++k) red[k][threadIdx.x] = acc[k];
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) {
#pragma unroll
            for (int k = 0; k < 10; ++k) red[k][threadIdx.x] += red[k][threadIdx.x + w];
        }
        __syncthreads();
    }
    if (threadIdx.x < 10) partial[10 * (size_t)c + threadIdx.x] = red[threadIdx.x][0];
}
// one block per structure: thread t adds chunks t, t + RED_THREADS, ... in order, then a fixed tree
__global__ void k_reduce_partials(int nstruc, const int32_t* schunk, const double* partial, bool with_w, double* Es, double* Ws) {
    const int s = blockIdx.x;
    __shared__ double red[10][RED_THREADS];
    double acc[10];
#pragma unroll
    for (int k = 0; k < 10; ++k) acc[k] = 0.0;
    for (int c = schunk[s] + threadIdx.x; c < schunk[s + 1]; c += blockDim.x) {
#pragma unroll
        for (int k = 0; k < 10; ++k) acc[k] += partial[10 * (size_t)c + k];
    }
#pragma unroll
    for (int k = 0; k < 10; ++k) red[k][threadIdx.x] = acc[k];
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) {
#pragma unroll
            for (int k = 0; k < 10; ++k) red[k][threadIdx.x] += red[k][threadIdx.x + w];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        Es[s] = red[0][0];
        if (with_w && Ws) for (int k = 0; k < 9; ++k) Ws[9 * (size_t)s + k] = red[1 + k][0];
    }
}
// The two steps in one launch, when every structure has at least one chunk: the chunk block that
// completes its structure's last chunk (per-structure arrival count) adds the structure's
// partials, with the same order and tree as k_reduce_partials, and resets the count.
template <typename real>
__global__ void k_reduce_fused(const int32_t* chunk, const int32_t* schunk, const double* Eatom, const real* W, const real* F,
                               double* partial, double* Fout, int32_t* arrive, bool with_w, double* Es, double* Ws) {
    const int c = blockIdx.x;
    const int s = chunk[3 * c], a0 = chunk[3 * c + 1], a1 = chunk[3 * c + 2];
    __shared__ double red[10][RED_THREADS];
    __shared__ int last;
    double acc[10];
#pragma unroll
    for (int k = 0; k < 10; ++k) acc[k] = 0.0;
    for (int i = a0 + threadIdx.x; i < a1; i += blockDim.x) {
        acc[0] += Eatom[i];
        if (W) {
#pragma unroll
            for (int k = 0; k < 9; ++k) acc[1 + k] += (double)W[9 * (size_t)i + k];
        }
        if (Fout) {
            Fout[3 * (size_t)i] = (double)F[3 * (size_t)i];
            Fout[3 * (size_t)i + 1] = (double)F[3 * (size_t)i + 1];
            Fout[3 * (size_t)i + 2] = (double)F[3 * (size_t)i + 2];
        }
    }
#pragma unroll
    for (int k = 0; k < 10; ++k) red[k][threadIdx.x] = acc[k];
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) {
#pragma unroll
            for (int k = 0; k < 10; ++k) red[k][threadIdx.x] += red[k][threadIdx.x + w];
        }
        __syncthreads();
    }
    if (threadIdx.x < 10) partial[10 * (size_t)c + threadIdx.x] = red[threadIdx.x][0];
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) last = (atomicAdd(&arrive[s], 1) == schunk[s + 1] - schunk[s] - 1);
    __syncthreads();
    if (!last) return;
    __threadfence();
#pragma unroll
    for (int k = 0; k < 10; ++k) acc[k] = 0.0;
    for (int cc = schunk[s] + threadIdx.x; cc < schunk[s + 1]; cc += blockDim.x) {
#pragma unroll
        for (int k = 0; k < 10; ++k) acc[k] += __ldcg(partial + 10 * (size_t)cc + k);   // other blocks' rows, from L2
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < 10; ++k) red[k][threadIdx.x] = acc[k];
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) {
#pragma unroll
            for (int k = 0; k < 10; ++k) red[k][threadIdx.x] += red[k][threadIdx.x + w];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        Es[s] = red[0][0];
        if (with_w && Ws) for (int k = 0; k < 9; ++k) Ws[9 * (size_t)s + k] = red[1 + k][0];
        arrive[s] = 0;
    }
}
template <typename real>
void launch_reduce_structures(int nstruc, const RedTable& t, const double* Eatom, const real* W, const real* F,
                              double* Es, double* Ws, double* Fout, cudaStream_t st) {
    if (nstruc <= 0) return;
    if (t.arrive && t.nchunks > 0) {
        ++::ann::g_launch_counter;
        k_reduce_fused<real><<<t.nchunks, RED_THREADS, 0, st>>>(t.chunk, t.schunk, Eatom, W, F, t.partial, Fout, t.arrive, W != nullptr, Es, Ws);
        return;
    }
    if (t.nchunks > 0) ++::ann::g_launch_counter, k_reduce_chunks<real><<<t.nchunks, RED_THREADS, 0, st>>>(t.chunk, Eatom, W, F, t.partial, Fout);
    ++::ann::g_launch_counter, k_reduce_partials<<<nstruc, RED_THREADS, 0, st>>>(nstruc, t.schunk, t.partial, W != nullptr, Es, Ws);
}
template void launch_reduce_structures<float>(int, const RedTable&, const double*, const float*, const float*, double*, double*, double*, cudaStream_t);
template void launch_reduce_structures<double>(int, const RedTable&, const double*, const double*, const double*, double*, double*, double*, cudaStream_t);

}  // namespace ann
