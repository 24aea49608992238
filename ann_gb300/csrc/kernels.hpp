// Kernel argument blocks and host-side launch wrappers of libann_gpu.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include "plan.hpp"

namespace ann {

// kernels launched by this thread (instrumentation; graph captures count their kernel nodes)
extern thread_local int64_t g_launch_counter;

struct StrucGeo {          // per structure (FP64), filled on the device by k_struc_setup
    double R[9];           // lattice matrix, column-major (R[3*c + r])
    double Ri[9];          // inverse, column-major
    int32_t nb[3];         // bins along each lattice direction
    int32_t sten[3];       // stencil half-width in bins
    int32_t bin0;          // first global bin of the structure
    int32_t atom0, natoms;
    int32_t pad;           // 1: singular or non-finite cell (no search)
    int32_t ortho;         // 1: lattice vectors along the axes (R diagonal): stencil rows are pruned
    float labs[3];         // |R_dd| of an orthogonal cell (A)
    float Rf[9], Rif[9];   // FP32 copies of R and R^-1 (the FP32 candidate test and row pruning)
};

// ---- neighbour list (neighbor.cu) ----------------------------------------------------------
struct NbrArgs {
    int32_t nstruc, natoms, ntypes, cap;
    double rc;                       // list cutoff
    const int32_t* off;              // [S+1]
    const double* cell;              // [9S]
    const double* pos;               // [3N] FP64 positions
    const int32_t* type;             // [N]
    const int32_t* sid;              // [N] structure of each atom
    StrucGeo* geo;                   // [S]
    float4* pos4;                    // [N] FP32 positions + type bits
    int32_t* abin;                   // [N] global bin
    int32_t* abc;                    // [N] packed bin coordinates
    int32_t* am;                     // [N] packed wrap shift m (s = frac + m)
    int32_t* aslot;                  // [N] slot inside the bin
    int32_t* bcount;                 // [nbins_cap+1]
    int32_t* bstart;                 // [nbins_cap+1]
    int32_t* bidx;                   // [N] atoms in bin order
    int32_t* bm;                     // [N] packed m in bin order
    float4* bpos4;                   // [N] positions in bin order
    double* bposd;                   // [3N] FP64 positions in bin order
    int32_t nbins_cap;
    int32_t* nn;                     // [N] entries per atom
    int32_t* ntc;                    // [N*T] entries per atom and neighbour type (type-sorted rows)
    int32_t* nj;                     // [N*cap]
    int32_t* nimg;                   // [N*cap] packed image n
    void* nr;                        // [N*cap] real4 (rx, ry, rz, d)
    int32_t* scan_tmp;               // scratch for the bin scan
    uint32_t* counter;               // [1] work counter
    int32_t* status;                 // [8]
    int32_t grid_per_sm;             // host side: blocks per SM of the search grid (0: 16)
    int32_t nsm;                     // host side: streaming multiprocessors of the device
    int32_t max_nat;                 // host side: atoms of the batch's largest structure
};
// the batch's structures are binned one block each in shared memory (else by the global chain:
// atom bins, scan, scatter, sort)
bool nbr_local_binning(int max_nat);
// shared memory of a neighbour-search block for row capacity cap
size_t nbr_smem_bytes(int cap, bool fp64);
void launch_neighbors(const NbrArgs& a, bool fp64, cudaStream_t st);
// recompute nr from positions and stored images (Verlet-list refresh between rebuilds)
void launch_refresh_geometry(const NbrArgs& a, bool fp64, cudaStream_t st);

// ---- symmetry functions / forces / tangents (bp.cu) ---------------------------------------
template <typename real>
struct BpArgs {
    int32_t natoms, ntypes, cap, newton_untranslated;
    const int32_t* type;
    const int32_t* nn;
    const int32_t* ntc;
    const int32_t* nj;
    const int32_t* nimg;
    const void* nr;                  // real4 rows
    real* G;                         // [N*imax] symmetry functions (symm pass)
    const real* dEdG;                // [N*imax] (force pass)
    real* F;                         // [3N] force accumulator (force pass)
    real* W;                         // [9N] per-atom virial (force pass)
    const real* lam;                 // [3N] tangent field (jvp pass)
    real* U;                         // [N*imax] tangent of G (jvp pass)
    const int32_t* self;             // [N] force index of each row's centre atom (NULL: the row index)
    DevParams<real> prm;
    uint32_t* counter;
    int32_t* status;
    int32_t grid_per_sm;             // host side: cap on resident blocks per SM (0: as many as fit)
    int32_t nsm;                     // host side: streaming multiprocessors of the device
    int32_t wait_polls;              // k > 0: a neighbour-row wait gives up after k - 1 non-blocking
                                     // polls (testing the timeout path); 0: the built-in bound
    int32_t out_zeroed;              // host side: the caller cleared the G / U rows already
};
// clear n reals on stream st (the G / U rows, which the passes do not write for blocks without
// neighbours or triplets)
template <typename real> void launch_zero_rows(real* p, size_t n, cudaStream_t st);
template <typename real> void launch_symm(const DevPot& pot, const BpArgs<real>& a, cudaStream_t st);
template <typename real> void launch_force(const DevPot& pot, const BpArgs<real>& a, cudaStream_t st);
template <typename real> void launch_jvp(const DevPot& pot, const BpArgs<real>& a, cudaStream_t st);

// ---- rows from a caller's neighbour list (extlist.cu) ----------------------------------------
struct ListArgs {
    int32_t nrows, nall, ntypes, cap;
    double rc2;                      // square of the potential's cutoff: entries at or beyond it are dropped
    int32_t hint;                    // largest row seen so far: longer rows record their length
    const int32_t* ilist;            // [nrows] centre atom of each row (NULL: row index)
    const int64_t* noff;             // [nrows+1] first entry of each row in neigh
    const int32_t* neigh;            // [noff[nrows]] neighbour atoms, indices into [0, nall)
    const double* x;                 // [3*nall] positions of local and ghost atoms
    const int32_t* type;             // [nall]
    float4* xh;                      // mixed form: [nall] FP32 hi parts of the positions + type bits
    float4* xl;                      // mixed form: [nall] FP32 lo parts (x - hi)
    float rc2f;                      // rc2 in FP32 (mixed form)
    int32_t* rtype;                  // [nrows] centre type of each row
    int32_t* nn;                     // [nrows]
    int32_t* ntc;                    // [nrows*T]
    int32_t* nj;                     // [nrows*cap]
    void* nr;                        // [nrows*cap] real4 (rx, ry, rz, d), r = x_centre - x_neighbour
    int32_t* status;                 // [8]: [1] longest row on overflow, [2] longest row above hint
    int32_t nsm;                     // host side: streaming multiprocessors of the device
};
void launch_list_rows(const ListArgs& a, bool fp64, cudaStream_t st);
template <typename real> void launch_to_double(size_t n, const real* in, double* out, int nsm, cudaStream_t st);

// ---- optimiser steps (optim.cu) ---------------------------------------------------------------
// algorithms with the values of opt::algo::Name (src/opt/algo.hpp:31-49)
enum OptAlgo { OPT_SGD = 1, OPT_SDM = 2, OPT_NAG = 3, OPT_ADAGRAD = 4, OPT_ADADELTA = 5, OPT_RMSPROP = 6, OPT_ADAM = 7, OPT_ADAMW = 8,
               OPT_ADAB = 9, OPT_YOGI = 10, OPT_NOGI = 11, OPT_NADAM = 12, OPT_AMSGRAD = 13, OPT_BFGS = 14, OPT_RPROP = 15, OPT_CG = 16 };
struct OptArgs {
    int64_t n;
    int algo, reg, inc;              // inc (RPROP): the loss rose since the previous step
    const double* g;                 // gradient, times scale
    double scale;
    double* p;                       // FP64 parameters
    double* s0; double* s1; double* s2;   // per-parameter state (s1 / s2 NULL where unused)
    double* gold;                    // previous gradient (RPROP, CG; else NULL)
    double* beta;                    // CG: device scalar from the reduction
    double gamma, eta, eps, w, b1, b2, b1ii, b2ii;
    double reg_eta;                  // weight-decay strength
    const int32_t* map;              // parameter map (bias / weight kind)
};
void launch_opt(const OptArgs& o, double* part, cudaStream_t st);

// ---- input statistics of a training set (stats.cu) -------------------------------------------
int stats_chunks_per_type(int natoms);
template <typename real>
void launch_input_stats(int natoms, int ntypes, int imax, const real* G, const int32_t* tstart, const int32_t* tlist, double* part,
                        int32_t* pcount, double* acc, double* accn, cudaStream_t st);

// ---- networks (mlp.cu) -----------------------------------------------------------------------
template <typename real>
struct MlpArgs {
    int32_t natoms, ntypes, imax;
    const int32_t* tstart;           // [T+1] start of each type in tlist
    const int32_t* tlist;            // [N] atoms grouped by type
    const real* G;                   // [N*imax]
    real* dEdG;                      // [N*imax]
    double* Eatom;                   // [N] network output + vacuum energy
    // training (double backward)
    const real* U;                   // [N*imax] tangent of G
    const double* ce;                // [N] energy-loss weight per atom
    double ct;                       // tangent-loss weight
    double* grad;                    // [P] parameter gradient accumulator (FP64 in both precisions)
    const int32_t* poff;             // [T] parameter offset of each type
    double* gpart;                   // [blocks * pstride] per-block sums of the training pass (see
    int32_t pstride;                 //   mlp_train_part_bytes), added into grad in block order
    DevParams<real> prm;
};
template <typename real> void launch_mlp_forward_backward(const DevPot& pot, const MlpArgs<real>& a, cudaStream_t st);
template <typename real> void launch_mlp_train_grad(const DevPot& pot, const MlpArgs<real>& a, cudaStream_t st);
// bytes of the training pass's per-block gradient sums for natoms atoms in tiles of `tile` atoms
// (MlpArgs::gpart) and its row stride (the largest per-type parameter count)
size_t mlp_train_part_bytes(const DevPot& pot, int natoms, int tile, int* pstride);
int mlp_train_tile();   // atoms per block of the SIMT training pass
// grad[poff[t] + k] += the per-tile sums of type t's tiles (tiles of `tile` atoms), in tile order
void launch_grad_blocks(const DevPot& pot, const int32_t* tstart, const int32_t* poff, const double* gpart, int pstride, double* grad,
                        int tile, cudaStream_t st);

// ---- small kernels (misc.cu) ---------------------------------------------------------------
void launch_type_lists(int natoms, int ntypes, const int32_t* type, int32_t* tcount, int32_t* tstart, int32_t* tlist,
                       int32_t* status, cudaStream_t st);
// chunk table of the per-structure reductions (built on the host with the batch)
constexpr int RED_CHUNK = 256;
struct RedTable {
    int32_t nchunks;
    const int32_t* chunk;            // [nchunks][3]: structure, first atom, end atom
    const int32_t* schunk;           // [S+1] first chunk of each structure
    double* partial;                 // [nchunks][10]
    int32_t* arrive = nullptr;       // [S] chunks of each structure done (zero between launches), or
                                     // nullptr: a second kernel adds the partials per structure
};
template <typename real>
void launch_reduce_structures(int nstruc, const RedTable& t, const double* Eatom, const real* W, const real* F,
                              double* Es, double* Ws, double* Fout, cudaStream_t st);
void launch_fill_sid(int nstruc, const int32_t* off, int32_t* sid, cudaStream_t st);
void launch_exclusive_scan(const int32_t* in, int32_t* out, int n, int32_t* tmp, cudaStream_t st);
size_t scan_tmp_ints(int n);

// raise the dynamic shared-memory limit of a kernel to what the device allows beside its static
// shared memory; returns the granted dynamic limit (0 on failure)
template <typename K>
inline int set_max_dynamic_smem(K kernel, int maxsmem) {
    cudaFuncAttributes fa{};
    if (cudaFuncGetAttributes(&fa, kernel) != cudaSuccess) { cudaGetLastError(); return 0; }
    const int dyn = maxsmem - (int)fa.sharedSizeBytes;
    if (cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn) != cudaSuccess) { cudaGetLastError(); return 0; }
    return dyn;
}
// ask for the largest shared-memory carveout of the SM for a kernel (a launch preference of this
// process: L1 takes what shared memory leaves)
template <typename K>
inline void prefer_max_shared(K kernel) {
    if (cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout, (int)cudaSharedmemCarveoutMaxShared) != cudaSuccess)
        cudaGetLastError();
}
// raise the dynamic shared-memory limit of every kernel once (outside any graph capture)
void configure_bp(int maxsmem);
void configure_mlp(int maxsmem);
void configure_nbr(int maxsmem);
size_t bp_smem_bytes(const DevPot& pot, int cap, bool fp64);
size_t mlp_smem_bytes(const DevPot& pot, bool fp64, bool train);

}  // namespace ann
