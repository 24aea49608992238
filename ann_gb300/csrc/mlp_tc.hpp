// Tensor-core (tcgen05) form of the per-element networks: host-built weight images and the
// per-type launch description shared by plan_tc.cpp (host) and mlp_tc.cu (device).
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <vector>
#include "plan.hpp"

namespace ann {

constexpr int TC_M = 128;          // atoms per tile (one TMEM lane each)
constexpr int TC_MAXH = 5;         // hidden layers
constexpr int TC_GROUPS = 4;       // most warps per TMEM lane quadrant (the epilogue's column split)
// shared memory after the A tiles: 2 mbarriers, the TMEM address, per-group energy partials
constexpr int TC_TAIL_BYTES = 32 + 4 * TC_GROUPS * TC_M;

// Operands live in shared memory in the canonical K-major no-swizzle layout of tcgen05:
// 8-row x 16-byte core matrices (128 B each); along K adjacent core matrices are 128 B apart
// (leading byte offset), along rows the 8-row groups are K/8 * 128 B apart (stride byte offset).
// The image of one type holds, for every hidden layer l, the B operand of the forward GEMM
// (W_l, N = nodes[l] x K = ni(l)) as BF16 hi and (split 3) lo parts, followed by FP32 vectors. The
// backward GEMM's operand W_l^T is the same bytes read as an MN-major operand.
struct TcType {
    int32_t nhidden;                 // hidden layers (the last layer is a dot product)
    int32_t nin, K0;                 // inputs and inputs padded to 16
    int32_t width[TC_MAXH];          // padded width of hidden layer l
    int32_t nodes[TC_MAXH];          // true width of hidden layer l
    uint32_t fwd_hi[TC_MAXH], fwd_lo[TC_MAXH];   // byte offsets of W_l's hi / lo parts in the image (lo = hi unless split 3)
    uint32_t bias[TC_MAXH];          // byte offset of the FP32 bias of hidden layer l (padded width)
    uint32_t wlast;                  // FP32 weights of the last layer (padded width of the last hidden layer)
    uint32_t inpw, inpb;             // FP32 input scaling (K0 entries)
    uint32_t blast;                  // FP32 bias of the last layer (one entry, padded to 16 B)
    uint32_t img_bytes;              // size of the image (multiple of 16)
    uint32_t img_off;                // offset of this type's image in the device buffer
    float outw, outb, c;
    double evac;
    int32_t neuron;
    int32_t wmax;                    // widest padded operand width (K0 or any hidden width)
    int32_t fwd_col[TC_MAXH];        // TMEM column of the forward accumulator of hidden layer l
    int32_t bwd_col;                 // TMEM column of the backward accumulators
    int32_t tmem_cols;               // allocated TMEM columns (power of two, <= 512)
    int32_t split;                   // 1: A and B single BF16; 2: A split hi+lo; 3: A and B split
};

// Warps per lane quadrant for a type's launch. A CTA is latency-bound on its chain of small GEMMs
// and epilogues; with 128 x G threads of up to 128 registers, 4 / G CTAs share an SM (as far as
// tensor memory allows, 512 / tmem_cols). More, narrower CTAs pay off only when each still gets
// a few tiles to amortise its prologue (weight image copy, TMEM allocation): the finest split
// whose CTAs get at least two tiles of est_atoms atoms, else G = 4 (one CTA per SM).
inline int tc_groups(const TcType& tt, long long est_atoms, int nsm) {
    const int allowed = 512 / (tt.tmem_cols > 32 ? tt.tmem_cols : 32);
    const long long tiles = (est_atoms + TC_M - 1) / TC_M;
    for (int per_sm = 4; per_sm >= 2; per_sm /= 2)
        if (per_sm <= allowed && tiles >= 2LL * nsm * per_sm) return 4 / per_sm;
    return 4;
}

struct TcPlan {
    bool ok = false;                 // every type fits the tensor-core kernel
    TcType t[MAXT];
    std::vector<uint8_t> image;      // all types' images, back to back (128-byte aligned)
    int smem_per_sm = 228 * 1024;    // shared memory of one SM (limits co-resident CTAs)
    size_t smem_bytes(int type) const;
};

// builds the images from the row-major FP64 weights of the plan (w[l][n*ni+m], b[l][n])
void build_tc_plan(const DevPot& pot, const std::vector<double>& w, const std::vector<double>& b,
                   const std::vector<double>& inpw, const std::vector<double>& inpb, int max_smem, int split_pref, TcPlan& out);

// Where every network parameter lives on the device, in the packing order of ann_get_params
// (per type: biases layer by layer, then weights layer by layer with the input index outer,
// nn.cpp:846-859): 8 ints per parameter, -1 where a destination does not apply.
enum ParamSlot { PM_KIND = 0, PM_I64, PM_IT, PM_F32, PM_FH, PM_FL, PM_BH, PM_BL, PM_N };
enum ParamKind { PK_BIAS = 0, PK_WEIGHT = 1 };
// weight decay of the optimiser step (Regularization, nnptefr2.hpp:173-181)
enum RegKind { REG_LASSO = 0, REG_RIDGE = 1, REG_HUBER = 2, REG_ASINH = 3, REG_NONE = 4 };
// PM_I64: index into the FP64/FP32 bias or row-major weight arrays; PM_IT: index into the
// transposed weights; PM_F32: byte offset of an FP32 copy in the tensor-core images (hidden bias,
// last-layer weight or bias); PM_FH/FL, PM_BH/BL: byte offsets of the BF16 hi/lo entries of the
// forward operand W (FL -1 unless the type's weights are split); PM_BH/BL are not used (-1): the
// backward GEMM reads W's image as W^T
void build_param_map(const DevPot& pot, const TcPlan& tc, std::vector<int32_t>& map);

struct TcArgs {
    int32_t natoms, imax, type;
    const int32_t* tstart;
    const int32_t* tlist;
    const float* G;                  // [N*imax] FP32 symmetry functions
    float* dEdG;                     // [N*imax]
    double* Eatom;                   // [N]
    const uint8_t* image;            // device copy of TcPlan::image
    int32_t* status;
    int32_t wait_polls;              // k > 0: image and MMA waits give up after k - 1 non-blocking
                                     // polls (testing the timeout path); 0: the built-in bound
};
// est_atoms: the expected atoms of the type (its count is known on the device only); groups:
// 1, 2 or 4 to force the split, 0 to choose it (tc_groups)
// nsm: streaming multiprocessors of the device (the persistent grid's size)
void launch_mlp_tc(const TcType& tt, const TcArgs& a, long long est_atoms, int groups, size_t smem, int nsm, cudaStream_t st);
void configure_mlp_tc(int maxsmem);

// ---- the training pass on the tensor cores (mlp_tc_train.cu) --------------------------------
// layout of a type: widths of the activation tiles H (inputs + a ones column) and of the delta
// tiles, TMEM columns of the forward accumulators, of the weight-gradient accumulators (per hidden
// layer and the output layer) and the shared-memory offsets
struct TcTrainLayout {
    int32_t WH, WZ;
    int32_t zc[TC_MAXH], zdc[TC_MAXH], gw[TC_MAXH];
    int32_t gwl, tmem_cols;
    uint32_t o_h, o_z, o_tail, smem;
};
// false: the type's networks do not fit the training kernel (the SIMT kernel takes them)
bool plan_tc_train(const TcType& tt, int max_smem, TcTrainLayout& ly);
struct TcTrainArgs {
    int32_t natoms, imax, ntypes;
    const int32_t* tstart;                    // [T+1] start of each type in tlist
    const int32_t* tlist;                     // [N] atoms grouped by type
    const float* G;                           // [N*imax]
    const float* U;                           // [N*imax] tangent of G
    const double* ce;                         // [N] energy-loss weight per atom
    float ct;                                 // tangent-loss weight
    const uint8_t* image;                     // device copy of TcPlan::image
    double* gpart;                            // [tiles of 128 atoms * pstride] per-tile gradient sums
    int32_t pstride;
    int32_t* status;
    int32_t wait_polls;
};
// one CTA per tile of 128 atoms (types one after the other); the per-tile sums go to gpart, to be
// added by launch_grad_blocks with tile = 128
void launch_mlp_train_tc(const TcPlan& tc, const TcTrainLayout* lay, const TcTrainArgs& a, cudaStream_t st);
void configure_mlp_train_tc(int maxsmem);

}  // namespace ann
