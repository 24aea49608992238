// K3 / K6a: per-element atomic networks over type-sorted atom tiles (SIMT form, FP32 or FP64).
//
// Reference: NN::ANN::fpbp / fpbp2 (src/ml/nn.cpp:1343-1409; input scaling ins = inpw*(inp+inpb),
// z_l = W_l a_{l-1} + b_l, a = f(c z) with a linear last layer nn.cpp:1314-1317, out =
// outb + outw*a_L), NN::DODZ::grad (nn.cpp:1801-1824: dE/dG = outw f'...W_0 diag(inpw)),
// NNH::energy (src/nnp/nnh.cpp:118-121: + the type's vacuum energy), NN::Cost::grad
// (nn.cpp:1712-1770) and the mixed second derivative of the force loss (the quantity
// NN::D2ODZDI assembles, nn.cpp:2012-2100) computed here as a forward-over-reverse product.
//
// A block owns TA atoms of one type; activations live in shared memory, weights are read
// through L1 (rows broadcast across the warp). Thread mapping: consecutive threads take
// consecutive atoms of the same neuron, so a weight row is one broadcast load.
#include <cuda_runtime.h>
#include <cstdint>
#include "dev_math.cuh"
#include "kernels.hpp"

namespace ann {

constexpr int TA = 32;        // atoms per block (energy/force network pass)
constexpr int TAT = 16;       // atoms per block (training pass, more state per atom)
constexpr int MLP_T = 128;    // threads per block
constexpr int MLP_TT = 256;   // threads per block of the training pass (two blocks per SM fit its shared memory)

// map block -> (type, first atom in the type list); returns false if the block is spare
template <int TAn>
__device__ __forceinline__ bool tile_of_block(int ntypes, const int32_t* tstart, int& type, int& a0, int& na) {
    int b = blockIdx.x;
    for (int t = 0; t < ntypes; ++t) {
        const int cnt = tstart[t + 1] - tstart[t];
        const int tiles = (cnt + TAn - 1) / TAn;
        if (b < tiles) { type = t; a0 = tstart[t] + b * TAn; na = min(TAn, cnt - b * TAn); return true; }
        b -= tiles;
    }
    return false;
}

// y[a][n] = b[n] + sum_m W[n][m] x[a][m]  for all atoms a of the tile (rows of length ld);
// bl == nullptr: no bias
template <typename real, int TAn = TA>
__device__ __forceinline__ void layer_fwd(const real* __restrict__ Wl, const real* __restrict__ bl, int no, int ni,
                                          const real* x, real* z, int ld) {
    for (int idx = threadIdx.x; idx < TAn * no; idx += MLP_T) {
        const int a = idx % TAn, n = idx / TAn;
        const real* wr = Wl + (size_t)n * ni;
        const real* xr = x + a * ld;
        real s = bl ? bl[n] : real(0);
        for (int m = 0; m < ni; ++m) s += wr[m] * xr[m];
        z[a * ld + n] = s;
    }
}
// y[a][m] = sum_n WT[m][n] x[a][n]   (WT = W^T, rows of length no)
template <typename real, int TAn = TA>
__device__ __forceinline__ void layer_bwd(const real* __restrict__ WTl, int no, int ni, const real* x, real* y, int ld) {
    for (int idx = threadIdx.x; idx < TAn * ni; idx += MLP_T) {
        const int a = idx % TAn, m = idx / TAn;
        const real* wr = WTl + (size_t)m * no;
        const real* xr = x + a * ld;
        real s = real(0);
        for (int n = 0; n < no; ++n) s += wr[n] * xr[n];
        y[a * ld + m] = s;
    }
}

// Register-tiled forms of the training pass, which carries a value and a tangent through every
// layer: each thread computes RT consecutive outputs of one atom for both, so one weight load
// feeds 2 FMAs and one activation load feeds RT of them.
constexpr int RT = 4;
// z[a][n] = b[n] + sum_m W[n][m] x[a][m] and zd[a][n] = sum_m W[n][m] xd[a][m]
template <typename real, int TAn>
__device__ __forceinline__ void layer_fwd2(const real* __restrict__ Wl, const real* __restrict__ bl, int no, int ni,
                                           const real* x, const real* xd, real* z, real* zd, int ld) {
    const int ng = (no + RT - 1) / RT;
    for (int idx = threadIdx.x; idx < TAn * ng; idx += blockDim.x) {
        const int a = idx % TAn, n0 = (idx / TAn) * RT;
        const real* xr = x + a * ld;
        const real* xdr = xd + a * ld;
        real s[RT], sd[RT];
#pragma unroll
        for (int k = 0; k < RT; ++k) { s[k] = (n0 + k < no) ? bl[n0 + k] : real(0); sd[k] = real(0); }
        const real* w0 = Wl + (size_t)n0 * ni;
        for (int m = 0; m < ni; ++m) {
            const real xv = xr[m], xdv = xdr[m];
#pragma unroll
            for (int k = 0; k < RT; ++k) {
                const real w = (n0 + k < no) ? w0[(size_t)k * ni + m] : real(0);
                s[k] += w * xv; sd[k] += w * xdv;
            }
        }
#pragma unroll
        for (int k = 0; k < RT; ++k)
            if (n0 + k < no) { z[a * ld + n0 + k] = s[k]; zd[a * ld + n0 + k] = sd[k]; }
    }
}
// y[a][m] = sum_n WT[m][n] x[a][n] and yd[a][m] = sum_n WT[m][n] xd[a][n]   (WT = W^T, rows of length no)
template <typename real, int TAn>
__device__ __forceinline__ void layer_bwd2(const real* __restrict__ WTl, int no, int ni, const real* x, const real* xd, real* y,
                                           real* yd, int ld) {
    const int mg = (ni + RT - 1) / RT;
    for (int idx = threadIdx.x; idx < TAn * mg; idx += blockDim.x) {
        const int a = idx % TAn, m0 = (idx / TAn) * RT;
        const real* xr = x + a * ld;
        const real* xdr = xd + a * ld;
        real s[RT], sd[RT];
#pragma unroll
        for (int k = 0; k < RT; ++k) { s[k] = real(0); sd[k] = real(0); }
        const real* w0 = WTl + (size_t)m0 * no;
        for (int n = 0; n < no; ++n) {
            const real xv = xr[n], xdv = xdr[n];
#pragma unroll
            for (int k = 0; k < RT; ++k) {
                const real w = (m0 + k < ni) ? w0[(size_t)k * no + n] : real(0);
                s[k] += w * xv; sd[k] += w * xdv;
            }
        }
#pragma unroll
        for (int k = 0; k < RT; ++k)
            if (m0 + k < ni) { y[a * ld + m0 + k] = s[k]; yd[a * ld + m0 + k] = sd[k]; }
    }
}

// ---------------------------------------------------------------- forward + dE/dG
template <typename real>
__global__ void __launch_bounds__(MLP_T) k_mlp_fb(const __grid_constant__ DevPot pot, const MlpArgs<real> A, int ld) {
    extern __shared__ __align__(16) unsigned char msm[];
    int type, a0, na;
    if (!tile_of_block<TA>(A.ntypes, A.tstart, type, a0, na)) return;
    const DevNet& net = pot.t[type].net;
    const int L = net.nlayer;
    real* bufA = reinterpret_cast<real*>(msm);
    real* bufB = bufA + TA * ld;
    real* dz = bufB + TA * ld;            // f'(z) of every layer: L * TA * ld
    __shared__ int32_t atoms[TA];
    if (threadIdx.x < TA) atoms[threadIdx.x] = (threadIdx.x < na) ? A.tlist[a0 + threadIdx.x] : -1;
    __syncthreads();
    const int nin = net.nin;
    const real* inpw = A.prm.inpw + net.inoff;
    const real* inpb = A.prm.inpb + net.inoff;
    for (int idx = threadIdx.x; idx < TA * nin; idx += MLP_T) {
        const int a = idx / nin, m = idx % nin;
        const int at = atoms[a];
        bufA[a * ld + m] = (at >= 0) ? inpw[m] * (A.G[(size_t)at * A.imax + m] + inpb[m]) : real(0);
    }
    __syncthreads();
    real* x = bufA;
    real* y = bufB;
    const real c = (real)net.c;
    for (int l = 0; l < L; ++l) {
        const int no = net.nodes[l], ni = (l == 0) ? nin : net.nodes[l - 1];
        layer_fwd<real>(A.prm.w + net.woff[l], A.prm.b + net.boff[l], no, ni, x, y, ld);
        __syncthreads();
        const int act = (l == L - 1) ? (int)N_LINEAR : net.neuron;
        for (int idx = threadIdx.x; idx < TA * no; idx += MLP_T) {
            const int a = idx % TA, n = idx / TA;
            real av, d1, d2;
            act_fd<real>(act, c, y[a * ld + n], av, d1, d2);
            y[a * ld + n] = av;
            dz[(size_t)l * TA * ld + a * ld + n] = d1;
        }
        __syncthreads();
        real* t = x; x = y; y = t;
    }
    // x holds a_L (one output): energy
    if (threadIdx.x < na) {
        const real out = (real)net.outb + x[threadIdx.x * ld] * (real)net.outw;
        A.Eatom[atoms[threadIdx.x]] = (double)out + pot.t[type].evac;
    }
    __syncthreads();
    // backward: delta_L = outw * f'(z_L)
    for (int a = threadIdx.x; a < TA; a += MLP_T) x[a * ld] = (real)net.outw * dz[(size_t)(L - 1) * TA * ld + a * ld];
    __syncthreads();
    for (int l = L - 1; l >= 1; --l) {
        const int no = net.nodes[l], ni = net.nodes[l - 1];
        layer_bwd<real>(A.prm.wt + net.woff[l], no, ni, x, y, ld);
        __syncthreads();
        for (int idx = threadIdx.x; idx < TA * ni; idx += MLP_T) {
            const int a = idx % TA, m = idx / TA;
            y[a * ld + m] *= dz[(size_t)(l - 1) * TA * ld + a * ld + m];
        }
        __syncthreads();
        real* t = x; x = y; y = t;
    }
    layer_bwd<real>(A.prm.wt + net.woff[0], net.nodes[0], nin, x, y, ld);
    __syncthreads();
    // rows are padded to the widest type: inputs beyond this type's nInput read as zero
    for (int idx = threadIdx.x; idx < TA * A.imax; idx += MLP_T) {
        const int a = idx / A.imax, m = idx % A.imax;
        const int at = atoms[a];
        if (at >= 0) A.dEdG[(size_t)at * A.imax + m] = (m < nin) ? y[a * ld + m] * inpw[m] : real(0);
    }
}

// ---------------------------------------------------------------- training: d/dp [ce E + ct dE/dG . u]
template <typename real>
__global__ void __launch_bounds__(MLP_TT) k_mlp_train(const __grid_constant__ DevPot pot, const MlpArgs<real> A, int ld) {
    extern __shared__ __align__(16) unsigned char msm[];
    int type, a0, na;
    if (!tile_of_block<TAT>(A.ntypes, A.tstart, type, a0, na)) return;
    const DevNet& net = pot.t[type].net;
    const int L = net.nlayer;
    const size_t tl = (size_t)TAT * ld;
    // per layer l (0..L): activations a_l (a_0 = ins) and tangents ad_l; per layer z-derivatives
    real* act = reinterpret_cast<real*>(msm);            // (L+1) * tl
    real* actd = act + (size_t)(L + 1) * tl;             // (L+1) * tl
    real* d1 = actd + (size_t)(L + 1) * tl;              // L * tl  f'
    real* d2 = d1 + (size_t)L * tl;                      // L * tl  f''
    real* zd = d2 + (size_t)L * tl;                      // L * tl  zdot
    real* ab = zd + (size_t)L * tl;                      // tl      abar
    real* adb = ab + tl;                                 // tl      adbar
    real* zb = adb + tl;                                 // tl      zbar
    real* zdb = zb + tl;                                 // tl      zdbar
    __shared__ int32_t atoms[TAT];
    __shared__ double ce[TAT];
    if (threadIdx.x < TAT) {
        const int at = (threadIdx.x < na) ? A.tlist[a0 + threadIdx.x] : -1;
        atoms[threadIdx.x] = at;
        ce[threadIdx.x] = (at >= 0) ? A.ce[at] : 0.0;
    }
    __syncthreads();
    const int nin = net.nin;
    const real* inpw = A.prm.inpw + net.inoff;
    const real* inpb = A.prm.inpb + net.inoff;
    for (int idx = threadIdx.x; idx < TAT * nin; idx += blockDim.x) {
        const int a = idx / nin, m = idx % nin;
        const int at = atoms[a];
        act[a * ld + m] = (at >= 0) ? inpw[m] * (A.G[(size_t)at * A.imax + m] + inpb[m]) : real(0);
        actd[a * ld + m] = (at >= 0) ? inpw[m] * A.U[(size_t)at * A.imax + m] : real(0);
    }
    __syncthreads();
    const real c = (real)net.c;
    for (int l = 0; l < L; ++l) {
        const int no = net.nodes[l], ni = (l == 0) ? nin : net.nodes[l - 1];
        real* xin = act + (size_t)l * tl;
        real* xind = actd + (size_t)l * tl;
        real* xo = act + (size_t)(l + 1) * tl;
        real* xod = actd + (size_t)(l + 1) * tl;
        layer_fwd2<real, TAT>(A.prm.w + net.woff[l], A.prm.b + net.boff[l], no, ni, xin, xind, xo, xod, ld);
        __syncthreads();
        const int actn = (l == L - 1) ? (int)N_LINEAR : net.neuron;
        for (int idx = threadIdx.x; idx < TAT * no; idx += blockDim.x) {
            const int a = idx % TAT, n = idx / TAT;
            real av, f1, f2;
            act_fd<real>(actn, c, xo[a * ld + n], av, f1, f2);
            const real zdot = xod[a * ld + n];
            xo[a * ld + n] = av;
            d1[(size_t)l * tl + a * ld + n] = f1;
            d2[(size_t)l * tl + a * ld + n] = f2;
            zd[(size_t)l * tl + a * ld + n] = zdot;
            xod[a * ld + n] = f1 * zdot;
        }
        __syncthreads();
    }
    // seeds at the output: abar_L = ce*outw, adbar_L = ct*outw
    for (int a = threadIdx.x; a < TAT; a += blockDim.x) {
        ab[a * ld] = (real)(ce[a] * net.outw);
        adb[a * ld] = (atoms[a] >= 0) ? (real)(A.ct * net.outw) : real(0);
    }
    __syncthreads();
    // the block's partial sums of every parameter of its type (each written once)
    double* gp = A.gpart + (size_t)blockIdx.x * A.pstride;
    // parameter offsets (reference packing): biases of all layers, then weights column-major
    int bias_at[MAXLAYER], wt_at[MAXLAYER];
    {
        int cnt = 0;
        for (int l = 0; l < L; ++l) { bias_at[l] = cnt; cnt += net.nodes[l]; }
        for (int l = 0; l < L; ++l) { wt_at[l] = cnt; cnt += net.nodes[l] * ((l == 0) ? nin : net.nodes[l - 1]); }
    }
    for (int l = L - 1; l >= 0; --l) {
        const int no = net.nodes[l], ni = (l == 0) ? nin : net.nodes[l - 1];
        for (int idx = threadIdx.x; idx < TAT * no; idx += blockDim.x) {
            const int a = idx % TAT, n = idx / TAT;
            const real f1 = d1[(size_t)l * tl + a * ld + n], f2 = d2[(size_t)l * tl + a * ld + n];
            const real adbv = adb[a * ld + n];
            zdb[a * ld + n] = f1 * adbv;
            zb[a * ld + n] = f1 * ab[a * ld + n] + f2 * zd[(size_t)l * tl + a * ld + n] * adbv;
        }
        __syncthreads();
        // bias gradient: sum over the tile's atoms of zbar, in the pass's precision (the products
        // are formed in it), stored as the block's FP64 partial (k_grad_blocks adds the blocks)
        for (int n = threadIdx.x; n < no; n += blockDim.x) {
            real s = real(0);
            for (int a = 0; a < TAT; ++a) s += zb[a * ld + n];
            gp[bias_at[l] + n] = (double)s;
        }
        // weight gradient: sum_a zbar[a][n] a_{l}[a][m] + zdbar[a][n] ad_{l}[a][m], column-major;
        // each thread a block of RT outputs n x 2 inputs m (every shared value used 2 or RT times)
        const real* xin = act + (size_t)l * tl;
        const real* xind = actd + (size_t)l * tl;
        const int ngw = (no + RT - 1) / RT, mgw = (ni + 1) / 2;
        for (int idx = threadIdx.x; idx < ngw * mgw; idx += blockDim.x) {
            const int n0 = (idx % ngw) * RT, m0 = (idx / ngw) * 2;
            real s[RT][2];
#pragma unroll
            for (int k = 0; k < RT; ++k) { s[k][0] = real(0); s[k][1] = real(0); }
            for (int a = 0; a < TAT; ++a) {
                const real x0 = xin[a * ld + m0], xd0 = xind[a * ld + m0];
                const real x1 = (m0 + 1 < ni) ? xin[a * ld + m0 + 1] : real(0), xd1 = (m0 + 1 < ni) ? xind[a * ld + m0 + 1] : real(0);
#pragma unroll
                for (int k = 0; k < RT; ++k) {
                    const int n = min(n0 + k, no - 1);
                    const real zv = zb[a * ld + n], zdv = zdb[a * ld + n];
                    s[k][0] += zv * x0 + zdv * xd0;
                    s[k][1] += zv * x1 + zdv * xd1;
                }
            }
#pragma unroll
            for (int k = 0; k < RT; ++k) {
                if (n0 + k >= no) continue;
                gp[wt_at[l] + m0 * no + n0 + k] = (double)s[k][0];
                if (m0 + 1 < ni) gp[wt_at[l] + (m0 + 1) * no + n0 + k] = (double)s[k][1];
            }
        }
        __syncthreads();
        if (l > 0) {
            layer_bwd2<real, TAT>(A.prm.wt + net.woff[l], no, ni, zb, zdb, ab, adb, ld);
            __syncthreads();
        }
    }
}

template <typename real>
static int mlp_ld(const DevPot& pot) {
    int w = 1;
    for (int t = 0; t < pot.ntypes; ++t) {
        w = std::max(w, pot.t[t].net.nin);
        for (int l = 0; l < pot.t[t].net.nlayer; ++l) w = std::max(w, pot.t[t].net.nodes[l]);
    }
    return w + 1;  // odd row stride: conflict-free column access
}
static int mlp_maxL(const DevPot& pot) { int L = 1; for (int t = 0; t < pot.ntypes; ++t) L = std::max(L, pot.t[t].net.nlayer); return L; }

template <typename real>
void launch_mlp_forward_backward(const DevPot& pot, const MlpArgs<real>& a, cudaStream_t st) {
    if (a.natoms <= 0) return;
    const int ld = mlp_ld<real>(pot);
    const size_t smem = (size_t)(2 + mlp_maxL(pot)) * TA * ld * sizeof(real);
    const int grid = (a.natoms + TA - 1) / TA + a.ntypes;
    ++::ann::g_launch_counter, k_mlp_fb<real><<<grid, MLP_T, smem, st>>>(pot, a, ld);
}
// grad[poff[t] + k] += sum over the blocks b of type t of gpart[b][k]: the training pass's per-tile
// sums added deterministically (no atomics, the same result on every run). A block of 32 x GB_SEG
// threads takes 32 consecutive parameters (coalesced rows); thread row y sums segment y of the
// type's block rows (independent loads, 8 in flight) and the segments are added in order.
constexpr int GB_SEG = 8;
__host__ __device__ inline int net_params(const DevNet& net) {
    int s = 0;
    for (int l = 0; l < net.nlayer; ++l) s += net.nodes[l] * (1 + ((l == 0) ? net.nin : net.nodes[l - 1]));
    return s;
}
__global__ void __launch_bounds__(32 * GB_SEG) k_grad_blocks(const __grid_constant__ DevPot pot, const int32_t* tstart, const int32_t* poff,
                                                             const double* gpart, int pstride, double* grad, int tile) {
    __shared__ double seg[GB_SEG][32];
    const int64_t g = blockIdx.x * (int64_t)32 + threadIdx.x;
    int b0 = 0, tiles = 0, type = -1, k = 0;
    int64_t p0 = 0;
    for (int t = 0; t < pot.ntypes; ++t) {
        const int nt = (tstart[t + 1] - tstart[t] + tile - 1) / tile;
        const int P = net_params(pot.t[t].net);
        if (type < 0 && g >= p0 && g < p0 + P) { type = t; k = (int)(g - p0); tiles = nt; }
        if (type < 0) b0 += nt;
        p0 += P;
    }
    double s = 0.0;
    if (type >= 0) {
        const int len = (tiles + GB_SEG - 1) / GB_SEG;
        const int lo = threadIdx.y * len, hi = min(tiles, lo + len);
        const double* col = gpart + (size_t)b0 * pstride + k;
        int b = lo;
        for (; b + 8 <= hi; b += 8) {
            double v[8];
#pragma unroll
            for (int q = 0; q < 8; ++q) v[q] = col[(size_t)(b + q) * pstride];
#pragma unroll
            for (int q = 0; q < 8; ++q) s += v[q];
        }
        for (; b < hi; ++b) s += col[(size_t)b * pstride];
    }
    seg[threadIdx.y][threadIdx.x] = s;
    __syncthreads();
    if (threadIdx.y == 0 && type >= 0) {
        double tsum = 0.0;
#pragma unroll
        for (int y = 0; y < GB_SEG; ++y) tsum += seg[y][threadIdx.x];
        grad[poff[type] + k] += tsum;
    }
}

int mlp_train_tile() { return TAT; }
size_t mlp_train_part_bytes(const DevPot& pot, int natoms, int tile, int* pstride) {
    int P = 1;
    for (int t = 0; t < pot.ntypes; ++t) P = std::max(P, net_params(pot.t[t].net));
    if (pstride) *pstride = P;
    const size_t blocks = (size_t)(std::max(natoms, 0) + tile - 1) / tile + pot.ntypes;
    return blocks * P * sizeof(double);
}

template <typename real>
void launch_mlp_train_grad(const DevPot& pot, const MlpArgs<real>& a, cudaStream_t st) {
    if (a.natoms <= 0) return;
    const int ld = mlp_ld<real>(pot);
    const int L = mlp_maxL(pot);
    const size_t smem = (size_t)(2 * (L + 1) + 3 * L + 4) * TAT * ld * sizeof(real);
    const int grid = (a.natoms + TAT - 1) / TAT + a.ntypes;
    ++::ann::g_launch_counter, k_mlp_train<real><<<grid, MLP_TT, smem, st>>>(pot, a, ld);
    launch_grad_blocks(pot, a.tstart, a.poff, a.gpart, a.pstride, a.grad, TAT, st);
}
void launch_grad_blocks(const DevPot& pot, const int32_t* tstart, const int32_t* poff, const double* gpart, int pstride, double* grad,
                        int tile, cudaStream_t st) {
    int64_t total = 0;
    for (int t = 0; t < pot.ntypes; ++t) total += net_params(pot.t[t].net);
    if (total <= 0) return;
    ++::ann::g_launch_counter, k_grad_blocks<<<(unsigned)((total + 31) / 32), dim3(32, GB_SEG), 0, st>>>(pot, tstart, poff, gpart, pstride, grad, tile);
}
void configure_mlp(int maxsmem) {
    set_max_dynamic_smem(k_mlp_fb<float>, maxsmem);
    set_max_dynamic_smem(k_mlp_fb<double>, maxsmem);
    set_max_dynamic_smem(k_mlp_train<float>, maxsmem);
    set_max_dynamic_smem(k_mlp_train<double>, maxsmem);
}
size_t mlp_smem_bytes(const DevPot& pot, bool fp64, bool train) {
    const int ld = mlp_ld<float>(pot), L = mlp_maxL(pot);
    const size_t rb = fp64 ? 8 : 4;
    return train ? (size_t)(2 * (L + 1) + 3 * L + 4) * TAT * ld * rb : (size_t)(2 + L) * TA * ld * rb;
}

template void launch_mlp_forward_backward<float>(const DevPot&, const MlpArgs<float>&, cudaStream_t);
template void launch_mlp_forward_backward<double>(const DevPot&, const MlpArgs<double>&, cudaStream_t);
template void launch_mlp_train_grad<float>(const DevPot&, const MlpArgs<float>&, cudaStream_t);
template void launch_mlp_train_grad<double>(const DevPot&, const MlpArgs<double>&, cudaStream_t);

}  // namespace ann
