// Training-loss seeds (K6 entry) and the velocity-Verlet integrator (K7).
//
// Loss (nnptefr2.cpp:1321-1374 energy term, any of its losses and normalisations, averaged over
// the batch as nnptefr2.cpp:984-995; force term as intended by nnptef.cpp:1715-1825):
//   L = wE/S sum_s loss(dU_s) + wF/(3N) sum_a 1/2 |F_a-Fref_a|^2,  dU_s = (E_s-Eref_s) normt(N_s)
// (MSE / LINEAR: loss = 1/2 dU^2, normt = 1/N). Seeds for the adjoint pass: ce_i = dL/dE_s(i) =
// wE/S d loss/dE_s for every atom i of s, lam_a = dL/dF_a = wF/(3N) (F_a - Fref_a).
//
// MD: Verlet::compute (src/torch/integrator.cpp:177-200) in metal units (x A, v A/fs, dt fs,
// m Da, F eV/A; a = F/(m mvv_to_e), mvv_to_e = 103.642696526805, src/chem/units.cpp:151).
#include <cuda_runtime.h>
#include <cstdint>
#include "kernels.hpp"
#include "mlp_tc.hpp"

namespace ann {

// energy term of one structure (nnptefr2.cpp:1339-1368, normalisation 606-612): the loss and
// gfac = d loss / dE for loss 1 MSE, 2 MAE, 3 HUBER, 4 ASINH and norm 0 IDENTITY, 1 LINEAR, 2 SQRT,
// 3 CBRT, 4 LOG
__device__ __forceinline__ void energy_loss(int lossf, int norm, double delta, double dE, double ns, double& L, double& gfac) {
    double normt = 1.0;
    switch (norm) {
        case 1: normt = 1.0 / ns; break;
        case 2: normt = 1.0 / sqrt(ns); break;
        case 3: normt = 1.0 / cbrt(ns); break;
        case 4: normt = 1.0 / (log(ns) + 1.0); break;
        default: break;
    }
    const double dU = dE * normt, deltai = 1.0 / delta;
    gfac = normt;
    switch (lossf) {
        case 2: L = fabs(dU); gfac *= (double)((dU > 0) - (dU < 0)); break;
        case 3: { const double arg = dU * deltai, sq = sqrt(1.0 + arg * arg); L = delta * delta * (sq - 1.0); gfac *= dU / sq; } break;
        case 4: {
            const double arg = dU * deltai, sq = sqrt(1.0 + arg * arg), lg = log(arg + sq);
            L = delta * delta * (1.0 - sq + arg * lg); gfac *= lg * delta;
        } break;
        default: L = 0.5 * dU * dU; gfac *= dU; break;
    }
}

template <typename real>
__global__ void k_train_loss(int nstruc, int natoms, const int32_t* off, const int32_t* sid, const double* Es, const double* Fout,
                             const double* Eref, const double* Fref, double wE, double wF, int lossf, int norm, double delta,
                             double* loss3, double* ce, real* lam) {
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    double le = 0.0, lf = 0.0;   // this atom's share of the two loss terms
    if (a < natoms) {
        const int s = sid[a];
        const double ns = (double)(off[s + 1] - off[s]);
        double Ls, gfac;
        energy_loss(lossf, norm, delta, Es[s] - Eref[s], ns, Ls, gfac);
        ce[a] = wE / nstruc * gfac;
        if (a == off[s]) le = wE / nstruc * Ls;
        const double sc = wF / (3.0 * natoms);
        double l2 = 0.0;
        for (int c = 0; c < 3; ++c) {
            const double df = Fout[3 * (size_t)a + c] - Fref[3 * (size_t)a + c];
            l2 += df * df;
            lam[3 * (size_t)a + c] = (real)(sc * df);
        }
        lf = 0.5 * l2 * sc;
    }
    // one atomic per warp and term (the loss words are shared by the whole batch)
    for (int o = 16; o > 0; o >>= 1) {
        le += __shfl_xor_sync(0xffffffffu, le, o);
        lf += __shfl_xor_sync(0xffffffffu, lf, o);
    }
    if ((threadIdx.x & 31) == 0) {
        if (le != 0.0) atomicAdd(&loss3[1], le);
        atomicAdd(&loss3[2], lf);
    }
}
__global__ void k_train_loss_final(double* loss3) { loss3[0] = loss3[1] + loss3[2]; }

void launch_train_loss(int nstruc, int natoms, const int32_t* off, const int32_t* sid, const double* Es, const double* Fout,
                       const double* Eref, const double* Fref, double wE, double wF, int lossf, int norm, double delta, double* loss3,
                       double* ce, void* lam, bool fp64, cudaStream_t st) {
    if (natoms > 0) {
        const int g = (natoms + 255) / 256;
        if (fp64)
            ++::ann::g_launch_counter, k_train_loss<double><<<g, 256, 0, st>>>(nstruc, natoms, off, sid, Es, Fout, Eref, Fref, wE, wF, lossf,
                                                                               norm, delta, loss3, ce, (double*)lam);
        else
            ++::ann::g_launch_counter, k_train_loss<float><<<g, 256, 0, st>>>(nstruc, natoms, off, sid, Es, Fout, Eref, Fref, wE, wF, lossf,
                                                                              norm, delta, loss3, ce, (float*)lam);
    }
    ++::ann::g_launch_counter, k_train_loss_final<<<1, 1, 0, st>>>(loss3);
}

// stage 0: v += dt/2 F/m; x += v dt; flag atoms that moved more than skin/2 since the last build
// stage 1: v += dt/2 F/m
// stage 2: wrap x into the cell (Cell::returnToCell)
template <typename real>
__global__ void k_md(int n, double* x, double* v, const real* F, const double* minv, const int32_t* type, double dt,
                     const double* R, const double* Ri, const double* xref, int32_t* flag, double half_skin2, int stage) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (stage == 2) {
        double s[3];
        for (int d = 0; d < 3; ++d) s[d] = Ri[d] * x[3 * i] + Ri[3 + d] * x[3 * i + 1] + Ri[6 + d] * x[3 * i + 2];
        for (int d = 0; d < 3; ++d) s[d] -= floor(s[d]);
        for (int c = 0; c < 3; ++c) x[3 * i + c] = R[c] * s[0] + R[3 + c] * s[1] + R[6 + c] * s[2];
        return;
    }
    const double hm = 0.5 * dt * minv[type[i]];
    for (int c = 0; c < 3; ++c) v[3 * i + c] += hm * (double)F[3 * (size_t)i + c];
    if (stage == 0) {
        double d2 = 0.0;
        for (int c = 0; c < 3; ++c) {
            x[3 * i + c] += v[3 * i + c] * dt;
            const double dd = x[3 * i + c] - xref[3 * i + c];
            d2 += dd * dd;
        }
        if (d2 > half_skin2) atomicOr(flag, 1);
    }
}
void launch_md_kick_drift(int natoms, double* pos, double* vel, const void* F, bool fp64, const double* minv, const int32_t* type,
                          double dt, const double* R, const double* Ri, double* disp_ref, int32_t* flag, double half_skin2,
                          int stage, cudaStream_t st) {
    if (natoms <= 0) return;
    const int g = (natoms + 255) / 256;
    if (fp64) ++::ann::g_launch_counter, k_md<double><<<g, 256, 0, st>>>(natoms, pos, vel, (const double*)F, minv, type, dt, R, Ri, disp_ref, flag, half_skin2, stage);
    else ++::ann::g_launch_counter, k_md<float><<<g, 256, 0, st>>>(natoms, pos, vel, (const float*)F, minv, type, dt, R, Ri, disp_ref, flag, half_skin2, stage);
}

__global__ void k_md_ke(int n, const double* v, const double* mass, const int32_t* type, double* ke) {
    __shared__ double red[256];
    double s = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        s += mass[type[i]] * (v[3 * i] * v[3 * i] + v[3 * i + 1] * v[3 * i + 1] + v[3 * i + 2] * v[3 * i + 2]);
    red[threadIdx.x] = s;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) { if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w]; __syncthreads(); }
    if (threadIdx.x == 0) atomicAdd(ke, 0.5 * 103.642696526805 * red[0]);
}
void launch_md_ke(int natoms, const double* vel, const double* mass, const int32_t* type, double* ke, cudaStream_t st) {
    cudaMemsetAsync(ke, 0, sizeof(double), st);
    if (natoms > 0) ++::ann::g_launch_counter, k_md_ke<<<std::min(1024, (natoms + 255) / 256), 256, 0, st>>>(natoms, vel, mass, type, ke);
}

void configure_kernels() {
    static bool done = false;
    if (done) return;
    int dev = 0, maxs = 48 * 1024;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&maxs, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    configure_bp(maxs);
    configure_mlp(maxs);
    configure_nbr(maxs);
    configure_mlp_tc(maxs);
    configure_mlp_train_tc(maxs);
    done = true;
}

}  // namespace ann
