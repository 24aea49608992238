// Optimiser steps on the device (every elementwise algorithm of opt::algo, and CG) and the refresh
// of every device copy of the network parameters from the packed FP64 vector, so that a training
// loop keeps its parameters resident.
//
// Reference: NN::ADAM::step (src/opt/algo.cpp:280-296): m = b1 m + (1-b1) g, v = b2 v + (1-b2) g^2,
// p -= gamma / (1 - b1^t) m / (sqrt(v / (1 - b2^t)) + eps); the packing order of the parameters is
// ANN::operator>> (src/ml/nn.cpp:846-859), types in NNP order.
#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <cstdint>
#include "kernels.hpp"
#include "mlp_tc.hpp"

namespace ann {

// One optimiser step of opt::algo (src/opt/algo.cpp:97-660), then the trainer's weight decay on
// weights (not biases; nnptefr2.cpp:909-921, 1028-1049): p -= gamma eta f(p_old) with f = sgn
// (LASSO), x (RIDGE), x / sqrt(1 + x^2) (HUBER), asinh (ASINH). State per parameter: s0, s1, s2 (the
// algorithm's running vectors) and gold (the previous gradient, for RPROP and CG). The Adam family
// uses beta1 = b1, beta2 = b2 and the bias corrections b1ii = 1/(1 - b1^t), b2ii = 1/(1 - b2^t).
__global__ void k_opt(OptArgs o) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= o.n) return;
    double g = o.g[i] * o.scale;
    const double p0 = o.p[i], gm = o.gamma, b1 = o.b1, b2 = o.b2, eps = o.eps, eta = o.eta;
    double p = p0;
    double s0 = o.s0[i], s1 = o.s1 ? o.s1[i] : 0.0, s2 = o.s2 ? o.s2[i] : 0.0;
    auto sgn = [](double x) { return (double)((x > 0) - (x < 0)); };
    switch (o.algo) {
        case OPT_SGD: p -= gm * g; break;
        case OPT_SDM: s0 = eta * s0 + gm * g; p -= s0; break;
        case OPT_NAG: s0 = eta * s0 + gm * (eta + 1.0) * g; p -= s0; break;
        case OPT_ADAGRAD: s0 += g * g; p -= gm * g / (sqrt(s0) + eps); break;
        case OPT_ADADELTA: {
            s0 = eta * s0 + (1.0 - eta) * g * g;
            const double dx = g * sqrt(s1) / (sqrt(s0) + eps);
            p -= dx;
            s1 = eta * s1 + (1.0 - eta) * dx * dx;
        } break;
        case OPT_RMSPROP: s0 = 0.9 * s0 + 0.1 * g * g; p -= gm * g / (sqrt(s0) + eps); break;
        case OPT_ADAM: case OPT_ADAMW: case OPT_ADAB: case OPT_YOGI: case OPT_NOGI: case OPT_NADAM: case OPT_AMSGRAD: {
            s0 = s0 * b1 + (1.0 - b1) * g;
            if (o.algo == OPT_ADAB) s1 = s1 * b2 + (1.0 - b2) * (g - s0) * (g - s0) + eps;
            else if (o.algo == OPT_YOGI || o.algo == OPT_NOGI) s1 -= (1.0 - b2) * sgn(s1 - g * g) * (g * g);
            else s1 = s1 * b2 + (1.0 - b2) * g * g;
            double vv = s1;
            if (o.algo == OPT_AMSGRAD) { if (s1 > s2) s2 = s1; vv = s2; }
            const double mm = (o.algo == OPT_NOGI || o.algo == OPT_NADAM) ? b1 * s0 + (1.0 - b1) * g : s0;
            if (o.algo == OPT_ADAMW) p -= gm * (o.b1ii * mm / (sqrt(o.b2ii * vv) + eps) + o.w * p0);
            else p -= gm * o.b1ii * mm / (sqrt(o.b2ii * vv) + eps);
        } break;
        case OPT_RPROP: {   // s0 = delta, s1 = dx; the gradient kept for the next step is zeroed on a sign change
            const double sg = g * o.gold[i];
            if (sg > 0) { s0 = fmin(s0 * 1.2, 50.0); s1 = -1.0 * sgn(g) * s0; p += s1; }
            else if (sg < 0) { s0 = fmax(s0 * 0.5, 1e-14); if (o.inc) p -= s1; g = 0.0; }
            else { s1 = -1.0 * sgn(g) * s0; p += s1; }
        } break;
        case OPT_CG: s0 = (*o.beta) * s0 - g; p += gm * s0; break;
        default: break;
    }
    if (o.reg != REG_NONE && o.map[PM_N * i + PM_KIND] != PK_BIAS) {
        double f = 0.0;
        switch (o.reg) {
            case REG_LASSO: f = sgn(p0); break;
            case REG_RIDGE: f = p0; break;
            case REG_HUBER: f = p0 / sqrt(1.0 + p0 * p0); break;
            default: f = asinh(p0); break;
        }
        p -= gm * o.reg_eta * f;
    }
    o.p[i] = p;
    o.s0[i] = s0;
    if (o.s1) o.s1[i] = s1;
    if (o.s2) o.s2[i] = s2;
    if (o.gold) o.gold[i] = g;
}

// CG: beta = g . (g - g_old) / (|g_old|^2 + eps) in a fixed order (block partials, then one block)
constexpr int CG_T = 256;
__global__ void k_cg_partial(int64_t n, const double* g, double scale, const double* gold, double* part) {
    __shared__ double a[CG_T], b[CG_T];
    double sa = 0.0, sb = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)CG_T + threadIdx.x; i < n; i += (int64_t)gridDim.x * CG_T) {
        const double gi = g[i] * scale;
        sa += gi * (gi - gold[i]);
        sb += gold[i] * gold[i];
    }
    a[threadIdx.x] = sa; b[threadIdx.x] = sb;
    __syncthreads();
    for (int w = CG_T / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) { a[threadIdx.x] += a[threadIdx.x + w]; b[threadIdx.x] += b[threadIdx.x + w]; }
        __syncthreads();
    }
    if (threadIdx.x == 0) { part[2 * blockIdx.x] = a[0]; part[2 * blockIdx.x + 1] = b[0]; }
}
__global__ void k_cg_beta(int nb, const double* part, double eps, double* beta) {
    if (threadIdx.x != 0) return;
    double a = 0.0, b = 0.0;
    for (int k = 0; k < nb; ++k) { a += part[2 * k]; b += part[2 * k + 1]; }
    *beta = a / (b + eps);
}

// one thread per parameter: FP64 and FP32 copies (row-major and transposed weights, biases) and,
// when the tensor-core images exist, their FP32 entries and BF16 hi/lo operand entries (the same
// roundings as the host-built images)
__global__ void k_param_refresh(int64_t n, const double* p, const int32_t* map, double* w64, double* wt64, double* b64, float* w32,
                                float* wt32, float* b32, uint8_t* img) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int32_t* e = map + PM_N * i;
    const double v = p[i];
    const float vf = (float)v;
    if (e[PM_KIND] == PK_BIAS) {
        b64[e[PM_I64]] = v;
        b32[e[PM_I64]] = vf;
    } else {
        w64[e[PM_I64]] = v; wt64[e[PM_IT]] = v;
        w32[e[PM_I64]] = vf; wt32[e[PM_IT]] = vf;
    }
    if (!img) return;
    if (e[PM_F32] >= 0) *reinterpret_cast<float*>(img + e[PM_F32]) = vf;
    if (e[PM_FH] >= 0) {
        const __nv_bfloat16 hi = __float2bfloat16_rn(vf);
        const __nv_bfloat16 lo = __float2bfloat16_rn(vf - __bfloat162float(hi));
        *reinterpret_cast<__nv_bfloat16*>(img + e[PM_FH]) = hi;
        if (e[PM_FL] >= 0) *reinterpret_cast<__nv_bfloat16*>(img + e[PM_FL]) = lo;
        if (e[PM_BH] >= 0) *reinterpret_cast<__nv_bfloat16*>(img + e[PM_BH]) = hi;
        if (e[PM_BL] >= 0) *reinterpret_cast<__nv_bfloat16*>(img + e[PM_BL]) = lo;
    }
}

void launch_opt(const OptArgs& o, double* part, cudaStream_t st) {
    if (o.n <= 0) return;
    if (o.algo == OPT_CG) {
        const int nb = (int)std::min<int64_t>((o.n + CG_T - 1) / CG_T, 64);
        ++::ann::g_launch_counter, k_cg_partial<<<nb, CG_T, 0, st>>>(o.n, o.g, o.scale, o.gold, part);
        ++::ann::g_launch_counter, k_cg_beta<<<1, 32, 0, st>>>(nb, part, o.eps, o.beta);
    }
    ++::ann::g_launch_counter, k_opt<<<(unsigned)((o.n + 255) / 256), 256, 0, st>>>(o);
}
void launch_param_refresh(int64_t n, const double* p, const int32_t* map, double* w64, double* wt64, double* b64, float* w32, float* wt32,
                          float* b32, uint8_t* img, cudaStream_t st) {
    if (n <= 0) return;
    ++::ann::g_launch_counter,
        k_param_refresh<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(n, p, map, w64, wt64, b64, w32, wt32, b32, img);
}

}  // namespace ann
