// Optimiser step on the device and the refresh of every device copy of the network parameters
// from the packed FP64 vector, so that a training loop keeps its parameters resident.
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

// one Adam step, then the trainer's weight decay on weights (not biases; nnptefr2.cpp:909-921,
// 1028-1049): p -= gamma eta f(p_old), f = sgn (LASSO), x (RIDGE), x / sqrt(1 + x^2) (HUBER),
// asinh (ASINH); reg = REG_NONE skips it
__global__ void k_adam(int64_t n, const double* g, double scale, double* m, double* v, double* p, double lr, double b1, double b2,
                       double b1ii, double b2ii, double eps, int reg, double eta, const int32_t* map) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double gi = g[i] * scale;
    const double mi = m[i] * b1 + (1.0 - b1) * gi;
    const double vi = v[i] * b2 + (1.0 - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const double p0 = p[i];
    double pn = p0 - lr * b1ii * mi / (sqrt(b2ii * vi) + eps);
    if (reg != REG_NONE && map[PM_N * i + PM_KIND] != PK_BIAS) {
        double f = 0.0;
        switch (reg) {
            case REG_LASSO: f = (double)((p0 > 0) - (p0 < 0)); break;
            case REG_RIDGE: f = p0; break;
            case REG_HUBER: f = p0 / sqrt(1.0 + p0 * p0); break;
            default: f = asinh(p0); break;
        }
        pn -= lr * eta * f;
    }
    p[i] = pn;
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
        *reinterpret_cast<__nv_bfloat16*>(img + e[PM_FL]) = lo;
        *reinterpret_cast<__nv_bfloat16*>(img + e[PM_BH]) = hi;
        *reinterpret_cast<__nv_bfloat16*>(img + e[PM_BL]) = lo;
    }
}

void launch_adam(int64_t n, const double* g, double scale, double* m, double* v, double* p, double lr, double b1, double b2, double b1ii,
                 double b2ii, double eps, int reg, double eta, const int32_t* map, cudaStream_t st) {
    if (n <= 0) return;
    ++::ann::g_launch_counter, k_adam<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(n, g, scale, m, v, p, lr, b1, b2, b1ii, b2ii, eps, reg, eta, map);
}
void launch_param_refresh(int64_t n, const double* p, const int32_t* map, double* w64, double* wt64, double* b64, float* w32, float* wt32,
                          float* b32, uint8_t* img, cudaStream_t st) {
    if (n <= 0) return;
    ++::ann::g_launch_counter,
        k_param_refresh<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(n, p, map, w64, wt64, b64, w32, wt32, b32, img);
}

}  // namespace ann
