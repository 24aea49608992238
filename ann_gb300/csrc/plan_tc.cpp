// Host side of the tensor-core network kernel: BF16 weight images in the canonical K-major
// no-swizzle layout of tcgen05 (see mlp_tc.hpp), per type.
#include <algorithm>
#include <cmath>
#include <cstring>

#include "mlp_tc.hpp"
#include "potential.hpp"

namespace ann {

static uint16_t f2bf(float f) {  // round to nearest even
    uint32_t u;
    std::memcpy(&u, &f, 4);
    if ((u & 0x7fffffffu) > 0x7f800000u) return 0x7fc0;
    const uint32_t r = u + 0x7fffu + ((u >> 16) & 1u);
    return (uint16_t)(r >> 16);
}
static float bf2f(uint16_t h) {
    const uint32_t u = (uint32_t)h << 16;
    float f;
    std::memcpy(&f, &u, 4);
    return f;
}
static int pad16(int n) { return (n + 15) / 16 * 16; }

// byte offset of element (r, k) of an R x K operand in the canonical layout
static size_t canon(int r, int k, int K) { return (size_t)(r / 8) * (K / 8) * 128 + (size_t)(k / 8) * 128 + (size_t)(r % 8) * 16 + (size_t)(k % 8) * 2; }

// image (rounded to 128 B) + A tiles + barriers; at most 512 / tmem_cols CTAs may share one SM's
// tensor memory, so the request is raised until no more CTAs than that fit in the SM's shared memory
size_t TcPlan::smem_bytes(int type) const {
    const TcType& tt = t[type];
    const size_t a = (size_t)TC_M * tt.wmax * 2 * (tt.split >= 2 ? 2 : 1);
    const size_t need = ((size_t)tt.img_bytes + 127) / 128 * 128 + a + TC_TAIL_BYTES;
    const size_t allowed = 512 / (size_t)std::max(tt.tmem_cols, 32);
    return std::max(need, (size_t)smem_per_sm / (allowed + 1) + 1);
}

void build_tc_plan(const DevPot& pot, const std::vector<double>& w, const std::vector<double>& b,
                   const std::vector<double>& inpw, const std::vector<double>& inpb, int max_smem, int split_pref, TcPlan& out) {
    out.ok = true;
    out.image.clear();
    std::memset(out.t, 0, sizeof(out.t));
    for (int ty = 0; ty < pot.ntypes; ++ty) {
        const DevNet& net = pot.t[ty].net;
        TcType& tt = out.t[ty];
        const int L = net.nlayer;
        tt.nhidden = L - 1;
        if (tt.nhidden < 1 || tt.nhidden > TC_MAXH || net.nodes[L - 1] != 1) { out.ok = false; continue; }
        tt.nin = net.nin;
        tt.K0 = pad16(net.nin);
        tt.wmax = tt.K0;
        for (int l = 0; l < tt.nhidden; ++l) {
            tt.nodes[l] = net.nodes[l];
            tt.width[l] = pad16(net.nodes[l]);
            tt.wmax = std::max(tt.wmax, tt.width[l]);
        }
        if (tt.wmax > 256) { out.ok = false; continue; }
        // TMEM: one column range per hidden layer's forward accumulator (kept for the backward
        // pass, which recomputes f'(z) from it) plus one range for the backward accumulators
        int cols = 0, maxkin = tt.K0;
        for (int l = 0; l < tt.nhidden; ++l) { tt.fwd_col[l] = cols; cols += tt.width[l]; maxkin = std::max(maxkin, tt.width[l]); }
        tt.bwd_col = cols;
        cols += maxkin;
        tt.tmem_cols = 32;
        while (tt.tmem_cols < cols) tt.tmem_cols *= 2;
        if (tt.tmem_cols > 512) { out.ok = false; continue; }
        tt.neuron = net.neuron;
        tt.c = (float)net.c;
        tt.outw = (float)net.outw;
        tt.outb = (float)net.outb;
        tt.evac = pot.t[ty].evac;
        // operand sizes
        size_t bf = 0;
        for (int l = 0; l < tt.nhidden; ++l) {
            const int Kin = (l == 0) ? tt.K0 : tt.width[l - 1];
            bf += (size_t)tt.width[l] * Kin * 2;      // W_l (the backward pass reads it as W_l^T)
        }
        size_t vec = 0;
        for (int l = 0; l < tt.nhidden; ++l) vec += (size_t)tt.width[l] * 4;
        vec += (size_t)tt.width[tt.nhidden - 1] * 4 + (size_t)tt.K0 * 8;
        auto total = [&](int split) {
            const size_t img = bf * (split == 3 ? 2 : 1) + vec + 16 * (4 * TC_MAXH + 5);
            return (img + 127) / 128 * 128 + (size_t)TC_M * tt.wmax * 2 * (split >= 2 ? 2 : 1) + TC_TAIL_BYTES;
        };
        // operand form: split 3 (A and W as BF16 hi + lo, three MMAs per k-step) keeps the products
        // within ~1e-5 relative of FP32; split 2 (A split, W single BF16) halves the image and the
        // MMAs; split 1 is plain BF16 x BF16 with FP32 accumulation. split_pref 0 takes the most
        // accurate form whose image fits a block's shared memory; a forced form that does not fit
        // leaves the type to the SIMT kernel
        tt.split = 0;
        for (int s = split_pref ? split_pref : 3; s >= (split_pref ? split_pref : 1); --s)
            if (total(s) + 1024 <= (size_t)max_smem) { tt.split = s; break; }
        if (tt.split == 0) { out.ok = false; continue; }
        // image
        std::vector<uint8_t> img;
        auto align16 = [&]() { while (img.size() % 16) img.push_back(0); };
        auto put_operand = [&](int R, int K, auto value, bool lo) {  // value(r,k) -> double, zero outside
            align16();
            const size_t base = img.size();
            img.resize(base + (size_t)R * K * 2, 0);
            for (int r = 0; r < R; ++r)
                for (int k = 0; k < K; ++k) {
                    const float v = (float)value(r, k);
                    const uint16_t hi = f2bf(v);
                    const uint16_t h = lo ? f2bf(v - bf2f(hi)) : hi;
                    std::memcpy(&img[base + canon(r, k, K)], &h, 2);
                }
            return (uint32_t)base;
        };
        auto put_floats = [&](int n, auto value) {
            align16();
            const size_t base = img.size();
            img.resize(base + (size_t)n * 4, 0);
            for (int k = 0; k < n; ++k) { const float v = (float)value(k); std::memcpy(&img[base + 4 * (size_t)k], &v, 4); }
            return (uint32_t)base;
        };
        for (int l = 0; l < tt.nhidden; ++l) {
            const int ni = (l == 0) ? net.nin : net.nodes[l - 1];
            const int no = net.nodes[l];
            const int Kin = (l == 0) ? tt.K0 : tt.width[l - 1];
            const double* W = w.data() + net.woff[l];   // W[n*ni + m]
            auto fwd = [&](int r, int k) { return (r < no && k < ni) ? W[(size_t)r * ni + k] : 0.0; };
            tt.fwd_hi[l] = put_operand(tt.width[l], Kin, fwd, false);
            tt.fwd_lo[l] = (tt.split == 3) ? put_operand(tt.width[l], Kin, fwd, true) : tt.fwd_hi[l];
        }
        for (int l = 0; l < tt.nhidden; ++l) {
            const int no = net.nodes[l];
            const double* B = b.data() + net.boff[l];
            tt.bias[l] = put_floats(tt.width[l], [&](int k) { return k < no ? B[k] : 0.0; });
        }
        {
            const int nl = net.nodes[L - 2];
            const double* WL = w.data() + net.woff[L - 1];   // 1 x nl
            tt.wlast = put_floats(tt.width[tt.nhidden - 1], [&](int k) { return k < nl ? WL[k] : 0.0; });
        }
        tt.blast = put_floats(1, [&](int) { return b[net.boff[L - 1]]; });
        tt.inpw = put_floats(tt.K0, [&](int k) { return k < net.nin ? inpw[net.inoff + k] : 0.0; });
        tt.inpb = put_floats(tt.K0, [&](int k) { return k < net.nin ? inpb[net.inoff + k] : 0.0; });
        align16();
        tt.img_bytes = (uint32_t)img.size();
        while (out.image.size() % 128) out.image.push_back(0);
        tt.img_off = (uint32_t)out.image.size();
        out.image.insert(out.image.end(), img.begin(), img.end());
    }
    if (out.image.empty()) out.image.resize(128, 0);
}

void build_param_map(const DevPot& pot, const TcPlan& tc, std::vector<int32_t>& map) {
    map.clear();
    auto put = [&](int kind, int i64, int iT, int64_t f32, int64_t fh, int64_t fl, int64_t bh, int64_t bl) {
        const int64_t v[PM_N] = {kind, i64, iT, f32, fh, fl, bh, bl};
        for (int k = 0; k < PM_N; ++k) map.push_back((int32_t)v[k]);
    };
    for (int ty = 0; ty < pot.ntypes; ++ty) {
        const DevNet& net = pot.t[ty].net;
        const int L = net.nlayer;
        const bool img = tc.ok;
        const TcType& tt = tc.t[ty];
        const int64_t base = img ? (int64_t)tt.img_off : 0;
        for (int l = 0; l < L; ++l)
            for (int n = 0; n < net.nodes[l]; ++n) {
                int64_t f32 = -1;
                if (img) f32 = base + ((l < tt.nhidden) ? tt.bias[l] + 4 * n : tt.blast);
                put(PK_BIAS, net.boff[l] + n, -1, f32, -1, -1, -1, -1);
            }
        for (int l = 0; l < L; ++l) {
            const int ni = (l == 0) ? net.nin : net.nodes[l - 1], no = net.nodes[l];
            for (int m = 0; m < ni; ++m)
                for (int n = 0; n < no; ++n) {
                    int64_t f32 = -1, fh = -1, fl = -1;
                    if (img && l < tt.nhidden) {
                        const int Kin = (l == 0) ? tt.K0 : tt.width[l - 1];
                        fh = base + tt.fwd_hi[l] + canon(n, m, Kin);
                        if (tt.split == 3) fl = base + tt.fwd_lo[l] + canon(n, m, Kin);   // lo parts only when split
                    } else if (img) {
                        f32 = base + tt.wlast + 4 * m;   // last layer: one output
                    }
                    put(PK_WEIGHT, net.woff[l] + n * ni + m, net.woff[l] + m * no + n, f32, fh, fl, -1, -1);
                }
        }
    }
}

}  // namespace ann
