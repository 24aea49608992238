// K1: periodic-image neighbour list, cell-binned, one warp per centre atom with warp-ballot
// compaction. Replaces the reference's NeighborList(struc, rc) (src/struc/, missing from the
// snapshot; contract from the call sites src/nnp/nnp.cpp:343-348, 478-486): every image
// j + R n with |x_i - x_j - R n| < rc except (j == i, n == 0), r = x_i - x_j - R n.
//
// Binning: fractional coordinates s = R^-1 x are wrapped (s = frac + m) and binned along each
// lattice direction (bins ~rc/2 wide). A centre atom in bin b visits the unwrapped bins
// u = b + e, |e_d| <= sten_d = ceil(rc |g_d| nb_d) (g_d = row d of R^-1), which covers every
// image of every atom within rc once, for any cell shape and for cells smaller than rc
// (u_d outside [0,nb_d) selects the image k_d = floor(u_d / nb_d)).
// The accepted entries are written grouped by neighbour type (a stable partition) so that the
// symmetry-function kernels iterate type blocks without branching.
#include <cuda_runtime.h>
#include <cstdint>
#include <cmath>
#include "kernels.hpp"

namespace ann {

static __device__ __forceinline__ int32_t pack3(int a, int b, int c) {
    return (int32_t)(((uint32_t)a & 1023u) | (((uint32_t)b & 1023u) << 10) | (((uint32_t)c & 1023u) << 20));
}
static __device__ __forceinline__ void unpack3(int32_t p, int& a, int& b, int& c) {
    a = ((int32_t)((uint32_t)p << 22)) >> 22;
    b = ((int32_t)((uint32_t)p << 12)) >> 22;
    c = ((int32_t)((uint32_t)p << 2)) >> 22;
}
// floor(a / b) for b >= 1 and |a| < 2^21 without an integer division: (a + 1/2) / b lies at least
// 1/(2b) from an integer and the product's rounding error is below 2^-22 |a + 1/2| / b
static __device__ __forceinline__ int floordiv_small(int a, int b) { return (int)floorf(((float)a + 0.5f) * __frcp_rn((float)b)); }

// ---------------------------------------------------------------- per-structure geometry
// one thread per structure (the FP64 inverse, norms and divisions spread over many SMs); bins per
// structure bounded by 2*natoms+1 so that the bin arrays can be sized from the atom count alone
constexpr int GEO_T = 32;
static __device__ void struc_geo(const NbrArgs& a, int s, StrucGeo& g) {
    const double* R = a.cell + 9 * s;
    for (int k = 0; k < 9; ++k) g.R[k] = R[k];
    auto at = [&](int r, int c) { return R[3 * c + r]; };
    const double det = at(0, 0) * (at(1, 1) * at(2, 2) - at(1, 2) * at(2, 1)) - at(0, 1) * (at(1, 0) * at(2, 2) - at(1, 2) * at(2, 0)) +
                       at(0, 2) * (at(1, 0) * at(2, 1) - at(1, 1) * at(2, 0));
    const double id = 1.0 / det;
    double m[3][3];
    m[0][0] = (at(1, 1) * at(2, 2) - at(1, 2) * at(2, 1)) * id; m[0][1] = (at(0, 2) * at(2, 1) - at(0, 1) * at(2, 2)) * id; m[0][2] = (at(0, 1) * at(1, 2) - at(0, 2) * at(1, 1)) * id;
    m[1][0] = (at(1, 2) * at(2, 0) - at(1, 0) * at(2, 2)) * id; m[1][1] = (at(0, 0) * at(2, 2) - at(0, 2) * at(2, 0)) * id; m[1][2] = (at(0, 2) * at(1, 0) - at(0, 0) * at(1, 2)) * id;
    m[2][0] = (at(1, 0) * at(2, 1) - at(1, 1) * at(2, 0)) * id; m[2][1] = (at(0, 1) * at(2, 0) - at(0, 0) * at(2, 1)) * id; m[2][2] = (at(0, 0) * at(1, 1) - at(0, 1) * at(1, 0)) * id;
    for (int r = 0; r < 3; ++r) for (int c = 0; c < 3; ++c) g.Ri[3 * c + r] = m[r][c];
    const int nat = a.off[s + 1] - a.off[s];
    const int maxbins = 2 * max(nat, 1) + 1;
    double gn[3];
    for (int d = 0; d < 3; ++d) gn[d] = sqrt(m[d][0] * m[d][0] + m[d][1] * m[d][1] + m[d][2] * m[d][2]);
    const bool ok = isfinite(det) && det != 0.0;
    for (int d = 0; d < 3; ++d) {
        const double h = ok ? 1.0 / gn[d] : 1.0;             // distance between lattice planes
        int nb = (int)floor(h / (0.5 * a.rc));
        g.nb[d] = max(1, min(nb, 1024));
    }
    while ((long long)g.nb[0] * g.nb[1] * g.nb[2] > maxbins) {
        int dm = 0;
        if (g.nb[1] > g.nb[dm]) dm = 1;
        if (g.nb[2] > g.nb[dm]) dm = 2;
        g.nb[dm] = max(1, g.nb[dm] / 2);
    }
    for (int d = 0; d < 3; ++d) g.sten[d] = ok ? (int)ceil(a.rc * gn[d] * g.nb[d] + 1e-9) : 0;
    // the structure's bins start at 2 atom0 + s: every structure has at most 2 n + 1 bins, so the
    // ranges never overlap and fit the 2N + S + 2 bins of the batch without a prefix over structures
    g.atom0 = a.off[s]; g.natoms = nat; g.bin0 = 2 * a.off[s] + s; g.pad = ok ? 0 : 1;
    g.ortho = (ok && at(1, 0) == 0.0 && at(2, 0) == 0.0 && at(0, 1) == 0.0 && at(2, 1) == 0.0 && at(0, 2) == 0.0 && at(1, 2) == 0.0) ? 1 : 0;
    for (int d = 0; d < 3; ++d) g.labs[d] = (float)fabs(at(d, d));
    for (int k = 0; k < 9; ++k) { g.Rf[k] = (float)g.R[k]; g.Rif[k] = (float)g.Ri[k]; }
}
__global__ void __launch_bounds__(GEO_T) k_struc_geo(NbrArgs a) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= a.nstruc) return;
    StrucGeo g;
    struc_geo(a, s, g);
    a.geo[s] = g;
}

// bin coordinates of one atom (fractional coordinates wrapped into the cell, s = frac + m), its
// FP32 position with the type bits, and the input checks
static __device__ __forceinline__ int bin_atom(const NbrArgs& a, const StrucGeo& g, int i, int b[3], int m[3]) {
    const double x = a.pos[3 * i], y = a.pos[3 * i + 1], z = a.pos[3 * i + 2];
    const int t = a.type[i];
    if (t < 0 || t >= a.ntypes) atomicOr(a.status, (int)ST_BAD_TYPE);
    a.pos4[i] = make_float4((float)x, (float)y, (float)z, __int_as_float(t));
    b[0] = b[1] = b[2] = 0; m[0] = m[1] = m[2] = 0;
    if (!(isfinite(x) && isfinite(y) && isfinite(z)) || g.pad) {
        atomicOr(a.status, (int)ST_NONFINITE);
    } else {
        for (int d = 0; d < 3; ++d) {
            const double sd = g.Ri[d] * x + g.Ri[3 + d] * y + g.Ri[6 + d] * z;
            const double fl = floor(sd);
            if (fabs(fl) > 500.0) { atomicOr(a.status, (int)ST_IMAGE_RANGE); continue; }
            m[d] = (int)fl;
            int bb = (int)floor((sd - fl) * g.nb[d]);
            b[d] = min(max(bb, 0), g.nb[d] - 1);
        }
    }
    a.abc[i] = pack3(b[0], b[1], b[2]);
    a.am[i] = pack3(m[0], m[1], m[2]);
    return (b[2] * g.nb[1] + b[1]) * g.nb[0] + b[0];
}

// ---------------------------------------------------------------- small structures: one block each
// Structures of at most BIN_LOCAL_MAX atoms are binned by one block in shared memory: bin counts,
// their exclusive scan, the scatter, a sort of every bin by atom index (the same order as the
// global path), then the bin starts and the bin-ordered copies. Shared: counts and starts
// [2 * (2 * BIN_LOCAL_MAX + 2)], local bins and sorted slots [2 * BIN_LOCAL_MAX].
constexpr int BIN_LOCAL_MAX = 1024;
constexpr int BIN_LOCAL_T = 256;
constexpr int BIN_LOCAL_WORDS = 2 * (2 * BIN_LOCAL_MAX + 2) + 2 * BIN_LOCAL_MAX;
__global__ void __launch_bounds__(BIN_LOCAL_T) k_bin_local(NbrArgs a) {
    __shared__ int32_t sm[BIN_LOCAL_WORDS];
    __shared__ int32_t part[BIN_LOCAL_T / 32];
    __shared__ StrucGeo g;   // the structure's geometry, formed here for the search as well
    const int s = blockIdx.x, t = threadIdx.x, T = blockDim.x;
    if (t == 0) {
        struc_geo(a, s, g);
        a.geo[s] = g;
    }
    __syncthreads();
    const int a0 = g.atom0, nat = g.natoms, bin0 = g.bin0;
    const int nbins = g.nb[0] * g.nb[1] * g.nb[2];
    if (nat > BIN_LOCAL_MAX || nbins > 2 * BIN_LOCAL_MAX + 1 || bin0 + nbins > a.nbins_cap) {   // excluded by the host
        if (t == 0) atomicOr(a.status, (int)ST_NBR_OVERFLOW);
        return;
    }
    int32_t* cnt = sm;                               // [nbins + 1] counts, then the scatter cursors
    int32_t* bst = cnt + (2 * BIN_LOCAL_MAX + 2);    // [nbins + 1] bin starts (structure-local)
    int32_t* lbin = bst + (2 * BIN_LOCAL_MAX + 2);   // [nat] local bin of each atom
    int32_t* sidx = lbin + BIN_LOCAL_MAX;            // [nat] structure-local atoms in bin order
    for (int k = t; k <= nbins; k += T) cnt[k] = 0;
    __syncthreads();
    for (int li = t; li < nat; li += T) {
        int b[3], m[3];
        const int lb = bin_atom(a, g, a0 + li, b, m);
        lbin[li] = lb;
        atomicAdd(&cnt[lb], 1);
    }
    __syncthreads();
    // exclusive scan of the counts: each thread a contiguous range, then over the threads
    {
        const int n = nbins + 1, per = (n + T - 1) / T, lo = min(n, t * per), hi = min(n, lo + per);
        int32_t local = 0;
        for (int k = lo; k < hi; ++k) local += cnt[k];
        const int lane = t & 31, wid = t >> 5;
        int32_t incl = local;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) { const int32_t v = __shfl_up_sync(0xffffffffu, incl, o); if (lane >= o) incl += v; }
        if (lane == 31) part[wid] = incl;
        __syncthreads();
        if (t == 0) { int32_t run = 0; for (int w = 0; w < T / 32; ++w) { const int32_t v = part[w]; part[w] = run; run += v; } }
        __syncthreads();
        int32_t run = part[wid] + incl - local;
        for (int k = lo; k < hi; ++k) { const int32_t c = cnt[k]; bst[k] = run; cnt[k] = run; run += c; }
    }
    __syncthreads();
    for (int li = t; li < nat; li += T) sidx[atomicAdd(&cnt[lbin[li]], 1)] = li;
    __syncthreads();
    for (int b = t; b < nbins; b += T) {   // bins hold a few atoms: insertion sort by index
        const int st = bst[b], en = bst[b + 1];
        for (int p = st + 1; p < en; ++p) {
            const int v = sidx[p];
            int q = p - 1;
            while (q >= st && sidx[q] > v) { sidx[q + 1] = sidx[q]; --q; }
            sidx[q + 1] = v;
        }
        a.bstart[bin0 + b] = a0 + st;
    }
    if (t == 0) a.bstart[bin0 + nbins] = a0 + nat;   // end of the structure's last bin
    __syncthreads();
    for (int p = t; p < nat; p += T) {
        const int i = a0 + sidx[p], P = a0 + p;
        a.bidx[P] = i;
        a.bm[P] = a.am[i];
        a.bpos4[P] = a.pos4[i];
        a.bposd[3 * P] = a.pos[3 * i]; a.bposd[3 * P + 1] = a.pos[3 * i + 1]; a.bposd[3 * P + 2] = a.pos[3 * i + 2];
    }
}

// ---------------------------------------------------------------- atom -> bin
__global__ void k_atom_bin(NbrArgs a) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.natoms) return;
    const StrucGeo& g = a.geo[a.sid[i]];
    int b[3], m[3];
    const int bin = g.bin0 + bin_atom(a, g, i, b, m);
    const int safe_bin = min(bin, a.nbins_cap - 1);
    a.abin[i] = safe_bin;
    a.aslot[i] = atomicAdd(&a.bcount[safe_bin], 1);
}

__global__ void k_bin_scatter(NbrArgs a) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.natoms) return;
    a.bidx[a.bstart[a.abin[i]] + a.aslot[i]] = i;
}

// deterministic order inside each bin (atom index), then the bin-ordered copies
__global__ void k_bin_sort(NbrArgs a, int nbins) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nbins) return;
    const int st = a.bstart[b], en = a.bstart[b + 1];
    for (int p = st + 1; p < en; ++p) {
        const int v = a.bidx[p];
        int q = p - 1;
        while (q >= st && a.bidx[q] > v) { a.bidx[q + 1] = a.bidx[q]; --q; }
        a.bidx[q + 1] = v;
    }
    for (int p = st; p < en; ++p) {
        const int i = a.bidx[p];
        a.bm[p] = a.am[i];
        a.bpos4[p] = a.pos4[i];
        a.bposd[3 * p] = a.pos[3 * i]; a.bposd[3 * p + 1] = a.pos[3 * i + 1]; a.bposd[3 * p + 2] = a.pos[3 * i + 2];
    }
}

// canonical FP64 pair vector, identical association to the oracle: no contraction
static __device__ __forceinline__ void pair_vec_d(const double* xi, const double* xj, const double* R, int n0, int n1, int n2,
                                                  double r[3], double& d2) {
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const double dx = __dsub_rn(xi[c], xj[c]);
        const double s = __dadd_rn(__dadd_rn(__dmul_rn((double)n0, R[c]), __dmul_rn((double)n1, R[3 + c])), __dmul_rn((double)n2, R[6 + c]));
        r[c] = __dsub_rn(dx, s);
    }
    d2 = __dadd_rn(__dadd_rn(__dmul_rn(r[0], r[0]), __dmul_rn(r[1], r[1])), __dmul_rn(r[2], r[2]));
}

// one candidate (j, image n) tested by one lane; accepted entries are compacted into the warp's
// staging row with a ballot
template <bool FP64>
struct Cand {
    int i, cap;
    unsigned lt;
    float4 xi4;
    double xid[3];
    float Rf[9];
    float rc2f;
    double rc2;
    int mi0, mi1, mi2;
    // FP32 lists keep the candidate's pair vector and squared distance in sv for the output pass
    __device__ __forceinline__ void test(const NbrArgs& a, const StrucGeo& g, int c, bool valid, int k0, int k1, int k2,
                                         int32_t* sj, int32_t* simg, int32_t* styp, float4* sv, int& cursor) const {
        bool acc = false;
        int j = 0, n0 = 0, n1 = 0, n2 = 0, tj = 0;
        float rx = 0.0f, ry = 0.0f, rz = 0.0f, d2f = 0.0f;
        if (valid) {
            j = a.bidx[c];
            int mj0, mj1, mj2;
            unpack3(a.bm[c], mj0, mj1, mj2);
            n0 = k0 + mi0 - mj0; n1 = k1 + mi1 - mj1; n2 = k2 + mi2 - mj2;
            const float4 pj = a.bpos4[c];
            tj = __float_as_int(pj.w);
            const float fn0 = (float)n0, fn1 = (float)n1, fn2 = (float)n2;
            rx = (xi4.x - pj.x) - (fn0 * Rf[0] + fn1 * Rf[3] + fn2 * Rf[6]);
            ry = (xi4.y - pj.y) - (fn0 * Rf[1] + fn1 * Rf[4] + fn2 * Rf[7]);
            rz = (xi4.z - pj.z) - (fn0 * Rf[2] + fn1 * Rf[5] + fn2 * Rf[8]);
            d2f = rx * rx + ry * ry + rz * rz;
            acc = d2f < rc2f;
            if (FP64 && acc) {
                double r[3], d2;
                pair_vec_d(xid, a.bposd + 3 * c, g.R, n0, n1, n2, r, d2);
                acc = d2 < rc2;
            }
            if (j == i && n0 == 0 && n1 == 0 && n2 == 0) acc = false;
        }
        const unsigned msk = __ballot_sync(0xffffffffu, acc);
        const int pos = cursor + __popc(msk & lt);
        if (acc && pos < cap) {
            sj[pos] = j; simg[pos] = pack3(n0, n1, n2); styp[pos] = tj;
            if (!FP64) sv[pos] = make_float4(rx, ry, rz, d2f);
        }
        cursor += __popc(msk);
    }
};

constexpr int NBR_WARPS = 4;
constexpr int MAX_RANGES = 128;   // atom ranges per centre atom in the flattened stencil walk (else per-bin walk)
// shared words per warp: staged entries (j, image, type; FP32 lists also the pair vector and d^2,
// 16-byte aligned since cap is a multiple of 32) and the stencil ranges
__host__ __device__ constexpr int nbr_warp_words(int cap, bool fp64) { return 3 * cap + 3 * MAX_RANGES + (fp64 ? 0 : 4 * cap); }

template <bool FP64>
// bounded for eight resident blocks per SM in FP32 (63 registers, no spills), five in FP64
__global__ void __launch_bounds__(NBR_WARPS * 32, FP64 ? 5 : 8) k_neighbors(NbrArgs a) {
    extern __shared__ int32_t nsm[];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int cap = a.cap;
    int32_t* sj = nsm + wid * nbr_warp_words(cap, FP64);
    int32_t* simg = sj + cap;
    int32_t* styp = simg + cap;
    int32_t* rstart = styp + cap;            // first bin-ordered atom of each range
    int32_t* rpre = rstart + MAX_RANGES;     // inclusive prefix of range lengths
    int32_t* rimg = rpre + MAX_RANGES;       // packed image shift k of the range
    float4* sv = reinterpret_cast<float4*>(rimg + MAX_RANGES);   // FP32: pair vector and d^2 per entry
    Cand<FP64> cd;
    const unsigned lt = (1u << lane) - 1u;
    cd.lt = lt;
    cd.cap = cap;
    const float rcf = (float)a.rc;
    cd.rc2f = FP64 ? (rcf + 0.05f) * (rcf + 0.05f) : rcf * rcf;
    cd.rc2 = a.rc * a.rc;
    int wmax = 0;   // the warp's longest row: the host sizes later lists by it (status word 3)
    for (;;) {
        int i = 0;
        if (lane == 0) i = (int)atomicAdd(a.counter, 1u);
        i = __shfl_sync(0xffffffffu, i, 0);
        if (i >= a.natoms) {
            if (lane == 0 && wmax > 0) atomicMax(a.status + 3, wmax);
            break;
        }
        cd.i = i;
        const StrucGeo& g = a.geo[a.sid[i]];
        int b0, b1, b2;
        unpack3(a.abc[i], b0, b1, b2);
        unpack3(a.am[i], cd.mi0, cd.mi1, cd.mi2);
        cd.xi4 = a.pos4[i];
        cd.xid[0] = a.pos[3 * i]; cd.xid[1] = a.pos[3 * i + 1]; cd.xid[2] = a.pos[3 * i + 2];
        const double* xid = cd.xid;
        const float4 xi4 = cd.xi4;
        float Rf[9];
#pragma unroll
        for (int k = 0; k < 9; ++k) { Rf[k] = g.Rf[k]; cd.Rf[k] = Rf[k]; }
        const int nb0 = g.nb[0], nb1 = g.nb[1], nb2 = g.nb[2];
        const int s0 = g.sten[0], s1 = g.sten[1], s2 = g.sten[2];
        const int w1 = 2 * s1 + 1, nrows = w1 * (2 * s2 + 1);
        const int segmax = (2 * s0) / nb0 + 2;
        // orthogonal cells: the centre's fractional coordinates within its cell, for pruning
        // stencil rows whose bins lie farther than rc + 0.05 A (the FP32 pre-filter's margin) and
        // trimming each row to the bins within reach along x. The cell image is the one the
        // binning chose (am) and the coordinate is clamped into the atom's own bin, so that a
        // rounding difference at a cell face cannot move it to the other side of the cell.
        // (FP32: the rounding is far inside the margin; FP64 arithmetic is slow on this part)
        float f0 = 0.0f, f1 = 0.0f, f2 = 0.0f;
        if (g.ortho) {
            const int mi[3] = {cd.mi0, cd.mi1, cd.mi2}, bi[3] = {b0, b1, b2}, nbd[3] = {nb0, nb1, nb2};
            float f[3];
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                const float sd = g.Rif[d] * xi4.x + g.Rif[3 + d] * xi4.y + g.Rif[6 + d] * xi4.z;
                const float inb = __frcp_rn((float)nbd[d]);
                f[d] = fminf(fmaxf(sd - (float)mi[d], (float)bi[d] * inb), (float)(bi[d] + 1) * inb);
            }
            f0 = f[0]; f1 = f[1]; f2 = f[2];
        }
        const float rcm = rcf + 0.05f;
        int cursor = 0;
        if (nrows * segmax <= MAX_RANGES) {
            // ---- flattened walk: each stencil row (e1,e2) contributes <= segmax contiguous atom
            //      ranges (one per x image). Lanes build the rows; the non-empty ranges are
            //      written compactly with the inclusive prefix of their lengths (a count pass,
            //      warp scans, a write pass), and lanes then take consecutive candidates across them
            int nr = 0, total = 0;
            for (int r0 = 0; r0 < nrows; r0 += 32) {
                const int r = r0 + lane;
                int k1 = 0, k2 = 0, rowbin = 0, ubeg = 0, uend = -1;
                if (r < nrows) {
                    const int q = floordiv_small(r, w1);
                    const int e1 = r - q * w1 - s1, e2 = q - s2;
                    const int u1 = b1 + e1, u2 = b2 + e2;
                    k1 = floordiv_small(u1, nb1); k2 = floordiv_small(u2, nb2);
                    const int q1 = u1 - k1 * nb1, q2 = u2 - k2 * nb2;
                    rowbin = g.bin0 + (q2 * nb1 + q1) * nb0;
                    ubeg = b0 - s0; uend = b0 + s0;
                    if (g.ortho) {
                        // distance from the centre to the row's bins across the row (y, z), then
                        // the reach along x: a row of bins beyond rcm is skipped, the others keep
                        // the bins that reach [x - h, x + h], h = sqrt(rcm^2 - dy^2 - dz^2)
                        const float i1 = __frcp_rn((float)nb1), i2 = __frcp_rn((float)nb2);
                        const float dy = fmaxf(0.0f, fmaxf((float)u1 * i1 - f1, f1 - (float)(u1 + 1) * i1)) * g.labs[1];
                        const float dz = fmaxf(0.0f, fmaxf((float)u2 * i2 - f2, f2 - (float)(u2 + 1) * i2)) * g.labs[2];
                        const float rest = rcm * rcm - dy * dy - dz * dz;
                        if (rest <= 0.0f) {
                            uend = ubeg - 1;
                        } else {
                            const float hx = sqrtf(rest) * __frcp_rn(g.labs[0]) * (float)nb0;   // reach in bins
                            const float c0 = f0 * (float)nb0;
                            ubeg = max(ubeg, (int)floorf(c0 - hx));
                            uend = min(uend, (int)floorf(c0 + hx));
                        }
                    }
                }
                int cnt = 0, len_tot = 0;
                for (int u = ubeg, seg = 0; u <= uend && seg < segmax; ++seg) {
                    const int k0 = floordiv_small(u, nb0), q0 = u - k0 * nb0;
                    const int len = min(uend - u + 1, nb0 - q0);
                    const int n = a.bstart[rowbin + q0 + len] - a.bstart[rowbin + q0];
                    cnt += (n > 0); len_tot += n;
                    u += len;
                }
                int ic = cnt, il = len_tot;
#pragma unroll
                for (int off = 1; off < 32; off <<= 1) {
                    const int tc = __shfl_up_sync(0xffffffffu, ic, off), tl = __shfl_up_sync(0xffffffffu, il, off);
                    if (lane >= off) { ic += tc; il += tl; }
                }
                int w = nr + ic - cnt, run = total + il - len_tot;
                for (int u = ubeg, seg = 0; u <= uend && seg < segmax; ++seg) {
                    const int k0 = floordiv_small(u, nb0), q0 = u - k0 * nb0;
                    const int len = min(uend - u + 1, nb0 - q0);
                    const int st = a.bstart[rowbin + q0], n = a.bstart[rowbin + q0 + len] - st;
                    if (n > 0) { rstart[w] = st; run += n; rpre[w] = run; rimg[w] = pack3(k0, k1, k2); ++w; }
                    u += len;
                }
                nr += __shfl_sync(0xffffffffu, ic, 31);
                total += __shfl_sync(0xffffffffu, il, 31);
            }
            __syncwarp();
            int rr = 0;   // this lane's current range (non-empty ranges only, so rpre[nr - 1] = total)
            for (int c0 = 0; c0 < total; c0 += 32) {
                const int c = c0 + lane;
                const bool valid = c < total;
                int k0 = 0, k1 = 0, k2 = 0, ca = 0;
                if (valid) {
                    while (rpre[rr] <= c) ++rr;
                    const int before = (rr == 0) ? 0 : rpre[rr - 1];
                    ca = rstart[rr] + (c - before);
                    unpack3(rimg[rr], k0, k1, k2);
                }
                cd.test(a, g, ca, valid, k0, k1, k2, sj, simg, styp, sv, cursor);
            }
        } else {
            // ---- per-bin walk for cells needing very many images
            for (int e2 = -s2; e2 <= s2; ++e2) {
                const int u2 = b2 + e2, k2 = floordiv_small(u2, nb2), q2 = u2 - k2 * nb2;
                for (int e1 = -s1; e1 <= s1; ++e1) {
                    const int u1 = b1 + e1, k1 = floordiv_small(u1, nb1), q1 = u1 - k1 * nb1;
                    for (int e0 = -s0; e0 <= s0; ++e0) {
                        const int u0 = b0 + e0, k0 = floordiv_small(u0, nb0), q0 = u0 - k0 * nb0;
                        const int bin = g.bin0 + (q2 * nb1 + q1) * nb0 + q0;
                        const int st = a.bstart[bin], en = a.bstart[bin + 1];
                        for (int c0 = st; c0 < en; c0 += 32) cd.test(a, g, c0 + lane, c0 + lane < en, k0, k1, k2, sj, simg, styp, sv, cursor);
                    }
                }
            }
        }
        int cnt = cursor;
        wmax = max(wmax, cnt);
        if (cnt > cap) {
            if (lane == 0) { atomicOr(a.status, (int)ST_NBR_OVERFLOW); atomicMax(a.status + 1, cnt); }
            cnt = cap;
        }
        __syncwarp();
        // stable partition by neighbour type into the output row, with the pair geometry
        const size_t row = (size_t)i * cap;
        int base = 0;
        for (int t = 0; t < a.ntypes; ++t) {
            int ct = 0;
            for (int e0 = 0; e0 < cnt; e0 += 32) {
                const int e = e0 + lane;
                const bool f = (e < cnt) && (styp[e] == t);
                const unsigned msk = __ballot_sync(0xffffffffu, f);
                if (f) {
                    const int o = base + ct + __popc(msk & lt);
                    const int j = sj[e];
                    int n0, n1, n2;
                    unpack3(simg[e], n0, n1, n2);
                    a.nj[row + o] = j;
                    a.nimg[row + o] = simg[e];
                    if (FP64) {
                        double r[3], d2;
                        pair_vec_d(xid, a.pos + 3 * (size_t)j, g.R, n0, n1, n2, r, d2);
                        reinterpret_cast<Vec4d*>(a.nr)[row + o] = Vec4d{r[0], r[1], r[2], sqrt(d2)};
                    } else {
                        const float4 v = sv[e];
                        reinterpret_cast<Vec4f*>(a.nr)[row + o] = Vec4f{v.x, v.y, v.z, sqrtf(v.w)};
                    }
                }
                ct += __popc(msk);
            }
            if (lane == 0) a.ntc[(size_t)i * a.ntypes + t] = ct;
            base += ct;
        }
        if (lane == 0) a.nn[i] = cnt;
        __syncwarp();
    }
}

// Verlet-list refresh: r from current positions and the stored images
template <bool FP64>
__global__ void k_refresh(NbrArgs a) {
    const int lane = threadIdx.x & 31;
    const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (i >= a.natoms) return;
    const StrucGeo& g = a.geo[a.sid[i]];
    double R[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) R[k] = g.R[k];
    const int cnt = a.nn[i];
    const size_t row = (size_t)i * a.cap;
    const double xid[3] = {a.pos[3 * i], a.pos[3 * i + 1], a.pos[3 * i + 2]};
    float Rf[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) Rf[k] = (float)R[k];
    const float4 xi4 = FP64 ? float4{} : a.pos4[i];
    for (int e = lane; e < cnt; e += 32) {
        const int j = a.nj[row + e];
        int n0, n1, n2;
        unpack3(a.nimg[row + e], n0, n1, n2);
        if (FP64) {   // the canonical FP64 pair vector of the list builder
            double r[3], d2;
            pair_vec_d(xid, a.pos + 3 * (size_t)j, R, n0, n1, n2, r, d2);
            reinterpret_cast<Vec4d*>(a.nr)[row + e] = Vec4d{r[0], r[1], r[2], sqrt(d2)};
        } else {      // FP32 from the FP32 position copy, as the list builder's mixed form
            const float4 pj = a.pos4[j];
            const float fn0 = (float)n0, fn1 = (float)n1, fn2 = (float)n2;
            const float rx = (xi4.x - pj.x) - (fn0 * Rf[0] + fn1 * Rf[3] + fn2 * Rf[6]);
            const float ry = (xi4.y - pj.y) - (fn0 * Rf[1] + fn1 * Rf[4] + fn2 * Rf[7]);
            const float rz = (xi4.z - pj.z) - (fn0 * Rf[2] + fn1 * Rf[5] + fn2 * Rf[8]);
            reinterpret_cast<Vec4f*>(a.nr)[row + e] = Vec4f{rx, ry, rz, sqrtf(rx * rx + ry * ry + rz * rz)};
        }
    }
}

bool nbr_local_binning(int max_nat) { return max_nat <= BIN_LOCAL_MAX; }

size_t nbr_smem_bytes(int cap, bool fp64) { return (size_t)NBR_WARPS * nbr_warp_words(cap, fp64) * sizeof(int32_t); }

void launch_neighbors(const NbrArgs& a, bool fp64, cudaStream_t st) {
    if (nbr_local_binning(a.max_nat)) {
        // every structure fits one block's shared memory: geometry and bins by one block each
        if (a.nstruc > 0) ++::ann::g_launch_counter, k_bin_local<<<a.nstruc, BIN_LOCAL_T, 0, st>>>(a);
    } else {
        if (a.nstruc > 0) ++::ann::g_launch_counter, k_struc_geo<<<(a.nstruc + GEO_T - 1) / GEO_T, GEO_T, 0, st>>>(a);
        cudaMemsetAsync(a.bcount, 0, sizeof(int32_t) * (a.nbins_cap + 1), st);
        const int nb = (a.natoms + 255) / 256;
        if (a.natoms > 0) ++::ann::g_launch_counter, k_atom_bin<<<nb, 256, 0, st>>>(a);
        launch_exclusive_scan(a.bcount, a.bstart, a.nbins_cap + 1, a.scan_tmp, st);
        if (a.natoms > 0) ++::ann::g_launch_counter, k_bin_scatter<<<nb, 256, 0, st>>>(a);
        ++::ann::g_launch_counter, k_bin_sort<<<(a.nbins_cap + 255) / 256, 256, 0, st>>>(a, a.nbins_cap);
    }
    cudaMemsetAsync(a.counter, 0, sizeof(uint32_t), st);
    const int warps = NBR_WARPS;
    const size_t smem = (size_t)warps * nbr_warp_words(a.cap, fp64) * sizeof(int32_t);
    int grid = (a.natoms + warps - 1) / warps;
    grid = std::min(grid, std::max(1, (int)a.nsm) * (a.grid_per_sm > 0 ? (int)a.grid_per_sm : 16));
    if (grid < 1) grid = 1;
    if (fp64) ++::ann::g_launch_counter, k_neighbors<true><<<grid, warps * 32, smem, st>>>(a);
    else ++::ann::g_launch_counter, k_neighbors<false><<<grid, warps * 32, smem, st>>>(a);
}

void configure_nbr(int maxsmem) {
    set_max_dynamic_smem(k_neighbors<true>, maxsmem);
    set_max_dynamic_smem(k_neighbors<false>, maxsmem);
}

// FP32 copy of the current positions (the type bits in w are kept)
__global__ void k_pos4(int n, const double* pos, float4* pos4) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 p = pos4[i];
    p.x = (float)pos[3 * (size_t)i]; p.y = (float)pos[3 * (size_t)i + 1]; p.z = (float)pos[3 * (size_t)i + 2];
    pos4[i] = p;
}

void launch_refresh_geometry(const NbrArgs& a, bool fp64, cudaStream_t st) {
    const int threads = 256;
    const int grid = (int)(((long long)a.natoms * 32 + threads - 1) / threads);
    if (grid < 1) return;
    if (!fp64) ++::ann::g_launch_counter, k_pos4<<<(a.natoms + 255) / 256, 256, 0, st>>>(a.natoms, a.pos, a.pos4);
    if (fp64) ++::ann::g_launch_counter, k_refresh<true><<<grid, threads, 0, st>>>(a);
    else ++::ann::g_launch_counter, k_refresh<false><<<grid, threads, 0, st>>>(a);
}

}  // namespace ann
