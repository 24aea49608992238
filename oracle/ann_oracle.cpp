// ============================================================================================
// ann_oracle.cpp -- CPU FP64 restatement of the AtomicNN (markdellostritto/ann) Behler-Parrinello
// energy / force / training path.
//
// TEST INFRASTRUCTURE ONLY. This file is the checker, never the product: only tests/,
// __graft_entry__.smoke() and bench.py's cpu_baseline / reference leg load it. The GPU library
// (ann_gb300/csrc) never links, calls or falls back to anything here.
//
// Every routine restates the reference's own source; the file:line of the followed code is given
// beside each one (paths relative to the reference project's root).
//
// Pinning, against the reference's own sources compiled unmodified by oracle/Makefile (with the
// stand-ins of oracle/ref_shim/ for Eigen and for the src/struc/ headers the snapshot lacks):
//   - special functions, cutoffs and basis functions bit for bit against math/special.cpp,
//     nnp/cutoff.cpp, nnp/basis_radial.cpp and nnp/basis_angular.cpp (_ref/libref_basis.so);
//   - the networks against ml/nn.cpp (_ref/libref_nn.so): initialisation bit for bit, values and
//     gradients within 1e-13;
//   - the assembly against nnp/nnp.cpp and nnp/nnh.cpp (_ref/libref_nnp.so): NNP::symm's
//     symmetry functions bit for bit, NNP::energy / NNP::force / NNP::compute within 1e-13.
// The training loss and the force-term adjoint (nnptef.cpp is stale and does not compile) are
// pinned by finite-difference identities.
//
// Neighbour list: src/struc/ (NeighborList) is missing from the reference snapshot. Its contract
// is rebuilt from the call sites (src/nnp/nnp.cpp:343-348, 478-486): every periodic image j+R*n
// with |x_i - x_j - R*n| < rc except (j==i, n==0); r() = x_i - x_j - R*n ("from J to I").
// The canonical arithmetic (no fused multiply-add, fixed association) is shared with the GPU
// FP64 path so that the two lists agree bit for bit.
// ============================================================================================
#include <array>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <climits>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <stdexcept>
#include <string>
#include <random>
#include <vector>
#include <map>
#include <thread>
#include <algorithm>
#include <sstream>
#include <fstream>

namespace orc {

// ---------------------------------------------------------------- constants (math/const.hpp:9-15)
static const double PI = 3.141592653589793;
static const double Rad2 = 1.414213562373095;
static const double LOG2 = 0.693147180559945;

// ---------------------------------------------------------------- special functions
// coscut / sincut: degree-15/16 Taylor series about pi/2 (math/special.cpp:22-28, 36-42)
static double coscut(double x) {
    x -= 0.5 * PI;
    const double x2 = x * x;
    return x * (-1.0 + x2 * (1.0 / 6.0 + x2 * (-1.0 / 120.0 + x2 * (1.0 / 5040.0 + x2 * (-1.0 / 362880.0 +
           x2 * (1.0 / 39916800.0 + x2 * (-1.0 / 6227020800.0 + x2 * 1.0 / 1307674368000.0)))))));
}
static double sincut(double x) {
    x -= 0.5 * PI;
    const double x2 = x * x;
    return 1.0 + x2 * (-1.0 / 2.0 + x2 * (1.0 / 24.0 + x2 * (-1.0 / 720.0 + x2 * (1.0 / 40320.0 +
           x2 * (-1.0 / 3628800.0 + x2 * (1.0 / 479001600.0 + x2 * (-1.0 / 87178291200.0 +
           x2 * 1.0 / 20922789888000.0)))))));
}
// powint: binary exponentiation (math/special.cpp:140-149)
static double powint(double x, int n) {
    if (n == 0) return 1.0;
    if (x == 0.0) return 0.0;
    int nn = (n > 0) ? n : -n;
    double y = 1.0, w = x;
    for (; nn != 0; nn >>= 1, w *= w)
        if (nn & 1) y *= w;
    return (n > 0) ? y : 1.0 / y;
}
// fmexp: exp(x) = exp2(x*log2(e)); exp2 split into 2^round(x) (exponent bits) times a [2/2]
// Pade approximant of 2^f on [-1/2,1/2] (the Cephes exp2 coefficients), clamped to 0 / +inf
// (math/special.cpp:236-285).
static double exp2_pade(double x) {
    static const double P0 = 2.30933477057345225087e-2, P1 = 2.02020656693165307700e1,
                        P2 = 1.51390680115615096133e3, Q0 = 2.33184211722314911771e2,
                        Q1 = 4.36821166879210612817e3;
    const double ip = std::floor(x + 0.5);
    const double fp = x - ip;
    const uint64_t bits = (uint64_t)(uint32_t)(((int)ip + 1023) << 20) << 32;
    double scale;
    std::memcpy(&scale, &bits, sizeof(double));
    const double x2 = fp * fp;
    double px = P0;
    px = px * x2 + P1;
    double qx = x2 + Q0;
    px = px * x2 + P2;
    qx = qx * x2 + Q1;
    px = px * fp;
    return scale * (1.0 + 2.0 * (px / (qx - px)));
}
static double fmexp(double x) {
    const double LOG2E = 1.4426950408889634074;
    if (x < -1022.0 / LOG2E) return 0;
    if (x > 1023.0 / LOG2E) return INFINITY;
    return exp2_pade(LOG2E * x);
}
// hyperbolic helpers (math/special.cpp:58-96)
static double sp_tanh(double x) {
    if (x >= 0) { const double e = std::exp(-2.0 * x); return (1.0 - e) / (1.0 + e); }
    const double e = std::exp(2.0 * x); return (e - 1.0) / (e + 1.0);
}
static double sp_sech(double x) {
    if (x >= 0) { const double e = std::exp(-x); return 2.0 * e / (1.0 + e * e); }
    const double e = std::exp(x); return 2.0 * e / (e * e + 1.0);
}
static double sp_cosh(double x) {
    if (x >= 0) { const double e = std::exp(-x); return (1.0 + e * e) / (2.0 * e); }
    const double e = std::exp(x); return (e * e + 1.0) / (2.0 * e);
}

// ---------------------------------------------------------------- cutoff (nnp/cutoff.cpp:50-146)
enum { CUT_NONE = 0, CUT_STEP = 1, CUT_COS = 2, CUT_TANH = 3, CUT_POLY3 = 4 };
struct Cutoff {
    int name = CUT_NONE;
    double rc = 0, rci = 0, pirci = 0;
    Cutoff() {}
    Cutoff(int n, double r) : name(n), rc(r) {
        if (n == CUT_NONE) throw std::invalid_argument("Cutoff: invalid name");
        if (r < 0) throw std::invalid_argument("Cutoff: invalid distance");
        rci = 1.0 / rc; pirci = PI / rc;
    }
    double f(double dr) const {  // cutoff.cpp:62-86
        switch (name) {
            case CUT_STEP: return (dr < rc) ? 1.0 : 0.0;
            case CUT_COS: return (dr < rc) ? 0.5 * (coscut(dr * pirci) + 1.0) : 0.0;
            case CUT_TANH: { const double t = (dr > rc) ? 0.0 : std::tanh(1.0 - dr * rci); return t * t * t; }
            case CUT_POLY3: { if (dr < rc) { dr *= rci; return (2.0 * dr - 3.0) * dr * dr + 1.0; } return 0; }
            default: throw std::invalid_argument("Cutoff::f: invalid type");
        }
    }
    double g(double dr) const {  // cutoff.cpp:88-114
        switch (name) {
            case CUT_STEP: return 0.0;
            case CUT_COS: return (dr < rc) ? -0.5 * pirci * sincut(dr * pirci) : 0.0;
            case CUT_TANH: { if (dr < rc) { const double t = std::tanh(1.0 - dr * rci); return -3.0 * t * t * (1.0 - t * t) * rci; } return 0; }
            case CUT_POLY3: { if (dr < rc) { dr *= rci; return 6.0 * dr * (dr - 1.0) * rci; } return 0; }
            default: throw std::invalid_argument("Cutoff::g: invalid type");
        }
    }
};

// ---------------------------------------------------------------- radial basis (nnp/basis_radial.cpp)
enum { R_NONE = 0, R_GAUSSIAN, R_SECH, R_LOGISTIC, R_TANH, R_LOGCOSH, R_LOGCOSH2 };
struct BasisR {
    Cutoff cut;
    int name = R_NONE;
    std::vector<double> rs, eta;
    int size() const { return (int)eta.size(); }
    // basis_radial.cpp:263-309 (writes size() values to out)
    void symm(double dr, double* out) const {
        const double cutf = cut.f(dr);
        const int n = size();
        switch (name) {
            case R_GAUSSIAN: for (int i = 0; i < n; ++i) { const double a = eta[i] * (dr - rs[i]); out[i] = fmexp(-a * a) * cutf; } break;
            case R_SECH: for (int i = 0; i < n; ++i) { const double e = fmexp(-eta[i] * (dr - rs[i])); out[i] = 2.0 * e / (1.0 + e * e) * cutf; } break;
            case R_LOGISTIC: for (int i = 0; i < n; ++i) { const double e = fmexp(-2.0 * eta[i] * (dr - rs[i])); out[i] = 4.0 * e / ((1.0 + e) * (1.0 + e)) * cutf; } break;
            case R_TANH: for (int i = 0; i < n; ++i) out[i] = 0.5 * (std::tanh(-eta[i] * (dr - rs[i])) + 1.0) * cutf; break;
            case R_LOGCOSH: for (int i = 0; i < n; ++i) out[i] = 0.5 * std::log1p(fmexp(-2.0 * eta[i] * (dr - rs[i]))) * cutf; break;
            case R_LOGCOSH2: for (int i = 0; i < n; ++i) { const double a = -eta[i] * (dr - rs[i]); const double e = fmexp(2.0 * Rad2 * a); out[i] = (a == 0.0) ? 0.5 * cutf / Rad2 : a * e / (e - 1.0) * cutf; } break;
            default: throw std::invalid_argument("BasisR::symm: invalid function");
        }
    }
    // basis_radial.cpp:316-376: amp = -sum_i dEdG_i * dG_i/dr
    double force(double dr, const double* dEdG) const {
        double amp = 0;
        const double cutf = cut.f(dr), cutg = cut.g(dr);
        const int n = size();
        switch (name) {
            case R_GAUSSIAN: for (int i = 0; i < n; ++i) { const double a = eta[i] * (dr - rs[i]); amp -= dEdG[i] * fmexp(-a * a) * (-2.0 * eta[i] * a * cutf + cutg); } break;
            case R_SECH: for (int i = 0; i < n; ++i) { const double e = fmexp(-eta[i] * (dr - rs[i])); const double e2 = e * e; const double den = 1.0 / (1.0 + e2); amp -= dEdG[i] * 2.0 * e * den * (-eta[i] * (1.0 - e2) * den * cutf + cutg); } break;
            case R_LOGISTIC: for (int i = 0; i < n; ++i) { const double e2 = fmexp(-2.0 * eta[i] * (dr - rs[i])); const double den = 1.0 / (1.0 + e2); const double th = (1.0 - e2) * den; const double s2 = 4.0 * e2 * den * den; amp -= dEdG[i] * s2 * (-2.0 * eta[i] * th * cutf + cutg); } break;
            case R_TANH: for (int i = 0; i < n; ++i) { const double th = std::tanh(-eta[i] * (dr - rs[i])); amp -= dEdG[i] * 0.5 * (-eta[i] * (1.0 - th * th) * cutf + (1.0 + th) * cutg); } break;
            case R_LOGCOSH: for (int i = 0; i < n; ++i) { const double e = fmexp(-2.0 * eta[i] * (dr - rs[i])); amp -= dEdG[i] * (-eta[i] * e / (1.0 + e) * cutf + 0.5 * std::log1p(e) * cutg); } break;
            case R_LOGCOSH2: for (int i = 0; i < n; ++i) { const double a = -eta[i] * (dr - rs[i]); const double e = fmexp(2.0 * Rad2 * a); const double den = 1.0 / (e - 1.0); const double v = (a == 0.0) ? 0.5 * (-eta[i] * cutg + cutf / Rad2) : e * (eta[i] * (1.0 + 2.0 * Rad2 * a - e) * den * cutf + a * cutg) * den; amp -= dEdG[i] * v; } break;
            default: throw std::invalid_argument("BasisR::force: invalid function");
        }
        return amp;
    }
    // basis_radial.cpp:213-257: dG_i/dr of one function
    double symmd(double dr, int i) const {
        const double cutf = cut.f(dr), cutg = cut.g(dr);
        const double e_ = eta[i], r_ = rs[i];
        switch (name) {
            case R_GAUSSIAN: { const double a = e_ * (dr - r_); return fmexp(-a * a) * (-2.0 * e_ * a * cutf + cutg); }
            case R_SECH: { const double e = fmexp(-e_ * (dr - r_)); const double e2 = e * e; const double den = 1.0 / (1.0 + e2); return 2.0 * e * den * (-1.0 * e_ * (1.0 - e2) * den * cutf + cutg); }
            case R_LOGISTIC: { const double s = sp_sech(e_ * (dr - r_)); const double t = sp_tanh(e_ * (dr - r_)); return s * s * (-2.0 * e_ * t * cutf + cutg); }
            case R_TANH: { const double t = sp_tanh(-e_ * (dr - r_)); return 0.5 * (-e_ * (1.0 - t * t) * cutf + (1.0 + t) * cutg); }
            case R_LOGCOSH: { const double e = fmexp(-2.0 * e_ * (dr - r_)); return -e_ * e / (1.0 + e) * cutf + 0.5 * std::log1p(e) * cutg; }
            case R_LOGCOSH2: { const double a = -e_ * (dr - r_); const double e = fmexp(2.0 * Rad2 * a); const double den = 1.0 / (e - 1.0); return (a == 0.0) ? 0.5 * (-e_ * cutg + cutf / Rad2) : e * (e_ * (1.0 + 2.0 * Rad2 * a - e) * den * cutf + a * cutg) * den; }
            default: throw std::invalid_argument("BasisR::symmd: invalid function");
        }
    }
};

// ---------------------------------------------------------------- angular basis (nnp/basis_angular.cpp)
enum { A_NONE = 0, A_GAUSS, A_GAUSS2, A_SECH, A_STUDENT3, A_STUDENT4, A_STUDENT5 };
struct BasisA {
    Cutoff cut;
    int name = A_NONE;
    std::vector<double> eta, zeta, ieta2, lambdaf, etar, ietar2;
    std::vector<int> lambda, rflag;
    int size() const { return (int)eta.size(); }
    // basis_angular.cpp:178-205: group consecutive equal eta (|d|<1e-6) to share the damping term
    void init() {
        const int n = size();
        ieta2.assign(n, 0); lambdaf.assign(n, 0); rflag.assign(n, 0);
        for (int i = 0; i < n; ++i) { ieta2[i] = 1.0 / (eta[i] * eta[i]); lambdaf[i] = 0.5 * lambda[i]; }
        etar.clear(); ietar2.clear();
        if (n > 0) {
            int flag = 0; rflag[0] = 0; etar.push_back(eta[0]);
            for (int i = 1; i < n; ++i) {
                if (std::fabs(eta[i] - eta[i - 1]) < 1.0e-6) rflag[i] = flag;
                else { rflag[i] = ++flag; etar.push_back(eta[i]); }
            }
            for (double e : etar) ietar2.push_back(1.0 / (e * e));
        }
    }
    static double damp_student(double x, int p) { return powint(1.0 / std::sqrt(1.0 + x), p); }
    // basis_angular.cpp:371-420
    void symm(double dij, double dik, double cs, double* out) const {
        const double cprod = cut.f(dij) * cut.f(dik);
        const double r2s = dij * dij + dik * dik;
        const int n = size(), ng = (int)etar.size();
        std::vector<double> fd(ng);
        switch (name) {
            case A_GAUSS:
                for (int j = 0; j < ng; ++j) fd[j] = cprod * fmexp(-ietar2[j] * r2s);
                for (int i = 0; i < n; ++i) out[i] = std::pow(std::fabs(0.5 + lambdaf[i] * cs), zeta[i]) * fd[rflag[i]];
                break;
            case A_GAUSS2:
                for (int j = 0; j < ng; ++j) fd[j] = fmexp(-0.5 * PI * ietar2[j] * r2s);
                for (int i = 0; i < n; ++i) out[i] = cprod * std::pow(std::fabs(0.5 + lambdaf[i] * cs), zeta[i]) * 2.0 * fd[rflag[i]] / (1.0 + fd[rflag[i]]);
                break;
            case A_SECH:
                for (int j = 0; j < ng; ++j) fd[j] = fmexp(-0.5 * PI * ietar2[j] * r2s);
                for (int i = 0; i < n; ++i) { const double e = fd[rflag[i]]; out[i] = cprod * std::pow(std::fabs(0.5 + lambdaf[i] * cs), zeta[i]) * 2.0 * e / (1.0 + e * e); }
                break;
            case A_STUDENT3: case A_STUDENT4: case A_STUDENT5: {
                const int p = (name == A_STUDENT3) ? 4 : (name == A_STUDENT4) ? 5 : 6;
                for (int j = 0; j < ng; ++j) fd[j] = cprod * damp_student(ietar2[j] * r2s, p);
                for (int i = 0; i < n; ++i) out[i] = std::pow(std::fabs(0.5 + lambdaf[i] * cs), zeta[i]) * fd[rflag[i]];
            } break;
            default: throw std::invalid_argument("BasisA::symm: invalid function");
        }
    }
    // basis_angular.cpp:430-563: phi = -sum dEdG dG/dcos, eta[0/1] = -sum dEdG dG/drij / drik
    void force(double dij, double dik, double cs, double& phi, double* et, const double* dEdG) const {
        const double c0 = cut.f(dij), c1 = cut.f(dik), g0 = cut.g(dij), g1 = cut.g(dik);
        phi = 0; et[0] = 0; et[1] = 0;
        const double r2s = dij * dij + dik * dik;
        const int n = size(), ng = (int)etar.size();
        std::vector<double> fd(ng);
        switch (name) {
            case A_GAUSS: {
                const double d0 = 2.0 * dij * c0, d1 = 2.0 * dik * c1;
                for (int j = 0; j < ng; ++j) fd[j] = fmexp(-ietar2[j] * r2s);
                for (int i = 0; i < n; ++i) {
                    const double cw = std::fabs(0.5 + lambdaf[i] * cs);
                    const double ga = dEdG[i] * std::pow(cw, zeta[i] - 1.0) * fd[rflag[i]];
                    const double fa = cw * ga;
                    phi -= zeta[i] * lambdaf[i] * ga;
                    et[0] -= fa * (-d0 * ieta2[i] + g0);
                    et[1] -= fa * (-d1 * ieta2[i] + g1);
                }
            } break;
            case A_GAUSS2: {
                const double d0 = PI * dij * c0, d1 = PI * dik * c1;
                for (int j = 0; j < ng; ++j) fd[j] = fmexp(-0.5 * PI * ietar2[j] * r2s);
                for (int i = 0; i < n; ++i) {
                    const double e = fd[rflag[i]];
                    const double den = 1.0 / (1.0 + e);
                    const double cw = std::fabs(0.5 + lambdaf[i] * cs);
                    const double ga = dEdG[i] * std::pow(cw, zeta[i] - 1.0) * 2.0 * e * den;
                    const double fa = cw * ga;
                    phi -= zeta[i] * lambdaf[i] * ga;
                    et[0] -= fa * (-d0 * ieta2[i] * den + g0);
                    et[1] -= fa * (-d1 * ieta2[i] * den + g1);
                }
            } break;
            case A_SECH: {
                const double d0 = PI * dij * c0, d1 = PI * dik * c1;
                for (int j = 0; j < ng; ++j) fd[j] = fmexp(-0.5 * PI * ietar2[j] * r2s);
                for (int i = 0; i < n; ++i) {
                    const double e = fd[rflag[i]];
                    const double e2 = e * e;
                    const double den = 1.0 / (1.0 + e2);
                    const double th = (1.0 - e2) * den;
                    const double sh = 2.0 * e * den;
                    const double cw = std::fabs(0.5 + lambdaf[i] * cs);
                    const double ga = std::pow(cw, zeta[i] - 1.0) * dEdG[i] * sh;
                    const double fa = cw * ga;
                    phi -= zeta[i] * lambdaf[i] * ga;
                    et[0] -= fa * (-d0 * ieta2[i] * th + g0);
                    et[1] -= fa * (-d1 * ieta2[i] * th + g1);
                }
            } break;
            case A_STUDENT3: case A_STUDENT4: case A_STUDENT5: {
                const int p = (name == A_STUDENT3) ? 4 : (name == A_STUDENT4) ? 5 : 6;
                const double d0 = p * dij * c0, d1 = p * dik * c1;
                for (int j = 0; j < ng; ++j) fd[j] = 1.0 / std::sqrt(1.0 + ietar2[j] * r2s);
                for (int i = 0; i < n; ++i) {
                    const double den = fd[rflag[i]];
                    const double cw = std::fabs(0.5 + lambdaf[i] * cs);
                    const double ga = std::pow(cw, zeta[i] - 1.0) * dEdG[i] * powint(den, p);
                    const double fa = cw * ga;
                    phi -= zeta[i] * lambdaf[i] * ga;
                    et[0] -= fa * (-d0 * ieta2[i] * den * den + g0);
                    et[1] -= fa * (-d1 * ieta2[i] * den * den + g1);
                }
            } break;
            default: throw std::invalid_argument("BasisA::force: invalid function");
        }
        phi *= c0 * c1; et[0] *= c1; et[1] *= c0;
    }
    // basis_angular.cpp:259-364: per-function partial derivatives (dG/dcos, dG/drij, dG/drik)
    void symmd(int i, double dij, double dik, double cs, double& fphi, double* feta) const {
        const double c0 = cut.f(dij), c1 = cut.f(dik), g0 = cut.g(dij), g1 = cut.g(dik);
        const double lf = 0.5 * lambda[i];
        const double ie2 = 1.0 / (eta[i] * eta[i]);
        const double r2s = dij * dij + dik * dik;
        const double d0 = 2.0 * dij * c0, d1 = 2.0 * dik * c1;
        const double cw = std::fabs(0.5 + lf * cs);
        double ga = 0, fa = 0;
        switch (name) {
            case A_GAUSS: ga = std::pow(cw, zeta[i] - 1.0) * fmexp(-ie2 * r2s); fa = cw * ga;
                fphi = zeta[i] * lf * ga; feta[0] = fa * (-d0 * ie2 + g0); feta[1] = fa * (-d1 * ie2 + g1); break;
            case A_GAUSS2: { const double e = fmexp(-0.5 * PI * ie2 * r2s); const double den = 1.0 / (1.0 + e);
                ga = std::pow(cw, zeta[i] - 1.0) * 2.0 * e * den; fa = cw * ga;
                fphi = zeta[i] * lf * ga; feta[0] = fa * (-d0 * ie2 * 0.5 * PI * den + g0); feta[1] = fa * (-d1 * ie2 * 0.5 * PI * den + g1); } break;
            case A_SECH: { const double e = fmexp(-0.5 * PI * ie2 * r2s); const double e2 = e * e; const double den = 1.0 / (1.0 + e2);
                const double th = (1.0 - e2) * den, sh = 2.0 * e * den;
                ga = std::pow(cw, zeta[i] - 1.0) * sh; fa = cw * ga;
                fphi = zeta[i] * lf * ga; feta[0] = fa * (-d0 * 0.5 * PI * ie2 * th + g0); feta[1] = fa * (-d1 * 0.5 * PI * ie2 * th + g1); } break;
            case A_STUDENT3: case A_STUDENT4: case A_STUDENT5: {
                const int p = (name == A_STUDENT3) ? 4 : (name == A_STUDENT4) ? 5 : 6;
                const double den = 1.0 / std::sqrt(1.0 + ie2 * r2s);
                ga = std::pow(cw, zeta[i] - 1.0) * powint(den, p); fa = cw * ga;
                fphi = zeta[i] * lf * ga; feta[0] = fa * (-d0 * ie2 * p / 2.0 * den * den + g0); feta[1] = fa * (-d1 * ie2 * p / 2.0 * den * den + g1); } break;
            default: throw std::invalid_argument("BasisA::symmd: invalid function");
        }
        fphi *= c0 * c1; feta[0] *= c1; feta[1] *= c0;
    }
};

// ---------------------------------------------------------------- network (ml/nn.cpp)
enum { N_UNKNOWN = 0, N_LINEAR, N_SIGMOID, N_TANH, N_ISRU, N_ARCTAN, N_RELU, N_ELU, N_TANHRE, N_SQRE,
       N_SWISH, N_GELU, N_MISH, N_PFLU, N_SERF, N_LOGISH, N_SOFTPLUS, N_SQPLUS, N_ATISH, N_TEST };
static int neuron_read(const std::string& s) {  // nn.cpp:120-140
    static const char* names[] = {"UNKNOWN", "LINEAR", "SIGMOID", "TANH", "ISRU", "ARCTAN", "RELU", "ELU", "TANHRE", "SQRE",
                                  "SWISH", "GELU", "MISH", "PFLU", "SERF", "LOGISH", "SOFTPLUS", "SQPLUS", "ATISH", "TEST"};
    for (int i = 1; i < 20; ++i) if (s == names[i]) return i;
    return N_UNKNOWN;
}
// activation value, first and second derivative: a and d follow AFFPBP::af_* (nn.cpp:149-810);
// d2 is the exact derivative of d (AFFPBP2 sets d2 = 0 for GELU, MISH, SERF, LOGISH, ATISH and
// TEST and has inexact d2 for ARCTAN, TANHRE and SQRE, nn.cpp:282-444); SERF's d uses erf(fl) for
// its a/z term so that it is finite at z = 0.
static void activate(int neuron, double c, double z, double& a, double& d, double& d2) {
    constexpr double PI = 3.141592653589793, RADPI = 1.772453850905516;   // math/const.hpp:9-10
    switch (neuron) {
        case N_LINEAR: a = z; d = 1.0; d2 = 0.0; return;
        case N_SIGMOID: {
            if (z >= 0) { const double e = std::exp(-c * z); const double f = 1.0 / (1.0 + e); a = f; d = c * e * f * f; d2 = -c * c * e * (1.0 - e) * f * f * f; }
            else { const double e = std::exp(c * z); const double f = 1.0 / (1.0 + e); a = e * f; d = c * e * f * f; d2 = -c * c * e * (e - 1.0) * f * f * f; }
            return;
        }
        case N_TANH: { const double t = std::tanh(c * z); a = t; d = c * (1.0 - t * t); d2 = c * c * (-2.0 * t * (1.0 - t * t)); return; }
        case N_ISRU: {  // nn.cpp:254-266
            const double zz = c * z, isr = 1.0 / std::sqrt(1.0 + zz * zz), isr3 = isr * isr * isr;
            if (zz < -100.0) a = -1.0 / (1.0 + 1.0 / (zz * zz));
            else if (zz > 100.0) a = 1.0 / (1.0 + 1.0 / (zz * zz));
            else a = zz * isr;
            d = c * isr3;
            d2 = -3.0 * c * c * zz * isr3 * isr * isr;
            return;
        }
        case N_ARCTAN: {  // nn.cpp:282-290
            const double zz = c * z * PI / 2.0, fr = 1.0 / (1.0 + zz * zz);
            a = (2.0 / PI) * std::atan(zz); d = c * fr; d2 = -PI * c * c * zz * fr * fr;
            return;
        }
        case N_RELU: if (z > 0.0) { a = z; d = 1.0; } else { a = 0.0; d = 0.0; } d2 = 0.0; return;   // nn.cpp:315-328
        case N_ELU: {  // nn.cpp:353-366
            if (z >= 0.0) { a = z; d = 1.0; d2 = 0.0; }
            else { const double e = std::exp(c * z); a = e - 1.0; d = c * e; d2 = c * c * e; }
            return;
        }
        case N_TANHRE: {  // nn.cpp:393-405
            if (z >= 0) { a = z; d = 1.0; d2 = 0.0; }
            else { const double fe = std::exp(2.0 * c * z); a = (fe - 1.0) / (fe + 1.0); d = c * (1.0 - a * a); d2 = -2.0 * c * a * d; }
            return;
        }
        case N_SQRE: {  // nn.cpp:432-444
            if (z >= 0) { a = z; d = 1.0; d2 = 0.0; }
            else { const double den = 1.0 / std::sqrt(1.0 + z * z), den3 = den * den * den; a = z * den; d = den3; d2 = -3.0 * z * den3 * den * den; }
            return;
        }
        case N_SWISH: {  // nn.cpp:480-498
            const double zz = c * z;
            if (zz > 0.0) {
                const double e = std::exp(-zz), den = 1.0 / (1.0 + e);
                a = z * den; d = (1.0 + e * (1.0 + zz)) * den * den; d2 = c * e * (2.0 - zz + e * (2.0 + zz)) * den * den * den;
            } else {
                const double e = std::exp(zz), den = 1.0 / (1.0 + e);
                a = z * e * den; d = e * (1.0 + zz + e) * den * den; d2 = c * e * (2.0 + zz + e * (2.0 - zz)) * den * den * den;
            }
            return;
        }
        case N_GELU: {  // nn.cpp:505-524
            const double zz = 0.5 * RADPI * c * z, erfp1 = 1.0 + std::erf(zz), g = std::exp(-zz * zz);
            a = 0.5 * z * erfp1; d = 0.5 * (erfp1 + c * z * g); d2 = c * g * (1.0 - zz * zz);
            return;
        }
        case N_MISH: {  // nn.cpp:548-586 (AFFPBP form)
            const double zz = c * z;
            if (zz > 0.0) {
                const double e = std::exp(-zz), e2 = e * e, den = 1.0 / ((1.0 + e) * (1.0 + e) + e2);
                a = z * (1.0 - 2.0 * e2 * den);
                d = 1.0 - 2.0 * e2 * den * (1.0 - 2.0 * zz * (1.0 + e) * den);
                const double t1 = 4.0 * e2 * (1.0 + e) * den * den;
                const double t2 = 4.0 * e2 * den * den * den * (-2.0 - 3.0 * e + 2.0 * e2 + 2.0 * e2 * e);
                d2 = c * (2.0 * t1 + zz * t2);
            } else {
                const double e = std::exp(zz), den = 1.0 / (e * (e + 2.0) + 2.0);
                a = z * e * (e + 2.0) * den;
                d = 1.0 + 2.0 * den * (-1.0 + 2.0 * zz * (1.0 - (e + 2.0) * den));
                const double t1 = 4.0 * e * (e + 1.0) * den * den;
                const double t2 = 4.0 * den * den * den * e * (2.0 + 2.0 * e - 3.0 * e * e - 2.0 * e * e * e);
                d2 = c * (2.0 * t1 + zz * t2);
            }
            return;
        }
        case N_PFLU: {  // nn.cpp:605-618
            const double zz = c * z, z2 = zz * zz, fs = 1.0 / std::sqrt(z2 + 1.0), fs3 = fs * fs * fs;
            a = 0.5 * z * (1.0 + zz * fs); d = 0.5 * (zz * (z2 + 2.0) * fs3 + 1.0); d2 = -0.5 * c * (z2 - 2.0) * fs3 * fs * fs;
            return;
        }
        case N_SERF: {  // nn.cpp:634-646 (no c)
            const double fe = std::exp(z), fl = std::log1p(fe), ef = std::erf(fl), g = std::exp(-fl * fl), s = 1.0 / (1.0 + 1.0 / fe);
            a = z * ef; d = ef + 2.0 / RADPI * g * z * s; d2 = 2.0 / RADPI * g * s * (2.0 - 2.0 * z * fl * s + z * (1.0 - s));
            return;
        }
        case N_LOGISH: {  // nn.cpp:662-680 (no c)
            const double l2i = 1.0 / LOG2, e = std::exp(-z), lf = std::log(1.0 + 1.0 / (1.0 + e));
            const double q = e / ((1.0 + e) * (2.0 + e)), qp = e * (e * e - 2.0) / ((1.0 + e) * (1.0 + e) * (2.0 + e) * (2.0 + e));
            a = l2i * z * lf; d = l2i * (lf + z * q); d2 = l2i * (2.0 * q + z * qp);
            return;
        }
        case N_SOFTPLUS: {
            const double ci = 1.0 / c;
            // AFFPBP::af_softplus branches on z>0 (nn.cpp:694-708); AFFPBP2 on z>=0; identical values.
            if (z > 0.0) { const double e = std::exp(-c * z); const double den = 1.0 / (e + 1.0); a = z + ci * (std::log1p(e) - LOG2); d = 1.0 / (e + 1.0); d2 = c * e * den * den; }
            else { const double e = std::exp(c * z); const double den = 1.0 / (e + 1.0); a = ci * (std::log1p(e) - LOG2); d = e / (e + 1.0); d2 = c * e * den * den; }
            return;
        }
        case N_SQPLUS: {  // nn.cpp:740-750
            const double zz = c * z, fs = std::sqrt(1.0 + zz * zz);
            a = 0.5 / c * (zz - 1.0 + fs); d = 0.5 * (zz / fs + 1.0); d2 = 0.5 * c / (fs * fs * fs);
            return;
        }
        case N_ATISH: {  // nn.cpp:769-779 (no c)
            const double zz = 0.5 * PI * z, fr = 1.0 / (1.0 + zz * zz), at = std::atan(zz);
            a = z * 0.5 * (1.0 + 2.0 / PI * at); d = 0.5 * (1.0 + z * fr) + at / PI; d2 = fr * fr;
            return;
        }
        case N_TEST: {  // nn.cpp:802-812
            const double zz = c * z, z2 = zz * zz, z4 = z2 * z2, den = 1.0 / std::sqrt(std::sqrt(z4 + 1.0));
            const double den4 = den * den * den * den;
            a = 0.5 * z * (1.0 + zz * den); d = 0.5 * (zz * den * (1.0 + 1.0 / (z4 + 1.0)) + 1.0);
            d2 = 0.5 * c * (den + (1.0 - z4) * den * den4 - 5.0 * z4 * den * den4 * den4);
            return;
        }
        default: throw std::invalid_argument("activation not supported by the oracle");
    }
}

struct ANN {
    int nin = 0;
    std::vector<int> nodes;          // nodes per layer (last = outputs)
    int neuron = N_UNKNOWN;
    double c = 1.0;
    std::vector<double> inpw, inpb, outw, outb;
    std::vector<std::vector<double>> b;   // b[l][n]
    std::vector<std::vector<double>> w;   // w[l][n*ni + m] : row-major (rows = outputs of layer l)
    // forward state
    std::vector<double> ins;
    std::vector<std::vector<double>> z, a, d, d2;
    int nlayer() const { return (int)nodes.size(); }
    int ni(int l) const { return l == 0 ? nin : nodes[l - 1]; }
    int size() const { int s = 0; for (int l = 0; l < nlayer(); ++l) s += nodes[l] + nodes[l] * ni(l); return s; }
    // ANN::fpbp2 (nn.cpp:1343-1409): ins = inpw*(inp+inpb); z_l = W_l a_{l-1} + b_l; last layer linear
    double forward(const double* inp) {
        const int L = nlayer();
        ins.assign(nin, 0);
        for (int m = 0; m < nin; ++m) ins[m] = inpw[m] * (inp[m] + inpb[m]);
        z.resize(L); a.resize(L); d.resize(L); d2.resize(L);
        for (int l = 0; l < L; ++l) {
            const int no = nodes[l], nI = ni(l);
            const double* prev = (l == 0) ? ins.data() : a[l - 1].data();
            z[l].assign(no, 0); a[l].assign(no, 0); d[l].assign(no, 0); d2[l].assign(no, 0);
            const int act = (l == L - 1) ? N_LINEAR : neuron;  // nn.cpp:1314-1317
            for (int n = 0; n < no; ++n) {
                double s = b[l][n];
                for (int m = 0; m < nI; ++m) s += w[l][n * nI + m] * prev[m];
                z[l][n] = s;
                activate(act, c, s, a[l][n], d[l][n], d2[l][n]);
            }
        }
        return outb[0] + a[L - 1][0] * outw[0];
    }
    // DODZ::grad (nn.cpp:1801-1824): dodi = outw*dadz_L ... W_0 diag(inpw), evaluated as a row-vector chain
    void dodi(std::vector<double>& out) const {
        const int L = nlayer();
        std::vector<double> cur(nodes[L - 1]);
        for (int n = 0; n < nodes[L - 1]; ++n) cur[n] = outw[n] * d[L - 1][n];
        for (int l = L - 1; l > 0; --l) {
            const int nI = ni(l);
            std::vector<double> nxt(nI, 0.0);
            for (int m = 0; m < nI; ++m) {
                double s = 0;
                for (int n = 0; n < nodes[l]; ++n) s += cur[n] * w[l][n * nI + m];
                nxt[m] = s * d[l - 1][m];
            }
            cur.swap(nxt);
        }
        out.assign(nin, 0.0);
        for (int m = 0; m < nin; ++m) {
            double s = 0;
            for (int n = 0; n < nodes[0]; ++n) s += cur[n] * w[0][n * nin + m];
            out[m] = s * inpw[m];
        }
    }
    // Cost::grad (nn.cpp:1712-1770) with dc/do = dcdo; adds into g (reference packing: all biases
    // by layer, then all weights by layer, each column-major: m outer, n inner; nn.cpp:846-859)
    void cost_grad(double dcdo, double* g) const {
        const int L = nlayer();
        std::vector<std::vector<double>> dz(L);
        dz[L - 1].assign(nodes[L - 1], 0);
        for (int n = 0; n < nodes[L - 1]; ++n) dz[L - 1][n] = dcdo * outw[n] * d[L - 1][n];
        for (int l = L - 1; l > 0; --l) {
            const int nI = ni(l);
            dz[l - 1].assign(nI, 0);
            for (int m = 0; m < nI; ++m) {
                double s = 0;
                for (int n = 0; n < nodes[l]; ++n) s += w[l][n * nI + m] * dz[l][n];
                dz[l - 1][m] = s * d[l - 1][m];
            }
        }
        int cnt = 0;
        for (int l = 0; l < L; ++l) for (int n = 0; n < nodes[l]; ++n) g[cnt++] += dz[l][n];
        for (int l = 0; l < L; ++l) {
            const int nI = ni(l);
            const double* prev = (l == 0) ? ins.data() : a[l - 1].data();
            for (int m = 0; m < nI; ++m) for (int n = 0; n < nodes[l]; ++n) g[cnt++] += dz[l][n] * prev[m];
        }
    }
    // d/dp [ ce*E(G) + ct*(dE/dG . u) ] accumulated into g (same packing as cost_grad).
    // Forward-over-reverse restatement of the mixed second derivative the force term needs
    // (the quantity nnptef.cpp:1748-1820 assembles from D2ODZDI, nn.cpp:2012-2100).
    void jvp_grad(const double* u, double ce, double ct, double* g) const {
        const int L = nlayer();
        // tangent forward: adot_0 = inpw*u ; zdot_l = W_l adot_{l-1} ; adot_l = f'(z_l) zdot_l
        std::vector<std::vector<double>> zd(L), ad(L);
        std::vector<double> ins_d(nin);
        for (int m = 0; m < nin; ++m) ins_d[m] = inpw[m] * u[m];
        for (int l = 0; l < L; ++l) {
            const int nI = ni(l);
            const double* prev = (l == 0) ? ins_d.data() : ad[l - 1].data();
            zd[l].assign(nodes[l], 0); ad[l].assign(nodes[l], 0);
            for (int n = 0; n < nodes[l]; ++n) {
                double s = 0;
                for (int m = 0; m < nI; ++m) s += w[l][n * nI + m] * prev[m];
                zd[l][n] = s; ad[l][n] = d[l][n] * s;
            }
        }
        // reverse: primal adjoint abar (of a_l) and tangent adjoint adbar (of adot_l)
        std::vector<double> abar(nodes[L - 1]), adbar(nodes[L - 1]);
        for (int n = 0; n < nodes[L - 1]; ++n) { abar[n] = ce * outw[n]; adbar[n] = ct * outw[n]; }
        std::vector<std::vector<double>> zbar(L), zdbar(L);
        for (int l = L - 1; l >= 0; --l) {
            const int no = nodes[l], nI = ni(l);
            zbar[l].assign(no, 0); zdbar[l].assign(no, 0);
            for (int n = 0; n < no; ++n) {
                zdbar[l][n] = d[l][n] * adbar[n];
                zbar[l][n] = d[l][n] * abar[n] + d2[l][n] * zd[l][n] * adbar[n];
            }
            if (l > 0) {
                std::vector<double> na(nI, 0), nad(nI, 0);
                for (int m = 0; m < nI; ++m) {
                    double s = 0, sd = 0;
                    for (int n = 0; n < no; ++n) { s += w[l][n * nI + m] * zbar[l][n]; sd += w[l][n * nI + m] * zdbar[l][n]; }
                    na[m] = s; nad[m] = sd;
                }
                abar.swap(na); adbar.swap(nad);
            }
        }
        int cnt = 0;
        for (int l = 0; l < L; ++l) for (int n = 0; n < nodes[l]; ++n) g[cnt++] += zbar[l][n];
        for (int l = 0; l < L; ++l) {
            const int nI = ni(l);
            const double* prev = (l == 0) ? ins.data() : a[l - 1].data();
            const double* prevd = (l == 0) ? ins_d.data() : ad[l - 1].data();
            for (int m = 0; m < nI; ++m)
                for (int n = 0; n < nodes[l]; ++n) g[cnt++] += zbar[l][n] * prev[m] + zdbar[l][n] * prevd[m];
        }
    }
    void pack(double* p) const {  // operator>> (nn.cpp:846-859)
        int cnt = 0;
        for (int l = 0; l < nlayer(); ++l) for (int n = 0; n < nodes[l]; ++n) p[cnt++] = b[l][n];
        for (int l = 0; l < nlayer(); ++l) { const int nI = ni(l); for (int m = 0; m < nI; ++m) for (int n = 0; n < nodes[l]; ++n) p[cnt++] = w[l][n * nI + m]; }
    }
    void unpack(const double* p) {  // operator<< (nn.cpp:867-880)
        int cnt = 0;
        for (int l = 0; l < nlayer(); ++l) for (int n = 0; n < nodes[l]; ++n) b[l][n] = p[cnt++];
        for (int l = 0; l < nlayer(); ++l) { const int nI = ni(l); for (int m = 0; m < nI; ++m) for (int n = 0; n < nodes[l]; ++n) w[l][n * nI + m] = p[cnt++]; }
    }
};

// ---------------------------------------------------------------- potential (nnp/nnh.cpp, nnp/nnp.cpp)
struct NNH {
    std::string name;
    double mass = 0, energy = 0;
    std::vector<BasisR> R;      // by neighbour type J
    std::vector<BasisA> A;      // TensorTri order: index(j,k) = max*(max+1)/2 + min (tensortri.hpp:194-199)
    std::vector<int> offR, offA;
    int nInputR = 0, nInputA = 0, nInput = 0;
    ANN nn;
    // NNH::init_input (nnh.cpp:94-116)
    void init_input() {
        nInputR = 0; offR.assign(R.size(), 0);
        for (size_t i = 0; i < R.size(); ++i) { nInputR += R[i].size(); offR[i] = (i == 0) ? 0 : offR[i - 1] + R[i - 1].size(); }
        nInputA = 0; offA.assign(A.size(), 0);
        for (size_t i = 0; i < A.size(); ++i) { nInputA += A[i].size(); offA[i] = (i == 0) ? 0 : offA[i - 1] + A[i - 1].size(); }
        nInput = nInputR + nInputA;
    }
};
static int tri(int i, int j) { return (i > j) ? i * (i + 1) / 2 + j : j * (j + 1) / 2 + i; }

struct NNP {
    double rc = 0;
    std::vector<NNH> h;
    std::map<std::string, int> index;
    int ntypes() const { return (int)h.size(); }
    int nparams() const { int s = 0; for (auto& x : h) s += x.nn.size(); return s; }
};

// ---- text reader for the reference 'ann' format (nnp.cpp:243-307, basis_radial.cpp:123-143,
// basis_angular.cpp:116-138, nn.cpp:1495-1578, type.cpp:35-80)
struct Lines {
    std::vector<std::vector<std::string>> v;
    size_t pos = 0;
    explicit Lines(const std::string& text) {
        std::istringstream is(text);
        std::string line;
        while (std::getline(is, line)) {
            std::vector<std::string> toks;
            std::istringstream ls(line);
            std::string t;
            while (ls >> t) toks.push_back(t);
            v.push_back(toks);
        }
    }
    const std::vector<std::string>& next() {
        if (pos >= v.size()) throw std::runtime_error("unexpected end of potential file");
        return v[pos++];
    }
};
static int cut_read(const std::string& s) {
    if (s == "STEP") return CUT_STEP; if (s == "COS") return CUT_COS; if (s == "TANH") return CUT_TANH; if (s == "POLY3") return CUT_POLY3;
    throw std::invalid_argument("invalid cutoff name " + s);
}
static int radial_read(const std::string& s) {
    if (s == "GAUSSIAN") return R_GAUSSIAN; if (s == "SECH") return R_SECH; if (s == "LOGISTIC") return R_LOGISTIC;
    if (s == "TANH") return R_TANH; if (s == "LOGCOSH") return R_LOGCOSH; if (s == "LOGCOSH2") return R_LOGCOSH2;
    throw std::invalid_argument("invalid radial function " + s);
}
static int angular_read(const std::string& s) {
    if (s == "GAUSS") return A_GAUSS; if (s == "GAUSS2") return A_GAUSS2; if (s == "SECH") return A_SECH;
    if (s == "STUDENT3") return A_STUDENT3; if (s == "STUDENT4") return A_STUDENT4; if (s == "STUDENT5") return A_STUDENT5;
    throw std::invalid_argument("invalid angular function " + s);
}
static const std::string& tok(const std::vector<std::string>& l, size_t i) {
    if (i >= l.size()) throw std::runtime_error("malformed potential line");
    return l[i];
}
static void read_basisR(Lines& L, BasisR& b) {
    const auto& hd = L.next();
    b.cut = Cutoff(cut_read(tok(hd, 1)), std::atof(tok(hd, 2).c_str()));
    b.name = radial_read(tok(hd, 3));
    const int n = std::atoi(tok(hd, 4).c_str());
    b.rs.assign(n, 0); b.eta.assign(n, 0);
    for (int i = 0; i < n; ++i) { const auto& l = L.next(); b.rs[i] = std::atof(tok(l, 0).c_str()); b.eta[i] = std::atof(tok(l, 1).c_str()); }
}
static void read_basisA(Lines& L, BasisA& b) {
    const auto& hd = L.next();
    b.cut = Cutoff(cut_read(tok(hd, 1)), std::atof(tok(hd, 2).c_str()));
    b.name = angular_read(tok(hd, 3));
    const int n = std::atoi(tok(hd, 4).c_str());
    b.eta.assign(n, 0); b.zeta.assign(n, 0); b.lambda.assign(n, 0);
    for (int i = 0; i < n; ++i) {
        const auto& l = L.next();
        b.eta[i] = std::atof(tok(l, 0).c_str()); b.zeta[i] = std::atof(tok(l, 1).c_str()); b.lambda[i] = std::atoi(tok(l, 2).c_str());
    }
    b.init();
}
static void read_ann(Lines& L, ANN& nn) {
    const auto& cfg = L.next();
    std::vector<int> nodes;
    for (size_t i = 1; i < cfg.size(); ++i) nodes.push_back(std::atoi(cfg[i].c_str()));
    if (nodes.size() < 2) throw std::runtime_error("invalid network configuration");
    nn.nin = nodes[0];
    nn.nodes.assign(nodes.begin() + 1, nodes.end());
    const auto& ne = L.next();
    nn.neuron = neuron_read(tok(ne, 1));
    nn.c = std::atof(tok(ne, 2).c_str());
    if (nn.neuron == N_UNKNOWN) throw std::invalid_argument("invalid neuron");
    const int nout = nn.nodes.back();
    auto readvec = [&](std::vector<double>& v, int n) {
        const auto& l = L.next(); v.assign(n, 0);
        for (int i = 0; i < n; ++i) v[i] = std::atof(tok(l, i + 1).c_str());
    };
    readvec(nn.inpw, nn.nin); readvec(nn.outw, nout); readvec(nn.inpb, nn.nin); readvec(nn.outb, nout);
    const int Lyr = nn.nlayer();
    nn.b.resize(Lyr); nn.w.resize(Lyr);
    for (int l = 0; l < Lyr; ++l) readvec(nn.b[l], nn.nodes[l]);
    for (int l = 0; l < Lyr; ++l) readvec(nn.w[l], nn.nodes[l] * nn.ni(l));  // written row-major (nn.cpp:1465-1473)
}
static void read_nnp(const std::string& text, NNP& p) {
    Lines L(text);
    L.next();  // header "ann"
    const int nt = std::atoi(tok(L.next(), 1).c_str());
    if (nt <= 0) throw std::invalid_argument("invalid number of types");
    p.h.assign(nt, NNH());
    p.index.clear();
    for (int n = 0; n < nt; ++n) {  // Type::read (type.cpp:35-80): tagged values
        const auto& l = L.next();
        for (size_t i = 0; i + 1 < l.size(); i += 2) {
            std::string tag = l[i];
            for (auto& ch : tag) ch = (char)std::toupper((unsigned char)ch);
            if (tag == "NAME") p.h[n].name = l[i + 1];
            else if (tag == "MASS") p.h[n].mass = std::atof(l[i + 1].c_str());
            else if (tag == "ENERGY") p.h[n].energy = std::atof(l[i + 1].c_str());
        }
        p.index[p.h[n].name] = n;
    }
    p.rc = std::atof(tok(L.next(), 1).c_str());
    if (p.rc <= 0) throw std::invalid_argument("invalid cutoff");
    for (auto& x : p.h) { x.R.assign(nt, BasisR()); x.A.assign(nt * (nt + 1) / 2, BasisA()); }
    auto idx = [&](const std::string& s) { auto it = p.index.find(s); if (it == p.index.end()) throw std::invalid_argument("unknown type " + s); return it->second; };
    for (int i = 0; i < nt; ++i) {
        const int II = idx(tok(L.next(), 1));
        for (int j = 0; j < nt; ++j) { const int JJ = idx(tok(L.next(), 1)); read_basisR(L, p.h[II].R[JJ]); }
        for (int j = 0; j < nt; ++j) for (int k = j; k < nt; ++k) {
            const auto& l = L.next();
            const int JJ = idx(tok(l, 1)), KK = idx(tok(l, 2));
            read_basisA(L, p.h[II].A[tri(JJ, KK)]);
        }
    }
    for (auto& x : p.h) x.init_input();
    for (int n = 0; n < nt; ++n) {
        const int II = idx(tok(L.next(), 1));
        read_ann(L, p.h[II].nn);
        if (p.h[II].nn.nin != p.h[II].nInput) throw std::invalid_argument("network input size does not match the basis");
    }
}

// ---------------------------------------------------------------- neighbour list
struct Neigh { int j; int n[3]; double r[3]; double d; };
static void inv3(const double* R, double* Ri) {  // R column-major: R[3*c + r]
    auto at = [&](int r, int c) { return R[3 * c + r]; };
    const double det = at(0, 0) * (at(1, 1) * at(2, 2) - at(1, 2) * at(2, 1)) - at(0, 1) * (at(1, 0) * at(2, 2) - at(1, 2) * at(2, 0)) + at(0, 2) * (at(1, 0) * at(2, 1) - at(1, 1) * at(2, 0));
    if (det == 0) throw std::invalid_argument("singular cell");
    const double id = 1.0 / det;
    double m[3][3];
    m[0][0] = (at(1, 1) * at(2, 2) - at(1, 2) * at(2, 1)) * id; m[0][1] = (at(0, 2) * at(2, 1) - at(0, 1) * at(2, 2)) * id; m[0][2] = (at(0, 1) * at(1, 2) - at(0, 2) * at(1, 1)) * id;
    m[1][0] = (at(1, 2) * at(2, 0) - at(1, 0) * at(2, 2)) * id; m[1][1] = (at(0, 0) * at(2, 2) - at(0, 2) * at(2, 0)) * id; m[1][2] = (at(0, 2) * at(1, 0) - at(0, 0) * at(1, 2)) * id;
    m[2][0] = (at(1, 0) * at(2, 1) - at(1, 1) * at(2, 0)) * id; m[2][1] = (at(0, 1) * at(2, 0) - at(0, 0) * at(2, 1)) * id; m[2][2] = (at(0, 0) * at(1, 1) - at(0, 1) * at(1, 0)) * id;
    for (int r = 0; r < 3; ++r) for (int c = 0; c < 3; ++c) Ri[3 * c + r] = m[r][c];
}
// canonical pair vector: r = (x_i - x_j) - ((n0*R[:,0] + n1*R[:,1]) + n2*R[:,2]); d2 = (rx^2+ry^2)+rz^2
static inline void pair_vec(const double* xi, const double* xj, const double* R, const int* n, double* r, double& d2) {
    for (int c = 0; c < 3; ++c) {
        const double dx = xi[c] - xj[c];
        const double s = (((double)n[0] * R[c]) + ((double)n[1] * R[3 + c])) + ((double)n[2] * R[6 + c]);
        r[c] = dx - s;
    }
    d2 = (r[0] * r[0] + r[1] * r[1]) + r[2] * r[2];
}
// The periodic-image neighbour list (the NeighborList(struc, rc) contract): every (j, n) with
// |x_i - x_j - R n| < rc except (i, 0), each row ordered by j ascending, then n lexicographic.
// Rows [i0, i1) are filled (out sized to N by the caller), so threads can share one structure.
// Small cells (fewer than three bins of width >= rc along some lattice direction) take the brute
// force over all atoms and images; larger ones a cell-binned search that tests the same pairs with
// the same formula and sorts each row into the same order.
struct NeighborGrid {
    int N = 0;
    const double* x = nullptr;
    const double* R = nullptr;
    double rc = 0, Ri[9], gn[3];
    std::vector<double> s;                 // fractional coordinates
    bool binned = false;
    int nb[3] = {1, 1, 1};
    std::vector<int> k, bin, start, list;  // floor(s) per atom and direction; bin of each atom; CSR of the bins
    NeighborGrid(int N_, const double* x_, const double* R_, double rc_) : N(N_), x(x_), R(R_), rc(rc_) {
        inv3(R, Ri);
        for (int d = 0; d < 3; ++d) gn[d] = std::sqrt(Ri[d] * Ri[d] + Ri[3 + d] * Ri[3 + d] + Ri[6 + d] * Ri[6 + d]);
        s.resize(3 * (size_t)N);
        for (int i = 0; i < N; ++i) for (int d = 0; d < 3; ++d) s[3 * i + d] = Ri[d] * x[3 * i] + Ri[3 + d] * x[3 * i + 1] + Ri[6 + d] * x[3 * i + 2];
        binned = N > 512;
        for (int d = 0; d < 3; ++d) {
            // bins at least rc (plus a margin for rounding) high along lattice direction d
            nb[d] = (int)std::floor(1.0 / (rc * gn[d] * (1.0 + 1e-9)));
            if (nb[d] < 3) binned = false;
        }
        if (!binned) return;
        k.resize(3 * (size_t)N);
        bin.resize(N);
        const long long nbins = (long long)nb[0] * nb[1] * nb[2];
        start.assign(nbins + 1, 0);
        for (int i = 0; i < N; ++i) {
            int b[3];
            for (int d = 0; d < 3; ++d) {
                const double fl = std::floor(s[3 * i + d]);
                k[3 * i + d] = (int)fl;
                b[d] = std::min(nb[d] - 1, std::max(0, (int)std::floor((s[3 * i + d] - fl) * nb[d])));
            }
            bin[i] = (b[0] * nb[1] + b[1]) * nb[2] + b[2];
            ++start[bin[i] + 1];
        }
        for (long long q = 0; q < nbins; ++q) start[q + 1] += start[q];
        list.resize(N);
        std::vector<int> fill(start.begin(), start.end() - 1);
        for (int i = 0; i < N; ++i) list[fill[bin[i]]++] = i;
    }
    void test(int i, int j, const int* n, std::vector<Neigh>& row) const {
        if (j == i && n[0] == 0 && n[1] == 0 && n[2] == 0) return;
        Neigh e; double d2;
        pair_vec(x + 3 * i, x + 3 * j, R, n, e.r, d2);
        if (d2 < rc * rc) { e.j = j; e.n[0] = n[0]; e.n[1] = n[1]; e.n[2] = n[2]; e.d = std::sqrt(d2); row.push_back(e); }
    }
    void rows(int i0, int i1, std::vector<std::vector<Neigh>>& out) const {
        for (int i = i0; i < i1; ++i) {
            std::vector<Neigh>& row = out[i];
            row.clear();
            if (!binned) {
                for (int j = 0; j < N; ++j) {
                    int lo[3], hi[3];
                    for (int d = 0; d < 3; ++d) {
                        const double ds = s[3 * i + d] - s[3 * j + d];
                        const double rr = rc * gn[d];
                        lo[d] = (int)std::floor(ds - rr) - 1; hi[d] = (int)std::ceil(ds + rr) + 1;
                    }
                    int n[3];
                    for (n[0] = lo[0]; n[0] <= hi[0]; ++n[0]) for (n[1] = lo[1]; n[1] <= hi[1]; ++n[1]) for (n[2] = lo[2]; n[2] <= hi[2]; ++n[2])
                        test(i, j, n, row);
                }
                continue;
            }
            // the 27 bins around i's (nb >= 3: each neighbour bin and image shift is visited once);
            // an atom j of bin t' = t mod nb, reached through t = b_i + delta, is the image whose
            // wrapped fractional position lies in t: n = floor(t / nb) + floor(s_i) - floor(s_j)
            const int bi = bin[i];
            const int b0 = bi / (nb[1] * nb[2]), b1 = (bi / nb[2]) % nb[1], b2 = bi % nb[2];
            for (int d0 = -1; d0 <= 1; ++d0) for (int d1 = -1; d1 <= 1; ++d1) for (int d2 = -1; d2 <= 1; ++d2) {
                const int t[3] = {b0 + d0, b1 + d1, b2 + d2};
                int tw[3], wrap[3];
                for (int d = 0; d < 3; ++d) {
                    wrap[d] = (t[d] < 0) ? -1 : (t[d] >= nb[d]) ? 1 : 0;
                    tw[d] = t[d] - wrap[d] * nb[d];
                }
                const int tb = (tw[0] * nb[1] + tw[1]) * nb[2] + tw[2];
                for (int q = start[tb]; q < start[tb + 1]; ++q) {
                    const int j = list[q];
                    int n[3];
                    for (int d = 0; d < 3; ++d) n[d] = wrap[d] + k[3 * i + d] - k[3 * j + d];
                    test(i, j, n, row);
                }
            }
            std::sort(row.begin(), row.end(), [](const Neigh& a, const Neigh& b) {
                if (a.j != b.j) return a.j < b.j;
                if (a.n[0] != b.n[0]) return a.n[0] < b.n[0];
                if (a.n[1] != b.n[1]) return a.n[1] < b.n[1];
                return a.n[2] < b.n[2];
            });
        }
    }
};
static void neighbors(int N, const double* x, const double* R, double rc, std::vector<std::vector<Neigh>>& out) {
    NeighborGrid g(N, x, R, rc);
    out.assign(N, {});
    g.rows(0, N, out);
}
// brute force over all atoms and all images (kept as the definition the binned search is checked against)
static void neighbors_brute(int N, const double* x, const double* R, double rc, std::vector<std::vector<Neigh>>& out) {
    double Ri[9];
    inv3(R, Ri);
    double gn[3];
    for (int d = 0; d < 3; ++d) gn[d] = std::sqrt(Ri[d] * Ri[d] + Ri[3 + d] * Ri[3 + d] + Ri[6 + d] * Ri[6 + d]);
    std::vector<double> s(3 * (size_t)N);
    for (int i = 0; i < N; ++i) for (int d = 0; d < 3; ++d) s[3 * i + d] = Ri[d] * x[3 * i] + Ri[3 + d] * x[3 * i + 1] + Ri[6 + d] * x[3 * i + 2];
    const double rc2 = rc * rc;
    out.assign(N, {});
    for (int i = 0; i < N; ++i) {
        for (int j = 0; j < N; ++j) {
            int lo[3], hi[3];
            for (int d = 0; d < 3; ++d) {
                const double ds = s[3 * i + d] - s[3 * j + d];
                const double rr = rc * gn[d];
                lo[d] = (int)std::floor(ds - rr) - 1; hi[d] = (int)std::ceil(ds + rr) + 1;
            }
            int n[3];
            for (n[0] = lo[0]; n[0] <= hi[0]; ++n[0]) for (n[1] = lo[1]; n[1] <= hi[1]; ++n[1]) for (n[2] = lo[2]; n[2] <= hi[2]; ++n[2]) {
                if (j == i && n[0] == 0 && n[1] == 0 && n[2] == 0) continue;
                Neigh e; double d2;
                pair_vec(x + 3 * i, x + 3 * j, R, n, e.r, d2);
                if (d2 < rc2) { e.j = j; e.n[0] = n[0]; e.n[1] = n[1]; e.n[2] = n[2]; e.d = std::sqrt(d2); out[i].push_back(e); }
            }
        }
    }
}

// ---------------------------------------------------------------- NNP loops (nnp/nnp.cpp)
struct Struc {
    int N = 0;
    const double* x = nullptr;
    const int* type = nullptr;
    const double* R = nullptr;
    std::vector<std::vector<Neigh>> nl;
    std::vector<std::vector<double>> symm;
};
// NNP::symm (nnp.cpp:333-375), rows [i0, i1) (s.symm sized to N by the caller)
static void compute_symm_rows(const NNP& p, Struc& s, int i0, int i1) {
    std::vector<double> buf(256);
    for (int i = i0; i < i1; ++i) {
        const NNH& h = p.h[s.type[i]];
        std::vector<double>& G = s.symm[i];
        G.assign(h.nInput, 0.0);
        const auto& nl = s.nl[i];
        for (size_t j = 0; j < nl.size(); ++j) {
            const int JJ = s.type[nl[j].j];
            const BasisR& br = h.R[JJ];
            if ((int)buf.size() < br.size()) buf.resize(br.size());
            br.symm(nl[j].d, buf.data());
            for (int m = 0; m < br.size(); ++m) G[h.offR[JJ] + m] += buf[m];
            for (size_t k = j + 1; k < nl.size(); ++k) {
                const int KK = s.type[nl[k].j];
                const double* rij = nl[j].r; const double* rik = nl[k].r;
                const double cs = (rij[0] * rik[0] + rij[1] * rik[1] + rij[2] * rik[2]) / (nl[j].d * nl[k].d);
                const BasisA& ba = h.A[tri(JJ, KK)];
                if ((int)buf.size() < ba.size()) buf.resize(ba.size());
                ba.symm(nl[j].d, nl[k].d, cs, buf.data());
                const int oA = h.nInputR + h.offA[tri(JJ, KK)];
                for (int m = 0; m < ba.size(); ++m) G[oA + m] += buf[m];
            }
        }
    }
}
static void compute_symm(const NNP& p, Struc& s) {
    s.symm.assign(s.N, {});
    compute_symm_rows(p, s, 0, s.N);
}
// newton: 1 = Newton-3rd term for every neighbour entry (images included);
//         0 = only for the untranslated image n == 0 (the verlet::List rule of nnp.cpp:550)
// Returns E (network outputs + per-type vacuum energies, as NNH::energy nnh.cpp:118-121 /
// PotNNPE::compute pot_nnpe.cpp:220); forces into F (3N); virial W = sum r_ij (x) v_ij into W (9, row-major W[a*3+b]).
// Optional: dEdG per atom (out), atomic energies.
// compute_force_rows adds the contributions of centre atoms [i0, i1) to F and W and returns their
// energy (dEdG_out sized to N by the caller).
static double compute_force_rows(NNP& p, Struc& s, double* F, double* W, int newton, std::vector<std::vector<double>>* dEdG_out,
                                 double* Eatom, int i0, int i1) {
    double E = 0;
    std::vector<double> dEdG;
    for (int i = i0; i < i1; ++i) {
        NNH& h = p.h[s.type[i]];
        const double ei = h.nn.forward(s.symm[i].data()) + h.energy;
        E += ei;
        if (Eatom) Eatom[i] = ei;
        h.nn.dodi(dEdG);
        if (dEdG_out) (*dEdG_out)[i] = dEdG;
        const auto& nl = s.nl[i];
        // nnp.cpp:623-664
        for (size_t j = 0; j < nl.size(); ++j) {
            const int JJ = s.type[nl[j].j];
            const int jj = nl[j].j;
            const bool jmin = newton ? true : (nl[j].n[0] == 0 && nl[j].n[1] == 0 && nl[j].n[2] == 0);
            const double* rIJ = nl[j].r;
            const double dIJ = nl[j].d, dIJi = 1.0 / dIJ;
            const double amp = h.R[JJ].force(dIJ, dEdG.data() + h.offR[JJ]) * dIJi;
            for (int c = 0; c < 3; ++c) { F[3 * i + c] += amp * rIJ[c]; if (jmin) F[3 * jj + c] -= amp * rIJ[c]; }
            if (W) for (int a = 0; a < 3; ++a) for (int b = 0; b < 3; ++b) W[3 * a + b] += rIJ[a] * amp * rIJ[b];
            for (size_t k = j + 1; k < nl.size(); ++k) {
                const int KK = s.type[nl[k].j];
                const int kk = nl[k].j;
                const bool kmin = newton ? true : (nl[k].n[0] == 0 && nl[k].n[1] == 0 && nl[k].n[2] == 0);
                const double* rIK = nl[k].r;
                const double dIK = nl[k].d, dIKi = 1.0 / dIK;
                const int oA = h.nInputR + h.offA[tri(JJ, KK)];
                double phi = 0, et[2] = {0, 0};
                const double cs = (rIJ[0] * rIK[0] + rIJ[1] * rIK[1] + rIJ[2] * rIK[2]) * dIJi * dIKi;
                h.A[tri(JJ, KK)].force(dIJ, dIK, cs, phi, et, dEdG.data() + oA);
                double vj[3], vk[3];
                for (int c = 0; c < 3; ++c) {
                    vj[c] = (-phi * cs * dIJi + et[0]) * rIJ[c] * dIJi + phi * dIJi * rIK[c] * dIKi;
                    vk[c] = (-phi * cs * dIKi + et[1]) * rIK[c] * dIKi + phi * dIKi * rIJ[c] * dIJi;
                    F[3 * i + c] += (phi * (dIKi - cs * dIJi) + et[0]) * rIJ[c] * dIJi + (phi * (dIJi - cs * dIKi) + et[1]) * rIK[c] * dIKi;
                    if (jmin) F[3 * jj + c] -= vj[c];
                    if (kmin) F[3 * kk + c] -= vk[c];
                }
                if (W) for (int a = 0; a < 3; ++a) for (int b = 0; b < 3; ++b) W[3 * a + b] += rIJ[a] * vj[b] + rIK[a] * vk[b];
            }
        }
    }
    return E;
}
static double compute_force(NNP& p, Struc& s, double* F, double* W, int newton,
                            std::vector<std::vector<double>>* dEdG_out = nullptr, double* Eatom = nullptr) {
    for (int i = 0; i < 3 * s.N; ++i) F[i] = 0;
    if (W) for (int i = 0; i < 9; ++i) W[i] = 0;
    if (dEdG_out) dEdG_out->assign(s.N, {});
    return compute_force_rows(p, s, F, W, newton, dEdG_out, Eatom, 0, s.N);
}
// One structure on nthreads threads, its atoms in contiguous blocks (the atom split of the
// reference's two-tier parallelism, nnptef.cpp:1607-1669): neighbour rows, symmetry functions and
// force contributions per block, each thread with its own NNP copy and force / virial buffers, the
// blocks' sums added in block order. Fills s.nl and s.symm; returns E.
static double compute_struc_threaded(const NNP& p0, Struc& s, double* F, double* W, int newton,
                                     std::vector<std::vector<double>>* dEdG_out, int nthreads) {
    const int N = s.N;
    nthreads = std::max(1, std::min(nthreads, N));
    auto block = [&](int t, int& lo, int& hi) {
        const int q = N / nthreads, r = N % nthreads;
        lo = t * q + std::min(t, r); hi = lo + q + (t < r ? 1 : 0);
    };
    std::vector<std::string> errs(nthreads);
    auto par = [&](auto fn) {
        std::vector<std::thread> th;
        auto run = [&](int t) { try { int lo, hi; block(t, lo, hi); fn(t, lo, hi); } catch (std::exception& e) { errs[t] = e.what(); } };
        for (int t = 1; t < nthreads; ++t) th.emplace_back(run, t);
        run(0);
        for (auto& x : th) x.join();
        for (auto& e : errs) if (!e.empty()) throw std::runtime_error(e);
    };
    NeighborGrid g(N, s.x, s.R, p0.rc);
    s.nl.assign(N, {});
    par([&](int, int lo, int hi) { g.rows(lo, hi, s.nl); });
    s.symm.assign(N, {});
    par([&](int, int lo, int hi) { compute_symm_rows(p0, s, lo, hi); });
    if (dEdG_out) dEdG_out->assign(N, {});
    std::vector<std::vector<double>> Ft(nthreads, std::vector<double>(F ? 3 * (size_t)N : 0, 0.0));
    std::vector<std::array<double, 9>> Wt(nthreads);
    std::vector<double> Et(nthreads, 0.0);
    par([&](int t, int lo, int hi) {
        NNP p = p0;
        Wt[t].fill(0.0);
        std::vector<double> Fl;
        double* Fp = F ? Ft[t].data() : (Fl.assign(3 * (size_t)N, 0.0), Fl.data());
        Et[t] = compute_force_rows(p, s, Fp, Wt[t].data(), newton, dEdG_out, nullptr, lo, hi);
    });
    double E = 0;
    if (F) for (size_t a = 0; a < 3 * (size_t)N; ++a) F[a] = 0;
    if (W) for (int a = 0; a < 9; ++a) W[a] = 0;
    for (int t = 0; t < nthreads; ++t) {
        E += Et[t];
        if (F) for (size_t a = 0; a < 3 * (size_t)N; ++a) F[a] += Ft[t][a];
        if (W) for (int a = 0; a < 9; ++a) W[a] += Wt[t][a];
    }
    return E;
}
// energy only: NNP::energy (nnp.cpp:436-447) with vacuum energies (nnh.cpp:118-121)
static double compute_energy(NNP& p, Struc& s) {
    double E = 0;
    for (int i = 0; i < s.N; ++i) { NNH& h = p.h[s.type[i]]; E += h.nn.forward(s.symm[i].data()) + h.energy; }
    return E;
}
// u_i = sum_a (dG_i/dx_a) . lam_a  (tangent of the symmetry functions along the field lam)
static void symm_jvp(const NNP& p, const Struc& s, const double* lam, std::vector<std::vector<double>>& u) {
    u.assign(s.N, {});
    for (int i = 0; i < s.N; ++i) {
        const NNH& h = p.h[s.type[i]];
        u[i].assign(h.nInput, 0.0);
        const auto& nl = s.nl[i];
        for (size_t j = 0; j < nl.size(); ++j) {
            const int JJ = s.type[nl[j].j];
            const double* rj = nl[j].r; const double dj = nl[j].d;
            double drj[3]; for (int c = 0; c < 3; ++c) drj[c] = lam[3 * i + c] - lam[3 * nl[j].j + c];
            const double ddj = (rj[0] * drj[0] + rj[1] * drj[1] + rj[2] * drj[2]) / dj;
            const BasisR& br = h.R[JJ];
            for (int m = 0; m < br.size(); ++m) u[i][h.offR[JJ] + m] += br.symmd(dj, m) * ddj;
            for (size_t k = j + 1; k < nl.size(); ++k) {
                const int KK = s.type[nl[k].j];
                const double* rk = nl[k].r; const double dk = nl[k].d;
                double drk[3]; for (int c = 0; c < 3; ++c) drk[c] = lam[3 * i + c] - lam[3 * nl[k].j + c];
                const double ddk = (rk[0] * drk[0] + rk[1] * drk[1] + rk[2] * drk[2]) / dk;
                const double cs = (rj[0] * rk[0] + rj[1] * rk[1] + rj[2] * rk[2]) / (dj * dk);
                const double dcos = (drj[0] * rk[0] + drj[1] * rk[1] + drj[2] * rk[2] + drk[0] * rj[0] + drk[1] * rj[1] + drk[2] * rj[2]) / (dj * dk)
                                    - cs * (ddj / dj + ddk / dk);
                const BasisA& ba = h.A[tri(JJ, KK)];
                const int oA = h.nInputR + h.offA[tri(JJ, KK)];
                for (int m = 0; m < ba.size(); ++m) {
                    double fphi, fe[2];
                    ba.symmd(m, dj, dk, cs, fphi, fe);
                    u[i][oA + m] += fphi * dcos + fe[0] * ddj + fe[1] * ddk;
                }
            }
        }
    }
}

// ---------------------------------------------------------------- Lennard-Jones labels
// pot_lj_cut.cpp:73-90: E = 1/2 sum_i sum_{j in N(i), d<rc} 4 eps (s/d)^6 ((s/d)^6 - 1), unshifted
static double lj(int N, const double* x, const double* R, double eps, double sig, double rcut, double* F) {
    std::vector<std::vector<Neigh>> nl;
    neighbors(N, x, R, rcut, nl);
    double E = 0;
    for (int i = 0; i < 3 * N; ++i) F[i] = 0;
    for (int i = 0; i < N; ++i) for (auto& e : nl[i]) {
        const double du = sig / e.d, du3 = du * du * du, du6 = du3 * du3;
        E += 0.5 * 4.0 * eps * du6 * (du6 - 1.0);
        const double fmag = 24.0 * eps * du6 * (2.0 * du6 - 1.0) / e.d;  // -dE_pair/dd (pair counted once per side)
        for (int c = 0; c < 3; ++c) F[3 * i + c] += fmag * e.r[c] / e.d;
    }
    return E;
}

}  // namespace orc

// ============================================================================================
// C interface (ctypes)
// ============================================================================================
using namespace orc;

static thread_local std::string g_err;
extern "C" {

const char* orc_last_error() { return g_err.c_str(); }

void* orc_load_text(const char* text) {
    try { NNP* p = new NNP(); read_nnp(text, *p); return p; }
    catch (std::exception& e) { g_err = e.what(); return nullptr; }
}
void* orc_load(const char* path) {
    std::ifstream f(path);
    if (!f) { g_err = std::string("cannot open ") + path; return nullptr; }
    std::stringstream ss; ss << f.rdbuf();
    return orc_load_text(ss.str().c_str());
}
void orc_free(void* p) { delete (NNP*)p; }
int orc_ntypes(void* p) { return ((NNP*)p)->ntypes(); }
double orc_rc(void* p) { return ((NNP*)p)->rc; }
int orc_ninput(void* p, int t) { return ((NNP*)p)->h[t].nInput; }
int orc_nparams(void* p) { return ((NNP*)p)->nparams(); }
int orc_nn_size(void* p, int t) { return ((NNP*)p)->h[t].nn.size(); }
int orc_type_index(void* p, const char* name) { auto& m = ((NNP*)p)->index; auto it = m.find(name); return it == m.end() ? -1 : it->second; }
void orc_get_params(void* p, double* out) { int c = 0; for (auto& h : ((NNP*)p)->h) { h.nn.pack(out + c); c += h.nn.size(); } }
void orc_set_params(void* p, const double* in) { int c = 0; for (auto& h : ((NNP*)p)->h) { h.nn.unpack(in + c); c += h.nn.size(); } }

int orc_activate(int neuron, double c, double z, double* a, double* d, double* d2) {
    try { activate(neuron, c, z, *a, *d, *d2); return 0; } catch (std::exception& e) { return -1; }
}
// One network of a loaded potential on one input, for pinning against the reference's own network
// code (ANN::fpbp2 + DODZ::grad + Cost::grad + D2ODZDI::grad, nn.cpp:1391-1409, 1712-2100):
// out = the network output (without the vacuum energy), dodi = dO/dI (nin), grad = dO/dp in the
// packing order (P), d2odpdi = d2O/(dp dI) (P x nin, row-major; NULL: skipped), the latter by the
// forward-over-reverse pass with unit tangents.
int orc_nn_eval(void* pp, int type, const double* inp, double* out, double* dodi, double* grad, double* d2odpdi) {
    try {
        NNP& p = *(NNP*)pp;
        if (type < 0 || type >= p.ntypes()) throw std::invalid_argument("invalid type index");
        ANN& nn = p.h[type].nn;
        const int nin = nn.nin, P = nn.size();
        *out = nn.forward(inp);
        std::vector<double> d;
        nn.dodi(d);
        for (int m = 0; m < nin; ++m) dodi[m] = d[m];
        for (int k = 0; k < P; ++k) grad[k] = 0;
        nn.cost_grad(1.0, grad);
        if (d2odpdi) {
            std::vector<double> u(nin, 0.0), g(P);
            for (int m = 0; m < nin; ++m) {
                u[m] = 1.0;
                std::fill(g.begin(), g.end(), 0.0);
                nn.jvp_grad(u.data(), 0.0, 1.0, g.data());
                for (int k = 0; k < P; ++k) d2odpdi[(size_t)k * nin + m] = g[k];
                u[m] = 0.0;
            }
        }
        return 0;
    } catch (std::exception& e) { g_err = e.what(); return 1; }
}

double orc_fmexp(double x) { return fmexp(x); }
double orc_coscut(double x) { return coscut(x); }
double orc_sincut(double x) { return sincut(x); }
double orc_powint(double x, int n) { return powint(x, n); }
int orc_cutoff(int name, double rc, double dr, double* f, double* g) {
    try { Cutoff c(name, rc); *f = c.f(dr); *g = c.g(dr); return 0; } catch (std::exception& e) { g_err = e.what(); return 1; }
}
int orc_basisR(int cutname, double rc, int name, int n, const double* rs, const double* eta, double dr,
               double* symm, const double* dEdG, double* amp, double* symmd) {
    try {
        BasisR b; b.cut = Cutoff(cutname, rc); b.name = name; b.rs.assign(rs, rs + n); b.eta.assign(eta, eta + n);
        b.symm(dr, symm); *amp = b.force(dr, dEdG);
        for (int i = 0; i < n; ++i) symmd[i] = b.symmd(dr, i);
        return 0;
    } catch (std::exception& e) { g_err = e.what(); return 1; }
}
int orc_basisA(int cutname, double rc, int name, int n, const double* eta, const double* zeta, const int* lambda,
               double dij, double dik, double cs, double* symm, const double* dEdG, double* phi, double* eta2, double* symmd3) {
    try {
        BasisA b; b.cut = Cutoff(cutname, rc); b.name = name; b.eta.assign(eta, eta + n); b.zeta.assign(zeta, zeta + n);
        b.lambda.assign(lambda, lambda + n); b.init();
        b.symm(dij, dik, cs, symm); b.force(dij, dik, cs, *phi, eta2, dEdG);
        for (int i = 0; i < n; ++i) b.symmd(i, dij, dik, cs, symmd3[3 * i], symmd3 + 3 * i + 1);
        return 0;
    } catch (std::exception& e) { g_err = e.what(); return 1; }
}

// neighbour list of one structure; returns the count, or -(count) if cap is too small.
// brute = 1 takes the all-pairs search whatever the cell (the definition the binned search must equal)
long long orc_neighbors(int N, const double* x, const double* R, double rc, long long cap,
                        int* iout, int* jout, int* nout, double* rout, double* dout, int brute) {
    try {
        std::vector<std::vector<Neigh>> nl;
        if (brute) neighbors_brute(N, x, R, rc, nl);
        else neighbors(N, x, R, rc, nl);
        long long cnt = 0;
        for (int i = 0; i < N; ++i) cnt += nl[i].size();
        if (cnt > cap) return -cnt;
        long long c = 0;
        for (int i = 0; i < N; ++i) for (auto& e : nl[i]) {
            iout[c] = i; jout[c] = e.j;
            for (int d = 0; d < 3; ++d) { nout[3 * c + d] = e.n[d]; rout[3 * c + d] = e.r[d]; }
            dout[c] = e.d; ++c;
        }
        return cnt;
    } catch (std::exception& e) { g_err = e.what(); return LLONG_MIN; }
}

// batched E(+F, virial, symmetry functions, dE/dG); structures split over nthreads with the
// thread::Dist block rule (thread/dist.hpp:21-53, nnpce.cpp:228): thread t owns a contiguous block.
// With fewer structures than threads, each structure is split into atom blocks instead.
int orc_compute(void* pp, int nstruc, const long long* off, const double* x, const int* type, const double* cell,
                double* energy, double* forces, double* virial, double* symm, double* dedg, int imax, int newton, int nthreads) {
    NNP* p0 = (NNP*)pp;
    if (nthreads < 1) nthreads = 1;
    if (nthreads > 1 && nstruc < nthreads) {
        try {
            for (int si = 0; si < nstruc; ++si) {
                Struc s; s.N = (int)(off[si + 1] - off[si]);
                s.x = x + 3 * off[si]; s.type = type + off[si]; s.R = cell + 9 * si;
                for (int i = 0; i < s.N; ++i) if (s.type[i] < 0 || s.type[i] >= p0->ntypes()) throw std::invalid_argument("invalid type index");
                if (s.N == 0) { energy[si] = 0; if (virial) for (int a = 0; a < 9; ++a) virial[9 * si + a] = 0; continue; }
                std::vector<std::vector<double>> dE;
                double W[9];
                energy[si] = compute_struc_threaded(*p0, s, forces ? forces + 3 * off[si] : nullptr, W, newton, dedg ? &dE : nullptr, nthreads);
                if (virial) std::memcpy(virial + 9 * si, W, sizeof(W));
                if (symm) for (int i = 0; i < s.N; ++i) { double* row = symm + (size_t)(off[si] + i) * imax; for (int m = 0; m < imax; ++m) row[m] = m < (int)s.symm[i].size() ? s.symm[i][m] : 0.0; }
                if (dedg) for (int i = 0; i < s.N; ++i) { double* row = dedg + (size_t)(off[si] + i) * imax; for (int m = 0; m < imax; ++m) row[m] = m < (int)dE[i].size() ? dE[i][m] : 0.0; }
            }
            return 0;
        } catch (std::exception& e) { g_err = e.what(); return 1; }
    }
    if (nthreads > nstruc) nthreads = nstruc > 0 ? nstruc : 1;
    std::vector<std::string> errs(nthreads);
    auto work = [&](int t) {
        try {
            NNP p = *p0;  // NNP keeps per-call scratch (not reentrant): one copy per thread
            const int q = nstruc / nthreads, r = nstruc % nthreads;
            const int lo = t * q + std::min(t, r), hi = lo + q + (t < r ? 1 : 0);
            for (int si = lo; si < hi; ++si) {
                Struc s; s.N = (int)(off[si + 1] - off[si]);
                s.x = x + 3 * off[si]; s.type = type + off[si]; s.R = cell + 9 * si;
                for (int i = 0; i < s.N; ++i) if (s.type[i] < 0 || s.type[i] >= p.ntypes()) throw std::invalid_argument("invalid type index");
                neighbors(s.N, s.x, s.R, p.rc, s.nl);
                compute_symm(p, s);
                if (symm) for (int i = 0; i < s.N; ++i) { double* row = symm + (size_t)(off[si] + i) * imax; for (int m = 0; m < imax; ++m) row[m] = m < (int)s.symm[i].size() ? s.symm[i][m] : 0.0; }
                if (forces || virial || dedg) {
                    std::vector<double> F(3 * (size_t)s.N);
                    double W[9];
                    std::vector<std::vector<double>> dE;
                    const double E = compute_force(p, s, F.data(), W, newton, dedg ? &dE : nullptr);
                    energy[si] = E;
                    if (forces) std::memcpy(forces + 3 * off[si], F.data(), sizeof(double) * 3 * s.N);
                    if (virial) std::memcpy(virial + 9 * si, W, sizeof(W));
                    if (dedg) for (int i = 0; i < s.N; ++i) { double* row = dedg + (size_t)(off[si] + i) * imax; for (int m = 0; m < imax; ++m) row[m] = m < (int)dE[i].size() ? dE[i][m] : 0.0; }
                } else {
                    energy[si] = compute_energy(p, s);
                }
            }
        } catch (std::exception& e) { errs[t] = e.what(); }
    };
    std::vector<std::thread> th;
    for (int t = 1; t < nthreads; ++t) th.emplace_back(work, t);
    work(0);
    for (auto& tt : th) tt.join();
    for (auto& e : errs) if (!e.empty()) { g_err = e; return 1; }
    return 0;
}

// Energy + force training loss and its gradient w.r.t. all network parameters (reference packing,
// types in NNP order). Energy term restates NNPTEFR::error_cost_o1 with MSE loss and LINEAR
// normalisation (nnptefr2.cpp:1321-1374, averaged over the batch as nnptefr2.cpp:984-995):
//   L_E = wE/S * sum_s 1/2 ((E_s - Eref_s)/N_s)^2
// Force term (nnptef.cpp:1715-1825 intent, all neighbour terms included):
//   L_F = wF/(3 Ntot) * sum_a 1/2 |F_a - Fref_a|^2
// loss3 = {L, L_E, L_F}; grad += dL/dp.
// Energy term of one structure (nnptefr2.cpp:1339-1368) with its normalisation normt
// (nnptefr2.cpp:606-612): loss 1 MSE, 2 MAE, 3 HUBER, 4 ASINH (opt/loss.hpp:18-24; HUBER and ASINH with
// the scale delta, used as 1/delta and delta^2 as nnptefr2.cpp:188-189); norm 0 IDENTITY, 1 LINEAR,
// 2 SQRT, 3 CBRT, 4 LOG (nnptefr2.hpp:119-126). L = the structure's loss, gfac = dL/dE.
static void energy_loss(int loss, int norm, double delta, double dE, double nAtoms, double& L, double& gfac) {
    double normt;
    switch (norm) {
        case 0: normt = 1.0; break;
        case 1: normt = 1.0 / nAtoms; break;
        case 2: normt = 1.0 / std::sqrt(nAtoms); break;
        case 3: normt = 1.0 / std::cbrt(nAtoms); break;
        case 4: normt = 1.0 / (std::log(nAtoms) + 1.0); break;
        default: throw std::invalid_argument("Invalid normalization method.");
    }
    const double dU = dE * normt, deltai = 1.0 / delta, delta2 = delta * delta;
    gfac = normt;
    switch (loss) {
        case 1: L = 0.5 * dU * dU; gfac *= dU; break;
        case 2: L = std::fabs(dU); gfac *= (double)((dU > 0) - (dU < 0)); break;
        case 3: {
            const double arg = dU * deltai, sq = std::sqrt(1.0 + arg * arg);
            L = delta2 * (sq - 1.0); gfac *= dU / sq;
        } break;
        case 4: {
            const double arg = dU * deltai, sq = std::sqrt(1.0 + arg * arg), lg = std::log(arg + sq);
            L = delta2 * (1.0 - sq + arg * lg); gfac *= lg * delta;
        } break;
        default: throw std::invalid_argument("Invalid loss function.");
    }
}

// Structures are split over nthreads with the thread::Dist block rule (each thread its own NNP copy
// and gradient); the per-thread sums are added in thread order, as the reference's MPI_Reduce adds
// the ranks' gradients (nnptefr2.cpp:984).
int orc_train_ex(void* pp, int nstruc, const long long* off, const double* x, const int* type, const double* cell,
                 const double* Eref, const double* Fref, double wE, double wF, int loss, int norm, double delta, double* loss3,
                 double* grad, int nthreads) {
    try {
        NNP& p0 = *(NNP*)pp;
        const int P = p0.nparams();
        std::vector<int> poff(p0.ntypes() + 1, 0);
        for (int t = 0; t < p0.ntypes(); ++t) poff[t + 1] = poff[t] + p0.h[t].nn.size();
        for (int k = 0; k < P; ++k) grad[k] = 0;
        const long long Ntot = off[nstruc];
        if (nthreads < 1) nthreads = 1;
        if (nthreads > nstruc) nthreads = nstruc > 0 ? nstruc : 1;
        std::vector<std::vector<double>> gt(nthreads, std::vector<double>(P, 0.0));
        std::vector<double> LEt(nthreads, 0.0), LFt(nthreads, 0.0);
        std::vector<std::string> errs(nthreads);
        auto work = [&](int th) {
          try {
            NNP p = p0;
            double* g = gt[th].data();
            double LE = 0, LF = 0;
            const int q = nstruc / nthreads, r = nstruc % nthreads;
            const int lo = th * q + std::min(th, r), hi = lo + q + (th < r ? 1 : 0);
            for (int si = lo; si < hi; ++si) {
                Struc s; s.N = (int)(off[si + 1] - off[si]);
                s.x = x + 3 * off[si]; s.type = type + off[si]; s.R = cell + 9 * si;
                neighbors(s.N, s.x, s.R, p.rc, s.nl);
                compute_symm(p, s);
                std::vector<double> F(3 * (size_t)s.N);
                const double E = compute_force(p, s, F.data(), nullptr, 1);
                double Ls, gfac;
                energy_loss(loss, norm, delta, E - Eref[si], (double)s.N, Ls, gfac);
                LE += Ls;
                const double ce = wE / nstruc * gfac;
                std::vector<double> lam(3 * (size_t)s.N);
                for (int a = 0; a < 3 * s.N; ++a) {
                    const double df = F[a] - Fref[3 * off[si] + a];
                    LF += 0.5 * df * df;
                    lam[a] = wF / (3.0 * Ntot) * df;
                }
                std::vector<std::vector<double>> u;
                symm_jvp(p, s, lam.data(), u);
                for (int i = 0; i < s.N; ++i) {
                    const int t = s.type[i];
                    p.h[t].nn.forward(s.symm[i].data());
                    p.h[t].nn.jvp_grad(u[i].data(), ce, -1.0, g + poff[t]);
                }
            }
            LEt[th] = LE; LFt[th] = LF;
          } catch (std::exception& e) { errs[th] = e.what(); }
        };
        std::vector<std::thread> ths;
        for (int th = 1; th < nthreads; ++th) ths.emplace_back(work, th);
        work(0);
        for (auto& tt : ths) tt.join();
        for (auto& e : errs) if (!e.empty()) throw std::runtime_error(e);
        double LE = 0, LF = 0;
        for (int th = 0; th < nthreads; ++th) {
            LE += LEt[th]; LF += LFt[th];
            for (int k = 0; k < P; ++k) grad[k] += gt[th][k];
        }
        LE *= wE / nstruc;
        LF *= wF / (3.0 * Ntot);
        loss3[0] = LE + LF; loss3[1] = LE; loss3[2] = LF;
        return 0;
    } catch (std::exception& e) { g_err = e.what(); return 1; }
}

int orc_train(void* pp, int nstruc, const long long* off, const double* x, const int* type, const double* cell,
              const double* Eref, const double* Fref, double wE, double wF, double* loss3, double* grad) {
    return orc_train_ex(pp, nstruc, off, x, type, cell, Eref, Fref, wE, wF, 1, 1, 1.0, loss3, grad, 1);
}

// NNPTEFR::error_cost_o1 restated literally (energy only, nnptefr2.cpp:1321-1374; MSE, LINEAR norm
// unless given),
// followed by the batch average of nnptefr2.cpp:984-995. Eref excludes vacuum energies, as the
// structure energies the trainer compares against (the network outputs only are summed, 1337).
int orc_error_cost_o1_ex(void* pp, int nstruc, const long long* off, const double* x, const int* type, const double* cell,
                         const double* Eref, int lossf, int norm, double delta, double* loss, double* grad) {
    try {
        NNP& p = *(NNP*)pp;
        const int P = p.nparams();
        std::vector<int> poff(p.ntypes() + 1, 0);
        for (int t = 0; t < p.ntypes(); ++t) poff[t + 1] = poff[t] + p.h[t].nn.size();
        std::vector<double> g(P, 0.0);
        double err = 0;
        for (int si = 0; si < nstruc; ++si) {
            Struc s; s.N = (int)(off[si + 1] - off[si]);
            s.x = x + 3 * off[si]; s.type = type + off[si]; s.R = cell + 9 * si;
            neighbors(s.N, s.x, s.R, p.rc, s.nl);
            compute_symm(p, s);
            std::vector<double> gs(P, 0.0);
            double pe = 0;
            for (int i = 0; i < s.N; ++i) {
                const int t = s.type[i];
                pe += p.h[t].nn.forward(s.symm[i].data());
                p.h[t].nn.cost_grad(1.0, gs.data() + poff[t]);
            }
            double Ls, gfac;
            energy_loss(lossf, norm, delta, pe - Eref[si], (double)s.N, Ls, gfac);
            err += Ls;
            for (int k = 0; k < P; ++k) g[k] += gs[k] * gfac;
        }
        *loss = err / nstruc;
        for (int k = 0; k < P; ++k) grad[k] = g[k] / nstruc;
        return 0;
    } catch (std::exception& e) { g_err = e.what(); return 1; }
}
int orc_error_cost_o1(void* pp, int nstruc, const long long* off, const double* x, const int* type, const double* cell,
                      const double* Eref, double* loss, double* grad) {
    return orc_error_cost_o1_ex(pp, nstruc, off, x, type, cell, Eref, 1, 1, 1.0, loss, grad);
}

// u = J lam for a batch (tangent of the symmetry functions), rows padded to imax
int orc_symm_jvp(void* pp, int nstruc, const long long* off, const double* x, const int* type, const double* cell,
                 const double* lam, double* u, int imax) {
    try {
        NNP& p = *(NNP*)pp;
        for (int si = 0; si < nstruc; ++si) {
            Struc s; s.N = (int)(off[si + 1] - off[si]);
            s.x = x + 3 * off[si]; s.type = type + off[si]; s.R = cell + 9 * si;
            neighbors(s.N, s.x, s.R, p.rc, s.nl);
            std::vector<std::vector<double>> uu;
            symm_jvp(p, s, lam + 3 * off[si], uu);
            for (int i = 0; i < s.N; ++i) { double* row = u + (size_t)(off[si] + i) * imax; for (int m = 0; m < imax; ++m) row[m] = m < (int)uu[i].size() ? uu[i][m] : 0.0; }
        }
        return 0;
    } catch (std::exception& e) { g_err = e.what(); return 1; }
}

double orc_lj(int N, const double* x, const double* R, double eps, double sig, double rcut, double* F) {
    try { return lj(N, x, R, eps, sig, rcut, F); } catch (std::exception& e) { g_err = e.what(); return NAN; }
}

// one velocity-Verlet step (integrator.cpp:177-200; metal units: x in A, v in A/fs, dt in fs,
// m in Da, F in eV/A, so a = F/(m * mvv_to_e) with mvv_to_e = 103.642696526805 eV/(Da A^2/fs^2),
// chem/units.cpp:151). Positions are wrapped back into the cell (Cell::returnToCell).
// F holds the forces of the current positions on entry and of the new positions on exit.
int orc_md_step(void* pp, int N, double* x, double* v, const int* type, const double* R, const double* mass,
                double dt, double* F, double* pe, double* ke) {
    try {
        NNP& p = *(NNP*)pp;
        const double mvv = 103.642696526805;
        double Ri[9]; inv3(R, Ri);
        for (int i = 0; i < N; ++i) {
            const double m = mass[type[i]] * mvv;
            for (int c = 0; c < 3; ++c) { v[3 * i + c] += 0.5 * dt * F[3 * i + c] / m; x[3 * i + c] += v[3 * i + c] * dt; }
            double s[3];
            for (int d = 0; d < 3; ++d) s[d] = Ri[d] * x[3 * i] + Ri[3 + d] * x[3 * i + 1] + Ri[6 + d] * x[3 * i + 2];
            for (int d = 0; d < 3; ++d) s[d] -= std::floor(s[d]);
            for (int c = 0; c < 3; ++c) x[3 * i + c] = R[c] * s[0] + R[3 + c] * s[1] + R[6 + c] * s[2];
        }
        Struc st; st.N = N; st.x = x; st.type = type; st.R = R;
        neighbors(N, x, R, p.rc, st.nl);
        compute_symm(p, st);
        *pe = compute_force(p, st, F, nullptr, 1);
        double k = 0;
        for (int i = 0; i < N; ++i) {
            const double m = mass[type[i]] * mvv;
            for (int c = 0; c < 3; ++c) { v[3 * i + c] += 0.5 * dt * F[3 * i + c] / m; k += mass[type[i]] * v[3 * i + c] * v[3 * i + c]; }
        }
        *ke = 0.5 * k * mvv;
        return 0;
    } catch (std::exception& e) { g_err = e.what(); return 1; }
}

// Input statistics of a training set (nnptefr2.cpp:686-775), per type t over its N_t atoms and per
// input k: max, min, harmonic mean N/sum(1/G), mean, standard deviation sqrt(sum (mean-G)^2 /
// (N-1)) and rms sqrt(sum G^2 / N), each a separate pass over the atoms as in the reference.
// G is natoms x imax (the first nin[t] entries of a row are the atom's inputs).
// out[t * 6 * imax + q * imax + k] for q = max, min, har, avg, dev, rms; count[t] = N_t.
// Deviation kept from the reference: a type with fewer than two atoms gets dev = 0 (the
// reference divides by N-1 = 0).
void orc_input_stats(int ntypes, const int* nin, long long natoms, const int* type, const double* G, int imax, double* out,
                     long long* count) {
    for (int t = 0; t < ntypes; ++t) {
        double* o = out + (size_t)t * 6 * imax;
        for (int k = 0; k < 6 * imax; ++k) o[k] = 0.0;
        for (int k = 0; k < nin[t]; ++k) { o[k] = -DBL_MAX; o[imax + k] = DBL_MAX; }
        count[t] = 0;
    }
    for (long long i = 0; i < natoms; ++i) ++count[type[i]];
    for (long long i = 0; i < natoms; ++i) {                       // max / min (702-713)
        double* o = out + (size_t)type[i] * 6 * imax;
        for (int k = 0; k < nin[type[i]]; ++k) {
            const double g = G[i * imax + k];
            if (g > o[k]) o[k] = g;
            if (g < o[imax + k]) o[imax + k] = g;
        }
    }
    for (long long i = 0; i < natoms; ++i) {                       // harmonic mean (720-730)
        double* o = out + (size_t)type[i] * 6 * imax;
        for (int k = 0; k < nin[type[i]]; ++k) o[2 * imax + k] += 1.0 / G[i * imax + k];
    }
    for (long long i = 0; i < natoms; ++i) {                       // mean (732-740)
        double* o = out + (size_t)type[i] * 6 * imax;
        for (int k = 0; k < nin[type[i]]; ++k) o[3 * imax + k] += G[i * imax + k];
    }
    for (int t = 0; t < ntypes; ++t) {
        double* o = out + (size_t)t * 6 * imax;
        for (int k = 0; k < nin[t]; ++k) { o[2 * imax + k] = count[t] / o[2 * imax + k]; o[3 * imax + k] /= count[t]; }
    }
    for (long long i = 0; i < natoms; ++i) {                       // deviation (742-754), rms (756-766)
        double* o = out + (size_t)type[i] * 6 * imax;
        for (int k = 0; k < nin[type[i]]; ++k) {
            const double d = o[3 * imax + k] - G[i * imax + k];
            o[4 * imax + k] += d * d;
            o[5 * imax + k] += G[i * imax + k] * G[i * imax + k];
        }
    }
    for (int t = 0; t < ntypes; ++t) {
        double* o = out + (size_t)t * 6 * imax;
        for (int k = 0; k < nin[t]; ++k) {
            o[4 * imax + k] = count[t] > 1 ? std::sqrt(o[4 * imax + k] / (count[t] - 1.0)) : 0.0;
            o[5 * imax + k] = std::sqrt(o[5 * imax + k] / count[t]);
        }
    }
}

// Input pre-conditioning from those statistics (nnptefr2.cpp:777-858): inpb by PreBias
// (0 IDENTITY, 1 MEAN, 2 HAR, 3 RMS, 4 MID, 5 MIN; nnptefr2.hpp:87-97) plus inbias, inpw by PreScale
// (0 IDENTITY, 1 DEV, 2 MINMAX, 3 MAX; nnptefr2.hpp:59-67) times inscale. Returns 1 for an enum value
// outside those (the reference's "Invalid input bias." / "Invalid input scaling.").
int orc_precondition(int n, const double* st /* 6 x n rows of one type, row stride imax */, int imax, int prebias,
                     int prescale, double inbias, double inscale, double* inpb, double* inpw) {
    const double *mx = st, *mn = st + imax, *har = st + 2 * imax, *avg = st + 3 * imax, *dev = st + 4 * imax, *rms = st + 5 * imax;
    for (int k = 0; k < n; ++k) {
        switch (prebias) {
            case 0: inpb[k] = 0.0; break;
            case 1: inpb[k] = -1.0 * avg[k]; break;
            case 2: inpb[k] = -1.0 * har[k]; break;
            case 3: inpb[k] = -1.0 * rms[k]; break;
            case 4: inpb[k] = -0.5 * (mx[k] + mn[k]); break;
            case 5: inpb[k] = -1.0 * mn[k]; break;
            default: g_err = "Invalid input bias."; return 1;
        }
        inpb[k] += inbias;
        switch (prescale) {
            case 0: inpw[k] = 1.0; break;
            case 1: inpw[k] = (dev[k] == 0) ? 1.0 : 1.0 / dev[k]; break;
            case 2: { const double s = mx[k] - mn[k]; inpw[k] = (s > 0) ? 1.0 / s : 1.0; } break;
            case 3: inpw[k] = (mx[k] > 0) ? 1.0 / mx[k] : 1.0; break;
            default: g_err = "Invalid input scaling."; return 1;
        }
        inpw[k] *= inscale;
    }
    return 0;
}

// Taylor-perturbed copies of structures with forces (nnptefr2.cpp:2409-2479): every structure is
// kept; one whose mean |F| exceeds 1e-12 gets nadd copies in which each atom j moves by
// dr = vr (sin t cos p, sin t sin p, cos t), cos t and p/pi uniform in [-1, 1)
// (std::uniform_real_distribution), vr from the radial distribution rdist with scale rdelta
// (rand/rng.cpp:64-146: 1 UNIFORM, 2 LAPLACE, 3 NORMAL, 5 SECH, 6 LOGISTIC, 7 COSINE) times
// rcov[j] when given (Perturb::COVALENT), and the energy becomes E - sum_j dr_j . F_j. Draws come
// from one std::mt19937(seed) in the order vr, cos t, p per atom. Writes the new structures'
// atom offsets, positions, energies and source structure when the output pointers are not NULL;
// returns the number of structures (-1 for an unknown distribution).
long long orc_taylor_perturb(int nstruc, const long long* off, const double* x, const double* F, const double* E, int nadd, int rdist,
                             double rdelta, unsigned seed, const double* rcov, long long* out_off, double* out_x, double* out_E,
                             int* out_src) {
    const double PI = 3.14159265358979323846;
    std::mt19937 gen(seed);
    const double gmax = (double)gen.max();
    std::uniform_real_distribution<double> dista(-1.0, 1.0);
    int ncache = 0;
    double cache_y = 0.0;
    auto unit_nonzero = [&]() { double p = 0; while (p == 0) p = (double)gen() / gmax; return p; };
    auto radial = [&]() -> double {
        switch (rdist) {
            case 1: return (double)gen() / gmax * rdelta;
            case 2: { double p = unit_nonzero() - 0.5; const double s = (p > 0) - (p < 0); return -1.0 * rdelta * s * std::log(1.0 - 2.0 * std::fabs(p)); }
            case 3: {
                if (ncache++ % 2 == 0) {
                    const double r1 = unit_nonzero(), r2 = (double)gen() / gmax;
                    const double mag = rdelta * std::sqrt(-2.0 * std::log(r1)), ang = 2.0 * PI * r2;
                    cache_y = mag * std::sin(ang);
                    return mag * std::cos(ang);
                }
                return cache_y;
            }
            case 5: { const double p = unit_nonzero(); return rdelta * 2.0 / PI * std::log(std::tan(0.5 * PI * p)); }
            case 6: { const double p = unit_nonzero(); return rdelta * std::log(p / (1.0 - p)); }
            case 7: {
                const double p = unit_nonzero();
                if (p < 0.5) { const double t = std::sqrt(-2.0 * std::log(p)); return rdelta * (0.820251 - 0.806770 * t + 0.093247 * t * t); }
                const double t = std::sqrt(-2.0 * std::log(1.0 - p));
                return -rdelta * (0.820251 - 0.806770 * t + 0.093247 * t * t);
            }
        }
        return NAN;
    };
    if (rdist != 1 && rdist != 2 && rdist != 3 && rdist != 5 && rdist != 6 && rdist != 7) return -1;
    long long ns = 0, na = 0;
    auto emit = [&](int s, const double* xs, double e) {
        const long long n = off[s + 1] - off[s];
        if (out_off) { out_off[ns] = na; out_off[ns + 1] = na + n; }
        if (out_x) std::memcpy(out_x + 3 * na, xs, sizeof(double) * 3 * n);
        if (out_E) out_E[ns] = e;
        if (out_src) out_src[ns] = s;
        ++ns; na += n;
    };
    std::vector<double> xp;
    for (int s = 0; s < nstruc; ++s) {
        const long long a0 = off[s], n = off[s + 1] - off[s];
        emit(s, x + 3 * a0, E[s]);
        double favg = 0;
        for (long long j = 0; j < n; ++j) {
            const double* f = F + 3 * (a0 + j);
            favg += std::sqrt(f[0] * f[0] + f[1] * f[1] + f[2] * f[2]);
        }
        favg /= n;
        if (!(favg > 1.0e-12)) continue;
        for (int m = 0; m < nadd; ++m) {
            xp.assign(x + 3 * a0, x + 3 * (a0 + n));
            double e = E[s];
            for (long long j = 0; j < n; ++j) {
                double vr = radial();
                if (rcov) vr *= rcov[a0 + j];
                const double ct = dista(gen), st = std::sqrt(1.0 - ct * ct), ph = dista(gen) * PI;
                const double dr[3] = {vr * st * std::cos(ph), vr * st * std::sin(ph), vr * ct};
                const double* f = F + 3 * (a0 + j);
                for (int c = 0; c < 3; ++c) xp[3 * j + c] += dr[c];
                e -= dr[0] * f[0] + dr[1] * f[1] + dr[2] * f[2];
            }
            emit(s, xp.data(), e);
        }
    }
    return ns;
}

}  // extern "C"
