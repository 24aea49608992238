// C entry points over the reference's OWN cutoff / basis / special-function code, compiled from
// the reference sources by oracle/Makefile into oracle/_ref/libref_basis.so.
//
// TEST INFRASTRUCTURE ONLY: tests/ load it to pin the oracle's restatement bit for bit.
// Nothing here is reference source; this file only calls the reference classes
// (nnp/cutoff.hpp, nnp/basis_radial.hpp, nnp/basis_angular.hpp, math/special.hpp).
#include <cstdio>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>
#include "math/special.hpp"
#include "nnp/cutoff.hpp"
#include "nnp/basis_radial.hpp"
#include "nnp/basis_angular.hpp"

static std::string g_err;

extern "C" {

const char* ref_last_error() { return g_err.c_str(); }
double ref_fmexp(double x) { return math::special::fmexp(x); }
double ref_coscut(double x) { return math::special::coscut(x); }
double ref_sincut(double x) { return math::special::sincut(x); }
double ref_powint(double x, int n) { return math::special::powint(x, n); }

int ref_cutoff(int name, double rc, double dr, double* f, double* g) {
    try {
        Cutoff c((Cutoff::Name::Type)name, rc);
        *f = c.cutf(dr); *g = c.cutg(dr);
        return 0;
    } catch (std::exception& e) { g_err = e.what(); return 1; }
}

// BasisR::symm / force / symmd for one distance (basis_radial.cpp:213-376)
int ref_basisR(int cutname, double rc, int name, int n, const double* rs, const double* eta, double dr,
               double* symm, const double* dEdG, double* amp, double* symmd) {
    try {
        BasisR b(rc, (Cutoff::Name::Type)cutname, n, (BasisR::Name::Type)name);
        for (int i = 0; i < n; ++i) { b.rs(i) = rs[i]; b.eta(i) = eta[i]; }
        std::vector<double> dv(2, 0.0); dv[0] = dr;
        b.symm(dv);
        for (int i = 0; i < n; ++i) symm[i] = b.symm()[i];
        *amp = b.force(dv, dEdG);
        for (int i = 0; i < n; ++i) symmd[i] = b.symmd(dr, eta[i], rs[i]);
        return 0;
    } catch (std::exception& e) { g_err = e.what(); return 1; }
}

// BasisA::init / symm / force / symmd for one triple (basis_angular.cpp:178-563)
int ref_basisA(int cutname, double rc, int name, int n, const double* eta, const double* zeta, const int* lambda,
               double dij, double dik, double cs, double* symm, const double* dEdG, double* phi, double* eta2, double* symmd3) {
    try {
        BasisA b(rc, (Cutoff::Name::Type)cutname, n, (BasisA::Name::Type)name);
        for (int i = 0; i < n; ++i) { b.eta(i) = eta[i]; b.zeta(i) = zeta[i]; b.lambda(i) = lambda[i]; }
        b.init();
        std::vector<double> dv(2); dv[0] = dij; dv[1] = dik;
        std::vector<double> cv(1, cs);
        b.symm(dv, cv);
        for (int i = 0; i < n; ++i) symm[i] = b.symm()[i];
        b.force(dv, cv, *phi, eta2, dEdG);
        const double d2[2] = {dij, dik};
        for (int i = 0; i < n; ++i) b.symmd(symmd3[3 * i], symmd3 + 3 * i + 1, cs, d2, eta[i], zeta[i], lambda[i]);
        return 0;
    } catch (std::exception& e) { g_err = e.what(); return 1; }
}

// BasisR::read / BasisA::read of one block from a file (basis_radial.cpp:123-143,
// basis_angular.cpp:116-138); returns the parsed parameters for comparison with other readers.
int ref_read_basisR(const char* path, int* cutname, double* rc, int* name, int* n, double* rs, double* eta, int cap) {
    try {
        FILE* f = fopen(path, "r");
        if (!f) { g_err = "cannot open"; return 1; }
        BasisR b;
        BasisR::read(f, b);
        fclose(f);
        *cutname = (int)b.cutoff().name(); *rc = b.cutoff().rc(); *name = (int)b.name(); *n = b.size();
        for (int i = 0; i < b.size() && i < cap; ++i) { rs[i] = b.rs(i); eta[i] = b.eta(i); }
        return 0;
    } catch (std::exception& e) { g_err = e.what(); return 1; }
}
int ref_read_basisA(const char* path, int* cutname, double* rc, int* name, int* n, double* eta, double* zeta, int* lambda, int* rflag, int cap) {
    try {
        FILE* f = fopen(path, "r");
        if (!f) { g_err = "cannot open"; return 1; }
        BasisA b;
        BasisA::read(f, b);
        fclose(f);
        *cutname = (int)b.cutoff().name(); *rc = b.cutoff().rc(); *name = (int)b.name(); *n = b.size();
        for (int i = 0; i < b.size() && i < cap; ++i) { eta[i] = b.eta(i); zeta[i] = b.zeta(i); lambda[i] = b.lambda(i); rflag[i] = b.rflag(i); }
        return 0;
    } catch (std::exception& e) { g_err = e.what(); return 1; }
}

}  // extern "C"
