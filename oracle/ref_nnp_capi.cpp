// C entry points over the reference's OWN potential code (src/nnp/nnp.cpp, nnh.cpp, type.cpp,
// the MD engine's src/torch/pot_nnpe.cpp, and the basis, network and helper sources they call),
// compiled from the reference sources by
// oracle/Makefile, with the stand-ins of ref_shim/ (Eigen, and the struc/ headers that the
// reference's sources include but do not contain), into oracle/_ref/libref_nnp.so.
//
// TEST INFRASTRUCTURE ONLY: tests/golden/make_golden.py and tests/ load it to pin the oracle's
// assembly of symmetry functions, energies and forces. Nothing here is reference source; this
// file fills a Structure and a neighbour list from arrays and calls the reference's NNP::read,
// NNP::write, NNP::init, NNP::symm, NNP::energy, NNP::force and NNP::compute, and the MD engine's
// ptnl::PotNNPE::read and PotNNPE::compute.
#include <iostream>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>
#include "struc/structure.hpp"
#include "struc/neighbor.hpp"
#include "struc/verlet.hpp"
#include "nnp/nnp.hpp"
#include "torch/pot_nnpe.hpp"

static std::string g_err;

// std::cout sent to a discarded buffer while in scope: NNP::compute prints its name on every call
// (nnp.cpp:604)
struct MuteCout {
    std::ostringstream sink;
    std::streambuf* old;
    MuteCout() : old(std::cout.rdbuf(sink.rdbuf())) {}
    ~MuteCout() { std::cout.rdbuf(old); }
};

extern "C" {

const char* ref_nnp_last_error() { return g_err.c_str(); }

// NNP::read of a potential file (nnp.cpp:243-307)
void* ref_nnp_read(const char* path) {
    try {
        NNP* p = new NNP();
        NNP::read(path, *p);
        return p;
    } catch (std::exception& e) { g_err = e.what(); return nullptr; }
}
void ref_nnp_free(void* h) { delete (NNP*)h; }
int ref_nnp_ntypes(void* h) { return ((NNP*)h)->ntypes(); }
int ref_nnp_ninput(void* h, int t) { return ((NNP*)h)->nnh(t).nInput(); }
double ref_nnp_rc(void* h) { return ((NNP*)h)->rc(); }
int ref_nnp_nparams(void* h) { return ((NNP*)h)->size(); }
// NNP::write to a file (nnp.cpp:197-236)
int ref_nnp_write(void* h, const char* path) {
    try {
        NNP::write(path, *(NNP*)h);
        return 0;
    } catch (std::exception& e) { g_err = e.what(); return 1; }
}

}  // extern "C"

// One structure, as the entry points below take it: natoms atoms with the potential's type
// indices `type`, positions `posn` (3 per atom) and lattice vectors as the columns of R
// (column-major, 9 values). Neighbour entry e belongs to centre atom ei[e] and is atom ej[e] seen
// through image img[3e..3e+2] (multiples of the lattice vectors); entries are appended to their
// centre's row in the order given. fill() builds the Structure (type names from `name_of`) and
// both list forms:
//   the NeighborList: this file forms the pair vectors r = (x_i - x_j) - R n and their lengths;
//           newton = 1 gives every entry the Newton's-third-law reaction (min() true), newton = 0
//           only the entries with a zero image;
//   the verlet::List: indices and images; its functions form the pair vectors themselves and
//           give the reaction to zero-image entries only (nnp.cpp:550).
template <typename NameOf>
static void fill(Structure& s, NeighborList& nl, verlet::List& vl, int ntypes, NameOf name_of, int natoms, const int* type,
                 const double* posn, const double* R, int nent, const int* ei, const int* ej, const int* img, int newton) {
    s.resize(natoms);
    for (int c = 0; c < 3; ++c)
        for (int r = 0; r < 3; ++r) s.R()(r, c) = R[3 * c + r];
    for (int i = 0; i < natoms; ++i) {
        if (type[i] < 0 || type[i] >= ntypes) throw std::invalid_argument("type index out of range");
        s.type(i) = type[i];
        s.name(i) = name_of(type[i]);
        for (int d = 0; d < 3; ++d) s.posn(i)[d] = posn[3 * i + d];
    }
    nl.resize(natoms);
    vl.resize(natoms);
    for (int e = 0; e < nent; ++e) {
        const int i = ei[e], j = ej[e];
        if (i < 0 || i >= natoms || j < 0 || j >= natoms) throw std::invalid_argument("neighbour index out of range");
        Eigen::Vector3d n;
        for (int d = 0; d < 3; ++d) n[d] = (double)img[3 * e + d];
        const bool zero = img[3 * e] == 0 && img[3 * e + 1] == 0 && img[3 * e + 2] == 0;
        NeighborEntry x;
        x.type_ = type[j];
        x.index_ = j;
        x.min_ = newton ? true : zero;
        s.diff(s.posn(i), s.posn(j), x.r_);
        x.r_ -= s.R() * n;
        x.dr_ = x.r_.norm();
        nl.add(i, x);
        verlet::Entry y;
        y.index_ = j;
        y.cell_ = n;
        vl.add(i, y);
    }
}

extern "C" {

// NNP's functions on one structure, on the NeighborList (form 0) or the verlet::List (form 1).
// Outputs: symm (natoms rows of `width`, zero-padded) after NNP::symm; energy = NNP::energy
// (networks + vacuum energies); force = NNP::force; pe_compute and force_compute = NNP::compute
// (its energy has no vacuum energies).
int ref_nnp_structure(void* h, int natoms, const int* type, const double* posn, const double* R, int nent, const int* ei,
                      const int* ej, const int* img, int newton, int form, int width, double* symm, double* energy,
                      double* force, double* pe_compute, double* force_compute) {
    try {
        NNP& nnp = *(NNP*)h;
        Structure s;
        NeighborList nl;
        verlet::List vl;
        fill(s, nl, vl, nnp.ntypes(), [&](int t) { return nnp.nnh(t).type().name(); }, natoms, type, posn, R, nent, ei, ej, img,
             newton);
        NNP::init(nnp, s);
        if (form == 0) NNP::symm(nnp, s, nl);
        else NNP::symm(nnp, s, vl);
        for (int i = 0; i < natoms; ++i) {
            const Eigen::VectorXd& g = s.symm(i);
            if (g.size() > width) throw std::invalid_argument("symm width too small");
            for (int k = 0; k < width; ++k) symm[(size_t)i * width + k] = k < g.size() ? g[k] : 0.0;
        }
        *energy = NNP::energy(nnp, s);
        if (form == 0) NNP::force(nnp, s, nl);
        else NNP::force(nnp, s, vl);
        for (int i = 0; i < natoms; ++i)
            for (int d = 0; d < 3; ++d) force[3 * i + d] = s.force(i)[d];
        {
            MuteCout mute;
            if (form == 0) NNP::compute(nnp, s, nl);
            else NNP::compute(nnp, s, vl);
        }
        *pe_compute = s.pe();
        for (int i = 0; i < natoms; ++i)
            for (int d = 0; d < 3; ++d) force_compute[3 * i + d] = s.force(i)[d];
        return 0;
    } catch (std::exception& e) { g_err = e.what(); return 1; }
}

// NNP::symm, NNP::energy and NNP::force on an MD engine's domain: nlocal atoms (the centres)
// followed by ghost atoms up to nall, positions already shifted by their images, and the caller's
// neighbour entries (centre ei[e] < nlocal, neighbour ej[e] < nall), each with the
// Newton's-third-law reaction. Outputs: the energy (networks + vacuum energies of the local atoms)
// and the forces of all nall atoms (ghost forces for the engine's reverse communication).
int ref_nnp_domain(void* h, int nlocal, int nall, const int* type, const double* posn, int nent, const int* ei, const int* ej,
                   double* energy, double* force) {
    try {
        NNP& nnp = *(NNP*)h;
        if (nlocal < 0 || nall < nlocal) throw std::invalid_argument("need 0 <= nlocal <= nall");
        Structure s;
        s.resize(nlocal, nall);
        for (int a = 0; a < nall; ++a) {
            if (type[a] < 0 || type[a] >= nnp.ntypes()) throw std::invalid_argument("type index out of range");
            s.type(a) = type[a];
            s.name(a) = nnp.nnh(type[a]).type().name();
            for (int d = 0; d < 3; ++d) s.posn(a)[d] = posn[3 * a + d];
        }
        NeighborList nl;
        nl.resize(nlocal);
        for (int e = 0; e < nent; ++e) {
            const int i = ei[e], j = ej[e];
            if (i < 0 || i >= nlocal || j < 0 || j >= nall) throw std::invalid_argument("neighbour index out of range");
            NeighborEntry x;
            x.type_ = type[j];
            x.index_ = j;
            x.min_ = true;
            s.diff(s.posn(i), s.posn(j), x.r_);
            x.dr_ = x.r_.norm();
            nl.add(i, x);
        }
        NNP::init(nnp, s);
        NNP::symm(nnp, s, nl);
        *energy = NNP::energy(nnp, s);
        NNP::force(nnp, s, nl);
        for (int a = 0; a < nall; ++a)
            for (int d = 0; d < 3; ++d) force[3 * a + d] = s.force(a)[d];
        return 0;
    } catch (std::exception& e) { g_err = e.what(); return 1; }
}

// ptnl::PotNNPE::read of a potential file (pot_nnpe.cpp:697-768) with the cutoff that the engine's
// "pot" line would set first (the reader refuses a file whose rc differs)
void* ref_potnnpe_read(const char* path, double rc) {
    try {
        ptnl::PotNNPE* p = new ptnl::PotNNPE();
        p->rc() = rc;
        p->rc2() = rc * rc;
        p->read(path);
        return p;
    } catch (std::exception& e) { g_err = e.what(); return nullptr; }
}
void ref_potnnpe_free(void* h) { delete (ptnl::PotNNPE*)h; }

// PotNNPE::compute (pot_nnpe.cpp:169-288), the MD engine's energy and force call, on the
// NeighborList form of the arrays above (forces cleared first; the call adds to them)
int ref_potnnpe_structure(void* h, int natoms, const int* type, const double* posn, const double* R, int nent, const int* ei,
                          const int* ej, const int* img, int newton, double* energy, double* force) {
    try {
        ptnl::PotNNPE& pot = *(ptnl::PotNNPE*)h;
        Structure s;
        NeighborList nl;
        verlet::List vl;
        fill(s, nl, vl, pot.ntypes(), [&](int t) { return pot.nnh(t).type().name(); }, natoms, type, posn, R, nent, ei, ej, img,
             newton);
        for (int i = 0; i < natoms; ++i) s.force(i).setZero();
        s.pe() = 0;
        *energy = pot.compute(s, nl);
        for (int i = 0; i < natoms; ++i)
            for (int d = 0; d < 3; ++d) force[3 * i + d] = s.force(i)[d];
        return 0;
    } catch (std::exception& e) { g_err = e.what(); return 1; }
}

}  // extern "C"
