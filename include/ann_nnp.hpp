// ann_nnp.hpp -- header-only C++ adapter that keeps the reference's call shapes over the C ABI of
// libann_gpu.so, so nnpce-style and torch-engine-style callers switch by changing one call.
//
//   reference (src/nnp/nnp.hpp:105-122, src/torch/pot_nnpe.hpp:57-63)   this adapter
//   NNP::read(file, nnp)                                                ann::gpu::NNP::read(file, nnp)
//   NNP::compute(nnp, struc, nlist)   (E into struc.pe(), F into force) ann::gpu::NNP::compute(nnp, struc)
//   NNP::energy(nnp, struc)                                             ann::gpu::NNP::energy(nnp, struc)
//   ptnl::PotNNPE::compute(struc, nlist)  (returns E, adds to pe())     ann::gpu::PotNNPE::compute(struc)
//
// StructureT is any type with the reference Structure's accessors used on this path
// (nAtoms(), posn(i)[c], force(i)[c], type(i), R()(r,c), pe()); the neighbour list is built on the
// GPU from the positions and the cell, so the NeighborList argument of the reference calls is
// not needed. Errors throw std::runtime_error carrying the library's message, as the reference
// throws std::runtime_error / std::invalid_argument.
#pragma once
#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "ann_gpu.h"

namespace ann {
namespace gpu {

inline void check(ann_ctx* c, int rc) {
    if (rc != ANN_OK) throw std::runtime_error(std::string("libann_gpu: ") + ann_last_error(c));
}

class NNP {
public:
    explicit NNP(int device = 0, int precision = ANN_FP64) : prec_(precision) {
        ann_options o;
        ann_default_options(&o);
        o.device = device;
        o.precision = precision;
        ann_ctx* c = nullptr;
        check(nullptr, ann_create(&c, &o));
        ctx_ = c;
    }
    ~NNP() { ann_destroy(ctx_); }
    NNP(const NNP&) = delete;
    NNP& operator=(const NNP&) = delete;
    ann_ctx* ctx() const { return ctx_; }
    int index(const char* name) const { int32_t i = -1; check(ctx_, ann_type_index(ctx_, name, &i)); return i; }
    double rc() const { double r = 0; check(ctx_, ann_cutoff(ctx_, &r)); return r; }
    // launch shapes timed on the structures of the last compute call (ann_autotune), kept for the
    // context's later calls; no counterpart in the reference's NNP
    ann_tuning autotune(int precision = -1, int reps = 5) {
        ann_tuning t{};
        check(ctx_, ann_autotune(ctx_, precision < 0 ? prec_ : precision, reps, &t));
        return t;
    }

    static void read(const char* file, NNP& nnp) { check(nnp.ctx_, ann_load_potential(nnp.ctx_, file)); }
    static void write(const char* file, const NNP& nnp) { check(nnp.ctx_, ann_write_potential(nnp.ctx_, file)); }

    // energy (with vacuum energies, NNH::energy) into struc.pe() and forces into struc.force(i)
    template <class StructureT>
    static double compute(NNP& nnp, StructureT& struc, int precision = -1) {
        return run(nnp, struc, true, precision);
    }
    template <class StructureT>
    static double energy(NNP& nnp, const StructureT& struc, int precision = -1) {
        return run(nnp, const_cast<StructureT&>(struc), false, precision);
    }

private:
    template <class StructureT>
    static double run(NNP& nnp, StructureT& struc, bool forces, int precision) {
        const int n = struc.nAtoms();
        std::vector<double> x(3 * (size_t)n), f(forces ? 3 * (size_t)n : 0);
        std::vector<int32_t> t(n);
        for (int i = 0; i < n; ++i) {
            for (int c = 0; c < 3; ++c) x[3 * i + c] = struc.posn(i)[c];
            t[i] = struc.type(i);
        }
        double cell[9];
        for (int c = 0; c < 3; ++c) for (int r = 0; r < 3; ++r) cell[3 * c + r] = struc.R()(r, c);
        const int64_t off[2] = {0, n};
        double e = 0.0;
        check(nnp.ctx_, ann_compute(nnp.ctx_, 1, off, x.data(), t.data(), cell, &e, forces ? f.data() : nullptr, nullptr,
                                    precision < 0 ? nnp.prec_ : precision));
        if (forces) {
            for (int i = 0; i < n; ++i) for (int c = 0; c < 3; ++c) struc.force(i)[c] = f[3 * i + c];
            struc.pe() = e;
        }
        return e;
    }
    ann_ctx* ctx_ = nullptr;
    int prec_ = ANN_FP64;   // precision of calls that do not name one
};

// ptnl::PotNNPE-shaped plugin (torch/pot_nnpe.cpp:169-288): compute() returns the energy, adds it
// to struc.pe() and adds the forces to struc.force(i) (Engine::compute zeroes them first).
class PotNNPE {
public:
    explicit PotNNPE(const char* ann_file, int device = 0, int precision = ANN_MIXED) : nnp_(device, precision), prec_(precision) {
        NNP::read(ann_file, nnp_);
    }
    template <class StructureT>
    double compute(StructureT& struc) {
        const int n = struc.nAtoms();
        std::vector<double> x(3 * (size_t)n), f(3 * (size_t)n);
        std::vector<int32_t> t(n);
        for (int i = 0; i < n; ++i) { for (int c = 0; c < 3; ++c) x[3 * i + c] = struc.posn(i)[c]; t[i] = struc.type(i); }
        double cell[9];
        for (int c = 0; c < 3; ++c) for (int r = 0; r < 3; ++r) cell[3 * c + r] = struc.R()(r, c);
        const int64_t off[2] = {0, n};
        double e = 0.0;
        check(nnp_.ctx(), ann_compute(nnp_.ctx(), 1, off, x.data(), t.data(), cell, &e, f.data(), nullptr, prec_));
        for (int i = 0; i < n; ++i) for (int c = 0; c < 3; ++c) struc.force(i)[c] += f[3 * i + c];
        struc.pe() += e;
        return e;
    }
    NNP& nnp() { return nnp_; }

private:
    NNP nnp_;
    int prec_;
};

}  // namespace gpu
}  // namespace ann
