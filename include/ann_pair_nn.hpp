// ann_pair_nn.hpp -- header-only adapter with the shape of a LAMMPS pair style for the reference's
// potential files: `pair_style nn <rc>` / `pair_coeff * * <ann file> <element per LAMMPS type>`
// (used by the reference at examples/Ar/Ar_md_npt.in:22-23; the pair style's source is not part
// of the reference). It takes the arrays LAMMPS hands a pair style and calls ann_compute_list.
//
//   LAMMPS Pair member                      this adapter
//   settings(narg, arg)  "nn <rc>"          PairNN::settings(rc)        (checked against the file's rc)
//   coeff(narg, arg)     "* * file el..."   PairNN::coeff(file, elements)  ("NULL": type not handled)
//   init_style()                            requires a FULL neighbour list and newton_pair on
//   init_one(i, j)                          PairNN::cutoff()
//   compute(eflag, vflag)                   PairNN::compute(...): adds to f[][], eng_vdwl, virial[6], eatom[]
//
// Ghost atoms get forces (Newton's third law); LAMMPS's reverse communication adds them to their
// owners, so newton_pair must be on. Neighbour indices are masked with `neighmask` (LAMMPS
// NEIGHMASK: the top bits carry special-bond flags). Rows may come from a list with a skin: entries
// beyond the potential's cutoff are ignored on the device. Errors throw std::runtime_error with
// the library's message (LAMMPS pair styles report through error->all, which the caller's
// wrapper does with the message).
#pragma once
#include <cmath>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "ann_nnp.hpp"

namespace ann {
namespace gpu {

class PairNN {
public:
    explicit PairNN(int device = 0, int precision = ANN_MIXED) : nnp_(device, precision), prec_(precision) {}

    // pair_style nn <rc>: the cutoff of the style line; coeff() checks it against the file's
    void settings(double rc) { rc_style_ = rc; }

    // pair_coeff * * <file> <el_1> ... <el_ntypes>: LAMMPS type k (1-based) is element elements[k-1]
    // of the potential, or not handled by this style when the name is "NULL"
    void coeff(const char* file, const std::vector<std::string>& elements) {
        NNP::read(file, nnp_);
        staged_ = false;
        map_.assign(elements.size() + 1, -1);
        for (size_t k = 0; k < elements.size(); ++k)
            if (elements[k] != "NULL") map_[k + 1] = nnp_.index(elements[k].c_str());
        const double rc = nnp_.rc();
        if (rc_style_ > 0.0 && std::fabs(rc_style_ - rc) > 1e-6 * rc)
            throw std::runtime_error("pair_style nn: cutoff " + std::to_string(rc_style_) + " differs from the potential's " +
                                     std::to_string(rc));
    }
    double cutoff() const { return nnp_.rc(); }

    // The body of Pair::compute(eflag, vflag). x[nall][3] and type[nall] (1-based LAMMPS types) of
    // local then ghost atoms; the full list (inum, ilist, numneigh, firstneigh). Adds the forces of
    // all nall atoms to f, and returns the energy of the listed atoms. eng_vdwl (eflag_global),
    // virial[6] (vflag_global: xx yy zz xy xz yz) and eatom[] (eflag_atom, by atom index) are added
    // to when not NULL. list_changed = false (LAMMPS: neighbor->ago != 0) keeps the list, types and
    // ghosts of the previous call on the device and sends only the positions.
    double compute(int inum, const int* ilist, const int* numneigh, int* const* firstneigh, int nall, double* const* x,
                   const int* type, double* const* f, double* eng_vdwl = nullptr, double* virial = nullptr,
                   double* eatom = nullptr, int neighmask = 0x1FFFFFFF, bool list_changed = true) {
        if (map_.empty()) throw std::runtime_error("pair_style nn: pair_coeff has not been set");
        xs_.resize(3 * (size_t)nall);
        for (int i = 0; i < nall; ++i)
            for (int c = 0; c < 3; ++c) xs_[3 * (size_t)i + c] = x[i][c];
        const bool keep = !list_changed && staged_ && nall == staged_nall_;
        if (!keep) stage_rows(inum, ilist, numneigh, firstneigh, nall, type, neighmask);
        fs_.assign(3 * (size_t)nall, 0.0);
        ea_.assign(rows_.size(), 0.0);
        double e = 0.0, W[9];
        check(nnp_.ctx(), ann_compute_list(nnp_.ctx(), (int32_t)rows_.size(), keep ? nullptr : rows_.data(), keep ? nullptr : nn_.data(),
                                           keep ? nullptr : neigh_.data(), nall, xs_.data(), keep ? nullptr : ts_.data(), &e,
                                           eatom ? ea_.data() : nullptr, fs_.data(), virial ? W : nullptr, prec_,
                                           keep ? ANN_LIST_KEEP : 0));
        staged_ = true;
        staged_nall_ = nall;
        for (int i = 0; i < nall; ++i) for (int c = 0; c < 3; ++c) f[i][c] += fs_[3 * (size_t)i + c];
        if (eng_vdwl) *eng_vdwl += e;
        if (virial) {
            virial[0] += W[0]; virial[1] += W[4]; virial[2] += W[8];
            virial[3] += W[1]; virial[4] += W[2]; virial[5] += W[5];
        }
        if (eatom) for (size_t r = 0; r < rows_.size(); ++r) eatom[rows_[r]] += ea_[r];
        return e;
    }
    NNP& nnp() { return nnp_; }

private:
    // the rows of the handled centre atoms, without neighbours of types this style does not handle
    void stage_rows(int inum, const int* ilist, const int* numneigh, int* const* firstneigh, int nall, const int* type,
                    int neighmask) {
        ts_.resize(nall);
        for (int i = 0; i < nall; ++i) {
            const int t = type[i];
            ts_[i] = (t > 0 && t < (int)map_.size()) ? map_[t] : -1;
        }
        rows_.clear(); nn_.clear(); neigh_.clear();
        for (int ii = 0; ii < inum; ++ii) {
            const int i = ilist[ii];
            if (ts_[i] < 0) continue;
            int cnt = 0;
            for (int k = 0; k < numneigh[i]; ++k) {
                const int j = firstneigh[i][k] & neighmask;
                if (j >= 0 && j < nall && ts_[j] < 0) continue;
                neigh_.push_back(j);   // an index outside [0, nall) is reported by the library
                ++cnt;
            }
            rows_.push_back(i);
            nn_.push_back(cnt);
        }
        for (int i = 0; i < nall; ++i) if (ts_[i] < 0) ts_[i] = 0;   // never referenced by a row
    }
    NNP nnp_;
    int prec_;
    double rc_style_ = 0.0;
    bool staged_ = false;                        // a list of a previous call is on the device
    int staged_nall_ = 0;
    std::vector<int> map_;                       // LAMMPS type -> potential type (-1: not handled)
    std::vector<double> xs_, fs_, ea_;
    std::vector<int32_t> ts_, rows_, nn_, neigh_;
};

}  // namespace gpu
}  // namespace ann
